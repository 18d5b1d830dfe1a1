"""Device-agnostic sparse products of the DSA V-cycle setup, run here on CPU
tensors against scipy: the expand-sort-reduce SpGEMM, transpose, diagonal, and
the smoothed-aggregation hierarchy against the same algorithm written with
scipy products (same aggregates)."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from allium_gb300.dsa import SparseCOO, _pair_aggregates, smoothed_aggregation_levels


def to_coo(M):
    M = sp.coo_matrix(M)
    return SparseCOO.coalesce(torch.from_numpy(M.row.astype(np.int64)), torch.from_numpy(M.col.astype(np.int64)),
                              torch.from_numpy(M.data), M.shape)


def to_scipy(A):
    return sp.csr_matrix((A.val.numpy(), (A.row.numpy(), A.col.numpy())), shape=A.shape)


def close(A, M, rtol=1e-13):
    D = (to_scipy(A) - sp.csr_matrix(M)).toarray()
    return np.max(np.abs(D)) <= rtol * max(1.0, np.max(np.abs(sp.csr_matrix(M).toarray())))


def laplacian(nx, ny, shift=1e-2):
    def lap1(m):
        return sp.diags([-np.ones(m - 1), 2 * np.ones(m), -np.ones(m - 1)], [-1, 0, 1])
    A = sp.kron(sp.eye(ny), lap1(nx)) + sp.kron(lap1(ny), sp.eye(nx)) + shift * sp.eye(nx * ny)
    return A.tocsr()


def test_spgemm_transpose_diagonal():
    rng = np.random.default_rng(4)
    A = sp.random(60, 45, density=0.08, random_state=1, format="csr")
    B = sp.random(45, 70, density=0.1, random_state=2, format="csr")
    # duplicates summed by coalesce
    r = np.concatenate([A.tocoo().row, A.tocoo().row])
    c = np.concatenate([A.tocoo().col, A.tocoo().col])
    v = np.concatenate([A.tocoo().data, A.tocoo().data])
    A2 = SparseCOO.coalesce(torch.from_numpy(r.astype(np.int64)), torch.from_numpy(c.astype(np.int64)),
                            torch.from_numpy(v), A.shape)
    assert close(A2, 2 * A)
    assert close(to_coo(A).matmul(to_coo(B)), A @ B)
    assert close(to_coo(A).transpose(), A.T)
    S = sp.random(50, 50, density=0.1, random_state=3) + sp.diags(rng.random(50))
    assert np.allclose(to_coo(S).diagonal().numpy(), S.diagonal(), rtol=0, atol=1e-15)
    assert to_coo(A).spmv_csr("cpu")[0].numpy().tolist() == A.indptr.tolist()


def test_smoothed_aggregation_matches_scipy():
    A = laplacian(37, 29)
    levels = smoothed_aggregation_levels(to_coo(A), coarse=60)
    assert len(levels) >= 3 and levels[-1]["A"].shape[0] <= 60
    M = A
    for lvl in levels[:-1]:
        assert close(lvl["A"], M, rtol=1e-12)
        # the same step with scipy products and the aggregates of the level's own
        # operator (roundoff-level differences could flip a greedy pairing tie)
        agg, nagg = _pair_aggregates(lvl["A"])
        agg = agg.numpy()
        T = sp.csr_matrix((np.ones(M.shape[0]), (np.arange(M.shape[0]), agg)), shape=(M.shape[0], nagg))
        Dinv = sp.diags(1.0 / M.diagonal())
        lam = float(np.max(np.asarray(abs(Dinv @ M).sum(axis=1)).ravel()))
        P = (T - (4.0 / 3.0 / lam) * (Dinv @ (M @ T))).tocsr()
        assert close(lvl["P"], P, rtol=1e-12)
        assert close(lvl["R"], P.T, rtol=1e-12)
        assert np.allclose(lvl["dinv"].numpy(), 1.0 / M.diagonal(), rtol=1e-14)
        M = (P.T @ M @ P).tocsr()
    assert close(levels[-1]["A"], M, rtol=1e-11)
    # aggregates of up to four rows, every row in one
    agg, nagg = _pair_aggregates(to_coo(A))
    counts = np.bincount(agg.numpy(), minlength=nagg)
    assert counts.min() >= 1 and counts.max() <= 4
