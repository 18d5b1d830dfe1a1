"""Host-side logic of the solvers that needs no GPU: splitting a psi-sized
RIGHT source q[(g Nw + a) Ndof + i] into its per-cell isotropic part, and the
restarted, flexibly preconditioned GMRES (Givens rotations, classical
Gram-Schmidt twice) on small dense systems held in CPU tensors."""
from types import SimpleNamespace

import pytest

torch = pytest.importorskip("torch")

from allium_gb300.solvers import split_isotropic


def _iso(G, Nw, ndof, seed=0):
    g = torch.Generator().manual_seed(seed)
    cell = torch.rand((G, 1, ndof), generator=g, dtype=torch.float64)
    return cell, cell.expand(G, Nw, ndof).contiguous().reshape(-1)


def test_isotropic_source_is_split():
    L = SimpleNamespace(G=2, Nw=5, ndof=7)
    cell, q = _iso(2, 5, 7)
    q_iso, rest = split_isotropic(L, q)
    assert rest is None
    assert torch.equal(q_iso, cell.reshape(-1))


@pytest.mark.parametrize("where", [0, 17, 69])
def test_one_direction_differs(where):
    L = SimpleNamespace(G=2, Nw=5, ndof=7)
    _, q = _iso(2, 5, 7, seed=1)
    q[where] += 1e-12
    q_iso, rest = split_isotropic(L, q)
    assert q_iso is None and rest is q


def test_nan_is_not_isotropic():
    L = SimpleNamespace(G=1, Nw=3, ndof=2)
    q = torch.full((6,), float("nan"), dtype=torch.float64)
    q_iso, rest = split_isotropic(L, q)
    assert q_iso is None and rest is q


# ---- restarted, flexibly preconditioned GMRES on small dense systems (CPU tensors)
from allium_gb300.solvers import gmres  # noqa: E402


def _system(n=60, seed=3, scale=None):
    g = torch.Generator().manual_seed(seed)
    A = torch.eye(n, dtype=torch.float64) * 4.0 + torch.randn((n, n), generator=g, dtype=torch.float64) / n ** 0.5
    if scale is not None:
        A = A * scale[:, None]
    b = torch.randn(n, generator=g, dtype=torch.float64)
    return A, b


def _apply(A):
    def f(v, out):
        torch.mv(A, v, out=out)
        return out
    return f


@pytest.mark.parametrize("restart", [5, 60])
def test_gmres_solves_dense_system(restart):
    A, b = _system()
    x, it, hist = gmres(_apply(A), b, tol=1e-12, restart=restart, maxiter=400)
    ref = torch.linalg.solve(A, b)
    assert float(torch.linalg.norm(b - A @ x) / torch.linalg.norm(b)) <= 1e-12
    assert float(torch.max(torch.abs(x - ref))) < 1e-10 * float(torch.max(torch.abs(ref)))
    assert hist[-1] <= 1e-12 and it <= 400


def test_gmres_right_preconditioner_cuts_iterations():
    n = 80
    scale = torch.logspace(0, 4, n, dtype=torch.float64)
    A, b = _system(n, seed=5, scale=scale)
    d = torch.diagonal(A).clone()

    def prec(v, out):
        torch.div(v, d, out=out)
        return out
    x0, it0, _ = gmres(_apply(A), b, tol=1e-10, restart=80, maxiter=400)
    x1, it1, _ = gmres(_apply(A), b, tol=1e-10, restart=80, maxiter=400, prec=prec)
    assert float(torch.linalg.norm(b - A @ x1) / torch.linalg.norm(b)) <= 1e-10
    assert it1 < it0


def test_gmres_initial_guess_and_zero_rhs():
    A, b = _system(40, seed=7)
    ref = torch.linalg.solve(A, b)
    x, it, hist = gmres(_apply(A), b, x0=ref.clone(), tol=1e-10)
    assert it == 0 and hist[0] <= 1e-10
    x, it, hist = gmres(_apply(A), torch.zeros(40, dtype=torch.float64), tol=1e-10)
    assert it == 0 and hist == [0.0] and float(torch.max(torch.abs(x))) == 0.0


def test_gmres_reduce_hook_on_one_shard_matches():
    """reduce(t) sums partial inner products over the shards of a distributed
    vector; with a single shard it is the identity and the iterates agree."""
    A, b = _system(50, seed=9)
    x0, it0, h0 = gmres(_apply(A), b, tol=1e-11, restart=10, maxiter=300)
    x1, it1, h1 = gmres(_apply(A), b, tol=1e-11, restart=10, maxiter=300, reduce=lambda t: None)
    assert it0 == it1
    assert float(torch.max(torch.abs(x0 - x1))) < 1e-12 * float(torch.max(torch.abs(x0)))


def test_gmres_without_final_residual_ends_on_the_estimate():
    A, b = _system(50, seed=11)
    x, it, hist = gmres(_apply(A), b, tol=1e-6, restart=50, final_residual=False)
    # the Arnoldi estimate met the tolerance; the true residual agrees with it to rounding
    assert hist[-1] <= 1e-6
    assert float(torch.linalg.norm(b - A @ x) / torch.linalg.norm(b)) <= 1.01e-6
