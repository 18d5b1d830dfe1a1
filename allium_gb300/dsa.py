"""Diffusion synthetic acceleration with the GPU MIP diffusion operator.

MIPDiffusion wraps the C ABI's MIP operator K (InteriorPenaltyDiscretization,
src/moment_discretization.cpp:73-110) and solves K x = b by preconditioned
conjugate gradients: allium applies CG with hypre's BoomerAMG; here the
preconditioner is AggregationVCycle (block-Jacobi smoothing on the DG level,
the continuous vertex space and smoothed aggregation below it, all built and
applied on the device) or plain block-Jacobi (the inverted cell blocks K_ee).  DSAPreconditioner is DiffusionSyntheticAccelerationOperator
(src/transport_op.hpp:38-59): y = x + K^{-1} (M_s x), M_s the within-group
scattering mass, for source iteration and as the right preconditioner of GMRES
on T phi = phi - D L^{-1} D^T M_s phi.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check


def _p(t):
    return C.c_void_p(t.data_ptr())


class MIPDiffusion:
    def __init__(self, Linv, sigma_s, kappa=-1.0, penalty_min=-1.0, alpha_bdr=-1.0, tau=0.0):
        self.L = Linv
        self.G, self.ndof = Linv.G, Linv.ndof
        sig = np.ascontiguousarray(sigma_s, dtype=np.float64).reshape(self.G, -1)
        self.sigma_s = sig
        check(_lib.lib().allium_sweep_dsa_setup(Linv.h, sig.ctypes.data, float(kappa), float(penalty_min),
                                                float(alpha_bdr), float(tau)), Linv.h)
        dev = torch.device("cuda")
        self.sig_dev = torch.from_numpy(sig).to(dev)
        n = Linv.n
        self.n = n
        self.cg_iterations = 0

    def apply(self, x, y):
        check(_lib.lib().allium_sweep_dsa_apply(self.L.h, _p(x), _p(y)), self.L.h)
        return y

    def use_vcycle(self, on=True, **kw):
        """Precondition the diffusion CG with AggregationVCycle instead of block-Jacobi."""
        self.vcycle = AggregationVCycle(self, **kw) if on else None

    def _prec(self, r):
        if getattr(self, "vcycle", None) is not None:
            return self.vcycle(r)
        z = torch.empty_like(r)
        return self.jacobi(r, z)

    def jacobi(self, x, y):
        check(_lib.lib().allium_sweep_dsa_jacobi(self.L.h, _p(x), _p(y)), self.L.h)
        return y

    def blocks(self):
        nface = 2 * self.L.dim
        out = np.empty(self.G * self.L.mesh.num_elements * (1 + nface) * self.n * self.n)
        check(_lib.lib().allium_sweep_dsa_blocks(self.L.h, out.ctypes.data), self.L.h)
        return out.reshape(self.G, self.L.mesh.num_elements, 1 + nface, self.n, self.n)

    def scattering_mass(self, x, y):
        """y = M_s x per group (MassIntegrator(sigma_s), the mass of the scattering source)."""
        L = _lib.lib()
        Nd = self.ndof
        for g in range(self.G):
            check(L.allium_sweep_block_apply(self.L.h, None, 2, C.c_void_p(x.data_ptr() + 8 * g * Nd), 0,
                                             C.c_void_p(y.data_ptr() + 8 * g * Nd), 1.0, 0), self.L.h)
        y.view(self.G, -1, self.n).mul_(self.sig_dev.view(self.G, -1, 1))
        return y

    def solve(self, b, tol=1e-10, maxiter=200):
        """PCG on K x = b (x = 0 start) with the V-cycle when one is set
        (use_vcycle), block-Jacobi otherwise; returns x."""
        x = torch.zeros_like(b)
        r = b.clone()
        z = self._prec(r)
        p = z.clone()
        q = torch.empty_like(b)
        rz = torch.dot(r, z)
        bn = torch.linalg.norm(b).item()
        if bn == 0.0:
            return x
        it = 0
        while it < maxiter:
            self.apply(p, q)
            alpha = rz / torch.dot(p, q)
            x.add_(alpha * p)
            r.sub_(alpha * q)
            it += 1
            if torch.linalg.norm(r).item() <= tol * bn:
                break
            z = self._prec(r)
            rz_new = torch.dot(r, z)
            p.mul_(rz_new / rz).add_(z)
            rz = rz_new
        self.cg_iterations += it
        return x


class DSAPreconditioner:
    """y = x + K^{-1} M_s x (DiffusionSyntheticAccelerationOperator::Mult)."""

    def __init__(self, Linv, sigma_s, cg_tol=1e-10, cg_maxiter=200, vcycle=False, **kw):
        self.K = MIPDiffusion(Linv, sigma_s, **kw)
        if vcycle:
            self.K.use_vcycle()
        self.cg_tol, self.cg_maxiter = cg_tol, cg_maxiter
        self.tmp = None
        self.applications = 0

    def __call__(self, x, out):
        if self.tmp is None or self.tmp.numel() != x.numel():
            self.tmp = torch.empty_like(x)
        self.K.scattering_mass(x, self.tmp)
        d = self.K.solve(self.tmp, tol=self.cg_tol, maxiter=self.cg_maxiter)
        torch.add(x, d, out=out)
        self.applications += 1
        return out


def _csr_spmv(rowptr, col, val, x, y, alpha=1.0, beta=0.0):
    _lib.lib().allium_csr_spmv(int(rowptr.numel() - 1), _p(rowptr), _p(col), _p(val), _p(x), _p(y), float(alpha),
                               float(beta), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return y


class SparseCOO:
    """Sparse matrix as (row, col, val) tensors sorted by (row, col), no
    duplicates, on any torch device; products and sums by expand-sort-reduce."""

    def __init__(self, row, col, val, shape):
        self.row, self.col, self.val, self.shape = row, col, val, (int(shape[0]), int(shape[1]))

    @staticmethod
    def coalesce(row, col, val, shape):
        """Sum the entries that share (row, col)."""
        ncols = int(shape[1])
        keys = row.to(torch.int64) * ncols + col.to(torch.int64)
        uk, inv = torch.unique(keys, return_inverse=True)
        acc = torch.zeros(uk.numel(), dtype=val.dtype, device=val.device).index_add_(0, inv, val)
        return SparseCOO(uk // ncols, uk % ncols, acc, shape)

    def rowptr(self):
        counts = torch.bincount(self.row, minlength=self.shape[0])
        return torch.cat([torch.zeros(1, dtype=torch.int64, device=counts.device), torch.cumsum(counts, 0)])

    def transpose(self):
        return SparseCOO.coalesce(self.col, self.row, self.val, (self.shape[1], self.shape[0]))

    def diagonal(self):
        on = self.row == self.col
        return torch.zeros(self.shape[0], dtype=self.val.dtype, device=self.val.device).index_add_(
            0, self.row[on], self.val[on])

    def matmul(self, B):
        """self @ B: every product a_ik b_kj, then summed per (i, j)."""
        bptr = B.rowptr()
        start = bptr[self.col]
        cnt = bptr[self.col + 1] - start
        which = torch.repeat_interleave(torch.arange(self.col.numel(), device=cnt.device), cnt)
        first = torch.cumsum(cnt, 0) - cnt
        bidx = start[which] + (torch.arange(which.numel(), device=cnt.device) - first[which])
        return SparseCOO.coalesce(self.row[which], B.col[bidx], self.val[which] * B.val[bidx],
                                  (self.shape[0], B.shape[1]))

    def spmv_csr(self, dev):
        """(rowptr, col, val, nrows) with int32 indices for allium_csr_spmv."""
        return (self.rowptr().to(torch.int32).to(dev), self.col.to(torch.int32).to(dev),
                self.val.to(torch.float64).to(dev), self.shape[0])

    def to_dense(self):
        out = torch.zeros(self.shape, dtype=self.val.dtype, device=self.val.device)
        out[self.row, self.col] = self.val
        return out


def _pairs(A):
    """One round of greedy pairwise matching (allium_pair_aggregates) on a host
    copy of A; returns (aggregate of every row, count)."""
    rp = np.ascontiguousarray(A.rowptr().cpu().numpy(), dtype=np.int32)
    cl = np.ascontiguousarray(A.col.cpu().numpy(), dtype=np.int32)
    vl = np.ascontiguousarray(A.val.cpu().numpy(), dtype=np.float64)
    agg = np.empty(A.shape[0], dtype=np.int32)
    nagg = _lib.lib().allium_pair_aggregates(A.shape[0], rp.ctypes.data, cl.ctypes.data, vl.ctypes.data,
                                             agg.ctypes.data)
    return torch.from_numpy(agg.astype(np.int64)).to(A.row.device), nagg


def _pair_aggregates(A):
    """Two rounds of greedy pairwise aggregation: aggregates of up to four
    rows; returns (aggregate of every row, count)."""
    a1, n1 = _pairs(A)
    A1 = SparseCOO.coalesce(a1[A.row], a1[A.col], A.val, (n1, n1))   # T1^T A T1
    a2, n2 = _pairs(A1)
    return a2[a1], n2


def smoothed_aggregation_levels(A, coarse=400):
    """Levels of the smoothed-aggregation hierarchy below the vertex operator
    A (a SparseCOO): per level the operator, its inverse diagonal and, except
    for the last, the prolongator P = (I - 4/(3 lam) D^-1 A) T (T the
    aggregate indicator, lam the largest absolute row sum of D^-1 A) and
    R = P^T; the next operator is R A P.  The last level keeps the operator
    for a dense solve."""
    levels = []
    while True:
        d = A.diagonal()
        lvl = {"A": A, "dinv": 1.0 / d}
        levels.append(lvl)
        if A.shape[0] <= coarse:
            break
        agg, nagg = _pair_aggregates(A)
        n = A.shape[0]
        rowsum = torch.zeros(n, dtype=A.val.dtype, device=A.val.device).index_add_(0, A.row, A.val.abs())
        lam = float((rowsum / d.abs()).max())
        AT = SparseCOO.coalesce(A.row, agg[A.col], A.val, (n, nagg))
        w = 4.0 / 3.0 / lam
        ar = torch.arange(n, device=A.row.device)
        P = SparseCOO.coalesce(torch.cat([ar, AT.row]), torch.cat([agg, AT.col]),
                               torch.cat([torch.ones(n, dtype=A.val.dtype, device=A.val.device),
                                          -w * AT.val / d[AT.row]]), (n, nagg))
        R = P.transpose()
        lvl["P"], lvl["R"] = P, R
        A = R.matmul(A.matmul(P))
    return levels


def _gll_nodes(p):
    """Gauss-Lobatto nodes on [0, 1] (the sweep's L2 basis nodes), p <= 3."""
    if p == 0:
        return np.array([0.5])
    if p == 1:
        return np.array([0.0, 1.0])
    if p == 2:
        return np.array([0.0, 0.5, 1.0])
    r = 1.0 / np.sqrt(5.0)
    return np.array([0.0, 0.5 * (1 - r), 0.5 * (1 + r), 1.0])


def _corner_weights(dim, order):
    """W[i][c]: multilinear corner shape c at DG node i (lexicographic nodes)."""
    x = _gll_nodes(order)
    n1 = order + 1
    n = n1 ** dim
    W = np.empty((n, 1 << dim))
    for i in range(n):
        idx = [(i // n1 ** d) % n1 for d in range(dim)]
        for c in range(1 << dim):
            w = 1.0
            for d in range(dim):
                t = x[idx[d]]
                w *= t if (c >> d) & 1 else 1.0 - t
            W[i, c] = w
    return W


_CORNER_TO_MFEM = {1: [0, 1], 2: [0, 1, 3, 2], 3: [0, 1, 3, 2, 4, 5, 7, 6]}


def _vertex_prolongation(mesh, order, G, dev):
    """P (a SparseCOO on dev): continuous multilinear vertex values -> DG nodal
    values, for G independent groups (rows g * Ndof + e * n + i, columns
    g * Nv + v)."""
    dim = mesh.dim
    W = torch.from_numpy(_corner_weights(dim, order)).to(dev)      # [n][corners]
    n, nc = W.shape
    ne, nv = mesh.num_elements, mesh.num_vertices
    verts = torch.from_numpy(mesh.elements[:, _CORNER_TO_MFEM[dim]].astype(np.int64)).to(dev)
    rows = (torch.arange(ne, device=dev)[:, None, None] * n + torch.arange(n, device=dev)[None, :, None]).expand(ne, n, nc)
    cols = verts[:, None, :].expand(ne, n, nc)
    vals = W[None, :, :].expand(ne, n, nc)
    keep = vals != 0.0
    r, c, v = rows[keep], cols[keep], vals[keep]
    return SparseCOO.coalesce(torch.cat([r + g * ne * n for g in range(G)]), torch.cat([c + g * nv for g in range(G)]),
                              v.repeat(G), (G * ne * n, G * nv))


class AggregationVCycle:
    """Symmetric V-cycle preconditioner for K, standing in for BoomerAMG:
    damped block-Jacobi smoothing on the DG level; below it the continuous
    multilinear (vertex) space, K_v = P^T K P with P the interpolation of
    vertex values at the DG nodes; below that smoothed aggregation (aggregates
    of up to four strongly coupled vertices, Jacobi-smoothed tentative
    prolongator, damped Jacobi smoothing) down to a dense solve.  Built on the
    device from K's blocks once per operator (the greedy pairing runs on a
    host copy of each level), applied on the device."""

    def __init__(self, mip, omega0=0.7, omega=0.67, coarse=400):
        self.mip, self.omega0, self.omega = mip, omega0, omega
        L = mip.L
        G, ne, n, nd = mip.G, L.mesh.num_elements, mip.n, 2 * L.dim
        nbr = np.empty(ne * nd, dtype=np.int32)
        check(_lib.lib().allium_sweep_neighbours(L.h, nbr.ctypes.data), L.h)
        nbr = nbr.reshape(ne, nd)
        dev = torch.device("cuda")
        # K_v = P^T K P from K's blocks on the device: every block B (self or
        # face neighbour) contributes W^T B W between the two cells' vertices
        W = torch.from_numpy(_corner_weights(L.dim, L.order)).to(dev)
        nc = W.shape[1]
        nv = L.mesh.num_vertices
        B = torch.empty((G, ne, 1 + nd, n, n), dtype=torch.float64, device=dev)
        check(_lib.lib().allium_sweep_dsa_blocks(L.h, _p(B)), L.h)
        Cb = torch.einsum("ia,gesij,jb->gesab", W, B, W)            # [G][Ne][1+nd][nc][nc]
        del B
        verts = torch.from_numpy(L.mesh.elements[:, _CORNER_TO_MFEM[L.dim]].astype(np.int64)).to(dev)
        other = torch.from_numpy(np.concatenate([np.arange(ne)[:, None], nbr], axis=1).astype(np.int64)).to(dev)
        valid = other >= 0                                           # [Ne][1+nd]
        rv = verts[:, None, :, None].expand(ne, 1 + nd, nc, nc)
        cv = verts[other.clamp(min=0)][:, :, None, :].expand(ne, 1 + nd, nc, nc)
        m = valid[:, :, None, None].expand(ne, 1 + nd, nc, nc)
        rows_l, cols_l, vals_l = [], [], []
        for g in range(G):
            rows_l.append(rv[m] + g * nv)
            cols_l.append(cv[m] + g * nv)
            vals_l.append(Cb[g][m])
        del Cb
        A = SparseCOO.coalesce(torch.cat(rows_l), torch.cat(cols_l), torch.cat(vals_l), (G * nv, G * nv))
        Pv = _vertex_prolongation(L.mesh, L.order, G, dev)
        self.P0, self.R0 = Pv.spmv_csr(dev), Pv.transpose().spmv_csr(dev)
        self.levels = []
        for lv in smoothed_aggregation_levels(A, coarse):
            lvl = {"A": lv["A"].spmv_csr(dev), "dinv": lv["dinv"], "n": lv["A"].shape[0]}
            if "P" in lv:
                lvl["P"], lvl["R"] = lv["P"].spmv_csr(dev), lv["R"].spmv_csr(dev)
            else:
                lvl["inv"] = torch.from_numpy(np.linalg.inv(lv["A"].to_dense().cpu().numpy())).to(dev)
            self.levels.append(lvl)

    @staticmethod
    def _mv(M, x, out=None, alpha=1.0, beta=0.0):
        rp, cl, vl, nrows = M
        if out is None:
            out = torch.empty(nrows, dtype=x.dtype, device=x.device)
        return _csr_spmv(rp, cl, vl, x, out, alpha, beta)

    def _scalar(self, l, r):
        lvl = self.levels[l]
        if "inv" in lvl:
            return torch.mv(lvl["inv"], r)
        x = self.omega * lvl["dinv"] * r
        res = r.clone()
        self._mv(lvl["A"], x, res, -1.0, 1.0)
        x += self._mv(lvl["P"], self._scalar(l + 1, self._mv(lvl["R"], res)))
        res.copy_(r)
        self._mv(lvl["A"], x, res, -1.0, 1.0)
        x += self.omega * lvl["dinv"] * res
        return x

    def __call__(self, r):
        K = self.mip
        z = torch.empty_like(r)
        K.jacobi(r, z)
        x = self.omega0 * z
        res = torch.empty_like(r)
        K.apply(x, res)
        res = r - res
        x += self._mv(self.P0, self._scalar(0, self._mv(self.R0, res)))
        K.apply(x, res)
        res = r - res
        K.jacobi(res, z)
        x += self.omega0 * z
        return x
