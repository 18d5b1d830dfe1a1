"""Outer iterations around the sweep, on the GPU.

The transport problem with isotropic within-group scattering,
    L psi = D^T S phi + q,   phi = D psi,
is solved in its scalar-flux (Schur) form
    T phi = (I - D L^{-1} D^T S) phi = D L^{-1} q = b
as allium's chive driver does (exe/chive.cpp:704-735, TransportOperator in
src/transport_op.hpp:9-35).  Provided here:

* source_iteration: phi <- D L^{-1} (D^T S phi + q) until the relative change of
  phi is below tol (SLISolver without a preconditioner, src/linalg.cpp:103-153);
* gmres: restarted GMRES with classical Gram-Schmidt and reorthogonalisation on
  T (the Krylov option of chive);
* refine: FP32-inner / FP64-outer iterative refinement.  The outer residual
  r = b - T phi uses the FP64 sweep; each correction solves T d = r with GMRES
  whose operator applies the FP32 sweep (moments accumulated in FP64); phi += d;
* refine_fused: the same refinement on the transport system with no FP64 sweep:
  psi kept in double-float, the residual q + D^T S D psi - L psi evaluated in
  double-float arithmetic, every sweep the fused FP32 operator.

All vectors are torch float64 CUDA tensors of length G * Ndof (phi) or
G * Nw * Ndof (psi).  Diffusion synthetic acceleration (allium_gb300.dsa) is
optional: the preconditioner of source iteration and the right preconditioner
of GMRES.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .sweep import (DiscreteToMoment, InverseAdvectionOperator, MomentsF32, MomentsF32Nodes, ScatteringSource,
                    ScatteringSourceF32, ScatteringSourceF32Nodes)


class SchurOperator:
    """T phi = phi - D L^{-1} D^T S phi, in FP64 (apply) or with the FP32 sweep (apply32)."""

    def __init__(self, Linv: InverseAdvectionOperator, sigma_s):
        self.L = Linv
        self.D = DiscreteToMoment(Linv)
        self.sigma_s = np.ascontiguousarray(sigma_s, dtype=np.float64).reshape(Linv.G, -1)
        dev = torch.device("cuda")
        self.n = Linv.G * Linv.ndof
        self.psi = torch.empty(Linv.width, dtype=torch.float64, device=dev)
        self.psi32 = None
        self.tmp = torch.empty(self.n, dtype=torch.float64, device=dev)
        self.sweeps64 = 0
        self.sweeps32 = 0

    def rhs(self, q):
        """b = D L^{-1} q (one FP64 sweep)."""
        self.psi.copy_(q)
        self.L.Mult(self.psi, self.psi)
        self.sweeps64 += 1
        b = torch.empty(self.n, dtype=torch.float64, device=self.psi.device)
        self.D.Mult(self.psi, b)
        return b

    def apply(self, x, out):
        ScatteringSource(self.L, self.sigma_s, x, None, self.psi)
        self.L.Mult(self.psi, self.psi)
        self.sweeps64 += 1
        self.D.Mult(self.psi, self.tmp)
        torch.sub(x, self.tmp, out=out)
        return out

    def apply32(self, x, out):
        """T with the FP32 sweep on node-major vectors (contiguous runs per level);
        orders above 1 and reflective boundaries use allium's RIGHT layout."""
        if self.L.order > 1 or getattr(self.L, "has_reflective", False):
            return self.apply32_right(x, out)
        if self.psi32 is None:
            self.psi32 = torch.empty(self.L.width, dtype=torch.float32, device=self.psi.device)
        ScatteringSourceF32Nodes(self.L, self.sigma_s, x, None, self.psi32)
        self.L.MultF32Nodes(self.psi32, self.psi32)
        self.sweeps32 += 1
        MomentsF32Nodes(self.L, self.psi32, self.tmp)
        torch.sub(x, self.tmp, out=out)
        return out

    def apply32_right(self, x, out):
        """T with the FP32 sweep on allium's RIGHT layout."""
        if self.psi32 is None:
            self.psi32 = torch.empty(self.L.width, dtype=torch.float32, device=self.psi.device)
        ScatteringSourceF32(self.L, self.sigma_s, x, None, self.psi32)
        self.L.MultF32(self.psi32, self.psi32)
        self.sweeps32 += 1
        MomentsF32(self.L, self.psi32, self.tmp)
        torch.sub(x, self.tmp, out=out)
        return out


@dataclass
class SolveResult:
    phi: torch.Tensor
    iterations: int
    converged: bool
    history: list = field(default_factory=list)
    seconds: float = 0.0
    sweeps64: int = 0
    sweeps32: int = 0


def source_iteration(op: SchurOperator, q, tol=1e-8, maxiter=10000, phi0=None, dsa=None):
    """phi_{k+1/2} = D L^{-1} (D^T S phi_k + q); with dsa (a DSAPreconditioner)
    phi_{k+1} = phi_k + P (phi_{k+1/2} - phi_k), P = I + K^{-1} M_s (SLISolver
    with the DSA preconditioner, src/linalg.cpp:103-153); stop on
    ||phi_{k+1} - phi_k|| < tol ||phi_{k+1}||."""
    t0 = time.perf_counter()
    L, D = op.L, op.D
    phi = torch.zeros(op.n, dtype=torch.float64, device=op.psi.device) if phi0 is None else phi0.clone()
    new = torch.empty_like(phi)
    hist = []
    it = 0
    conv = False
    while it < maxiter:
        ScatteringSource(L, op.sigma_s, phi, q, op.psi)
        L.Mult(op.psi, op.psi)
        op.sweeps64 += 1
        D.Mult(op.psi, new)
        if dsa is not None:
            r = new - phi
            dsa(r, r)
            torch.add(phi, r, out=new)
        it += 1
        change = (torch.linalg.norm(new - phi) / torch.linalg.norm(new)).item()
        hist.append(change)
        phi, new = new, phi
        if change < tol:
            conv = True
            break
    torch.cuda.synchronize()
    return SolveResult(phi, it, conv, hist, time.perf_counter() - t0, op.sweeps64, op.sweeps32)


def gmres(apply, b, x0=None, tol=1e-8, restart=30, maxiter=2000, atol=0.0, prec=None, final_residual=True,
          reduce=None):
    """Restarted GMRES on torch vectors; stops when ||b - A x|| <= max(tol ||b||, atol)
    (the Arnoldi residual estimate).  prec(v, out) is a right preconditioner,
    kept in flexible form (the preconditioned directions are stored), so it
    may be an inner iterative solve.  With final_residual the residual of the
    iterate is recomputed with one more application of A after each cycle
    (restart or stop); without it the last cycle that meets the tolerance ends on
    the Arnoldi estimate (for inner solves whose caller checks the residual
    itself).  reduce(t), when given, sums a tensor of partial inner products
    over the shards of a distributed vector in place (every vector here is then
    one shard); the Hessenberg work is repeated identically on every shard.
    Returns (x, iterations, history)."""
    dev, n = b.device, b.numel()
    x = torch.zeros_like(b) if x0 is None else x0.clone()

    def norm(v):
        if reduce is None:
            return torch.linalg.norm(v).item()
        s = torch.dot(v, v).reshape(1)
        reduce(s)
        return math.sqrt(max(s.item(), 0.0))

    def dots(Vk, v):
        h = torch.mv(Vk, v)
        if reduce is not None:
            reduce(h)
        return h

    bnorm = norm(b)
    if bnorm == 0.0:
        return x, 0, [0.0]
    target = max(tol * bnorm, atol)
    V = torch.empty((restart + 1, n), dtype=b.dtype, device=dev)
    Z = torch.empty((restart, n), dtype=b.dtype, device=dev) if prec is not None else None
    w = torch.empty_like(b)
    hist = []
    it = 0
    r = b.clone()
    if x0 is not None:
        apply(x, w)
        r = b - w
    beta = norm(r)
    hist.append(beta / bnorm)
    while it < maxiter and beta > target:
        V[0] = r / beta
        H = np.zeros((restart + 1, restart))
        cs, sn = np.zeros(restart), np.zeros(restart)
        g = np.zeros(restart + 1)
        g[0] = beta
        k_used = 0
        for k in range(restart):
            if prec is not None:
                prec(V[k], Z[k])
                apply(Z[k], w)
            else:
                apply(V[k], w)
            it += 1
            # classical Gram-Schmidt, twice
            h = dots(V[: k + 1], w)
            w -= torch.mv(V[: k + 1].t(), h)
            h2 = dots(V[: k + 1], w)
            w -= torch.mv(V[: k + 1].t(), h2)
            if reduce is None:
                # the Hessenberg column and ||w||^2 in one device-to-host copy
                col = torch.cat([h + h2, torch.dot(w, w).reshape(1)]).cpu().numpy()
                hk, hn = col[:-1], math.sqrt(max(float(col[-1]), 0.0))
            else:
                hk = (h + h2).cpu().numpy()
                hn = norm(w)
            H[: k + 1, k] = hk
            H[k + 1, k] = hn
            for i in range(k):
                t = cs[i] * H[i, k] + sn[i] * H[i + 1, k]
                H[i + 1, k] = -sn[i] * H[i, k] + cs[i] * H[i + 1, k]
                H[i, k] = t
            den = math.hypot(H[k, k], H[k + 1, k])
            cs[k], sn[k] = H[k, k] / den, H[k + 1, k] / den
            H[k, k] = den
            H[k + 1, k] = 0.0
            g[k + 1] = -sn[k] * g[k]
            g[k] = cs[k] * g[k]
            k_used = k + 1
            hist.append(abs(g[k + 1]) / bnorm)
            if hn > 0.0:
                V[k + 1] = w / hn
            if abs(g[k + 1]) <= target or it >= maxiter or hn == 0.0:
                break
        y = np.linalg.solve(np.triu(H[:k_used, :k_used]), g[:k_used])
        basis = Z if prec is not None else V
        x += torch.mv(basis[:k_used].t(), torch.from_numpy(y).to(dev))
        if not final_residual and abs(g[k_used]) <= target:
            break
        apply(x, w)
        r = b - w
        beta = norm(r)
        hist[-1] = beta / bnorm
    return x, it, hist


def solve_gmres(op: SchurOperator, q, tol=1e-8, restart=30, maxiter=2000, prec=None):
    """FP64 GMRES on T phi = b (prec: a right preconditioner such as DSA)."""
    t0 = time.perf_counter()
    b = op.rhs(q)
    phi, it, hist = gmres(op.apply, b, tol=tol, restart=restart, maxiter=maxiter, prec=prec)
    torch.cuda.synchronize()
    conv = hist[-1] <= tol
    return SolveResult(phi, it, conv, hist, time.perf_counter() - t0, op.sweeps64, op.sweeps32)


def refine(op: SchurOperator, q, tol=1e-8, inner_tol=1e-4, restart=30, max_outer=20, inner_maxiter=500, prec=None):
    """FP32-inner / FP64-outer iterative refinement on T phi = b."""
    t0 = time.perf_counter()
    res = refine_rhs(op, op.rhs(q), tol=tol, inner_tol=inner_tol, restart=restart, max_outer=max_outer,
                     inner_maxiter=inner_maxiter, prec=prec)
    res.seconds = time.perf_counter() - t0
    return res


def refine_rhs(op, b, x0=None, tol=1e-8, inner_tol=1e-4, restart=30, max_outer=20, inner_maxiter=500, prec=None):
    """Iterative refinement on T phi = b from phi = x0 (zero when None): the
    residual with op.apply (FP64 sweep), corrections by GMRES on op.apply32."""
    t0 = time.perf_counter()
    bnorm = torch.linalg.norm(b).item()
    if bnorm == 0.0:
        res = SolveResult(torch.zeros_like(b), 0, True, [0.0], 0.0, op.sweeps64, op.sweeps32)
        res.inner_iterations = 0
        return res
    w = torch.empty_like(b)
    if x0 is None:
        phi = torch.zeros_like(b)
        r = b.clone()
    else:
        phi = x0.clone()
        op.apply(phi, w)
        r = b - w
    hist = []
    conv = False
    outer = 0
    inner_total = 0
    while outer < max_outer:
        rel = torch.linalg.norm(r).item() / bnorm
        hist.append(rel)
        if rel <= tol:
            conv = True
            break
        d, it, _ = gmres(op.apply32, r, tol=inner_tol, restart=restart, maxiter=inner_maxiter, prec=prec)
        inner_total += it
        phi += d
        op.apply(phi, w)
        torch.sub(b, w, out=r)
        outer += 1
    torch.cuda.synchronize()
    res = SolveResult(phi, outer, conv, hist, time.perf_counter() - t0, op.sweeps64, op.sweeps32)
    res.inner_iterations = inner_total
    return res


class FusedSchur:
    """T = I - D L^{-1} D^T S with the fused FP32 sweep: per application one small
    kernel builds the per-cell source (S x)/sum(w) and one CUDA graph sweeps
    (one launch per wavefront level) and sums D psi (allium_sweep_fused_mult_f32);
    psi stays in a scratch vector of the fused layout."""

    def __init__(self, Linv: InverseAdvectionOperator, sigma_s, allreduce=None):
        self.L = Linv
        self.allreduce = allreduce
        dev = torch.device("cuda")
        self.sigma_s = torch.as_tensor(np.ascontiguousarray(sigma_s, dtype=np.float64).reshape(-1), device=dev)
        self.n = Linv.G * Linv.ndof
        self.iso = torch.empty(self.n, dtype=torch.float32, device=dev)
        self.psi32 = torch.empty(Linv.width, dtype=torch.float32, device=dev)
        self.tmp = torch.empty(self.n, dtype=torch.float64, device=dev)
        self.sweeps32 = 0

    def apply32(self, x, out):
        # the inner GMRES's operator: moments summed in FP32 (phi_mode 3)
        self.L.IsotropicSource(self.sigma_s, x, None, out=self.iso)
        self.L.FusedMultF32(self.iso, None, self.psi32, phi=self.tmp, phi_mode=3)
        if self.allreduce is not None:
            self.allreduce(self.tmp)
        self.sweeps32 += 1
        torch.sub(x, self.tmp, out=out)
        return out


def split_isotropic(Linv: InverseAdvectionOperator, q):
    """(q_iso, q_rest) for a psi-sized RIGHT source q: q_iso [G*Ndof] when q is the
    same in every direction (FormTransportSource of an isotropic density with
    vacuum boundaries), else (None, q)."""
    v = q.view(Linv.G, Linv.Nw, Linv.ndof)
    lo, hi = torch.aminmax(v, dim=1)   # one pass over q, no psi-sized temporary
    if torch.equal(lo, hi):
        return v[:, 0, :].reshape(-1).contiguous(), None
    return None, q


def refine_fused(Linv: InverseAdvectionOperator, sigma_s, q=None, q_iso=None, tol=1e-8, inner_tol=1e-4, restart=30,
                 max_outer=20, inner_maxiter=500, prec=None, incremental=None, allreduce=None):
    """FP32-inner / FP64-outer refinement on the transport system itself,
    L psi - D^T S D psi = q, with no FP64 sweep.

    psi is kept as a double-float pair (hi + lo, about 48 bits).  Each outer step
    takes the residual r = q + D^T S phi - L psi in double-float arithmetic
    (allium_sweep_transport_residual_df, phi = D psi), projects it with one FP32
    sweep, rho = D L^{-1} r, which is the residual b - T phi of the scalar-flux
    system T phi = b = D L^{-1} q (exe/chive.cpp:704-735) that the FP64 solvers
    iterate on, solves T d = rho by GMRES on the fused FP32 operator, and
    corrects psi += L^{-1} (r + D^T S d) with one more FP32 sweep, whose graph
    also sums D of the correction (double-float sums) into phi.  The first
    residual is evaluated in double-float; later ones (incremental, the default
    for tol >= 1e-10) take a closed form: the correction sweep solved
    L dpsi = r + D^T S d, so the new residual r + D^T S D dpsi - L dpsi is
    D^T S (dphi - d), exact up to the FP32 solve error of dpsi (the same order
    as an FP32 evaluation of L dpsi, ~1e-7 of the correction), and per cell:
    the sweeps after it read no psi-sized source.  Stops when
    ||rho|| <= tol ||rho_0||.
    q is the psi-sized RIGHT FP64 source (a CUDA tensor) or q_iso its per-cell
    part when it is the same in every direction.  Returns a SolveResult whose
    phi is the FP64 scalar flux.

    allreduce(t), when given, sums a moment vector over the ranks that hold the
    other directions (in place): Linv then sweeps one slice of the directions,
    sigma_s is scaled by the slice's share of the weight sum, and every moment
    vector the sweeps produce is completed by one allreduce, so the moment-space
    (GMRES) work is repeated identically on every rank while psi and the
    residual stay sharded."""
    t0 = time.perf_counter()
    L = Linv
    dev = torch.device("cuda")
    fs = FusedSchur(L, sigma_s, allreduce)
    red = allreduce if allreduce is not None else (lambda t: t)
    W, n = L.width, fs.n
    q_rest = None
    if q_iso is None:
        q_iso, q_rest = split_isotropic(L, q)
    q_hi = q_lo = None
    if q_rest is not None:
        q_hi = torch.empty(W, dtype=torch.float32, device=dev)
        q_lo = torch.empty(W, dtype=torch.float32, device=dev)
        L.ToFusedLayout(q_rest, q_hi, q_lo)
    hi = torch.zeros(W, dtype=torch.float32, device=dev)
    lo = torch.zeros(W, dtype=torch.float32, device=dev)
    r32 = torch.empty(W, dtype=torch.float32, device=dev)
    phi = torch.zeros(n, dtype=torch.float64, device=dev)
    dphi = torch.empty(n, dtype=torch.float64, device=dev)
    rho = torch.empty(n, dtype=torch.float64, device=dev)
    iso_hi = torch.empty(n, dtype=torch.float32, device=dev)
    iso_lo = torch.empty(n, dtype=torch.float32, device=dev)
    if incremental is None:
        incremental = tol >= 1e-10
    # rho_0 = D L^{-1} q (the residual of psi = 0)
    if q_iso is not None:
        L.IsotropicSource(None, None, q_iso, out=fs.iso)
    # right-hand sides and projections need only FP32 moments (phi_mode 3); the
    # corrections of phi (phi_mode 1 below) are summed in double-float
    L.FusedMultF32(fs.iso if q_iso is not None else None, q_hi, fs.psi32, phi=rho, phi_mode=3)
    red(rho)
    fs.sweeps32 += 1
    r0 = torch.linalg.norm(rho).item()
    hist, outer, inner_total, conv, residuals, updates = [], 0, 0, False, 0, 0
    r_cell = None   # m with r = D^T S m when the residual is per cell, else r is in r32
    if r0 == 0.0:
        res = SolveResult(phi, 0, True, [0.0], time.perf_counter() - t0, 0, fs.sweeps32)
        res.inner_iterations, res.residuals_df, res.residual_updates = 0, 0, 0
        return res
    while outer <= max_outer:
        rn = torch.linalg.norm(rho).item()
        hist.append(rn / r0)
        if rn <= tol * r0:
            conv = True
            break
        if outer == max_outer:
            break
        # enough accuracy to land below tol in this step, never looser than needed
        eta = max(inner_tol, 0.5 * tol * r0 / rn)
        d, it, _ = gmres(fs.apply32, rho, tol=eta, restart=restart, maxiter=inner_maxiter, prec=prec,
                         final_residual=False)
        inner_total += it
        # psi += dpsi = L^{-1} (r + D^T S d); phi += D dpsi (double-float sums)
        if outer == 0:
            L.IsotropicSource(fs.sigma_s, d, q_iso, out=fs.iso)
            src = q_hi
        elif r_cell is None:
            L.IsotropicSource(fs.sigma_s, d, None, out=fs.iso)
            src = r32
        else:
            r_cell += d
            L.IsotropicSource(fs.sigma_s, r_cell, None, out=fs.iso)
            src = None
        L.FusedMultF32(fs.iso, src, fs.psi32, phi=dphi, phi_mode=1, acc=(hi, lo))
        red(dphi)
        fs.sweeps32 += 1
        phi += dphi
        # the new residual r, then rho = D L^{-1} r
        if outer == 0 or not incremental:
            # r = q + D^T S phi - L psi in double-float arithmetic
            L.IsotropicSource(fs.sigma_s, phi, q_iso, out_hi=iso_hi, out_lo=iso_lo)
            L.TransportResidualDF(iso_hi, iso_lo, hi, lo, r32, q_hi, q_lo)
            residuals += 1
            r_cell = None
            L.FusedMultF32(None, r32, fs.psi32, phi=rho, phi_mode=3)
        else:
            # the sweep solved L dpsi = r + D^T S d, so the new residual
            # r + D^T S D dpsi - L dpsi is D^T S (dphi - d): per cell, isotropic
            r_cell = torch.sub(dphi, d)
            updates += 1
            L.IsotropicSource(fs.sigma_s, r_cell, None, out=fs.iso)
            L.FusedMultF32(fs.iso, None, fs.psi32, phi=rho, phi_mode=3)
        red(rho)
        fs.sweeps32 += 1
        outer += 1
    torch.cuda.synchronize()
    res = SolveResult(phi, outer, conv, hist, time.perf_counter() - t0, 0, fs.sweeps32)
    res.inner_iterations = inner_total
    res.residuals_df = residuals
    res.residual_updates = updates
    res.psi = (hi, lo)
    return res


def true_residual(op: SchurOperator, b, phi):
    """||b - T phi|| / ||b|| with the FP64 operator."""
    w = torch.empty_like(phi)
    op.apply(phi, w)
    return (torch.linalg.norm(b - w) / torch.linalg.norm(b)).item()
