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
  whose operator applies the FP32 sweep (moments accumulated in FP64); phi += d.

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


def gmres(apply, b, x0=None, tol=1e-8, restart=30, maxiter=2000, atol=0.0, prec=None):
    """Restarted GMRES on torch vectors; stops when ||b - A x|| <= max(tol ||b||, atol)
    (the Arnoldi residual estimate).  prec(v, out) is a right preconditioner,
    kept in flexible form (the preconditioned directions are stored), so it
    may be an inner iterative solve.  Returns (x, iterations, history)."""
    dev, n = b.device, b.numel()
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    bnorm = torch.linalg.norm(b).item()
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
    beta = torch.linalg.norm(r).item()
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
            h = torch.mv(V[: k + 1], w)
            w -= torch.mv(V[: k + 1].t(), h)
            h2 = torch.mv(V[: k + 1], w)
            w -= torch.mv(V[: k + 1].t(), h2)
            hk = (h + h2).cpu().numpy()
            hn = torch.linalg.norm(w).item()
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
        apply(x, w)
        r = b - w
        beta = torch.linalg.norm(r).item()
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


def true_residual(op: SchurOperator, b, phi):
    """||b - T phi|| / ||b|| with the FP64 operator."""
    w = torch.empty_like(phi)
    op.apply(phi, w)
    return (torch.linalg.norm(b - w) / torch.linalg.norm(b)).item()
