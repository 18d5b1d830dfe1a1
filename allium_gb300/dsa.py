"""Diffusion synthetic acceleration with the GPU MIP diffusion operator.

MIPDiffusion wraps the C ABI's MIP operator K (InteriorPenaltyDiscretization,
src/moment_discretization.cpp:73-110) and solves K x = b with block-Jacobi
preconditioned conjugate gradients (allium applies CG with BoomerAMG;
BoomerAMG is a hypre library component, replaced here by the inverted cell
blocks K_ee).  DSAPreconditioner is DiffusionSyntheticAccelerationOperator
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
        """Block-Jacobi PCG on K x = b (x = 0 start); returns x."""
        x = torch.zeros_like(b)
        r = b.clone()
        z = torch.empty_like(b)
        self.jacobi(r, z)
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
            self.jacobi(r, z)
            rz_new = torch.dot(r, z)
            p.mul_(rz_new / rz).add_(z)
            rz = rz_new
        self.cg_iterations += it
        return x


class DSAPreconditioner:
    """y = x + K^{-1} M_s x (DiffusionSyntheticAccelerationOperator::Mult)."""

    def __init__(self, Linv, sigma_s, cg_tol=1e-10, cg_maxiter=200, **kw):
        self.K = MIPDiffusion(Linv, sigma_s, **kw)
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
