"""Linearized multigroup thermal radiative transfer steps on the GPU.

Backward-Euler time steps of grey-material, multigroup radiation transport
(allium's scallion driver with solver "linearized", exe/scallion.cpp:1352-1470)
built from the sweep and the TRT operators of the C ABI:

* per step: the power-law opacity sigma_g = C nu_g^a T^b at the cell centres
  (src/opacity.cpp:47-63, projected piecewise constant), reassembly of the
  sweep's local matrices and the time absorption 1/(c dt) (scallion.cpp:1456-1463);
* sources: q_psi = q_inflow + 1/(c dt) M psi_prev (scallion.cpp:1358-1359,
  src/tvector.cpp:76-95) and q_T = c_v/dt M T_prev;
* LinearizedTRTOperator::Mult (src/trt_linearized.cpp:230-312): with the
  emission B(T), its gradient dB, the energy-balance residual Bt(T) and the
  inverse of its gradient dBt^{-1}, solve the Schur system
      (I - D L^{-1} D^T dB dBt^{-1} M_sigma) phi = D L^{-1} (D^T e + q_psi),
      e = B(T) + dB dBt^{-1} (q_T - Bt(T)),
  by GMRES (FP64 sweep) or FP32-inner/FP64-outer refinement, sweep once more
  for psi and update T += dBt^{-1} (M_sigma D psi + q_T - Bt(T)), floored at 1e-8.

Units are the caller's: ac is allium's "StefanBoltzmann" (a c), c the speed of
light.  All state lives in torch float64 CUDA tensors.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._lib import check
from .solvers import SolveResult, gmres, refine_rhs
from .sweep import DiscreteToMoment, FormTransportSource, InverseAdvectionOperator, MomentsF32, MomentsF32Nodes


def log_spaced_groups(emin, emax, G):
    """MultiGroupEnergyGrid::MakeLogSpaced (src/multigroup.cpp:40-59): bounds[G+1], midpoints[G]."""
    lo, hi = math.log(emin), math.log(emax)
    d = (hi - lo) / G
    bounds = np.empty(G + 1)
    bounds[0] = emin
    for g in range(1, G + 1):
        bounds[g] = math.exp(lo + g * d)
    mid = np.sqrt(bounds[:-1] * bounds[1:])
    return bounds, mid


def planck_spectrum(bounds, T, kind=0):
    """Group fractions of the normalised Planck (kind 0) or Rosseland (1) spectrum."""
    b = np.ascontiguousarray(bounds, dtype=np.float64)
    out = np.empty(b.size - 1)
    check(_lib.lib().allium_planck_spectrum(b.ctypes.data, b.size - 1, float(T), int(kind), out.ctypes.data))
    return out


def _p(t):
    return C.c_void_p(t.data_ptr())


class TRTOperators:
    """The TRT operators of one sweep handle (device tensors in, device tensors out)."""

    def __init__(self, Linv: InverseAdvectionOperator, bounds, ac=1.0):
        self.L = Linv
        self.bounds = np.ascontiguousarray(bounds, dtype=np.float64)
        assert self.bounds.size == Linv.G + 1
        self.ac = float(ac)
        self.lib = _lib.lib()

    def _check(self, st):
        check(st, self.L.h)

    def emission(self, T, sigma, out=None, grad=None):
        self._check(self.lib.allium_sweep_planck_emission(self.L.h, self.bounds.ctypes.data, _p(sigma), _p(T),
                                                          self.ac, _p(out) if out is not None else None,
                                                          _p(grad) if grad is not None else None))

    def energy_balance(self, T, sigma, cv_dt, residual=None, grad_inv=None):
        self._check(self.lib.allium_sweep_energy_balance(self.L.h, self.bounds.ctypes.data, _p(sigma), _p(T),
                                                         self.ac, float(cv_dt),
                                                         _p(residual) if residual is not None else None,
                                                         _p(grad_inv) if grad_inv is not None else None))

    def block_apply(self, blocks, nsets, x, y, shared=False, alpha=1.0, accumulate=False):
        self._check(self.lib.allium_sweep_block_apply(self.L.h, _p(blocks) if blocks is not None else None,
                                                      int(nsets), _p(x), int(shared), _p(y), float(alpha),
                                                      int(accumulate)))

    def mass(self, which, x, y, alpha=1.0, accumulate=False):
        """which 1: unit sigma mass, 2: MassIntegrator mass."""
        self.block_apply(None, which, x, y, alpha=alpha, accumulate=accumulate)

    def absorption(self, sigma, phi, y, alpha=1.0, accumulate=False):
        self._check(self.lib.allium_sweep_absorption(self.L.h, _p(sigma), _p(phi), _p(y), float(alpha),
                                                     int(accumulate)))

    def time_source(self, psi_prev, q, tau, out):
        self._check(self.lib.allium_sweep_time_source(self.L.h, _p(psi_prev), _p(q) if q is not None else None,
                                                      float(tau), _p(out)))

    def powerlaw_opacity(self, T, nu, Cc, a, b, out):
        nu = np.ascontiguousarray(nu, dtype=np.float64)
        self._check(self.lib.allium_sweep_powerlaw_opacity(self.L.h, _p(T), nu.ctypes.data, float(Cc), float(a),
                                                           float(b), _p(out)))


class TRTSchurOperator:
    """x -> x - D L^{-1} D^T dB dBt^{-1} M_sigma x on [G][Ndof] moment vectors."""

    def __init__(self, step):
        self.s = step
        self.n = step.G * step.ndof
        self.sweeps64 = 0
        self.sweeps32 = 0

    def _emission_of(self, x):
        s = self.s
        s.ops.absorption(s.sigma, x, s.t1)
        s.ops.block_apply(s.bt_inv, 1, s.t1, s.t2)
        s.ops.block_apply(s.dB, s.G, s.t2, s.em, shared=True)
        return s.em

    def apply(self, x, out):
        s = self.s
        em = self._emission_of(x)
        s.D.MultTranspose(em, s.psi)
        s.L.Mult(s.psi, s.psi)
        self.sweeps64 += 1
        s.D.Mult(s.psi, s.mom)
        torch.sub(x, s.mom, out=out)
        return out

    def apply32(self, x, out):
        """The same operator with the FP32 sweep on the node-major layout
        [cell][angle][group][DOF] (isotropic source broadcast over angles)."""
        s = self.s
        em = self._emission_of(x)
        n = s.n
        src = (em.view(s.G, s.ne, n) / s.wsum).permute(1, 0, 2)          # [Ne][G][n]
        s.psi32.view(s.ne, s.Nw, s.G, n).copy_(src[:, None, :, :].expand(s.ne, s.Nw, s.G, n))
        s.L.MultF32Nodes(s.psi32, s.psi32)
        self.sweeps32 += 1
        MomentsF32Nodes(s.L, s.psi32, s.mom)
        torch.sub(x, s.mom, out=out)
        return out


@dataclass
class StepResult:
    iterations: int
    converged: bool
    seconds: float
    residual: float
    sweeps64: int
    sweeps32: int
    history: list = field(default_factory=list)


class LinearizedTRT:
    """State (psi, T) of a linearized TRT calculation and its time step.

    mesh/order/quad: the sweep's discretisation; bounds[G+1], nu[G]: group
    bounds and midpoints; opacity (C, a, b): sigma_g = C nu_g^a T^b; cv: heat
    capacity; dt: time step; inflow: {attribute: temperature} of isotropic
    Planck inflow; T0: initial temperature (radiation in equilibrium with it);
    tune: pick the sweep's launch configuration with the autotuner first."""

    def __init__(self, mesh, order, quad, bounds, nu, opacity, cv, dt, T0, inflow=None, ac=1.0, c=1.0,
                 method="fp64", tol=1e-8, inner_tol=1e-4, restart=30, tune=True):
        dev = torch.device("cuda")
        self.G = len(nu)
        self.nu = np.ascontiguousarray(nu, dtype=np.float64)
        self.bounds = np.ascontiguousarray(bounds, dtype=np.float64)
        self.opacity = tuple(float(v) for v in opacity)
        self.cv, self.dt, self.ac, self.c = float(cv), float(dt), float(ac), float(c)
        self.method, self.tol, self.inner_tol, self.restart = method, tol, inner_tol, restart
        ne = mesh.num_elements
        n = (order + 1) ** mesh.dim
        self.ne, self.n = ne, n
        self.ndof = ne * n
        T = torch.full((self.ndof,), float(T0), dtype=torch.float64, device=dev)
        self.T = T
        self.sigma = torch.empty((self.G, ne), dtype=torch.float64, device=dev)
        sig0 = np.ones((self.G, ne))
        self.L = InverseAdvectionOperator(mesh, order, quad, sig0)
        self.Nw = self.L.Nw
        self.D = DiscreteToMoment(self.L)
        self.ops = TRTOperators(self.L, self.bounds, ac)
        self.wsum = float(np.sum(quad.weights))
        G, Nd = self.G, self.ndof
        f64 = dict(dtype=torch.float64, device=dev)
        self.psi = torch.empty(self.L.width, **f64)
        self.psi32 = torch.empty(self.L.width, dtype=torch.float32, device=dev)
        self.q_psi = torch.empty(self.L.width, **f64)
        self.mom = torch.empty(G * Nd, **f64)
        self.em = torch.empty(G * Nd, **f64)
        self.t1 = torch.empty(Nd, **f64)
        self.t2 = torch.empty(Nd, **f64)
        self.bt = torch.empty(Nd, **f64)
        self.qT = torch.empty(Nd, **f64)
        self.bt_inv = torch.empty(ne * n * n, **f64)
        self.dB = torch.empty(G * ne * n * n, **f64)
        # isotropic Planck inflow psi = ac T^4 b_g(T) / (4 pi) (src/phase_coefficient.cpp:75)
        nattr = 1 + max([0] + list((inflow or {}).keys()))
        inf = np.zeros((G, nattr))
        for attr, Tin in (inflow or {}).items():
            inf[:, attr] = self.ac * Tin ** 4 * planck_spectrum(self.bounds, Tin) / (4.0 * math.pi)
        self.q_inflow = torch.from_numpy(FormTransportSource(self.L, None, inf)).to(dev)
        # radiation in equilibrium with T0: psi = ac T0^4 b_g(T0) / (4 pi)
        spec0 = planck_spectrum(self.bounds, T0) * self.ac * T0 ** 4 / (4.0 * math.pi)
        self.psi.view(G, self.Nw, Nd).copy_(torch.from_numpy(spec0).to(dev).view(G, 1, 1).expand(G, self.Nw, Nd))
        self.schur = TRTSchurOperator(self)
        self.steps = 0
        if tune:   # schedule and threads per block of this handle's sweeps (results do not change)
            from .autotune import autotune
            self.tuned = autotune(self.L, reps=3, fp32=(method != "fp64"))

    def phi(self):
        """Scalar flux [G][Ndof] of the current psi."""
        out = torch.empty(self.G * self.ndof, dtype=torch.float64, device=self.T.device)
        self.D.Mult(self.psi, out)
        return out

    def step(self, phi0=None):
        """One backward-Euler step; phi0 is the initial iterate of the Schur solve
        (D psi of the previous step when None)."""
        t0 = time.perf_counter()
        ops, L, D = self.ops, self.L, self.D
        Cc, a, b = self.opacity
        # opacity and sweep data for this step (scallion.cpp:1456-1463)
        ops.powerlaw_opacity(self.T, self.nu, Cc, a, b, self.sigma)
        L.AssembleLocalMatrices(self.sigma)
        tau = 1.0 / (self.c * self.dt)
        L.SetTimeAbsorption(tau)
        cv_dt = self.cv / self.dt
        # sources
        ops.time_source(self.psi, self.q_inflow, tau, self.q_psi)
        ops.mass(2, self.T, self.qT, alpha=cv_dt)
        # LinearizedTRTOperator::Mult
        phi_init = self.phi() if phi0 is None else phi0.clone()
        ops.energy_balance(self.T, self.sigma, cv_dt, self.bt, self.bt_inv)
        temp_resid = self.qT - self.bt
        ops.emission(self.T, self.sigma, self.em, self.dB)
        e_src = self.em.clone()
        ops.block_apply(self.bt_inv, 1, temp_resid, self.t1)
        ops.block_apply(self.dB, self.G, self.t1, e_src, shared=True, accumulate=True)
        D.MultTranspose(e_src, self.psi)
        self.psi += self.q_psi
        L.Mult(self.psi, self.psi)
        b_rhs = torch.empty_like(self.mom)
        D.Mult(self.psi, b_rhs)
        op = self.schur
        s64, s32 = op.sweeps64, op.sweeps32
        if self.method == "fp64":
            phi, it, hist = gmres(op.apply, b_rhs, x0=phi_init, tol=self.tol, restart=self.restart, maxiter=2000)
            conv = hist[-1] <= self.tol
        else:
            res = refine_rhs(op, b_rhs, x0=phi_init, tol=self.tol, inner_tol=self.inner_tol, restart=self.restart)
            phi, it, hist, conv = res.phi, res.iterations, res.history, res.converged
            it = res.inner_iterations
        # psi from phi, then the temperature update
        op._emission_of(phi)
        e_src += self.em
        D.MultTranspose(e_src, self.psi)
        self.psi += self.q_psi
        L.Mult(self.psi, self.psi)
        D.Mult(self.psi, self.mom)
        ops.absorption(self.sigma, self.mom, self.t1)
        self.t1 += temp_resid
        ops.block_apply(self.bt_inv, 1, self.t1, self.t2)
        self.T += self.t2
        self.T.clamp_(min=1e-8)
        torch.cuda.synchronize()
        self.steps += 1
        return StepResult(it, bool(conv), time.perf_counter() - t0, float(hist[-1]) if hist else 0.0,
                          op.sweeps64 - s64 + 2, op.sweeps32 - s32, hist)


def marshak_wave(cells=128, order=1, sn=8, G=32, emin=1e-2, emax=10.0, opacity_coef=10.0, cv=1.0, dt=1e-3,
                 T0=1e-3, T_inflow=1.0, method="fp64", tol=1e-8):
    """The multigroup Marshak-wave workload: [0,1]^2 with cells x cells quads,
    Planck inflow at T_inflow on x = 0 (boundary attribute 4), vacuum elsewhere,
    sigma_g = C nu_g^-3 T^-1/2 at the geometric group midpoints, non-dimensional
    units a = c = 1 (ac = 1)."""
    from . import mesh as M
    from . import quadrature as Q
    mesh = M.cartesian((cells, cells))
    quad = Q.level_symmetric(sn, 2)
    bounds, nu = log_spaced_groups(emin, emax, G)
    return LinearizedTRT(mesh, order, quad, bounds, nu, (opacity_coef, -3.0, -0.5), cv, dt, T0,
                         inflow={4: T_inflow}, method=method, tol=tol)
