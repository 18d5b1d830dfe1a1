"""CPU ORACLE -- test infrastructure only.

A numpy restatement of one linearized thermal-radiative-transfer time step
(LinearizedTRTOperator::Mult, src/trt_linearized.cpp:230-312, with the source
and opacity updates of exe/scallion.cpp:1352-1470) on top of the C++ oracle's
operators.  The Schur system is solved directly (its dense matrix is built
column by column with oracle sweeps), so the result is the exact solution of
each linearized step; meant for small meshes."""
from __future__ import annotations

import math

import numpy as np

from .oracle import OracleSweep, planck_spectrum


class OracleTRT:
    def __init__(self, mesh, order, quad, bounds, nu, opacity, cv, dt, T0, inflow=None, ac=1.0, c=1.0):
        self.mesh, self.order, self.quad = mesh, order, quad
        self.bounds = np.asarray(bounds, dtype=np.float64)
        self.nu = np.asarray(nu, dtype=np.float64)
        self.G = self.nu.size
        self.opacity = opacity
        self.cv, self.dt, self.ac, self.c = cv, dt, ac, c
        self.ne = mesh.num_elements
        self.n = (order + 1) ** mesh.dim
        self.ndof = self.ne * self.n
        self.Nw = quad.size
        self.T = np.full(self.ndof, float(T0))
        nattr = 1 + max([0] + list((inflow or {}).keys()))
        self.inflow = np.zeros((self.G, nattr))
        for attr, Tin in (inflow or {}).items():
            self.inflow[:, attr] = ac * Tin ** 4 * planck_spectrum(self.bounds, Tin) / (4.0 * math.pi)
        spec0 = planck_spectrum(self.bounds, T0) * ac * T0 ** 4 / (4.0 * math.pi)
        self.psi = np.repeat(spec0, self.Nw * self.ndof)

    def step(self):
        G, Nd, n, ne = self.G, self.ndof, self.n, self.ne
        C0, a, b = self.opacity
        o0 = OracleSweep(self.mesh, self.order, self.quad, np.ones((G, ne)))
        sigma = o0.powerlaw_opacity(self.T, self.nu, C0, a, b)
        o = OracleSweep(self.mesh, self.order, self.quad, sigma)
        tau = 1.0 / (self.c * self.dt)
        o.set_time_absorption(tau)
        cv_dt = self.cv / self.dt
        q_inflow = o.form_source(inflow=self.inflow)
        q_psi = o.time_source(self.psi, q_inflow, tau)
        qT = cv_dt * o.mass_apply(2, self.T)
        bt, dBt = o.energy_balance(self.bounds, sigma, self.T, self.ac, cv_dt)
        dBt_inv = np.linalg.inv(dBt)
        em, dB = o.planck_emission(self.bounds, sigma, self.T, self.ac)

        def binv(x):
            return np.einsum("eij,ej->ei", dBt_inv, x.reshape(ne, n)).reshape(-1)

        def dBx(x):
            return np.einsum("geij,ej->gei", dB, x.reshape(ne, n)).reshape(-1)

        temp_resid = qT - bt
        e_src = em + dBx(binv(temp_resid))
        psi = o.mult(o.moments_transpose(e_src, 1) + q_psi)
        rhs = o.moments(psi)

        def schur(x):
            y = o.mult(o.moments_transpose(dBx(binv(o.absorption(sigma, x))), 1))
            return x - o.moments(y)

        m = G * Nd
        A = np.empty((m, m))
        for k in range(m):
            ek = np.zeros(m)
            ek[k] = 1.0
            A[:, k] = schur(ek)
        phi = np.linalg.solve(A, rhs)
        e_src = e_src + dBx(binv(o.absorption(sigma, phi)))
        self.psi = o.mult(o.moments_transpose(e_src, 1) + q_psi)
        dT = binv(o.absorption(sigma, o.moments(self.psi)) + temp_resid)
        self.T = np.maximum(self.T + dT, 1e-8)
        return phi
