"""CPU checks of the thermal-radiative-transfer restatement: the Planck and
Rosseland group integrals against adaptive quadrature of their definitions, the
library's host spectrum against the oracle's, and one oracle TRT step."""
import math
import warnings

import numpy as np
import pytest

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q
from allium_gb300.trt import log_spaced_groups, planck_spectrum
from oracle.oracle import planck_spectrum as oracle_spectrum
from oracle.trt_oracle import OracleTRT

integrate = pytest.importorskip("scipy.integrate")


def _b_exact(x):
    if x == 0.0:
        return 0.0
    f = lambda t: t ** 3 * math.exp(-t) / -math.expm1(-t) if t > 0 else 0.0
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        v, _ = integrate.quad(f, 0.0, min(x, 200.0), epsabs=1e-16, epsrel=1e-14, limit=400)
    return 15.0 / math.pi ** 4 * v


def _r_exact(x):
    # Rosseland weight: 15/(4 pi^4) t^4 e^t / (e^t - 1)^2
    if x == 0.0:
        return 0.0
    f = lambda t: t ** 4 * math.exp(-t) / math.expm1(-t) ** 2 if t > 0 else 0.0
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        v, _ = integrate.quad(f, 0.0, min(x, 200.0), epsabs=1e-16, epsrel=1e-14, limit=400)
    return 15.0 / (4.0 * math.pi ** 4) * v


@pytest.mark.parametrize("T", [1e-3, 0.05, 0.3, 1.0, 3.0])
def test_planck_groups_match_quadrature(T):
    # src/planck.hpp:157-236 (Taylor through x^21 / 9-term polylogarithm): the
    # truncations are accurate to ~1e-10 of the normalised spectrum
    bounds, _ = log_spaced_groups(1e-2, 10.0, 32)
    F = [0.0] + [_b_exact(bounds[k] / T) for k in range(1, 32)] + [1.0]
    R = [0.0] + [_r_exact(bounds[k] / T) for k in range(1, 32)] + [1.0]
    b = oracle_spectrum(bounds, T, 0)
    r = oracle_spectrum(bounds, T, 1)
    assert abs(b.sum() - 1.0) < 1e-14 and abs(r.sum() - 1.0) < 1e-14
    assert np.max(np.abs(b - np.diff(F))) < 2e-10
    assert np.max(np.abs(r - np.diff(R))) < 2e-10
    # the library's host evaluation (no GPU needed) agrees to rounding
    assert np.max(np.abs(planck_spectrum(bounds, T, 0) - b)) < 1e-15
    assert np.max(np.abs(planck_spectrum(bounds, T, 1) - r)) < 1e-15


def test_log_spaced_groups():
    # MultiGroupEnergyGrid::MakeLogSpaced (src/multigroup.cpp:40-59)
    b, mid = log_spaced_groups(1e-2, 10.0, 3)
    assert np.allclose(b, [1e-2, 1e-1, 1.0, 10.0], rtol=1e-14)
    assert np.allclose(mid, np.sqrt(b[:-1] * b[1:]), rtol=1e-15)


def test_oracle_trt_step_heats_from_the_inflow():
    # Marshak-type wave: Planck inflow at T = 1 on x = 0 heats the cold slab
    # step after step; temperatures stay positive, the problem is symmetric in y
    mesh = M.cartesian((4, 4))
    quad = Q.level_symmetric(4, 2)
    bounds, nu = log_spaced_groups(1e-2, 10.0, 4)
    o = OracleTRT(mesh, 1, quad, bounds, nu, (10.0, -3.0, -0.5), cv=1.0, dt=1e-2, T0=1e-2, inflow={4: 1.0})
    first = []
    for _ in range(3):
        o.step()
        Tc = o.T.reshape(16, 4).mean(axis=1).reshape(4, 4)   # [j][i], x fastest
        first.append(Tc[:, 0].mean())
        assert np.all(o.T > 0)
        assert np.allclose(Tc, Tc[::-1], rtol=1e-10)
    assert first[0] > 1.1e-2 and first[2] > first[1] > first[0]


def _oracle_cells(dim=2, p=1, G=6, jitter=0.0):
    from oracle.oracle import OracleSweep
    mesh = M.cartesian((3,) * dim, jitter=jitter, seed=5)
    quad = Q.level_symmetric(4, dim)
    sig = np.ones((G, mesh.num_elements))
    return mesh, OracleSweep(mesh, p, quad, sig)


def test_emission_sums_to_gray_emission():
    # sum_g b_g = 1: with a group-independent opacity and a cellwise-constant T
    # the multigroup emission sums to sigma ac T^4 int phi_i, which the
    # energy-balance residual (another rule) also gives for cv_dt = 0
    mesh, o = _oracle_cells(G=6)
    bounds, _ = log_spaced_groups(1e-2, 10.0, 6)
    ne, n = mesh.num_elements, o.n
    Tc = np.linspace(0.3, 2.0, ne)
    T = np.repeat(Tc, n)
    sigma = np.tile(np.linspace(1.0, 3.0, ne), (6, 1))
    em, _ = o.planck_emission(bounds, sigma, T, ac=1.7)
    gray = em.reshape(6, ne * n).sum(axis=0)
    ones = o.mass_apply(1, np.ones(ne * n))          # int phi_i (sum_j M_ij)
    ref = np.repeat(sigma[0] * 1.7 * Tc ** 4, n) * ones
    assert np.max(np.abs(gray - ref)) < 1e-13 * np.max(np.abs(ref))
    res, _ = o.energy_balance(bounds, sigma, T, 1.7, 0.0)
    assert np.max(np.abs(res - ref)) < 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("dim,p", [(2, 1), (2, 2), (3, 1)])
def test_emission_gradients_are_derivatives(dim, p):
    # d/dT [T^4 b_g(E/T)] = 4 T^3 r_g(E/T): the Rosseland-weighted blocks of
    # PlanckEmissionNFI::AssembleElementGrad and the gray gradient are the
    # Jacobians of the emission and of the energy-balance residual
    mesh, o = _oracle_cells(dim, p, G=5, jitter=0.2)
    bounds, _ = log_spaced_groups(1e-2, 10.0, 5)
    ne, n = mesh.num_elements, o.n
    rng = np.random.default_rng(9)
    T = rng.uniform(0.3, 1.5, ne * n)
    sigma = 10.0 ** rng.uniform(-1, 1, size=(5, ne))
    _, dB = o.planck_emission(bounds, sigma, T, ac=1.0)
    _, dBt = o.energy_balance(bounds, sigma, T, 1.0, 2.0)
    h = 1e-6
    for e in (0, ne - 1):
        for j in range(n):
            Tp, Tm = T.copy(), T.copy()
            Tp[e * n + j] += h
            Tm[e * n + j] -= h
            ep, _ = o.planck_emission(bounds, sigma, Tp, ac=1.0)
            em_, _ = o.planck_emission(bounds, sigma, Tm, ac=1.0)
            fd = ((ep - em_) / (2 * h)).reshape(5, ne, n)[:, e, :]
            assert np.max(np.abs(fd - dB[:, e, :, j])) < 1e-6 * np.max(np.abs(dB[:, e]))
            rp, _ = o.energy_balance(bounds, sigma, Tp, 1.0, 2.0)
            rm, _ = o.energy_balance(bounds, sigma, Tm, 1.0, 2.0)
            fd = ((rp - rm) / (2 * h)).reshape(ne, n)[e]
            assert np.max(np.abs(fd - dBt[e, :, j])) < 1e-6 * np.max(np.abs(dBt[e]))
