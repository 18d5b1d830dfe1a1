"""GPU parity of the thermal-radiative-transfer operators and of whole
linearized TRT steps with the CPU oracle, through the C ABI.

Tolerances: operators 1e-12 relative (max norm); inverse gradient blocks 1e-10
(explicit Gauss-Jordan inverse against numpy's); whole steps 1e-8 relative for
T and psi (the GPU Schur solve runs GMRES to 1e-13, the oracle solves it
directly; with opacities up to 1e8 in the low groups the temperature update is
a difference of nearly equal absorption and emission terms, which turns the
1e-13 solve tolerance into ~1e-9 in T); FP32-inner refinement 1e-7 against the
FP64 step."""
import numpy as np
import pytest

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q
from allium_gb300.sweep import InverseAdvectionOperator
from allium_gb300.trt import LinearizedTRT, TRTOperators, log_spaced_groups
from oracle.oracle import OracleSweep
from oracle.trt_oracle import OracleTRT
from tests.helpers import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [
    # dim, cells, p, G
    (2, (6, 5), 1, 5),
    (2, (4, 3), 2, 3),
    (2, (3, 3), 3, 2),
    (3, (3, 3, 2), 1, 3),
    (2, (5, 5), 1, 40),
]


@pytest.mark.parametrize("case", CASES, ids=[f"d{c[0]}p{c[2]}G{c[3]}" for c in CASES])
def test_trt_operators(case):
    dim, cells, p, G = case
    mesh = M.cartesian(cells, jitter=0.15, seed=3)
    quad = Q.level_symmetric(4, dim)
    ne, n = mesh.num_elements, (p + 1) ** dim
    rng = np.random.default_rng(4)
    sigma = 10.0 ** rng.uniform(-1, 2, size=(G, ne))
    bounds, nu = log_spaced_groups(1e-2, 10.0, G)
    T = rng.uniform(0.2, 2.0, size=ne * n)
    o = OracleSweep(mesh, p, quad, sigma)
    L = InverseAdvectionOperator(mesh, p, quad, sigma)
    ops = TRTOperators(L, bounds, ac=1.3)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    dT, dsig = dev(T), dev(sigma)
    f64 = dict(dtype=torch.float64, device="cuda")

    em = torch.empty(G * ne * n, **f64)
    dB = torch.empty(G * ne * n * n, **f64)
    ops.emission(dT, dsig, em, dB)
    em_o, dB_o = o.planck_emission(bounds, sigma, T, 1.3)
    assert rel_err(em.cpu().numpy(), em_o) < 1e-12
    assert rel_err(dB.cpu().numpy(), dB_o.reshape(-1)) < 1e-12

    bt = torch.empty(ne * n, **f64)
    binv = torch.empty(ne * n * n, **f64)
    ops.energy_balance(dT, dsig, 7.0, bt, binv)
    bt_o, grad_o = o.energy_balance(bounds, sigma, T, 1.3, 7.0)
    assert rel_err(bt.cpu().numpy(), bt_o) < 1e-12
    assert rel_err(binv.cpu().numpy(), np.linalg.inv(grad_o).reshape(-1)) < 1e-10

    phi = rng.random(G * ne * n)
    y = torch.empty(ne * n, **f64)
    ops.absorption(dsig, dev(phi), y)
    assert rel_err(y.cpu().numpy(), o.absorption(sigma, phi)) < 1e-12
    for which in (1, 2):
        x = rng.random(ne * n)
        ops.mass(which, dev(x), y)
        assert rel_err(y.cpu().numpy(), o.mass_apply(which, x)) < 1e-12
    # block products: one shared vector through G block sets, accumulate
    x = rng.random(ne * n)
    out = dev(phi).clone()
    ops.block_apply(dB, G, dev(x), out, shared=True, alpha=0.5, accumulate=True)
    ref = phi + 0.5 * np.einsum("geij,ej->gei", dB_o, x.reshape(ne, n)).reshape(-1)
    assert rel_err(out.cpu().numpy(), ref) < 1e-12

    psi = rng.random(o.psi_size)
    q = rng.random(o.psi_size)
    o.set_time_absorption(1.0)
    d_psi = dev(psi)
    ops.time_source(d_psi, dev(q), 3.5, d_psi)          # in place
    assert rel_err(d_psi.cpu().numpy(), o.time_source(psi, q, 3.5)) < 1e-12

    s_out = torch.empty(G * ne, **f64)
    ops.powerlaw_opacity(dT, nu, 10.0, -3.0, -0.5, s_out)
    assert rel_err(s_out.cpu().numpy(), o.powerlaw_opacity(T, nu, 10.0, -3.0, -0.5).reshape(-1)) < 1e-13


def _pair(G=4, cells=(4, 4), sn=4, dt=1e-2, method="fp64", tol=1e-13):
    mesh = M.cartesian(cells)
    quad = Q.level_symmetric(sn, 2)
    bounds, nu = log_spaced_groups(1e-2, 10.0, G)
    kw = dict(opacity=(10.0, -3.0, -0.5), cv=1.0, dt=dt, T0=1e-2, inflow={4: 1.0})
    gpu = LinearizedTRT(mesh, 1, quad, bounds, nu, method=method, tol=tol, **kw)
    cpu = OracleTRT(mesh, 1, quad, bounds, nu, **kw)
    return gpu, cpu


def test_trt_steps_match_oracle():
    # LinearizedTRTOperator::Mult step by step against the oracle's exact Schur solve
    gpu, cpu = _pair()
    for _ in range(3):
        r = gpu.step()
        cpu.step()
        assert r.converged
        assert rel_err(gpu.T.cpu().numpy(), cpu.T) < 1e-8
        assert rel_err(gpu.psi.cpu().numpy(), cpu.psi) < 1e-8


def test_trt_refinement_matches_fp64():
    # FP32 sweeps inside the Schur solve, FP64 residual: same steps to 1e-7
    a, _ = _pair(G=6, cells=(8, 8), method="fp64", tol=1e-10)
    b, _ = _pair(G=6, cells=(8, 8), method="ir", tol=1e-10)
    for _ in range(3):
        ra, rb = a.step(), b.step()
        assert ra.converged and rb.converged and rb.sweeps32 > 0
        assert rel_err(b.T.cpu().numpy(), a.T.cpu().numpy()) < 1e-7
