"""Parity of the CUDA sweep path with the CPU oracle, through the C ABI.

Tolerances: FP64 results within 1e-12 relative (max-norm over the vector) of
the oracle; integer levels and the moment sums bit-exact; the FP32 sweep within
2e-5 relative of the FP64 oracle."""
import math

import numpy as np
import pytest

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q
from allium_gb300._lib import AlliumError
from allium_gb300.sweep import (AdvectionOperator, DiscreteToMoment, FormTransportSource,
                                InverseAdvectionOperator, ScatteringSource)
from oracle.oracle import OracleSweep
from tests.helpers import mms_phi, mms_source, problem, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5

CASES = [
    # dim, cells, p, S_N, G, jitter, lump
    (1, (12,), 0, 4, 2, 0.0, 0),
    (1, (12,), 1, 4, 2, 0.0, 0),
    (1, (12,), 2, 4, 1, 0.0, 0),
    (1, (12,), 3, 4, 1, 0.0, 0),
    (2, (9, 7), 0, 4, 2, 0.0, 0),
    (2, (9, 7), 1, 6, 2, 0.0, 0),
    (2, (9, 7), 2, 4, 1, 0.0, 0),
    (2, (6, 5), 3, 4, 1, 0.0, 0),
    (2, (10, 10), 1, 8, 1, 0.2, 0),
    (2, (8, 8), 2, 6, 1, 0.2, 0),
    (2, (10, 10), 1, 4, 2, 0.0, 7),
    (3, (5, 4, 3), 0, 4, 1, 0.0, 0),
    (3, (5, 4, 3), 1, 4, 2, 0.0, 0),
    (3, (6, 6, 6), 1, 12, 1, 0.1, 0),
    (3, (4, 4, 4), 1, 4, 1, 0.0, 7),
    (3, (4, 3, 3), 2, 4, 1, 0.0, 0),
    (3, (4, 4, 4), 2, 6, 2, 0.1, 0),
    (3, (3, 3, 2), 3, 4, 1, 0.0, 0),
    (3, (3, 3, 3), 3, 2, 2, 0.1, 0),
]


def build(dim, cells, p, sn, G, jitter, lump, seed=11):
    mesh, quad, sig = problem(dim, cells, p, sn=sn, G=G, jitter=jitter, seed=seed, lump=lump)
    return mesh, quad, sig, OracleSweep(mesh, p, quad, sig, lump=lump), InverseAdvectionOperator(mesh, p, quad, sig, lump=lump)


@pytest.mark.parametrize("case", CASES, ids=[f"d{c[0]}p{c[2]}S{c[3]}G{c[4]}j{c[5]}l{c[6]}" for c in CASES])
def test_sweep_parity(case):
    mesh, quad, sig, o, L = build(*case)
    nl, lev_o = o.levels()
    assert L.num_levels == nl
    assert np.array_equal(L.levels(), lev_o)

    rng = np.random.default_rng(5)
    src = rng.random(o.psi_size)
    ref = o.mult(src)
    psi = np.empty_like(src)
    L.Mult(src, psi)
    assert rel_err(psi, ref) < TOL64

    # device pointers, in place
    d = torch.from_numpy(src).cuda()
    L.Mult(d, d)
    L.synchronize()
    assert np.array_equal(d.cpu().numpy(), psi)

    # FP32 sweep
    f = torch.from_numpy(src.astype(np.float32)).cuda()
    L.MultF32(f, f)
    L.synchronize()
    assert rel_err(f.cpu().numpy(), ref) < TOL32

    # FP32 sweep in the node-major layout
    if case[2] == 1:
        fn = torch.empty(o.psi_size, dtype=torch.float32, device="cuda")
        L.ToNodeLayoutF32(torch.from_numpy(src).cuda(), fn)
        L.MultF32Nodes(fn, fn)
        back64 = torch.empty(o.psi_size, dtype=torch.float64, device="cuda")
        L.FromNodeLayoutF32(fn, back64)
        L.synchronize()
        assert rel_err(back64.cpu().numpy(), ref) < TOL32

    # forward operator and L L^{-1} = I
    y = np.empty_like(src)
    AdvectionOperator(L).Mult(src, y)
    assert rel_err(y, o.apply_L(src)) < TOL64
    back = np.empty_like(src)
    L.Mult(y, back)
    assert np.linalg.norm(back - src) < 1e-12 * max(1.0, np.linalg.norm(src))

    # balance
    b = AdvectionOperator(L).ComputeBalance(ref)
    assert abs(b - o.balance(ref)) < TOL64 * abs(o.balance(ref))


@pytest.mark.parametrize("case", [c for c in CASES if c[2] == 1], ids=[f"d{c[0]}S{c[3]}G{c[4]}l{c[6]}" for c in CASES if c[2] == 1])
def test_factor_cache(case):
    # the FP64 factor cache (stored local inverses) against the plain sweep and
    # the oracle; repeated Mults replay the same captured launches bit for bit
    mesh, quad, sig, o, L = build(*case)
    src = np.random.default_rng(8).random(o.psi_size)
    L.SetFactorCache(0)
    plain = np.empty_like(src)
    L.Mult(src, plain)
    L.SetFactorCache(1)
    d_src = torch.from_numpy(src).cuda()
    out = torch.empty_like(d_src)
    L.Mult(d_src, out)          # factors and stores the inverses
    first = out.cpu().numpy()
    L.Mult(d_src, out)          # applies the stored inverses
    second = out.cpu().numpy()
    L.Mult(d_src, out)
    L.synchronize()
    assert np.array_equal(first, second) and np.array_equal(second, out.cpu().numpy())
    assert rel_err(first, plain) < TOL64
    assert rel_err(first, o.mult(src)) < TOL64
    # new cross sections invalidate the stored inverses
    sig2 = sig * 2.0 + 0.3
    L.AssembleLocalMatrices(sig2)
    L.Mult(d_src, out)
    L.synchronize()
    assert rel_err(out.cpu().numpy(), OracleSweep(mesh, case[2], quad, sig2, lump=case[6]).mult(src)) < TOL64


@pytest.mark.parametrize("case", CASES[:: 2], ids=[f"d{c[0]}p{c[2]}" for c in CASES[:: 2]])
def test_moments_bit_exact(case):
    mesh, quad, sig, o, L = build(*case)
    rng = np.random.default_rng(9)
    psi = rng.random(o.psi_size)
    for nmom in (1, mesh.dim + 1):
        D = DiscreteToMoment(L, nmom)
        phi = np.empty(D.height)
        D.Mult(psi, phi)
        assert np.array_equal(phi, o.moments(psi, nmom))
        out = np.empty(o.psi_size)
        D.MultTranspose(phi, out)
        assert np.array_equal(out, o.moments_transpose(phi, nmom))
        acc = psi.copy()
        D.AddMultTranspose(phi, acc, 0.7)
        assert np.array_equal(acc, o.moments_transpose(phi, nmom, psi=psi.copy(), alpha=0.7, add=True))


@pytest.mark.parametrize("case", CASES[1:: 2], ids=[f"d{c[0]}p{c[2]}" for c in CASES[1:: 2]])
def test_sources(case):
    mesh, quad, sig, o, L = build(*case)
    G = sig.shape[0]
    rng = np.random.default_rng(4)
    q = rng.random((G, mesh.num_elements))
    inflow = rng.random((G, 8))
    assert rel_err(FormTransportSource(L, q, inflow), o.form_source(q_cell=q, inflow=inflow)) < 1e-13
    phi = rng.random(G * L.ndof)
    sig_s = rng.random((G, mesh.num_elements))
    qf = rng.random(o.psi_size)
    assert rel_err(ScatteringSource(L, sig_s, phi, qf), o.scattering_source(sig_s, phi, qf)) < 1e-13


@pytest.mark.parametrize("case", CASES[1:: 3], ids=[f"d{c[0]}p{c[2]}" for c in CASES[1:: 3]])
def test_general_source(case):
    # point densities and direction-dependent inflow: constant data reproduce
    # allium_sweep_form_source bit for bit; a density varying in x and with the
    # direction (a PhaseSpaceCoefficient) matches the oracle's integration
    from allium_gb300.sweep import FormTransportSourceGeneral, SourcePoints
    mesh, quad, sig, o, L = build(*case)
    G, dim = sig.shape[0], mesh.dim
    rng = np.random.default_rng(8)
    q = rng.random((G, mesh.num_elements))
    inflow = rng.random((G, 8))
    x = SourcePoints(L)
    assert x.shape[0] == mesh.num_elements and x.shape[2] == dim
    lo, hi = mesh.vertices.min(0), mesh.vertices.max(0)
    assert np.all(x >= lo - 1e-12) and np.all(x <= hi + 1e-12)
    ref = FormTransportSource(L, q, inflow)
    gen = FormTransportSourceGeneral(L, lambda xx, g: np.repeat(q[g][:, None], xx.shape[1], axis=1),
                                     np.repeat(inflow[:, None, :], quad.size, axis=1))
    assert np.array_equal(gen, ref)

    def qx(xx, om, g):   # the oracle's callback form, one point at a time
        return (1.0 + g) * (2.0 + math.sin(3.0 * xx[0]) * (1.0 + 0.5 * om[0]) + (xx[1] if dim > 1 else 0.0) ** 2)

    def qv(xx, om, g):   # the same, vectorised over the rule points
        y = xx[..., 1] ** 2 if dim > 1 else 0.0
        return (1.0 + g) * (2.0 + np.sin(3.0 * xx[..., 0]) * (1.0 + 0.5 * om[0]) + y)

    fin = rng.random((G, quad.size, 8))
    gen = FormTransportSourceGeneral(L, qv, fin, per_direction=True)
    want = o.form_source(qfn=qx, inflow_fn=lambda xx, om, g, attr: fin[g, _angle(quad, om), attr])
    assert rel_err(gen, want) < 1e-13


def _angle(quad, om):
    """Index of the quadrature direction om (a ctypes pointer from the oracle)."""
    v = np.array([om[i] for i in range(quad.dim)])
    return int(np.argmin(np.abs(quad.omega - v[None, :]).sum(1)))


@pytest.mark.parametrize("dim,cells", [(2, (9, 7)), (3, (6, 5, 4))])
def test_time_absorption(dim, cells):
    mesh, quad, sig, o, L = build(dim, cells, 1, 4, 2, 0.2, 0)
    o.set_time_absorption(3.7)
    L.SetTimeAbsorption(3.7)
    src = np.random.default_rng(1).random(o.psi_size)
    psi = np.empty_like(src)
    L.Mult(src, psi)
    assert rel_err(psi, o.mult(src)) < TOL64
    y = np.empty_like(src)
    AdvectionOperator(L).Mult(src, y)
    assert rel_err(y, o.apply_L(src)) < TOL64
    # new cross sections (AssembleLocalMatrices) keep the time absorption
    sig2 = sig * 0.5 + 0.1
    o2 = OracleSweep(mesh, 1, quad, sig2)
    o2.set_time_absorption(3.7)
    L.AssembleLocalMatrices(sig2)
    L.Mult(src, psi)
    assert rel_err(psi, o2.mult(src)) < TOL64


@pytest.mark.parametrize("dim,cells,p", [(1, (10,), 3), (2, (10, 10), 2), (2, (10, 10), 3), (3, (6, 6, 6), 1),
                                         (3, (10, 10, 10), 0), (3, (3, 3, 3), 2), (3, (3, 3, 3), 3)])
def test_constant_solution(dim, cells, p):
    # test_sweep.cpp:7-108 on the GPU: sigma = 0, q = 0, unit inflow -> psi == 1
    mesh = M.cartesian(cells)
    L = InverseAdvectionOperator(mesh, p, Q.level_symmetric(4, dim), np.zeros((2, mesh.num_elements)))
    src = FormTransportSource(L, None, np.ones((2, 8)))
    psi = np.empty_like(src)
    L.Mult(src, psi)
    assert np.max(np.abs(psi - 1.0)) < 1e-10


def _mms_error_gpu(ne, p, lump):
    mesh = M.cartesian((ne, ne))
    quad = Q.level_symmetric(6, 2)
    total, scat = 1.0, 0.25
    sig = np.full((1, mesh.num_elements), total)
    o = OracleSweep(mesh, p, quad, sig, lump=lump)   # builds the manufactured source and measures the error
    src = torch.from_numpy(o.form_source(qfn=mms_source(total, scat),
                                         inflow_fn=lambda x, om, g, a: 2.0 / 4 / math.pi)).cuda()
    L = InverseAdvectionOperator(mesh, p, quad, sig, lump=lump)
    D = DiscreteToMoment(L)
    sig_s = np.full((1, mesh.num_elements), scat)
    psi = torch.empty_like(src)
    phi_old = torch.zeros(L.ndof, dtype=torch.float64, device="cuda")
    phi = torch.empty_like(phi_old)
    for _ in range(200):
        ScatteringSource(L, sig_s, phi_old, src, psi)
        L.Mult(psi, psi)
        D.Mult(psi, phi)
        L.synchronize()
        norm = torch.linalg.norm(phi_old - phi).item()
        phi_old.copy_(phi)
        if norm < 1e-10:
            break
    return o.l2_error(phi.cpu().numpy(), 0, 0, mms_phi)


@pytest.mark.parametrize("p,lump", [(1, 0), (2, 0), (3, 0), (1, 7)])
def test_transport_mms_order(p, lump):
    # test_transport_mms.cpp:89-197 with the GPU sweep inside source iteration
    e1 = _mms_error_gpu(10, p, lump)
    e2 = _mms_error_gpu(20, p, lump)
    assert abs(math.log2(e1 / e2) - (p + 1)) < 0.2


def test_chive_2d_workload_parity():
    # 64 x 64 quads, p = 1, S8 (40 directions), sigma_t = 1, q = 1, vacuum
    mesh = M.cartesian((64, 64))
    quad = Q.level_symmetric(8, 2)
    sig = np.ones((1, mesh.num_elements))
    o = OracleSweep(mesh, 1, quad, sig)
    L = InverseAdvectionOperator(mesh, 1, quad, sig)
    src = FormTransportSource(L, np.ones((1, mesh.num_elements)))
    assert rel_err(src, o.form_source(q_cell=np.ones((1, mesh.num_elements)))) < 1e-13
    psi = np.empty_like(src)
    L.Mult(src, psi)
    assert rel_err(psi, o.mult(src)) < TOL64
    assert L.num_levels == 127


def test_jittered_hex_s12_parity():
    # the 3D workload's ingredients at 12^3: jittered hexes, S12 (168 directions), log-uniform sigma
    mesh, quad, sig, o, L = build(3, (12, 12, 12), 1, 12, 1, 0.1, 0, seed=20261203)
    nl, lev = o.levels()
    assert np.array_equal(L.levels(), lev)
    src = np.random.default_rng(2).random(o.psi_size)
    psi = np.empty_like(src)
    L.Mult(src, psi)
    assert rel_err(psi, o.mult(src)) < TOL64


def test_full_size_3d_properties():
    # 64^3 jittered hexes, p = 1, S12: size-independent checks at full size.
    mesh, quad, sig = problem(3, (64, 64, 64), 1, sn=12, G=1, jitter=0.1, seed=20261203)
    L = InverseAdvectionOperator(mesh, 1, quad, sig)
    n = L.width
    q = torch.from_numpy(FormTransportSource(L, np.random.default_rng(3).random((1, mesh.num_elements)))).cuda()
    psi = torch.empty_like(q)
    L.Mult(q, psi)
    y = torch.empty_like(q)
    AdvectionOperator(L).Mult(psi, y)
    L.synchronize()
    # L (L^{-1} q) = q
    assert (torch.linalg.norm(y - q) / torch.linalg.norm(q)).item() < 1e-12
    # vacuum balance: absorption + leakage = total source
    total = float((q.view(quad.size, -1).sum(1).cpu().numpy() * quad.weights).sum())
    bal = AdvectionOperator(L).ComputeBalance(psi)
    assert abs(bal - total) < 1e-11 * abs(total)
    # FP32 sweep against the FP64 sweep
    f = q.float()
    L.MultF32(f, f)
    L.synchronize()
    assert (torch.max(torch.abs(f.double() - psi)) / torch.max(torch.abs(psi))).item() < TOL32
    del q, psi, y, f
    assert n == 64 ** 3 * 8 * 168


def test_cycle_is_reported():
    # +-0.2h jitter with S12's grazing directions gives a cyclic upwind graph;
    # the reference aborts (sweep.cpp:205-208), the library returns NOT_DAG
    mesh, quad, sig = problem(3, (16, 16, 16), 1, sn=12, jitter=0.2, seed=20261203)
    assert OracleSweep(mesh, 1, quad, sig).levels()[0] == -1
    with pytest.raises(AlliumError) as e:
        InverseAdvectionOperator(mesh, 1, quad, sig)
    assert e.value.status == 2


@pytest.mark.parametrize("case", [c for c in CASES if c[2] <= 1], ids=[f"d{c[0]}p{c[2]}S{c[3]}G{c[4]}" for c in CASES if c[2] <= 1])
def test_schedules_agree(case):
    # the persistent dataflow launch and one launch per level run the same
    # per-node arithmetic: results are identical bit for bit
    mesh, quad, sig, o, L = build(*case)
    src = torch.from_numpy(np.random.default_rng(6).random(o.psi_size)).cuda()
    outs = {}
    for sched in (0, 1):
        L.SetSchedule(sched)
        for cache in (0, 1):
            L.SetFactorCache(cache)
            y = torch.empty_like(src)
            L.Mult(src, y)
            y32 = torch.empty(o.psi_size, dtype=torch.float32, device="cuda")
            L.MultF32(src.float(), y32)
            yn = torch.empty_like(y32)
            L.ToNodeLayoutF32(src, yn)
            L.MultF32Nodes(yn, yn)
            L.synchronize()
            outs[(sched, cache)] = (y.cpu().numpy(), y32.cpu().numpy(), yn.cpu().numpy())
    for cache in (0, 1):
        for k in range(3):
            assert np.array_equal(outs[(0, cache)][k], outs[(1, cache)][k])
    assert rel_err(outs[(1, 1)][0], o.mult(src.cpu().numpy())) < TOL64


def test_bounded_wait_reports_timeout():
    # failure detection without a GPU fault: a wait on a flag nothing sets gives
    # up after its poll limit, the call returns TIMEOUT and the device still works
    mesh, quad, sig = problem(2, (6, 6), 1)
    L = InverseAdvectionOperator(mesh, 1, quad, sig)
    from allium_gb300 import _lib
    st = _lib.lib().allium_sweep_selftest_wait(L.h, 1000)
    assert st == 4
    src = np.random.default_rng(1).random(L.width)
    psi = np.empty_like(src)
    L.Mult(src, psi)
    o = OracleSweep(mesh, 1, quad, sig)
    assert rel_err(psi, o.mult(src)) < TOL64


@pytest.mark.parametrize("dim,cells", [(2, (16, 16)), (3, (8, 8, 8))])
@pytest.mark.parametrize("kind", [1, 2, 3, 4])
def test_fixup_parity(dim, cells, kind):
    # optically thick cells next to a point source: p = 1 DG fluxes dip below
    # zero; the zero (1), zero-and-scale (2), Ryosuke (3) and local-optimization
    # (4) fixups of src/fixup.cpp remove them
    mesh = M.cartesian(cells, jitter=0.1, seed=2)
    quad = Q.level_symmetric(4, dim)
    sig = np.full((2, mesh.num_elements), 50.0)
    sig[1] *= 0.2
    q = np.zeros((2, mesh.num_elements))
    q[:, 0] = 100.0
    o = OracleSweep(mesh, 1, quad, sig)
    L = InverseAdvectionOperator(mesh, 1, quad, sig)
    src = FormTransportSource(L, q)
    plain = np.empty_like(src)
    L.Mult(src, plain)
    assert plain.min() < 0
    o.set_fixup(kind, 0.0)
    L.SetFixup(kind, 0.0)
    ref = o.mult(src)
    psi = np.empty_like(src)
    if o.fixup_unsupported():
        # Ryosuke with more than three positive entries: the reference aborts
        with pytest.raises(AlliumError) as e:
            L.Mult(src, psi)
        assert e.value.status == 7
        L.SetFixup(0)
        return
    L.Mult(src, psi)
    assert psi.min() >= 0.0
    assert rel_err(psi, ref) < 1e-11
    if kind >= 2 and o.fixup_counts()[1] == 0:   # the conservative fixups keep the balance
        assert abs(AdvectionOperator(L).ComputeBalance(psi) - o.balance(plain)) < 1e-9 * abs(o.balance(plain))
    applied, failed = L.FixupCounts(reset=True)
    ra, rf = o.fixup_counts()
    assert abs(applied - ra) <= max(3, ra // 100) and abs(failed - rf) <= max(3, rf // 100)
    f32 = torch.from_numpy(src.astype(np.float32)).cuda()
    L.MultF32(f32, f32)
    L.synchronize()
    assert f32.min().item() >= 0.0
    L.SetFixup(0)
    L.Mult(src, psi)
    assert np.array_equal(psi, plain)


@pytest.mark.parametrize("dim,cells,p", [(2, (10, 10), 2), (2, (8, 8), 3), (3, (4, 4, 4), 2), (3, (3, 3, 3), 3)])
@pytest.mark.parametrize("kind", [1, 2, 3, 4])
def test_fixup_high_order(dim, cells, p, kind):
    # the fixups on the lane-per-row (9..27 DOFs) and block-per-node (64 DOFs)
    # kernels: one lane of the team applies them to the staged solution
    mesh = M.cartesian(cells, jitter=0.1, seed=2)
    quad = Q.level_symmetric(4, dim)
    sig = np.full((1, mesh.num_elements), 50.0)
    q = np.zeros((1, mesh.num_elements))
    q[:, 0] = 100.0
    o = OracleSweep(mesh, p, quad, sig)
    L = InverseAdvectionOperator(mesh, p, quad, sig)
    src = FormTransportSource(L, q)
    plain = np.empty_like(src)
    L.Mult(src, plain)
    assert plain.min() < 0
    o.set_fixup(kind, 0.0)
    L.SetFixup(kind, 0.0)
    ref = o.mult(src)
    psi = np.empty_like(src)
    if o.fixup_unsupported():
        with pytest.raises(AlliumError) as e:
            L.Mult(src, psi)
        assert e.value.status == 7
    else:
        L.Mult(src, psi)
        assert psi.min() >= 0.0
        assert rel_err(psi, ref) < 1e-10
        applied, failed = L.FixupCounts(reset=True)
        ra, rf = o.fixup_counts()
        assert abs(applied - ra) <= max(3, ra // 100) and abs(failed - rf) <= max(3, rf // 100)
    L.SetFixup(0)
    L.Mult(src, psi)
    assert np.array_equal(psi, plain)


def test_errors_are_reported():
    mesh, quad, sig = problem(2, (4, 4), 1)
    m3, q3, s3 = problem(3, (2, 2, 2), 3)
    with pytest.raises(AlliumError) as e:
        InverseAdvectionOperator(m3, 4, q3, s3)   # p > 3
    assert e.value.status == 7
    L = InverseAdvectionOperator(mesh, 1, quad, sig)
    x = np.zeros(L.width)
    with pytest.raises(AlliumError) as e:
        AdvectionOperator(L).Mult(x, x)
    assert e.value.status == 1
    with pytest.raises(ValueError):
        L.Mult(np.zeros(3), np.zeros(3))


# --------------------------------------------------------------- reflective boundaries
REFL_CASES = [
    # dim, cells, p, S_N, G, reflective attributes
    (1, (12,), 1, 4, 2, (2,)),
    (2, (9, 7), 0, 4, 2, (2,)),
    (2, (9, 7), 1, 6, 2, (2, 3)),
    (2, (8, 6), 2, 4, 1, (1, 2)),
    (2, (6, 5), 3, 4, 1, (3,)),
    (3, (5, 4, 3), 1, 4, 2, (3, 4, 6)),
    (3, (6, 6, 6), 1, 12, 1, (1, 2, 5)),
    (3, (4, 3, 3), 2, 4, 1, (3,)),
    (3, (3, 3, 2), 3, 4, 1, (2, 5)),
]


@pytest.mark.parametrize("case", REFL_CASES, ids=[f"d{c[0]}p{c[2]}S{c[3]}r{''.join(map(str, c[5]))}" for c in REFL_CASES])
def test_reflective_parity(case):
    # reflective edges (sweep.cpp:177-195) and the reflected-angle face term
    # (sweep.cpp:432-437) against the oracle: levels exact, FP64 to 1e-12
    dim, cells, p, sn, G, attrs = case
    mesh, quad, sig = problem(dim, cells, p, sn=sn, G=G, seed=13)
    o = OracleSweep(mesh, p, quad, sig)
    o.set_reflective(attrs)
    L = InverseAdvectionOperator(mesh, p, quad, sig, bc={a: "reflective" for a in attrs})
    nl, lev = o.levels()
    assert L.num_levels == nl and np.array_equal(L.levels(), lev)
    src = np.random.default_rng(3).random(o.psi_size)
    ref = o.mult(src)
    psi = np.empty_like(src)
    L.Mult(src, psi)
    assert rel_err(psi, ref) < TOL64
    d = torch.from_numpy(src).cuda()
    L.Mult(d, d)
    f = torch.from_numpy(src.astype(np.float32)).cuda()
    L.MultF32(f, f)
    L.synchronize()
    assert np.array_equal(d.cpu().numpy(), psi)
    assert rel_err(f.cpu().numpy(), ref) < TOL32
    if p == 1:
        L.SetFactorCache(1)
        L.Mult(d.copy_(torch.from_numpy(src)), d)
        L.Mult(torch.from_numpy(src).cuda(), d)
        L.synchronize()
        assert rel_err(d.cpu().numpy(), ref) < TOL64
        with pytest.raises(AlliumError) as e:
            fn = torch.empty(o.psi_size, dtype=torch.float32, device="cuda")
            L.MultF32Nodes(fn, fn)
        assert e.value.status == 7
    # the forward operator and the balance ignore the reflective coupling, as
    # AdvectionOperator::Mult / ComputeBalance do (sweep.cpp:1246-1462)
    y = np.empty_like(src)
    AdvectionOperator(L).Mult(src, y)
    assert rel_err(y, o.apply_L(src)) < TOL64
    assert abs(AdvectionOperator(L).ComputeBalance(ref) - o.balance(ref)) < TOL64 * abs(o.balance(ref))


def test_reflective_mirror_3d():
    # 16 x 8 x 8 symmetric box against its 8^3 half with a reflective x = 1 face
    full = M.cartesian((16, 8, 8), extents=(2.0, 1.0, 1.0))
    half = M.cartesian((8, 8, 8))
    quad = Q.level_symmetric(8, 3)

    def centres(m):
        return m.vertices[m.elements].mean(axis=1)

    def sig(m):
        c = centres(m)
        return (1.0 + 3.0 * np.abs(c[:, 0] - 1.0) + c[:, 1] ** 2 + c[:, 2])[None, :]

    def q(m):
        c = centres(m)
        return (1.0 + c[:, 0] * (2.0 - c[:, 0]) + 0.5 * c[:, 1])[None, :]

    Lf = InverseAdvectionOperator(full, 1, quad, sig(full))
    Lh = InverseAdvectionOperator(half, 1, quad, sig(half), bc={3: "reflective"})
    pf = np.empty(Lf.width)
    ph = np.empty(Lh.width)
    Lf.Mult(FormTransportSource(Lf, q(full)), pf)
    Lh.Mult(FormTransportSource(Lh, q(half)), ph)
    cf, ch = centres(full), centres(half)
    match = np.array([np.argmin(np.linalg.norm(cf - c, axis=1)) for c in ch])
    pf = pf.reshape(1, quad.size, full.num_elements, 8)[:, :, match, :]
    ph = ph.reshape(1, quad.size, half.num_elements, 8)
    assert np.max(np.abs(pf - ph)) <= 1e-12 * np.max(np.abs(pf))


def test_reflective_errors():
    quad = Q.level_symmetric(4, 2)
    mesh = M.cartesian((3, 3))
    c, s = math.cos(0.3), math.sin(0.3)
    mesh.vertices[:] = mesh.vertices @ np.array([[c, s], [-s, c]])
    with pytest.raises(AlliumError) as e:
        InverseAdvectionOperator(mesh, 1, quad, np.ones((1, 9)), bc={2: "reflective"})
    assert e.value.status == 8
    mesh, quad, sig = problem(2, (4, 3), 1)
    with pytest.raises(AlliumError) as e:
        InverseAdvectionOperator(mesh, 1, quad, sig, bc={2: "reflective", 4: "reflective"})
    assert e.value.status == 2


def test_autotune_keeps_results():
    # every launch configuration computes each node with the same arithmetic
    from allium_gb300.autotune import autotune
    mesh, quad, sig = problem(3, (8, 8, 8), 1, sn=6, jitter=0.1, seed=3)
    L = InverseAdvectionOperator(mesh, 1, quad, sig)
    src = torch.rand(L.width, dtype=torch.float64, device="cuda")
    a = torch.empty_like(src)
    L.Mult(src, a)
    f = torch.empty(L.width, dtype=torch.float32, device="cuda")
    L.ToNodeLayoutF32(src, f)
    fa = torch.empty_like(f)
    L.MultF32Nodes(f, fa)
    res = autotune(L, reps=2)
    assert res["fp64"]["block"] in (32, 64, 128) and len(res["trials"]) >= 4
    b = torch.empty_like(src)
    L.Mult(src, b)
    fb = torch.empty_like(f)
    L.MultF32Nodes(f, fb)
    L.synchronize()
    assert torch.equal(a, b) and torch.equal(fa, fb)


@pytest.mark.parametrize("dim,cells,sn,G", [(3, (6, 5, 4), 6, 2), (2, (12, 9), 8, 3)])
def test_f32_inverse_layouts(dim, cells, sn, G):
    # both orders of the FP32 inverse copy give the same node-major FP32 sweep,
    # within the FP32 tolerance of the oracle
    mesh, quad, sig, o, L = build(dim, cells, 1, sn, G, 0.1, 0)
    src = np.random.default_rng(2).random(o.psi_size)
    ref = o.mult(src)
    f = torch.empty(L.width, dtype=torch.float32, device="cuda")
    out = {}
    for layout in (1, 0, 1):
        L.SetF32InverseLayout(layout)
        L.ToNodeLayoutF32(torch.from_numpy(src).cuda(), f)
        L.MultF32Nodes(f, f)
        back = torch.empty(L.width, dtype=torch.float64, device="cuda")
        L.FromNodeLayoutF32(f, back)
        L.synchronize()
        assert rel_err(back.cpu().numpy(), ref) < TOL32
        if layout in out:
            assert torch.equal(back, out[layout])
        out[layout] = back
    assert torch.equal(out[0], out[1])
    with pytest.raises(AlliumError):
        L.SetF32InverseLayout(2)


@pytest.mark.parametrize("dim,cells,sn,G", [(3, (6, 5, 4), 6, 2), (2, (12, 9), 8, 3)])
def test_pinned_host_mult_pipeline(dim, cells, sn, G):
    # page-locked host vectors take the chunked copy/sweep/copy pipeline; every
    # node is computed with the same arithmetic, so psi matches the device Mult
    # bit for bit, also in place
    mesh, quad, sig = problem(dim, cells, 1, sn=sn, G=G, jitter=0.1, seed=5)
    L = InverseAdvectionOperator(mesh, 1, quad, sig)
    src = torch.rand(L.width, dtype=torch.float64)
    ref = torch.empty(L.width, dtype=torch.float64, device="cuda")
    L.Mult(src.cuda(), ref)
    L.synchronize()
    h_src = src.pin_memory()
    h_psi = torch.empty_like(src).pin_memory()
    for _ in range(2):
        L.Mult(h_src, h_psi)
        assert torch.equal(h_psi, ref.cpu())
    h_io = src.clone().pin_memory()
    L.Mult(h_io, h_io)
    assert torch.equal(h_io, ref.cpu())
    # the pipeline's shape (slices, compute streams) changes nothing
    for chunks, streams, taper in [(2, 1, 0), (4, 4, 1), (16, 3, 2), (32, 2, 3), (8, 4, 3)]:
        L.SetPipeline(chunks, streams, taper)
        h_psi.zero_()
        L.Mult(h_src, h_psi)
        assert torch.equal(h_psi, ref.cpu()), (chunks, streams, taper)
    with pytest.raises(AlliumError):
        L.SetPipeline(1, 2)
    with pytest.raises(AlliumError):
        L.SetPipeline(8, 5)
    with pytest.raises(AlliumError):
        L.SetPipeline(8, 4, 4)


@pytest.mark.parametrize("dim,cells,p,sn,G", [(2, (9, 7), 1, 4, 3), (3, (4, 3, 3), 2, 4, 2), (1, (33,), 0, 8, 1)])
def test_left_layout(dim, cells, p, sn, G):
    # a caller built with the LEFT layout (tvector.hpp:47-53) converts at the
    # boundary: relayout -> Mult -> relayout equals the oracle's sweep in LEFT
    from oracle.oracle import relayout
    mesh, quad, sig, o, L = build(dim, cells, p, sn, G, 0.0, 0)
    rng = np.random.default_rng(3)
    src_r = rng.random(o.psi_size)
    ref_left = relayout(o.mult(src_r), G, quad.size, L.ndof, to_left=True)
    src_left = torch.from_numpy(relayout(src_r, G, quad.size, L.ndof, to_left=True)).cuda()
    right = torch.empty_like(src_left)
    L.Relayout(src_left, L.LEFT, right, L.RIGHT)
    L.synchronize()
    assert np.array_equal(right.cpu().numpy(), src_r)   # bit-exact permutation
    L.Mult(right, right)
    out_left = torch.empty_like(right)
    L.Relayout(right, L.RIGHT, out_left, L.LEFT)
    L.synchronize()
    assert rel_err(out_left.cpu().numpy(), ref_left) < TOL64
    same = torch.empty_like(right)
    L.Relayout(right, L.RIGHT, same, L.RIGHT)
    L.synchronize()
    assert torch.equal(same, right)
    with pytest.raises(AlliumError):
        L.Relayout(right, L.RIGHT, right, L.LEFT)      # in place is refused
    with pytest.raises(AlliumError):
        L.Relayout(right, 2, out_left, L.LEFT)
