"""Parity of the fused FP32 inner operator and the double-float residual with the
CPU oracle, through the C ABI.

Tolerances: the FP32 sweep and its moments within 2e-5 relative (max norm) of
the FP64 oracle (as for the other FP32 sweeps); the double-float residual of
the oracle's FP64 solution below 1e-12 of |q| (an FP32 evaluation would leave
about 1e-7); double-float moments within 1e-13 of sum_a w_a |psi_a|; the
FP32-inner refinement at the FP64 solvers' 1e-8 residual."""
import numpy as np
import pytest

from allium_gb300._lib import AlliumError
from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator
from oracle.oracle import OracleSweep
from tests.helpers import problem, rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL32 = 2e-5

CASES = [
    # dim, cells, p, S_N, G, jitter
    (1, (14,), 0, 4, 2, 0.0),
    (1, (14,), 1, 6, 2, 0.0),
    (2, (9, 7), 0, 4, 1, 0.0),
    (2, (9, 7), 1, 6, 2, 0.2),
    (2, (16, 16), 1, 8, 1, 0.2),
    (3, (5, 4, 3), 0, 4, 2, 0.0),
    (3, (6, 5, 4), 1, 4, 2, 0.1),
    (3, (8, 8, 8), 1, 12, 1, 0.1),
]
IDS = [f"d{c[0]}p{c[2]}S{c[3]}G{c[4]}j{c[5]}" for c in CASES]


def fused_of_right(L, x):
    """RIGHT [G][Nw][Ndof] -> fused [G][Ne][Nw][n] (numpy)."""
    ne = L.mesh.num_elements
    return np.ascontiguousarray(x.reshape(L.G, L.Nw, ne, L.n).transpose(0, 2, 1, 3)).reshape(-1)


def right_of_fused(L, v):
    ne = L.mesh.num_elements
    return np.ascontiguousarray(v.reshape(L.G, ne, L.Nw, L.n).transpose(0, 2, 1, 3)).reshape(-1)


def setup(case, seed=5, tau=None):
    dim, cells, p, sn, G, jit = case
    mesh, quad, sig = problem(dim, cells, p, sn=sn, G=G, jitter=jit, seed=seed)
    L = InverseAdvectionOperator(mesh, p, quad, sig)
    o = OracleSweep(mesh, p, quad, sig)
    if tau is not None:
        L.SetTimeAbsorption(tau)
        o.set_time_absorption(tau)
    return L, o


@pytest.mark.parametrize("case", CASES + [CASES[6] + ("td",), CASES[3] + ("td",)],
                         ids=IDS + [IDS[6] + "-td", IDS[3] + "-td"])
def test_fused_sweep_matches_oracle(case):
    # "td": with a time absorption tau M_t (per-unit tables carry M_t)
    td = len(case) > 6
    L, o = setup(case[:6], tau=2.5 if td else None)
    rng = np.random.default_rng(3)
    nd = L.G * L.ndof
    iso = rng.uniform(0.0, 1.0, nd)
    src = rng.uniform(-0.2, 1.0, L.width)
    full = src + np.tile(iso.reshape(L.G, 1, L.ndof), (1, L.Nw, 1)).reshape(-1)
    ref = o.mult(full)
    phi_ref = o.moments(ref)
    d_iso = torch.tensor(iso, dtype=torch.float32, device="cuda")
    d_src = torch.tensor(fused_of_right(L, src), dtype=torch.float32, device="cuda")
    psi = torch.empty(L.width, dtype=torch.float32, device="cuda")
    phi = torch.full((nd,), 7.0, dtype=torch.float64, device="cuda")
    L.FusedMultF32(d_iso, d_src, psi, phi=phi, phi_mode=1)
    L.synchronize()
    got = right_of_fused(L, psi.cpu().numpy().astype(np.float64))
    assert rel_err(got, ref) < TOL32
    assert rel_err(phi.cpu().numpy(), phi_ref) < TOL32
    # the moments summed in plain FP32 (phi_mode 3, the inner operator's)
    phi3 = torch.full((nd,), 7.0, dtype=torch.float64, device="cuda")
    L.FusedMultF32(d_iso, d_src, psi, phi=phi3, phi_mode=3)
    L.synchronize()
    assert rel_err(phi3.cpu().numpy(), phi_ref) < TOL32
    # the same through the conversion back to RIGHT FP64
    back = torch.empty(L.width, dtype=torch.float64, device="cuda")
    L.FromFusedLayout(psi, None, back)
    assert rel_err(back.cpu().numpy(), ref) < TOL32


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_fused_schedule_orders_every_node_after_its_upwind_nodes(case):
    """The unit levels are at least as many as the node levels (a unit waits for
    the slowest of its angles) and a sweep with and without launch overlap agrees
    bit for bit."""
    L, o = setup(case)
    nl, _ = o.levels()
    n, unit = L.FusedLevels()
    assert unit == 1 and n >= nl
    src = torch.rand(L.width, dtype=torch.float32, device="cuda")
    a = torch.empty_like(src)
    b = torch.empty_like(src)
    L.FusedMultF32(None, src, a)
    L.SetFusedPDL(0)
    L.FusedMultF32(None, src, b)
    L.SetFusedPDL(1)
    L.synchronize()
    assert torch.equal(a, b)


@pytest.mark.parametrize("case", [CASES[3], CASES[7]], ids=[IDS[3], IDS[7]])
def test_fused_in_place_and_accumulation(case):
    L, o = setup(case)
    rng = np.random.default_rng(4)
    nd = L.G * L.ndof
    src = rng.uniform(0.0, 1.0, L.width)
    ref = o.mult(src)
    phi_ref = o.moments(ref)
    v = torch.tensor(fused_of_right(L, src), dtype=torch.float32, device="cuda")
    phi = torch.ones(nd, dtype=torch.float64, device="cuda")
    hi = torch.full((L.width,), 0.5, dtype=torch.float32, device="cuda")
    lo = torch.zeros(L.width, dtype=torch.float32, device="cuda")
    L.FusedMultF32(None, v, v, phi=phi, phi_mode=2, acc=(hi, lo))   # in place: source == psi
    L.synchronize()
    got = right_of_fused(L, v.cpu().numpy().astype(np.float64))
    assert rel_err(got, ref) < TOL32
    assert rel_err(phi.cpu().numpy() - 1.0, phi_ref) < TOL32
    acc = hi.double() + lo.double()
    assert rel_err(right_of_fused(L, acc.cpu().numpy()) - 0.5, ref) < TOL32
    # the accumulator is exact: hi + lo - 0.5 equals the FP32 psi to FP64 rounding
    assert float(torch.max(torch.abs(acc - 0.5 - v.double())).item()) <= 1e-12 * float(torch.max(torch.abs(v)).item())


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_isotropic_source_matches_scattering_source(case):
    L, o = setup(case)
    rng = np.random.default_rng(6)
    ne = L.mesh.num_elements
    sigma_s = rng.uniform(0.1, 0.9, (L.G, ne))
    phi = rng.uniform(0.0, 1.0, L.G * L.ndof)
    q_iso = rng.uniform(0.0, 1.0, L.G * L.ndof)
    qfull = np.tile(q_iso.reshape(L.G, 1, L.ndof), (1, L.Nw, 1)).reshape(-1)
    ref = o.scattering_source(sigma_s, phi, qfull).reshape(L.G, L.Nw, L.ndof)[:, 0, :].reshape(-1)
    hi = torch.empty(L.G * L.ndof, dtype=torch.float32, device="cuda")
    lo = torch.empty_like(hi)
    out = torch.empty_like(hi)
    L.IsotropicSource(sigma_s, torch.tensor(phi, device="cuda"), torch.tensor(q_iso, device="cuda"), out=out,
                      out_hi=hi, out_lo=lo)
    L.synchronize()
    dd = hi.double().cpu().numpy() + lo.double().cpu().numpy()
    assert rel_err(dd, ref) < 1e-13
    assert np.array_equal(out.cpu().numpy(), hi.cpu().numpy())


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_moments_df_of_fp64_psi(case):
    """D of a double-float psi matches the oracle's FP64 moments to 1e-13."""
    L, o = setup(case)
    psi = np.random.default_rng(7).uniform(-1.0, 1.0, L.width)
    hi = torch.empty(L.width, dtype=torch.float32, device="cuda")
    lo = torch.empty_like(hi)
    L.ToFusedLayout(torch.tensor(psi, device="cuda"), hi, lo)
    phi = torch.empty(L.G * L.ndof, dtype=torch.float64, device="cuda")
    L.MomentsDF(hi, lo, phi)
    L.synchronize()
    ref = o.moments(psi)
    assert float(np.max(np.abs(phi.cpu().numpy() - ref))) < 1e-13 * float(np.max(o.moments(np.abs(psi))))


@pytest.mark.parametrize("case", CASES + [CASES[6] + ("td",)], ids=IDS + [IDS[6] + "-td"])
def test_residual_df_of_fp64_solution(case):
    """r = q + D^T S phi - L psi at psi = the FP64 solution of L psi = q + D^T S phi
    (one FP64 oracle sweep with that source) is FP64 rounding: below 1e-12 |q|."""
    td = len(case) > 6
    L, o = setup(case[:6], tau=3.0 if td else None)
    rng = np.random.default_rng(8)
    ne = L.mesh.num_elements
    sigma_s = rng.uniform(0.1, 0.9, (L.G, ne))
    phi = rng.uniform(0.0, 1.0, L.G * L.ndof)
    q_iso = rng.uniform(0.0, 1.0, L.G * L.ndof)
    q_ang = rng.uniform(-0.3, 0.3, L.width)
    total = o.scattering_source(sigma_s, phi, np.tile(q_iso.reshape(L.G, 1, L.ndof), (1, L.Nw, 1)).reshape(-1) + q_ang)
    psi = o.mult(total)
    d = lambda x: torch.tensor(x, device="cuda")
    nd = L.G * L.ndof
    iso_hi = torch.empty(nd, dtype=torch.float32, device="cuda")
    iso_lo = torch.empty_like(iso_hi)
    L.IsotropicSource(sigma_s, d(phi), d(q_iso), out_hi=iso_hi, out_lo=iso_lo)
    f32 = lambda: torch.empty(L.width, dtype=torch.float32, device="cuda")
    p_hi, p_lo, q_hi, q_lo, r = f32(), f32(), f32(), f32(), f32()
    L.ToFusedLayout(d(psi), p_hi, p_lo)
    L.ToFusedLayout(d(q_ang), q_hi, q_lo)
    L.TransportResidualDF(iso_hi, iso_lo, p_hi, p_lo, r, q_hi, q_lo)
    L.synchronize()
    scale = np.max(np.abs(total))
    assert float(torch.max(torch.abs(r)).item()) < 1e-12 * scale
    # against the oracle's FP64 residual of a perturbed psi (the residual is not small there)
    pert = psi * (1.0 + 1e-3 * rng.standard_normal(psi.size))
    L.ToFusedLayout(d(pert), p_hi, p_lo)
    L.TransportResidualDF(iso_hi, iso_lo, p_hi, p_lo, r, q_hi, q_lo)
    L.synchronize()
    ref = total - o.apply_L(pert)
    got = right_of_fused(L, r.cpu().numpy().astype(np.float64))
    assert float(np.max(np.abs(got - ref))) < 1e-12 * scale + 1e-6 * float(np.max(np.abs(ref)))


@pytest.mark.parametrize("case", [CASES[4], CASES[7]], ids=[IDS[4], IDS[7]])
def test_refine_fused_reaches_fp64_solution(case):
    from allium_gb300.solvers import SchurOperator, refine_fused, solve_gmres, true_residual
    L, o = setup(case)
    rng = np.random.default_rng(9)
    ne = L.mesh.num_elements
    sigma_s = L._keep[6] * rng.uniform(0.5, 0.99, (L.G, ne))
    q = torch.from_numpy(FormTransportSource(L, rng.uniform(0.0, 1.0, (L.G, ne)))).cuda()
    res = refine_fused(L, sigma_s, q, tol=1e-8, inner_tol=1e-4)
    assert res.converged and res.sweeps64 == 0
    op = SchurOperator(L, sigma_s)
    b = op.rhs(q)
    assert true_residual(op, b, res.phi) < 2e-8
    plain = solve_gmres(SchurOperator(L, sigma_s), q, tol=1e-10)
    err = float((torch.max(torch.abs(res.phi - plain.phi)) / torch.max(torch.abs(plain.phi))).item())
    assert err < 1e-6


@pytest.mark.parametrize("directional", [False, True])
def test_refine_fused_many_outer_steps(directional):
    """A loose inner tolerance forces several outer steps, so the per-cell
    closed-form residual D^T S (dphi - d) is carried through more than one
    correction (and, with an inflow boundary, follows a psi-sized one)."""
    from allium_gb300.solvers import SchurOperator, refine_fused, true_residual
    L, o = setup(CASES[4])
    rng = np.random.default_rng(21)
    ne = L.mesh.num_elements
    sigma_s = L._keep[6] * rng.uniform(0.5, 0.99, (L.G, ne))
    inflow = np.ones((1, 8)) if directional else None
    q = torch.from_numpy(FormTransportSource(L, rng.uniform(0.0, 1.0, (L.G, ne)), inflow)).cuda()
    res = refine_fused(L, sigma_s, q, tol=1e-8, inner_tol=0.2, max_outer=60)
    assert res.converged and res.sweeps64 == 0
    assert res.iterations >= 3 and res.residuals_df == 1 and res.residual_updates == res.iterations - 1
    op = SchurOperator(L, sigma_s)
    assert true_residual(op, op.rhs(q), res.phi) < 2e-8


def test_refine_fused_with_directional_source():
    """An inflow boundary makes q direction dependent: the psi-sized part goes
    through the fused-layout double-float source."""
    from allium_gb300.solvers import SchurOperator, refine_fused, true_residual
    L, o = setup(CASES[4])
    ne = L.mesh.num_elements
    sigma_s = 0.8 * L._keep[6]
    q = torch.from_numpy(FormTransportSource(L, np.ones((1, ne)), np.ones((1, 8)))).cuda()
    res = refine_fused(L, sigma_s, q, tol=1e-8)
    assert res.converged
    op = SchurOperator(L, sigma_s)
    assert true_residual(op, op.rhs(q), res.phi) < 2e-8


def test_fused_rejects_unsupported():
    mesh, quad, sig = problem(2, (4, 4), 2, sn=4)
    L = InverseAdvectionOperator(mesh, 2, quad, sig)
    psi = torch.empty(L.width, dtype=torch.float32, device="cuda")
    with pytest.raises(AlliumError) as e:
        L.FusedMultF32(None, psi, psi)
    assert e.value.status == 7


@pytest.mark.parametrize("case", CASES + [CASES[6] + ("td",)], ids=IDS + [IDS[6] + "-td"])
def test_residual_update_f32(case):
    """From r = 0 the FP32 update gives D^T S D x - L x: the FP64 oracle's
    scattering source of D x minus its forward operator, to FP32 accuracy."""
    td = len(case) > 6
    L, o = setup(case[:6], tau=3.0 if td else None)
    rng = np.random.default_rng(10)
    ne = L.mesh.num_elements
    sigma_s = rng.uniform(0.1, 0.9, (L.G, ne))
    x = rng.uniform(-1.0, 1.0, L.width)
    ref = o.scattering_source(sigma_s, o.moments(x)) - o.apply_L(x)
    xf = torch.tensor(fused_of_right(L, x), dtype=torch.float32, device="cuda")
    phi = torch.empty(L.G * L.ndof, dtype=torch.float64, device="cuda")
    xh = torch.empty(L.width, dtype=torch.float32, device="cuda")
    L.ToFusedLayout(torch.tensor(x, device="cuda"), xh, torch.empty_like(xh))
    assert torch.equal(xh, xf)
    L.MomentsDF(xf, torch.zeros_like(xf), phi)
    iso = torch.empty(L.G * L.ndof, dtype=torch.float32, device="cuda")
    L.IsotropicSource(sigma_s, phi, None, out=iso)
    r = torch.zeros_like(xf)
    L.TransportResidualUpdateF32(iso, xf, r)
    L.synchronize()
    got = right_of_fused(L, r.cpu().numpy().astype(np.float64))
    scale = max(np.max(np.abs(o.apply_L(np.abs(x)))), 1e-300)
    assert float(np.max(np.abs(got - ref))) < 2e-6 * scale
