"""Pins the CPU oracle against the reference's own known answers and identities
(test/test_integrators.cpp, test/test_sweep.cpp, test/test_transport_mms.cpp,
test/test_angle_quad.cpp).  CPU only."""
import math

import numpy as np
import pytest

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q
from oracle.oracle import OracleSweep
from tests.helpers import mms_phi, mms_source, problem


@pytest.mark.parametrize("lump", [0, 7])
def test_face_blocks_known_answer(lump):
    # test_integrators.cpp:269-347: 2x1 quads, p = 1 Lobatto, interior face x = 1/2
    mesh = M.cartesian((2, 1))
    o = OracleSweep(mesh, 1, Q.level_symmetric(4, 2), np.ones((1, 2)), lump=lump)
    faces = [f for f in range(o.num_faces()) if o.face_info(f)[0][2] >= 0]
    assert len(faces) == 1
    F = o.face_matrices(faces[0])
    a, b = (0.5, 0.0) if lump else (1.0 / 3, 1.0 / 6)
    ex11 = np.zeros((4, 4)); ex11[1, 1] = ex11[3, 3] = a; ex11[1, 3] = ex11[3, 1] = b
    ex12 = np.zeros((4, 4)); ex12[1, 0] = ex12[3, 2] = a; ex12[1, 2] = ex12[3, 0] = b
    ex22 = np.zeros((4, 4)); ex22[0, 0] = ex22[2, 2] = a; ex22[0, 2] = ex22[2, 0] = b
    assert np.linalg.norm(F[0, 0] - ex11) < 1e-14
    assert np.linalg.norm(F[0, 1] - ex12) < 1e-14
    assert np.linalg.norm(F[1, 0].T - F[0, 1]) < 1e-14
    assert np.linalg.norm(F[1, 1] - ex22) < 1e-14


CONST_CASES = [(1, (10,), 0, 0), (1, (10,), 1, 0), (1, (10,), 1, 7), (1, (10,), 2, 0), (1, (10,), 3, 0),
               (2, (10, 10), 0, 0), (2, (10, 10), 1, 0), (2, (10, 10), 1, 7), (2, (10, 10), 2, 0),
               (2, (6, 6), 3, 0),
               (3, (10, 10, 10), 0, 0), (3, (6, 6, 6), 1, 0), (3, (6, 6, 6), 1, 7), (3, (3, 3, 3), 2, 0),
               (3, (3, 3, 2), 3, 0)]


@pytest.mark.parametrize("dim,cells,p,lump", CONST_CASES)
def test_constant_solution(dim, cells, p, lump):
    # test_sweep.cpp:7-108: sigma = 0, q = 0, unit inflow everywhere -> psi == 1
    mesh = M.cartesian(cells)
    quad = Q.level_symmetric(4, dim)
    o = OracleSweep(mesh, p, quad, np.zeros((2, mesh.num_elements)), lump=lump)
    src = o.form_source(inflow=np.ones((2, 8)))
    psi = o.mult(src)
    assert np.max(np.abs(psi - 1.0)) < 1e-10


@pytest.mark.parametrize("dim,cells,lump,p", [(1, (10,), 0, 1), (2, (3, 3), 0, 1), (3, (3, 3, 3), 0, 1),
                                              (1, (10,), 7, 1), (2, (3, 3), 7, 1), (3, (3, 3, 3), 7, 1),
                                              (3, (2, 2, 2), 0, 3)])
def test_L_Linv_identity(dim, cells, lump, p):
    # test_sweep.cpp:289-361: || L^{-1} (L x) - x || < 1e-12, sigma = (1, 0.5); also 3D p = 3
    mesh = M.cartesian(cells)
    quad = Q.level_symmetric(4, dim)
    sig = np.array([[1.0], [0.5]]) * np.ones((2, mesh.num_elements))
    o = OracleSweep(mesh, p, quad, sig, lump=lump)
    x = np.random.default_rng(12345).random(o.psi_size)
    psi = o.mult(o.apply_L(x))
    assert np.linalg.norm(psi - x) < 1e-12


def _exp_error(cells, p, exact, lump=0):
    mesh = M.cartesian(cells)
    dim = mesh.dim
    quad = Q.single_angle(Q.level_symmetric(4, dim), 0)
    sig = np.array([[1.0], [0.5]]) * np.ones((2, mesh.num_elements))
    o = OracleSweep(mesh, p, quad, sig, lump=lump)
    src = o.form_source(inflow=np.ones((2, 8)))
    psi = o.mult(src)
    return sum(o.l2_error(psi, g, 0, lambda x, om, gg: exact(sig[gg, 0], x, om)) for g in range(2))


def _exp1(alpha, x, om):
    return math.exp(-x[0] / om[0] * alpha)


def _exp2(alpha, x, om):
    return math.exp(-x[1] / om[0] * alpha) if x[0] > x[1] else math.exp(-x[0] / om[1] * alpha)


@pytest.mark.parametrize("p,lump", [(1, 0), (1, 7), (2, 0), (3, 0)])
def test_exponential_order_1d(p, lump):
    # test_sweep.cpp:178-220: order p + 1 in 1D
    e1 = _exp_error((10,), p, _exp1, lump)
    e2 = _exp_error((20,), p, _exp1, lump)
    assert abs(math.log2(e1 / e2) - (p + 1)) < 0.1


def test_exponential_order_2d():
    # test_sweep.cpp:222-230: discontinuity not mesh aligned -> order ~1
    e1 = _exp_error((50, 50), 1, _exp2)
    e2 = _exp_error((100, 100), 1, _exp2)
    assert abs(math.log2(e1 / e2) - 1.0) < 0.2


def _mms_error(ne, p, lump):
    mesh = M.cartesian((ne, ne))
    quad = Q.level_symmetric(6, 2)
    total, scat = 1.0, 0.25
    o = OracleSweep(mesh, p, quad, np.full((1, mesh.num_elements), total), lump=lump)
    src = o.form_source(qfn=mms_source(total, scat), inflow_fn=lambda x, om, g, a: 2.0 / 4 / math.pi)
    sig_s = np.full((1, mesh.num_elements), scat)
    phi_old = np.zeros(o.ndof)
    for _ in range(200):
        psi = o.scattering_source(sig_s, phi_old, src)
        o.mult(psi, psi)
        phi = o.moments(psi)
        norm = np.linalg.norm(phi_old - phi)
        phi_old = phi
        if norm < 1e-10:
            break
    return o.l2_error(phi, 0, 0, mms_phi)


@pytest.mark.parametrize("p,lump", [(1, 0), (2, 0), (3, 0), (1, 7)])
def test_transport_mms_order(p, lump):
    # test_transport_mms.cpp:89-197: source iteration, L2 order p + 1 +- 0.2
    e1 = _mms_error(10, p, lump)
    e2 = _mms_error(20, p, lump)
    assert abs(math.log2(e1 / e2) - (p + 1)) < 0.2


def test_moments_known_answers():
    # test_angle_quad.cpp:86-123 on one DOF: D of a quadratic and a linear psi
    mesh = M.cartesian((1,) * 2)
    quad = Q.level_symmetric(4, 2)
    o = OracleSweep(mesh, 0, quad, np.ones((1, 1)))
    om = quad.omega
    psi = 2 * om[:, 0] ** 2 + om[:, 1] ** 2 + om[:, 0] * om[:, 1]
    assert abs(o.moments(psi)[0] - 4 * math.pi) < 1e-13
    psi = ((om ** 2).sum(1) + om[:, 0] + om[:, 1]) / 4 / math.pi
    phi = o.moments(psi, nmom=3)
    assert abs(phi[0] - 2.0 / 3) < 1e-13 and abs(phi[1] - 1.0 / 3) < 1e-13 and abs(phi[2] - 1.0 / 3) < 1e-13


def test_levels_structured():
    # on a structured grid the Kahn frontier of (cell i,j) in an octant is i + j
    mesh, quad, sig = problem(2, (7, 5), 1)
    o = OracleSweep(mesh, 1, quad, sig)
    nl, lev = o.levels()
    assert nl == 7 + 5 - 1
    lev = lev.reshape(mesh.num_elements, quad.size)
    for a in range(quad.size):
        sx, sy = np.sign(quad.omega[a])
        for e in range(mesh.num_elements):
            i, j = e % 7, e // 7
            ii = i if sx > 0 else 6 - i
            jj = j if sy > 0 else 4 - j
            assert lev[e, a] == ii + jj


def test_balance_vacuum():
    # with vacuum boundaries and no scattering, absorption + leakage of L^{-1} q
    # equals the total source sum_a w_a sum_i q(a, i)
    mesh, quad, sig = problem(2, (6, 6), 1, jitter=0.2, G=2)
    o = OracleSweep(mesh, 1, quad, sig)
    src = o.form_source(q_cell=np.ones((2, mesh.num_elements)))
    psi = o.mult(src)
    total = sum(quad.weights[a] * src.reshape(2, quad.size, -1)[g, a].sum() for g in range(2) for a in range(quad.size))
    assert abs(o.balance(psi) - total) < 1e-12 * abs(total)


def test_in_place_and_threads():
    mesh, quad, sig = problem(3, (4, 4, 4), 1, jitter=0.2)
    o = OracleSweep(mesh, 1, quad, sig)
    x = np.random.default_rng(3).random(o.psi_size)
    a = o.mult(x, threads=1)
    b = x.copy()
    o.mult(b, b, threads=4)
    assert np.array_equal(a, b)


# --------------------------------------------------------------- reflective boundaries
def _centres(mesh):
    v = mesh.vertices[mesh.elements]          # [ne][2^dim][dim]
    return v.mean(axis=1)


def _mirror_problem(dim, n, p, sn=4, G=2):
    """Full box [0,2] x [0,1]^(dim-1) and its half [0,1]^dim with the x = 1 face
    reflective; source and cross sections symmetric about x = 1."""
    full = M.cartesian((2 * n,) + (n,) * (dim - 1), extents=(2.0,) + (1.0,) * (dim - 1))
    half = M.cartesian((n,) * dim)
    quad = Q.level_symmetric(sn, dim)

    def sig(mesh):
        c = _centres(mesh)
        s = 1.0 + 3.0 * np.abs(c[:, 0] - 1.0) + c[:, 1] ** 2 + (c[:, 2] if dim == 3 else 0.0)
        return np.stack([s * (g + 1) for g in range(G)])

    def qfn(x, om, g):
        return 1.0 + x[0] * (2.0 - x[0]) + 0.5 * x[1] + (0.25 * x[2] if dim == 3 else 0.0) + g

    refl_attr = 2 if dim == 2 else 3          # x = max face
    return full, half, quad, sig, qfn, refl_attr


@pytest.mark.parametrize("dim,n,p", [(2, 4, 1), (2, 3, 2), (3, 3, 1)])
def test_reflective_half_domain_equals_full_domain(dim, n, p):
    # a reflective face is a mirror (sweep.cpp:177-195, 432-437): the half domain
    # with reflection reproduces the symmetric full-domain solution cell by cell
    full, half, quad, sig, qfn, attr = _mirror_problem(dim, n, p)
    of = OracleSweep(full, p, quad, sig(full))
    oh = OracleSweep(half, p, quad, sig(half))
    oh.set_reflective([attr])
    pf = of.mult(of.form_source(qfn=qfn))
    ph = oh.mult(oh.form_source(qfn=qfn))
    cf, ch = _centres(full), _centres(half)
    match = np.array([np.argmin(np.linalg.norm(cf - c, axis=1)) for c in ch])
    n_loc = (p + 1) ** dim
    pf = pf.reshape(of.G, of.Nw, full.num_elements, n_loc)[:, :, match, :]
    ph = ph.reshape(oh.G, oh.Nw, half.num_elements, n_loc)
    assert np.max(np.abs(pf - ph)) <= 1e-12 * np.max(np.abs(pf))
    # the reflective face adds in-edges: more levels than the vacuum half domain
    assert oh.levels()[0] > OracleSweep(half, p, quad, sig(half)).levels()[0]


def _reflect_mms(ne, p):
    # test/chive/mms.lua without scattering: [0, 0.5] x [0, 1], reflective at x = 0.5
    alpha, beta, delta, total = 0.25, 0.5, 2.0, 1.0
    pi = math.pi

    def psi(x, om, g):
        mu, eta = om[0], om[1]
        return (math.sin(pi * x[0]) * math.sin(pi * x[1])
                + beta * (mu + eta) * math.sin(2 * pi * x[0]) * math.sin(2 * pi * x[1])
                + alpha * (mu * mu + eta * eta) * math.sin(3 * pi * x[0]) * math.sin(3 * pi * x[1]) + delta) / 4 / pi

    def q(x, om, g):
        mu, eta = om[0], om[1]
        dx = (math.cos(pi * x[0]) * math.sin(pi * x[1]) / 4
              + beta * (mu + eta) * math.cos(2 * pi * x[0]) * math.sin(2 * pi * x[1]) / 2
              + alpha * (mu * mu + eta * eta) * math.cos(3 * pi * x[0]) * math.sin(3 * pi * x[1]) * 3 / 4)
        dy = (math.sin(pi * x[0]) * math.cos(pi * x[1]) / 4
              + beta * (mu + eta) * math.sin(2 * pi * x[0]) * math.cos(2 * pi * x[1]) / 2
              + alpha * (mu * mu + eta * eta) * math.sin(3 * pi * x[0]) * math.cos(3 * pi * x[1]) * 3 / 4)
        return mu * dx + eta * dy + total * psi(x, om, g)

    mesh = M.cartesian((ne // 2, ne), extents=(0.5, 1.0))
    quad = Q.level_symmetric(4, 2)
    o = OracleSweep(mesh, p, quad, np.full((1, mesh.num_elements), total))
    o.set_reflective([2])
    # inflow on every boundary face; on the reflective face the manufactured
    # solution is mirror symmetric, so the exact trace is the reflected one
    src = o.form_source(qfn=q, inflow_fn=lambda x, om, g, a: 0.0 if a == 2 else psi(x, om, g))
    sol = o.mult(src)
    return max(o.l2_error(sol, 0, a, psi) for a in range(quad.size))


@pytest.mark.parametrize("p", [1, 2])
def test_reflective_mms_order(p):
    # test/chive/mms.lua + test_ooa.py: L2 order p + 1 +- 0.2 with a reflective side
    e1 = _reflect_mms(10, p)
    e2 = _reflect_mms(20, p)
    assert abs(math.log2(e1 / e2) - (p + 1)) < 0.2


def test_reflective_errors():
    # a rotated box: the mirror images of S4 directions are not in the set
    mesh = M.cartesian((3, 3))
    c, s = math.cos(0.3), math.sin(0.3)
    mesh.vertices[:] = mesh.vertices @ np.array([[c, s], [-s, c]])
    quad = Q.level_symmetric(4, 2)
    o = OracleSweep(mesh, 1, quad, np.ones((1, 9)))
    with pytest.raises(ValueError):
        o.set_reflective([2])
    # two opposite reflective sides close a cycle, which the reference rejects
    mesh, quad, sigma = problem(2, (4, 3), 1)
    o = OracleSweep(mesh, 1, quad, sigma)
    o.set_reflective([2, 4])
    assert o.levels()[0] == -1
    with pytest.raises(RuntimeError):
        o.mult(np.ones(o.psi_size))
    # adjacent reflective sides (a symmetric quarter) stay a DAG
    o.set_reflective([2, 3])
    assert o.levels()[0] > 0


def test_layout_maps():
    # test_linalg.cpp:116-135: extents (G, Nw, Ndof) = (2, 4, 8); LEFT is Kokkos
    # layout_left (g fastest), RIGHT layout_right (i fastest)
    from oracle.oracle import relayout
    G, Nw, nd = 2, 4, 8
    right = np.arange(G * Nw * nd, dtype=np.float64)   # value = RIGHT offset
    left = relayout(right, G, Nw, nd, to_left=True)
    assert left[1 + 2 * (2 + 4 * 3)] == 3 + 8 * (2 + 4 * 1)   # (g, a, i) = (1, 2, 3)
    assert left[0 + 2 * (1 + 4 * 6)] == 6 + 8 * (1 + 4 * 0)   # (0, 1, 6)
    assert np.array_equal(relayout(left, G, Nw, nd, to_left=False), right)
    # the LEFT vector is the RIGHT one viewed as [G][Nw][Ndof] and transposed
    assert np.array_equal(left, right.reshape(G, Nw, nd).transpose(2, 1, 0).ravel())


@pytest.mark.parametrize("kind", [2, 3, 4])
def test_oracle_conservative_fixups(kind):
    # src/fixup.cpp: zero-and-scale (2), Ryosuke (3) and local optimization (4)
    # make psi >= 0 and keep every cell's balance w . x = sum b, so the global
    # balance of the sweep (absorption + leakage) equals the unfixed one
    mesh = M.cartesian((16, 16), jitter=0.1, seed=2)
    quad = Q.level_symmetric(4, 2)
    sig = np.full((1, mesh.num_elements), 50.0)
    q = np.zeros((1, mesh.num_elements))
    q[:, 0] = 100.0
    o = OracleSweep(mesh, 1, quad, sig)
    src = o.form_source(q_cell=q)
    plain = o.mult(src)
    assert plain.min() < 0
    o.set_fixup(kind, 0.0)
    psi = o.mult(src)
    applied, failed = o.fixup_counts()
    assert applied > 0 and failed == 0 and o.fixup_unsupported() == 0
    assert psi.min() >= 0.0
    assert abs(o.balance(psi) - o.balance(plain)) < 1e-12 * abs(o.balance(plain))


def test_oracle_ryosuke_abort_case():
    # 3D p = 1: cells with more than three positive entries after the zeroing,
    # where RyosukeFixupOperator::perform_nff aborts (src/fixup.cpp:155)
    mesh = M.cartesian((6, 6, 6), jitter=0.1, seed=2)
    quad = Q.level_symmetric(4, 3)
    sig = np.full((1, mesh.num_elements), 50.0)
    q = np.zeros((1, mesh.num_elements))
    q[:, 0] = 100.0
    o = OracleSweep(mesh, 1, quad, sig)
    o.set_fixup(3, 0.0)
    o.mult(o.form_source(q_cell=q))
    assert o.fixup_unsupported() > 0


def _gll(p):
    if p == 2:
        return np.array([0.0, 0.5, 1.0])
    r = 1.0 / math.sqrt(5.0)
    return np.array([0.0, 0.5 * (1 - r), 0.5 * (1 + r), 1.0])


def _lagrange(nodes, t):
    """Values and derivatives of the Lagrange polynomials on nodes at points t."""
    n = len(nodes)
    V = np.ones((n, len(t)))
    D = np.zeros((n, len(t)))
    for a in range(n):
        for b in range(n):
            if b == a:
                continue
            V[a] *= (t - nodes[b]) / (nodes[a] - nodes[b])
        for c in range(n):
            if c == a:
                continue
            term = np.full(len(t), 1.0 / (nodes[a] - nodes[c]))
            for b in range(n):
                if b not in (a, c):
                    term *= (t - nodes[b]) / (nodes[a] - nodes[b])
            D[a] += term
    return V, D


@pytest.mark.parametrize("dim,p", [(2, 2), (2, 3), (3, 2)])
def test_high_order_matrices_on_affine_cells(dim, p):
    # p >= 2 on affine cells: every integrand is a polynomial that the
    # integration rules integrate exactly, so the oracle's blocks must equal the
    # exact integrals, computed here independently by 12-point Gauss-Legendre
    # on the Lagrange-Gauss-Lobatto basis.  2 x 1 (x 1) cells of the unit square
    # (cube): 0.5 x 1 (x 1).
    mesh = M.cartesian((2,) + (1,) * (dim - 1))
    o = OracleSweep(mesh, p, Q.level_symmetric(4, dim), np.ones((1, 2)))
    x, w = np.polynomial.legendre.leggauss(12)
    t, w = 0.5 * (x + 1.0), 0.5 * w
    V, Dv = _lagrange(_gll(p), t)
    m1 = (V * w) @ V.T                     # int l_a l_b
    d1 = (Dv * w) @ V.T                    # d1[a, b] = int l_a' l_b
    n1 = p + 1
    h = [0.5] + [1.0] * (dim - 1)
    vol = float(np.prod(h))

    def kron_axes(mats):
        # local DOF i = i0 + n1 i1 + n1^2 i2: the last axis varies slowest
        out = np.ones((1, 1))
        for m in mats[::-1]:
            out = np.kron(out, m)
        return out

    Gm, Mm = o.element_matrices(0)
    assert np.max(np.abs(Mm - kron_axes([m1] * dim) * vol)) < 1e-14
    # the MassIntegrator mass of time absorption and scattering: the same integral
    assert np.max(np.abs(o.time_mass(0) - kron_axes([m1] * dim) * vol)) < 1e-14
    # G_d(i, j) = -int phi_j d_d phi_i = -(vol / h_d) * (int l'_i l_j along d) * masses across
    for d in range(dim):
        mats = [d1 if k == d else m1 for k in range(dim)]
        assert np.max(np.abs(Gm[d] - (-kron_axes(mats) * vol / h[d]))) < 1e-13
    # interior face x = 1/2 (area 1): blocks on the face DOFs, i0 = p of cell 0, i0 = 0 of cell 1
    f = [k for k in range(o.num_faces()) if o.face_info(k)[0][2] >= 0][0]
    F = o.face_matrices(f)
    tang = kron_axes([m1] * (dim - 1))
    nf = n1 ** (dim - 1)
    ex = np.zeros((2, 2, n1 ** dim, n1 ** dim))
    side = {0: p, 1: 0}
    for a in (0, 1):
        for b in (0, 1):
            for r in range(nf):
                for c in range(nf):
                    ex[a, b, side[a] + n1 * r, side[b] + n1 * c] = tang[r, c]
    assert np.max(np.abs(F - ex)) < 1e-14


@pytest.mark.parametrize("p", [2, 3])
def test_transport_source_on_affine_cells(p):
    # FormTransportSource (src/sweep.cpp:1135-1185) on a 0.5 x 1 affine cell:
    # q = int Q phi_i = Q vol (int l_ix)(int l_iy), and the inflow term of the
    # face x = 0 for directions entering through it, |Omega_x| psi_in int_face phi_i
    mesh = M.cartesian((2, 1))
    quad = Q.level_symmetric(4, 2)
    o = OracleSweep(mesh, p, quad, np.ones((1, 2)))
    x, w = np.polynomial.legendre.leggauss(12)
    t, w = 0.5 * (x + 1.0), 0.5 * w
    V, _ = _lagrange(_gll(p), t)
    s1 = V @ w                              # int l_a
    n1 = p + 1
    qv = 1.7
    src = o.form_source(q_cell=np.full((1, 2), qv)).reshape(quad.size, 2, n1 * n1)
    exact = qv * 0.5 * np.kron(s1, s1)
    assert np.max(np.abs(src[:, 0, :] - exact[None, :])) < 1e-14
    # inflow psi_in = 2 on the left boundary (attribute 4 of the cartesian mesh)
    attrs = np.unique(mesh.boundary_attributes)
    left = [a for a in attrs if np.allclose(mesh.vertices[mesh.boundary_faces[mesh.boundary_attributes == a]][..., 0], 0.0)]
    assert len(left) == 1
    inflow = np.zeros((1, int(attrs.max()) + 1))
    inflow[0, left[0]] = 2.0
    srcb = o.form_source(inflow=inflow).reshape(quad.size, 2, n1 * n1)
    for a in range(quad.size):
        ox = quad.omega[a, 0]
        want = np.zeros(n1 * n1)
        if ox > 0:   # enters through x = 0: DOFs with ix = 0, weight |Omega_x| * 2 * int l_iy
            want[0::n1] = ox * 2.0 * s1
        assert np.max(np.abs(srcb[a, 0] - want)) < 1e-14


@pytest.mark.parametrize("dim,cells", [(2, (6, 5)), (3, (4, 3, 3))])
def test_constant_solution_product_sets(dim, cells):
    # test_sweep.cpp:7-108 with product sets (pole directions included) and a rotated set
    mesh = M.cartesian(cells)
    for quad in (Q.product(dim, 4, 4), Q.product(dim, 5, 3, "lobatto"), Q.rotate(Q.product(dim, 4, 4), 0.2, 0.1, 0.3)):
        o = OracleSweep(mesh, 1, quad, np.zeros((1, mesh.num_elements)))
        psi = o.mult(o.form_source(inflow=np.ones((1, 8))))
        assert np.max(np.abs(psi - 1.0)) < 1e-12
