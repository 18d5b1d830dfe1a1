"""GPU MIP diffusion operator (DSA) against the oracle's dense operator, and
DSA-accelerated source iteration and GMRES against the unaccelerated solves.

Tolerances: operator blocks and products 1e-12 relative (max norm); solves
agree with each other to 1e-6 relative at a 1e-8 stopping tolerance."""
import numpy as np
import pytest

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q
from allium_gb300.dsa import DSAPreconditioner, MIPDiffusion
from allium_gb300.solvers import SchurOperator, solve_gmres, source_iteration
from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator
from oracle.oracle import OracleSweep
from tests.helpers import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [
    # dim, cells, p, G, jitter
    (1, (7,), 2, 2, 0.0),
    (2, (5, 4), 1, 2, 0.2),
    (2, (4, 3), 2, 1, 0.15),
    (2, (3, 3), 3, 1, 0.1),
    (3, (3, 3, 2), 1, 2, 0.15),
]


def _dense_from_blocks(o, blocks, g):
    ne, n, nd = o.ne, o.n, 2 * o.dim
    nbr = -np.ones((ne, nd), dtype=int)
    for f in range(o.num_faces()):
        info, _ = o.face_info(f)
        e1, k1, e2, k2 = info[:4]
        if e2 >= 0:
            nbr[e1, k1] = e2
            nbr[e2, k2] = e1
    K = np.zeros((ne * n, ne * n))
    for e in range(ne):
        K[e * n:(e + 1) * n, e * n:(e + 1) * n] = blocks[g, e, 0]
        for k in range(nd):
            m = nbr[e, k]
            if m >= 0:
                K[e * n:(e + 1) * n, m * n:(m + 1) * n] = blocks[g, e, 1 + k]
            else:
                assert np.all(blocks[g, e, 1 + k] == 0.0)
    return K


@pytest.mark.parametrize("case", CASES, ids=[f"d{c[0]}p{c[2]}G{c[3]}" for c in CASES])
def test_mip_operator_parity(case):
    dim, cells, p, G, jit = case
    mesh = M.cartesian(cells, jitter=jit, seed=6)
    quad = Q.level_symmetric(4, dim)
    rng = np.random.default_rng(2)
    st = 10.0 ** rng.uniform(-1, 1.5, size=(G, mesh.num_elements))
    ss = st * rng.uniform(0.3, 0.99, size=st.shape)
    o = OracleSweep(mesh, p, quad, st)
    L = InverseAdvectionOperator(mesh, p, quad, st)
    K = MIPDiffusion(L, ss, tau=0.7)
    blocks = K.blocks()
    x = rng.random(G * L.ndof)
    y = torch.empty(G * L.ndof, dtype=torch.float64, device="cuda")
    K.apply(torch.from_numpy(x).cuda(), y)
    y = y.cpu().numpy()
    for g in range(G):
        Ko = o.dsa_matrix(ss, g, tau=0.7)
        assert rel_err(_dense_from_blocks(o, blocks, g), Ko) < 1e-12
        assert rel_err(y[g * L.ndof:(g + 1) * L.ndof], Ko @ x[g * L.ndof:(g + 1) * L.ndof]) < 1e-12
    # block-Jacobi PCG converges on the SPD operator
    b = torch.from_numpy(rng.random(G * L.ndof)).cuda()
    xs = K.solve(b, tol=1e-11, maxiter=2000)
    r = torch.empty_like(b)
    K.apply(xs, r)
    assert torch.linalg.norm(r - b).item() <= 1e-10 * torch.linalg.norm(b).item()


def _scattering_problem(cells=(24, 24), sn=8, c=0.99, sigma_t=1.0):
    mesh = M.cartesian(cells)
    quad = Q.level_symmetric(sn, 2)
    st = np.full((1, mesh.num_elements), sigma_t)
    L = InverseAdvectionOperator(mesh, 1, quad, st)
    q = torch.from_numpy(FormTransportSource(L, np.ones((1, mesh.num_elements)))).cuda()
    return L, st * c, q


def test_dsa_source_iteration():
    # chive's SLI with the MIP-DSA preconditioner converges in far fewer sweeps
    L, ss, q = _scattering_problem(c=0.99, sigma_t=10.0)
    plain = source_iteration(SchurOperator(L, ss), q, tol=1e-8, maxiter=5000)
    dsa = DSAPreconditioner(L, ss)
    acc = source_iteration(SchurOperator(L, ss), q, tol=1e-8, maxiter=5000, dsa=dsa)
    assert plain.converged and acc.converged
    assert acc.iterations * 5 < plain.iterations
    assert torch.max(torch.abs(acc.phi - plain.phi)).item() < 1e-5 * torch.max(torch.abs(plain.phi)).item()


def test_dsa_gmres():
    L, ss, q = _scattering_problem(c=0.999, sigma_t=10.0)
    plain = solve_gmres(SchurOperator(L, ss), q, tol=1e-10, restart=50)
    acc = solve_gmres(SchurOperator(L, ss), q, tol=1e-10, restart=50, prec=DSAPreconditioner(L, ss))
    assert plain.converged and acc.converged
    assert acc.iterations < plain.iterations
    assert torch.max(torch.abs(acc.phi - plain.phi)).item() < 1e-7 * torch.max(torch.abs(plain.phi)).item()


@pytest.mark.parametrize("dim,cells,p", [(2, (24, 24), 1), (2, (12, 12), 2), (3, (8, 8, 8), 1)])
def test_vcycle_preconditioned_cg(dim, cells, p):
    # the vertex-space smoothed-aggregation V-cycle against block-Jacobi on one
    # heterogeneous, highly scattering operator: same solution, far fewer CG steps
    mesh = M.cartesian(cells, jitter=0.1, seed=1)
    quad = Q.level_symmetric(4, dim)
    rng = np.random.default_rng(0)
    st = 10.0 ** rng.uniform(-1, 1.7, size=(1, mesh.num_elements))
    L = InverseAdvectionOperator(mesh, p, quad, st)
    K = MIPDiffusion(L, 0.99 * st)
    b = torch.from_numpy(rng.random(L.ndof)).cuda()
    K.cg_iterations = 0
    xj = K.solve(b, tol=1e-10, maxiter=5000)
    itj = K.cg_iterations
    K.use_vcycle()
    K.cg_iterations = 0
    xv = K.solve(b, tol=1e-10, maxiter=5000)
    itv = K.cg_iterations
    assert itv * 4 < itj
    assert torch.max(torch.abs(xv - xj)).item() < 1e-7 * torch.max(torch.abs(xj)).item()
