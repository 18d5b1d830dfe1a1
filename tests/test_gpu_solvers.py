"""Outer iterations on the GPU: source iteration, GMRES and FP32-inner /
FP64-outer refinement reach the same scalar flux as the CPU oracle's source
iteration, and their FP64 residuals meet the tolerance."""
import numpy as np
import pytest

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q
from allium_gb300.solvers import SchurOperator, gmres, refine, solve_gmres, source_iteration, true_residual
from allium_gb300.sweep import FormTransportSource, InverseAdvectionOperator
from oracle.oracle import OracleSweep
from tests.helpers import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def oracle_si(o, sig_s, src, tol):
    phi = np.zeros(o.ndof * o.G)
    for _ in range(5000):
        psi = o.scattering_source(sig_s, phi, src)
        o.mult(psi, psi)
        new = o.moments(psi)
        change = np.linalg.norm(new - phi) / np.linalg.norm(new)
        phi = new
        if change < tol:
            break
    return phi


@pytest.mark.parametrize("dim,cells,sn,jitter", [(2, (16, 16), 4, 0.0), (3, (6, 6, 6), 4, 0.1)])
def test_solvers_agree(dim, cells, sn, jitter):
    mesh = M.cartesian(cells, jitter=jitter, seed=3)
    quad = Q.level_symmetric(sn, dim)
    rng = np.random.default_rng(4)
    sig_t = 10.0 ** rng.uniform(-1, 1, size=(1, mesh.num_elements))
    sig_s = sig_t * rng.uniform(0.5, 0.95, size=sig_t.shape)
    q = rng.uniform(0, 1, size=(1, mesh.num_elements))
    o = OracleSweep(mesh, 1, quad, sig_t)
    src_h = o.form_source(q_cell=q)
    ref = oracle_si(o, sig_s, src_h, 1e-12)

    L = InverseAdvectionOperator(mesh, 1, quad, sig_t)
    src = torch.from_numpy(FormTransportSource(L, q)).cuda()
    assert rel_err(src.cpu().numpy(), src_h) < 1e-13
    op = SchurOperator(L, sig_s)
    si = source_iteration(op, src, tol=1e-12)
    assert si.converged
    assert rel_err(si.phi.cpu().numpy(), ref) < 1e-9

    op2 = SchurOperator(L, sig_s)
    gm = solve_gmres(op2, src, tol=1e-10)
    assert gm.converged
    b = op2.rhs(src)
    assert true_residual(op2, b, gm.phi) < 1e-9
    assert rel_err(gm.phi.cpu().numpy(), ref) < 1e-8

    op3 = SchurOperator(L, sig_s)
    ir = refine(op3, src, tol=1e-10, inner_tol=1e-4)
    assert ir.converged and ir.iterations <= 6
    assert true_residual(op3, b, ir.phi) < 1e-9
    assert rel_err(ir.phi.cpu().numpy(), ref) < 1e-8
    assert op3.sweeps32 > op3.sweeps64


def test_gmres_on_a_matrix():
    # the Krylov kernel alone on a nonsymmetric system
    n = 200
    rng = np.random.default_rng(0)
    A = np.eye(n) * 4 + rng.standard_normal((n, n)) / np.sqrt(n)
    b = rng.standard_normal(n)
    At = torch.from_numpy(A).cuda()
    bt = torch.from_numpy(b).cuda()
    x, it, hist = gmres(lambda v, out: out.copy_(At @ v), bt, tol=1e-12, restart=20)
    assert np.linalg.norm(A @ x.cpu().numpy() - b) < 1e-10 * np.linalg.norm(b)
