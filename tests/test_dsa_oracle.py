"""CPU checks of the oracle's MIP diffusion operator (the DSA operator of
InteriorPenaltyDiscretization, src/moment_discretization.cpp:73-110): symmetry
and positivity, and the diffusion MMS convergence order p + 1."""
import math

import numpy as np
import pytest

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q
from oracle.oracle import OracleSweep


@pytest.mark.parametrize("dim,cells,p", [(1, (6,), 2), (2, (4, 3), 1), (2, (3, 3), 2), (3, (3, 2, 2), 1)])
def test_mip_symmetric_positive(dim, cells, p):
    mesh = M.cartesian(cells, jitter=0.2 if dim > 1 else 0.0, seed=4)
    quad = Q.level_symmetric(4, dim)
    rng = np.random.default_rng(1)
    st = 10.0 ** rng.uniform(-1, 1, size=(1, mesh.num_elements))
    ss = st * rng.uniform(0.5, 0.99, size=st.shape)
    o = OracleSweep(mesh, p, quad, st)
    K = o.dsa_matrix(ss)
    assert np.max(np.abs(K - K.T)) < 1e-13 * np.max(np.abs(K))
    assert np.linalg.eigvalsh(0.5 * (K + K.T)).min() > 0


def _mms(ne, p):
    # -div(D grad u) + sigma_a u = f with natural (Neumann) boundaries:
    # u = cos(pi x) cos(pi y), D = 1/3, sigma_a = 1/2
    mesh = M.cartesian((ne, ne), jitter=0.1, seed=2)
    quad = Q.level_symmetric(4, 2)
    st = np.ones((1, mesh.num_elements))
    o = OracleSweep(mesh, p, quad, st)
    K = o.dsa_matrix(0.5 * st, marshak=False)
    u = lambda x, om, g: math.cos(math.pi * x[0]) * math.cos(math.pi * x[1])
    f = lambda x, om, g: (2 * math.pi ** 2 / 3 + 0.5) * u(x, om, g)
    F = o.form_source(qfn=f)[: o.ndof]
    uh = np.linalg.solve(K, F)
    return o.l2_error(uh, 0, 0, u)


@pytest.mark.parametrize("p", [1, 2])
def test_mip_mms_order(p):
    e1, e2 = _mms(6, p), _mms(12, p)
    assert abs(math.log2(e1 / e2) - (p + 1)) < 0.25


@pytest.mark.parametrize("kappa,pmin", [(4.0, 0.0), (4.0, 50.0), (1.0, 0.25)])
def test_mip_1d_known_matrix(kappa, pmin):
    # The MIP form written out from its definition on a 1D p = 1 mesh of
    # uneven cells (independently of the oracle's MFEM-style assembly):
    #   K = sum_e int D u'v' + sigma_a u v
    #     - sum_faces ({D u'}[v] + {D v'}[u]) + kappa_f [u][v]
    #     + alpha (u v) at the two boundary points (Marshak),
    # D = 1/(3 sigma_t), sigma_a = sigma_t - sigma_s, [v] = v_left - v_right,
    # {w} the average, kappa_f = max(kappa (D_l/h_l + D_r/h_r) / 2, pmin).
    ne = 5
    mesh = M.cartesian((ne,))
    x = np.array([0.0, 0.1, 0.3, 0.45, 0.8, 1.0])
    mesh.vertices[:, 0] = x                                  # uneven widths
    h = np.diff(x)
    st = np.array([[1.0, 3.0, 0.5, 2.0, 10.0]])
    ss = st * np.array([[0.5, 0.9, 0.2, 0.7, 0.99]])
    o = OracleSweep(mesh, 1, Q.level_symmetric(2, 1), st)
    K = o.dsa_matrix(ss, kappa=kappa, penalty_min=pmin, alpha_bdr=0.5)
    D = 1.0 / (3.0 * st[0])
    sa = st[0] - ss[0]
    N = 2 * ne
    E = np.zeros((N, N))
    for e in range(ne):
        i = slice(2 * e, 2 * e + 2)
        E[i, i] += D[e] / h[e] * np.array([[1.0, -1.0], [-1.0, 1.0]])
        E[i, i] += sa[e] * h[e] / 6.0 * np.array([[2.0, 1.0], [1.0, 2.0]])
    for f in range(ne - 1):            # face between cell f (left) and f + 1 (right)
        l, r = f, f + 1
        ul, ur = 2 * l + 1, 2 * r      # trace DOFs: right end of l, left end of r
        # jump [v] = v(ul) - v(ur); flux average {D u'} from both cells' gradients
        jump = np.zeros(N); jump[ul], jump[ur] = 1.0, -1.0
        avg = np.zeros(N)
        avg[2 * l], avg[2 * l + 1] = -0.5 * D[l] / h[l], 0.5 * D[l] / h[l]
        avg[2 * r], avg[2 * r + 1] = -0.5 * D[r] / h[r], 0.5 * D[r] / h[r]
        kf = max(kappa * (D[l] / h[l] + D[r] / h[r]) / 2.0, pmin)
        E -= np.outer(jump, avg) + np.outer(avg, jump)
        E += kf * np.outer(jump, jump)
    E[0, 0] += 0.5
    E[N - 1, N - 1] += 0.5
    assert np.max(np.abs(K - E)) < 1e-12 * np.max(np.abs(E))
