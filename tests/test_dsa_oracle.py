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
