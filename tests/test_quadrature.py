"""Level-symmetric generator vs allium's tables and moment conditions
(test/test_angle_quad.cpp:16-84).  CPU only."""
import json
import math
import os

import numpy as np
import pytest

from allium_gb300 import quadrature as Q

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "lsquad.json")))


@pytest.mark.parametrize("order", [2, 4, 6, 8, 10, 12])
@pytest.mark.parametrize("dim", [2, 3])
def test_matches_reference_tables(order, dim):
    q = Q.level_symmetric(order, dim)
    ref = GOLD[str(order)][str(dim)]
    assert q.omega.shape == (len(ref["weights"]), dim)
    assert np.max(np.abs(q.omega - np.array(ref["omega"]))) < 1e-12
    assert np.max(np.abs(q.weights - np.array(ref["weights"]))) < 1e-12


@pytest.mark.parametrize("order", [2, 4, 6, 8, 10, 12])
@pytest.mark.parametrize("dim", [2, 3])
def test_moments(order, dim):
    q = Q.level_symmetric(order, dim)
    assert abs(q.weights.sum() - 4 * math.pi) < 1e-13
    om = q.omega
    f = 2 * om[:, 0] ** 2 + om[:, 1] ** 2 + om[:, 0] * om[:, 1]
    assert abs((f * q.weights).sum() - 4 * math.pi) < 1e-13


@pytest.mark.parametrize("order", range(2, 25, 2))
def test_legendre_1d(order):
    q = Q.legendre_1d(order)
    assert q.size == order
    assert abs((q.omega[:, 0] ** 2 * q.weights).sum() / 4 / math.pi - 1.0 / 3) < 1e-13
    assert q.omega[0, 0] > 0


@pytest.mark.parametrize("dim", [2, 3])
def test_reflection(dim):
    q = Q.level_symmetric(4, dim)
    nor = np.zeros(dim); nor[0] = 1.0
    for a in range(q.size):
        r = q.reflected_index(a, nor)
        assert np.allclose(q.omega[r, 0], -q.omega[a, 0]) and np.allclose(q.omega[r, 1:], q.omega[a, 1:])


def test_layouts():
    # test_linalg.cpp:116-135: RIGHT transport layout and the moment layout
    G, Nw, Ndof = 2, 4, 8
    psi_index = lambda g, a, i: i + Ndof * (a + Nw * g)
    assert psi_index(1, 2, 3) == np.ravel_multi_index((1, 2, 3), (G, Nw, Ndof))
    assert psi_index(0, 1, 6) == np.ravel_multi_index((0, 1, 6), (G, Nw, Ndof))
    mom_index = lambda g, m, i: i + Ndof * (g + G * m)
    assert mom_index(1, 2, 3) == 3 + 8 * (1 + 2 * 2)


def test_disjoint_union():
    from allium_gb300 import mesh as M
    a, b = M.cartesian((2, 3)), M.cartesian((4, 1))
    u, off = M.disjoint_union([a, b])
    assert list(off) == [0, 6, 10]
    assert u.num_vertices == a.num_vertices + b.num_vertices
    assert np.array_equal(u.elements[6:], b.elements + a.num_vertices)
    assert np.array_equal(u.boundary_attributes, np.concatenate([a.boundary_attributes, b.boundary_attributes]))
