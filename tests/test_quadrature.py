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


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("polar,azimuthal,ptype,tri", [(4, 4, "legendre", False), (6, 3, "legendre", False),
                                                       (5, 4, "lobatto", False), (6, 6, "legendre", True),
                                                       (5, 5, "legendre", True)])
def test_product_quadrature(dim, polar, azimuthal, ptype, tri):
    # ProductQuadrature (angular_quadrature.cpp:190-264)
    q = Q.product(dim, polar, azimuthal, ptype, tri)
    mid = polar // 2
    if tri:
        levels = [i + 2 for i in range(mid)] + [i + 2 for i in range(mid)][::-1] + [0] * (polar - 2 * mid)
    else:
        levels = [azimuthal] * polar
    if ptype == "lobatto":
        levels[0] = levels[-1] = 1
    assert q.size == sum(levels) * (2 if dim == 3 else 1)
    if dim == 3:
        assert np.allclose((q.omega ** 2).sum(1), 1.0, atol=1e-14)
    else:
        assert np.all((q.omega ** 2).sum(1) <= 1.0 + 1e-14)
    if tri and polar % 2:
        # the reference leaves the last level of an odd triangular set empty
        assert levels[-1] == 0
        return
    assert abs(q.sum_weights() - 4 * np.pi) < 1e-12
    # first moments vanish (symmetric polar points, azimuths symmetric about pi/2)
    assert np.max(np.abs(q.weights @ q.omega[:, :2])) < 1e-12
    if ptype == "lobatto":
        assert np.isclose(q.omega[0, 0], -1.0) and np.isclose(q.omega[-1, 0], 1.0)
    # polar levels in ascending Omega_x
    assert np.all(np.diff(q.omega[:, 0]) >= -1e-15)


def test_product_quadrature_polar_rule():
    # the polar points are the Gauss rule on [0, 1]: sum_l w_l (2 x_l - 1)^2 = 1/3 exactly
    q = Q.product(2, 8, 4)
    assert abs(q.weights @ q.omega[:, 0] ** 2 - 4 * np.pi / 3) < 1e-12
    lob_x, lob_w = Q._gauss_lobatto01(5)
    assert abs(lob_w.sum() - 1.0) < 1e-15 and lob_x[0] == 0.0 and lob_x[-1] == 1.0
    # Lobatto with n points integrates degree 2n - 3 exactly
    assert abs(lob_w @ lob_x ** 7 - 1.0 / 8) < 1e-14


@pytest.mark.parametrize("dim", [2, 3])
def test_rotate(dim):
    # AngularQuadrature::Rotate (angular_quadrature.cpp:38-80): directions stay unit
    # vectors, weights are kept, and a rotation by zero is the identity
    q = Q.level_symmetric(6, dim)
    r = Q.rotate(q, 0.3, -0.2, 0.7)
    assert np.array_equal(r.weights, q.weights)
    if dim == 3:
        assert np.allclose((r.omega ** 2).sum(1), 1.0, atol=1e-14)
        # the second moment tensor of a level-symmetric set is (4 pi / 3) I: rotation invariant
        assert np.allclose((r.omega * r.weights[:, None]).T @ r.omega, 4 * np.pi / 3 * np.eye(3), atol=1e-12)
    z = Q.rotate(q, 0.0, 0.0, 0.0)
    assert np.allclose(z.omega, q.omega, atol=1e-15)
    with pytest.raises(ValueError):
        Q.rotate(Q.legendre_1d(4), 0.1, 0.0, 0.0)


def _quadratic(om):
    return 2 * om[:, 0] ** 2 + om[:, 1] ** 2 + om[:, 0] * om[:, 1]


@pytest.mark.parametrize("tri", [True, False])
@pytest.mark.parametrize("ptype", ["legendre", "lobatto"])
def test_product_quadratic_known_answer(tri, ptype):
    # test_angle_quad.cpp:137-151: sum w (2 Ox^2 + Oy^2 + Ox Oy) = 4 pi, 2D, orders 4..12
    for order in range(4, 14, 2):
        q = Q.product(2, order, order, ptype, tri)
        assert abs(q.weights @ _quadratic(q.omega) - 4 * np.pi) < 1e-11


def test_rotate_known_answers():
    # test_angle_quad.cpp:153-173: the same integral after Rotate(pi/2, pi/4, pi/4)
    for q in (Q.level_symmetric(4, 2), Q.product(2, 4, 6)):
        r = Q.rotate(q, np.pi / 2, np.pi / 4, np.pi / 4)
        assert abs(r.weights @ _quadratic(r.omega) - 4 * np.pi) < 1e-11
