"""Shared problem builders for the tests."""
import math

import numpy as np

from allium_gb300 import mesh as M
from allium_gb300 import quadrature as Q


def problem(dim, cells, order, sn=4, G=1, jitter=0.0, seed=7, sigma=None, lump=0):
    mesh = M.cartesian(cells, jitter=jitter, seed=seed)
    quad = Q.level_symmetric(sn, dim)
    if sigma is None:
        rng = np.random.default_rng(seed + 1)
        sigma = 10.0 ** rng.uniform(-1, 2, size=(G, mesh.num_elements))
    return mesh, quad, np.ascontiguousarray(sigma, dtype=np.float64)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def mms_source(total, scat):
    """Manufactured source of test_transport_mms.cpp:29-38."""
    def q(x, om, g):
        quadratic = om[0] * om[0] + om[1] * om[1]
        px, py = math.pi * x[0], math.pi * x[1]
        dx = math.cos(px) * math.sin(py) / 4 + quadratic * math.cos(2 * px) * math.sin(2 * py) / 2
        dy = math.sin(px) * math.cos(py) / 4 + quadratic * math.sin(2 * px) * math.cos(2 * py) / 2
        return (om[0] * dx + om[1] * dy
                + total * (math.sin(px) * math.sin(py) + quadratic * math.sin(2 * px) * math.sin(2 * py) + 2.0) / 4 / math.pi
                - scat * (math.sin(px) * math.sin(py) + 2.0 / 3 * math.sin(2 * px) * math.sin(2 * py) + 2.0) / 4 / math.pi)
    return q


def mms_phi(x, om, g):
    return (math.sin(math.pi * x[0]) * math.sin(math.pi * x[1])
            + 2.0 / 3 * math.sin(2 * math.pi * x[0]) * math.sin(2 * math.pi * x[1]) + 2.0)
