"""Angular quadratures for the sweep: level-symmetric (LQn) sets, 1D Gauss-Legendre,
product sets (Gauss-Legendre or Gauss-Lobatto polar levels x Chebyshev azimuths) and
the rotation of a set.

allium reads its level-symmetric sets from tables (src/angular_quadrature.cpp:98-147,
data/lsquad/LS_N.txt).  Here the same sets are generated from the LQn construction:

* one octant holds the points (mu_i, mu_j, mu_k) with i + j + k = N/2 + 2 (1-based),
  ordered by i, then j;
* mu_i^2 = mu_1^2 + (i - 1) * 2 (1 - 3 mu_1^2) / (N - 2);
* points in the same permutation class share a weight;
* mu_1 and the class weights make the octant rule integrate mu^(2m) exactly for
  m = 0, 2, 3, ..., N/2 (m = 1 holds by symmetry).

For N <= 12 these conditions fix the set uniquely (the positive-weight root).
The octants follow the table order (+,+,+), (-,+,+), (+,-,+), (-,-,+),
(+,+,-), (-,+,-), (+,-,-), (-,-,-); each octant weight sums to pi/2.  In 2D the
first four octants are kept and their weights doubled, as the reference does
(angular_quadrature.cpp:125,137); the third component is dropped.  In 1D the
set is the Gauss-Legendre rule with positive directions first
(angular_quadrature.cpp:103-115).
"""
from __future__ import annotations

import functools
import math
from dataclasses import dataclass

import numpy as np


@dataclass
class AngularQuadrature:
    dim: int
    omega: np.ndarray    # [Nw, dim] float64
    weights: np.ndarray  # [Nw] float64

    @property
    def size(self) -> int:
        return int(self.weights.shape[0])

    def sum_weights(self) -> float:
        return float(np.sum(self.weights))

    def reflected_index(self, angle: int, nor) -> int:
        """Index of Omega - 2 (Omega.n) n (angular_quadrature.cpp:27-36)."""
        om = self.omega[angle]
        nor = np.asarray(nor, dtype=np.float64)
        target = om - 2.0 * float(om @ nor) * nor
        d = np.sqrt(((self.omega - target) ** 2).sum(axis=1))
        k = int(np.argmin(d))
        if d[k] >= 1e-14:
            raise ValueError("no reflected direction in the set")
        return k


def _octant_points(N: int):
    s = N // 2 + 2
    return [(i, j, s - i - j) for i in range(1, N // 2 + 1) for j in range(1, N // 2 + 1) if s - i - j >= 1]


def _levels(N: int, mu1: float) -> np.ndarray:
    if N == 2:
        return np.array([mu1])
    delta = 2.0 * (1.0 - 3.0 * mu1 * mu1) / (N - 2)
    return np.sqrt(mu1 * mu1 + delta * np.arange(N // 2))


def _system(N: int, mu1: float):
    pts = _octant_points(N)
    keys = sorted({tuple(sorted(p)) for p in pts})
    cls = [keys.index(tuple(sorted(p))) for p in pts]
    K = len(keys)
    mu = _levels(N, mu1)
    powers = [0] + list(range(2, N // 2 + 1))
    A = np.zeros((len(powers), K))
    b = np.zeros(len(powers))
    for r, m in enumerate(powers):
        for p, c in zip(pts, cls):
            A[r, c] += mu[p[0] - 1] ** (2 * m)
        b[r] = 1.0 / (2 * m + 1)
    return A, b, pts, cls, K


def _residual(N: int, mu1: float):
    A, b, _, _, K = _system(N, mu1)
    try:
        w = np.linalg.solve(A[:K], b[:K])
    except np.linalg.LinAlgError:
        return math.nan, np.full(K, math.nan)
    return float(A[K] @ w - b[K]), w


@functools.lru_cache(maxsize=None)
def _solve_mu1(N: int) -> float:
    """The first level of the LQn set (a scan and bisection; cached per N)."""
    if N == 2:
        return 1.0 / math.sqrt(3.0)
    lo_lim, hi_lim = 1e-3, 1.0 / math.sqrt(3.0) - 1e-9
    grid = np.linspace(lo_lim, hi_lim, 2000)
    vals = [_residual(N, x)[0] for x in grid]
    for i in range(len(grid) - 1):
        if not (np.isfinite(vals[i]) and np.isfinite(vals[i + 1])):
            continue
        if vals[i] == 0.0 or np.sign(vals[i]) != np.sign(vals[i + 1]):
            a, b = float(grid[i]), float(grid[i + 1])
            fa = _residual(N, a)[0]
            for _ in range(200):
                c = 0.5 * (a + b)
                if c in (a, b):
                    break
                fc = _residual(N, c)[0]
                if fc == 0.0:
                    a = b = c
                    break
                if np.sign(fc) == np.sign(fa):
                    a, fa = c, fc
                else:
                    b = c
            root = 0.5 * (a + b)
            if np.all(_residual(N, root)[1] > 0):
                return root
    raise ValueError(f"no positive level-symmetric set for N={N}")


def level_symmetric(order: int, dim: int) -> AngularQuadrature:
    """LevelSymmetricQuadrature(order, dim) (angular_quadrature.cpp:98-147)."""
    if dim == 1:
        return legendre_1d(order)
    if order % 2 or order < 2 or order > 12:
        raise ValueError("level-symmetric sets are generated for N = 2, 4, ..., 12")
    mu1 = _solve_mu1(order)
    mu = _levels(order, mu1)
    if order == 2:
        pts, cls, w = [(1, 1, 1)], [0], np.array([1.0])
    else:
        A, b, pts, cls, K = _system(order, mu1)
        w = np.linalg.solve(A[:K], b[:K])
    octant = []
    for (i, j, _k), c in zip(pts, cls):
        mx, my = mu[i - 1], mu[j - 1]
        mz = math.sqrt(1.0 - mx * mx - my * my)
        octant.append((mx, my, mz, w[c] * math.pi / 2.0))
    dirs, wts = [], []
    n_oct = 4 if dim == 2 else 8
    for o in range(n_oct):
        sx = -1.0 if o & 1 else 1.0
        sy = -1.0 if o & 2 else 1.0
        sz = -1.0 if o & 4 else 1.0
        for mx, my, mz, wt in octant:
            dirs.append((sx * mx, sy * my, sz * mz)[:dim])
            wts.append(wt * (2.0 if dim == 2 else 1.0))
    return AngularQuadrature(dim, np.array(dirs, dtype=np.float64), np.array(wts, dtype=np.float64))


def legendre_1d(order: int) -> AngularQuadrature:
    """1D Gauss-Legendre directions, positive first, weights sum to 4 pi."""
    x, w = np.polynomial.legendre.leggauss(order)
    # ascending nodes on [-1, 1]; the reference stores directions descending
    omega = x[::-1].reshape(-1, 1).copy()
    return AngularQuadrature(1, omega, (2.0 * math.pi * w).astype(np.float64))


def single_angle(quad: AngularQuadrature, angle: int) -> AngularQuadrature:
    """SingleAngleQuadratureRule (angular_quadrature.hpp:45-56): one direction, weight 4 pi."""
    return AngularQuadrature(quad.dim, quad.omega[angle:angle + 1].copy(), np.array([4.0 * math.pi]))


def _gauss_lobatto01(n: int):
    """n-point Gauss-Lobatto rule on [0, 1] (ascending nodes, weights sum to 1)."""
    if n < 2:
        raise ValueError("Gauss-Lobatto needs at least 2 points")
    if n == 2:
        return np.array([0.0, 1.0]), np.array([0.5, 0.5])
    # interior nodes: roots of P'_{n-1}; weights 2 / (n (n - 1) P_{n-1}(x)^2) on [-1, 1]
    pn1 = np.polynomial.legendre.Legendre.basis(n - 1)
    inner = np.sort(pn1.deriv().roots().real)
    x = np.concatenate([[-1.0], inner, [1.0]])
    w = 2.0 / (n * (n - 1) * pn1(x) ** 2)
    return 0.5 * (x + 1.0), 0.5 * w


def product(dim: int, polar: int, azimuthal: int, polar_type: str = "legendre",
            triangular: bool = False) -> AngularQuadrature:
    """ProductQuadrature (angular_quadrature.cpp:190-264): `polar` levels
    theta_l = acos(2 x_l - 1) at the Gauss-Legendre (or Gauss-Lobatto, whose
    end levels are the poles with one direction each) points x_l of [0, 1] in
    ascending order; on level l, N_l azimuths phi_c = pi (2c + 1) / (2 N_l),
    c = 0..N_l-1, with N_l = azimuthal, or 2, 3, .. up to the equator and back
    when triangular.  Omega = (cos theta, sin theta cos phi[, sin theta sin phi]);
    in 3D the reference's loop over two half-ranges computes the same azimuths
    both times, so every 3D direction appears twice, kept here so that psi
    vectors index the same set; weights scale * w_l * pi / N_l with scale 4 (2D)
    or 2 (3D), so they sum to 4 pi."""
    if dim not in (2, 3):
        raise ValueError("product quadratures are 2D or 3D")
    if polar_type == "legendre":
        xg, wg = np.polynomial.legendre.leggauss(polar)
        x, w = 0.5 * (xg + 1.0), 0.5 * wg
        poles = False
    elif polar_type == "lobatto":
        x, w = _gauss_lobatto01(polar)
        poles = True
    else:
        raise ValueError("polar_type is 'legendre' or 'lobatto'")
    theta = np.arccos(2.0 * x - 1.0)
    mid = polar // 2
    if triangular:
        # as the reference fills them: 2, 3, .. for the first half, mirrored for
        # the second; with an odd level count the last level keeps no azimuths
        levels = [i + 2 for i in range(mid)]
        levels = levels + levels[::-1] + [0] * (polar - 2 * mid)
    else:
        levels = [azimuthal] * polar
    if poles:
        levels[0] = levels[-1] = 1
    scale = 4.0 if dim == 2 else 2.0
    dirs, wts = [], []
    for lvl in range(polar):
        naz = levels[lvl]
        for _ in range(1 if dim == 2 else 2):
            for c in range(naz):
                phi = math.pi * (2 * (c + 1) - 1) / 2 / naz
                om = [math.cos(theta[lvl]), math.sin(theta[lvl]) * math.cos(phi)]
                if dim == 3:
                    om.append(math.sin(theta[lvl]) * math.sin(phi))
                dirs.append(om)
                wts.append(scale * w[lvl] * math.pi / naz)
    return AngularQuadrature(dim, np.array(dirs, dtype=np.float64), np.array(wts, dtype=np.float64))


def rotate(quad: AngularQuadrature, x: float, y: float, z: float) -> AngularQuadrature:
    """AngularQuadrature::Rotate (angular_quadrature.cpp:38-80): every direction
    (lifted to 3D with its positive third component in 2D) multiplied by
    R = Rx(x) Ry(y) Rz(z), then cut back to the set's dimension."""
    if quad.dim == 1:
        raise ValueError("rotation needs a 2D or 3D set")
    cx, sx, cy, sy, cz, sz = math.cos(x), math.sin(x), math.cos(y), math.sin(y), math.cos(z), math.sin(z)
    Rx = np.array([[1.0, 0.0, 0.0], [0.0, cx, -sx], [0.0, sx, cx]])
    Ry = np.array([[cy, 0.0, sy], [0.0, 1.0, 0.0], [-sy, 0.0, cy]])
    Rz = np.array([[cz, -sz, 0.0], [sz, cz, 0.0], [0.0, 0.0, 1.0]])
    R = Rx @ Ry @ Rz
    om = quad.omega
    if quad.dim == 2:
        om = np.column_stack([om, np.sqrt(np.clip(1.0 - (om * om).sum(1), 0.0, None))])
    out = om @ R.T
    return AngularQuadrature(quad.dim, np.ascontiguousarray(out[:, :quad.dim]), quad.weights.copy())
