"""ctypes view of the CPU oracle (test infrastructure only).

The oracle restates allium's sweep path on the CPU in FP64 (sweep_oracle.cpp).
Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module, as
the checker and as the CPU baseline; the CUDA product never calls it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
FN = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int, C.c_int)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [C.c_int, C.c_int, dp, C.c_int, ip, C.c_int, ip, ip,
                                    C.c_int, C.c_int, C.c_int, dp, dp, C.c_int, dp]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_time_absorption.argtypes = [vp, C.c_double]
        L.oracle_num_faces.argtypes = [vp]
        L.oracle_face_info.argtypes = [vp, C.c_int, ip, dp]
        L.oracle_element_matrices.argtypes = [vp, C.c_int, C.c_int, dp, dp]
        L.oracle_time_mass.argtypes = [vp, C.c_int, dp]
        L.oracle_face_matrices.argtypes = [vp, C.c_int, dp]
        L.oracle_levels.argtypes = [vp, ip]
        L.oracle_sweep.argtypes = [vp, dp, dp, C.c_int]
        L.oracle_apply_L.argtypes = [vp, dp, dp]
        L.oracle_balance.argtypes = [vp, dp]
        L.oracle_balance.restype = C.c_double
        L.oracle_moments.argtypes = [vp, dp, dp, C.c_int]
        L.oracle_moments_transpose.argtypes = [vp, dp, dp, C.c_int, C.c_double, C.c_int]
        L.oracle_form_source.argtypes = [vp, dp, FN, dp, C.c_int, FN, dp]
        L.oracle_set_fixup.argtypes = [vp, C.c_int, C.c_double]
        L.oracle_set_reflective.argtypes = [vp, C.c_int, ip]
        L.oracle_dsa_matrix.argtypes = [vp, dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, dp]
        L.oracle_planck_spectrum.argtypes = [dp, C.c_int, C.c_double, C.c_int, dp]
        L.oracle_planck_emission.argtypes = [vp, dp, dp, dp, C.c_double, dp, dp]
        L.oracle_energy_balance.argtypes = [vp, dp, dp, dp, C.c_double, C.c_double, dp, dp]
        L.oracle_time_source.argtypes = [vp, dp, dp, C.c_double, dp]
        L.oracle_mass_apply.argtypes = [vp, C.c_int, dp, dp]
        L.oracle_absorption.argtypes = [vp, dp, dp, dp]
        L.oracle_powerlaw_opacity.argtypes = [vp, dp, dp, C.c_double, C.c_double, C.c_double, dp]
        L.oracle_fixup_counts.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
        L.oracle_fixup_unsupported.argtypes = [vp]
        L.oracle_fixup_unsupported.restype = C.c_longlong
        L.oracle_scattering_source.argtypes = [vp, dp, dp, dp, dp]
        L.oracle_l2_error.argtypes = [vp, dp, C.c_int, C.c_int, FN]
        L.oracle_l2_error.restype = C.c_double
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def planck_spectrum(bounds, T, kind=0):
    """Group fractions of the normalised Planck (0) or Rosseland (1) spectrum."""
    b = _f64(bounds)
    out = np.empty(b.size - 1)
    lib().oracle_planck_spectrum(_dp(b), b.size - 1, float(T), int(kind), _dp(out))
    return out


def relayout(psi, G, Nw, ndof, to_left):
    """Transport-vector layouts of src/tvector.hpp:47-53 (IndexMap<SPACE,
    ANGLE, ENERGY> for RIGHT, <ENERGY, ANGLE, SPACE> for LEFT): element
    (g, a, i) sits at i + ndof (a + Nw g) in RIGHT and g + G (a + Nw i) in LEFT,
    written here as an explicit index scatter."""
    psi = np.asarray(psi)
    out = np.empty_like(psi)
    g, a, i = np.meshgrid(np.arange(G), np.arange(Nw), np.arange(ndof), indexing="ij")
    right = (i + ndof * (a + Nw * g)).ravel()
    left = (g + G * (a + Nw * i)).ravel()
    if to_left:
        out[left] = psi[right]
    else:
        out[right] = psi[left]
    return out


class OracleSweep:
    """InverseAdvectionOperator restated on the CPU (plus D, L, balance, source)."""

    def __init__(self, mesh, order, quad, sigma, lump=0):
        L = lib()
        self.mesh, self.order, self.quad, self.lump = mesh, order, quad, lump
        self.dim = mesh.dim
        self.ne = mesh.num_elements
        self.n = (order + 1) ** self.dim
        sigma = _f64(sigma).reshape(-1, self.ne)
        self.G = sigma.shape[0]
        self.Nw = quad.size
        self.ndof = self.ne * self.n
        self._keep = [_f64(mesh.vertices), _i32(mesh.elements), _i32(mesh.boundary_faces),
                      _i32(mesh.boundary_attributes), _f64(quad.omega), _f64(quad.weights), sigma]
        v, e, bf, ba, om, w, s = self._keep
        self.h = L.oracle_create(self.dim, mesh.num_vertices, _dp(v), self.ne, _ip(e),
                                 int(ba.shape[0]), _ip(bf), _ip(ba), order, lump,
                                 self.Nw, _dp(om), _dp(w), self.G, _dp(s))
        if not self.h:
            raise ValueError("oracle_create rejected the problem")

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    @property
    def psi_size(self):
        return self.G * self.Nw * self.ndof

    def set_time_absorption(self, tau):
        lib().oracle_set_time_absorption(self.h, float(tau))

    # --- thermal radiative transfer operators (src/planck.hpp, src/trt_integrators.cpp)
    def planck_emission(self, bounds, sigma, T, ac=1.0):
        em = np.empty(self.G * self.ndof)
        grad = np.empty(self.G * self.ne * self.n * self.n)
        lib().oracle_planck_emission(self.h, _dp(_f64(bounds)), _dp(_f64(sigma)), _dp(_f64(T)), float(ac),
                                     _dp(em), _dp(grad))
        return em, grad.reshape(self.G, self.ne, self.n, self.n)

    def energy_balance(self, bounds, sigma, T, ac, cv_dt):
        res = np.empty(self.ndof)
        grad = np.empty(self.ne * self.n * self.n)
        lib().oracle_energy_balance(self.h, _dp(_f64(bounds)), _dp(_f64(sigma)), _dp(_f64(T)), float(ac),
                                    float(cv_dt), _dp(res), _dp(grad))
        return res, grad.reshape(self.ne, self.n, self.n)

    def time_source(self, psi_prev, q, tau):
        out = np.empty(self.psi_size)
        qq = _f64(q) if q is not None else None
        lib().oracle_time_source(self.h, _dp(_f64(psi_prev)), _dp(qq) if qq is not None else None, float(tau),
                                 _dp(out))
        return out

    def mass_apply(self, which, x):
        y = np.empty(self.ndof)
        lib().oracle_mass_apply(self.h, int(which), _dp(_f64(x)), _dp(y))
        return y

    def absorption(self, sigma, phi):
        y = np.empty(self.ndof)
        lib().oracle_absorption(self.h, _dp(_f64(sigma)), _dp(_f64(phi)), _dp(y))
        return y

    def powerlaw_opacity(self, T, nu, C0, a, b):
        out = np.empty(self.G * self.ne)
        lib().oracle_powerlaw_opacity(self.h, _dp(_f64(T)), _dp(_f64(nu)), float(C0), float(a), float(b), _dp(out))
        return out.reshape(self.G, self.ne)

    def dsa_matrix(self, sigma_s, g=0, kappa=None, penalty_min=None, alpha_bdr=0.5, tau=0.0, marshak=True):
        """Dense MIP diffusion operator of group g (InteriorPenaltyDiscretization)."""
        if kappa is None:
            kappa = (self.order + 1) ** 2
        if penalty_min is None:
            w = self.quad.weights
            penalty_min = 0.5 * float(np.sum(np.abs(self.quad.omega[:, 0]) * w) / np.sum(w))
        K = np.empty((self.ndof, self.ndof))
        lib().oracle_dsa_matrix(self.h, _dp(_f64(sigma_s)), int(g), float(kappa), float(penalty_min),
                                float(alpha_bdr), float(tau), int(marshak), _dp(K))
        return K

    def set_reflective(self, attributes):
        """Mark boundary attributes reflective (BoundaryCondition::REFLECTIVE)."""
        a = np.ascontiguousarray(list(attributes), dtype=np.int32)
        if lib().oracle_set_reflective(self.h, int(a.size), _ip(a)) != 0:
            raise ValueError("a reflected direction is not in the angular quadrature")

    def set_fixup(self, kind, minimum=0.0):
        lib().oracle_set_fixup(self.h, int(kind), float(minimum))

    def fixup_counts(self):
        a, f = C.c_longlong(), C.c_longlong()
        lib().oracle_fixup_counts(self.h, C.byref(a), C.byref(f))
        return a.value, f.value

    def fixup_unsupported(self):
        """Ryosuke solves with more than three positive entries (the reference aborts there)."""
        return lib().oracle_fixup_unsupported(self.h)

    def levels(self):
        lev = np.zeros(self.ne * self.Nw, dtype=np.int32)
        nl = lib().oracle_levels(self.h, _ip(lev))
        return nl, lev

    def mult(self, source, psi=None, threads=0):
        src = _f64(source)
        out = np.empty_like(src) if psi is None else psi
        st = lib().oracle_sweep(self.h, _dp(src), _dp(out), int(threads))
        if st != 0:
            raise RuntimeError(f"oracle sweep failed with status {st}")
        return out

    def apply_L(self, x):
        x = _f64(x)
        y = np.empty_like(x)
        lib().oracle_apply_L(self.h, _dp(x), _dp(y))
        return y

    def balance(self, psi):
        return lib().oracle_balance(self.h, _dp(_f64(psi)))

    def moments(self, psi, nmom=1):
        phi = np.empty(self.G * nmom * self.ndof)
        lib().oracle_moments(self.h, _dp(_f64(psi)), _dp(phi), nmom)
        return phi

    def moments_transpose(self, phi, nmom=1, psi=None, alpha=1.0, add=False):
        out = np.zeros(self.psi_size) if psi is None else psi
        lib().oracle_moments_transpose(self.h, _dp(_f64(phi)), _dp(out), nmom, float(alpha), int(add))
        return out

    def form_source(self, q_cell=None, inflow=None, qfn=None, inflow_fn=None):
        """FormTransportSource with per-cell Q[g, e] (or qfn(x, omega, g)) and an
        isotropic inflow[g, attr] table (or inflow_fn(x, omega, g, attr))."""
        out = np.empty(self.psi_size)
        q = _f64(q_cell if q_cell is not None else np.zeros((self.G, self.ne)))
        inf = _f64(inflow if inflow is not None else np.zeros((self.G, 1)))
        nattr = inf.shape[1] if inf.ndim == 2 else 1
        cb_q = FN(lambda x, om, g, a: qfn(x, om, g)) if qfn else FN()
        cb_in = FN(lambda x, om, g, a: inflow_fn(x, om, g, a)) if inflow_fn else FN()
        lib().oracle_form_source(self.h, _dp(q), cb_q, _dp(inf), nattr, cb_in, _dp(out))
        return out

    def scattering_source(self, sigma_s, phi, q_fixed=None):
        out = np.empty(self.psi_size)
        qf = _f64(q_fixed) if q_fixed is not None else None
        lib().oracle_scattering_source(self.h, _dp(_f64(sigma_s)), _dp(_f64(phi)),
                                       _dp(qf) if qf is not None else None, _dp(out))
        return out

    def l2_error(self, psi, g, angle, exact):
        cb = FN(lambda x, om, gg, a: exact(x, om, gg))
        return lib().oracle_l2_error(self.h, _dp(_f64(psi)), g, angle, cb)

    # --- matrices, for known-answer tests
    def element_matrices(self, e, g=0):
        nn = self.n * self.n
        G = np.empty(self.dim * nn)
        M = np.empty(nn)
        lib().oracle_element_matrices(self.h, e, g, _dp(G), _dp(M))
        return G.reshape(self.dim, self.n, self.n), M.reshape(self.n, self.n)

    def time_mass(self, e):
        M = np.empty(self.n * self.n)
        lib().oracle_time_mass(self.h, e, _dp(M))
        return M.reshape(self.n, self.n)

    def num_faces(self):
        return lib().oracle_num_faces(self.h)

    def face_info(self, f):
        info = np.zeros(5, dtype=np.int32)
        nrm = np.zeros(3)
        lib().oracle_face_info(self.h, f, _ip(info), _dp(nrm))
        return info, nrm[: self.dim]

    def face_matrices(self, f):
        out = np.empty(4 * self.n * self.n)
        lib().oracle_face_matrices(self.h, f, _dp(out))
        return out.reshape(2, 2, self.n, self.n)
