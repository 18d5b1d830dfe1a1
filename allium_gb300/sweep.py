"""Python mirror of allium's sweep-path operators, backed by liballium_sweep.so.

Names, argument meaning and in-place behaviour follow the reference:
  InverseAdvectionOperator   src/sweep.hpp:13-130   (Mult, AssembleLocalMatrices,
                                                     SetTimeAbsorption, UseParallelBlockJacobi)
  AdvectionOperator          src/sweep.hpp:155-166  (Mult, ComputeBalance)
  DiscreteToMoment           src/transport_op.hpp:97-122
  TransportOperator          src/transport_op.hpp:9-35
  FormTransportSource        src/sweep.cpp:1135-1185 (isotropic, piecewise constant data)

Vectors may be numpy arrays (host) or torch tensors (CUDA or pinned host),
float64 in allium's RIGHT layout psi[g, a, i] -> i + Ndof (a + Nw g).  Calls on
host arrays return when the result is on the host; calls on CUDA tensors are
ordered on the torch stream that was current when the operator was built.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import BcDesc, FeDesc, MeshDesc, QuadDesc, check

try:  # torch is plumbing only: device memory and streams
    import torch
except Exception:  # pragma: no cover
    torch = None


def _ptr(x, dtype, size=None, what="array"):
    """Raw pointer of a numpy array or torch tensor after dtype/size checks."""
    if torch is not None and isinstance(x, torch.Tensor):
        want = torch.float64 if dtype == np.float64 else (torch.float32 if dtype == np.float32 else torch.int32)
        if x.dtype != want or not x.is_contiguous():
            raise TypeError(f"{what} must be a contiguous {want} tensor")
        if size is not None and x.numel() != size:
            raise ValueError(f"{what} has {x.numel()} entries, expected {size}")
        return x.data_ptr()
    if not isinstance(x, np.ndarray) or x.dtype != dtype or not x.flags.c_contiguous:
        raise TypeError(f"{what} must be a contiguous {np.dtype(dtype).name} numpy array")
    if size is not None and x.size != size:
        raise ValueError(f"{what} has {x.size} entries, expected {size}")
    return x.ctypes.data


class InverseAdvectionOperator:
    """L^{-1}: the upwind DG sweep on one GPU.

    mesh: allium_gb300.mesh.Mesh; order: DG order (0..3, Gauss-Lobatto basis);
    quad: allium_gb300.quadrature.AngularQuadrature; sigma_t: [G, Ne] total cross
    section per cell; lump: allium lumping bit mask; bc: {attribute: "inflow" |
    "reflective"} (attributes not listed are inflow/vacuum).
    """

    def __init__(self, mesh, order, quad, sigma_t, lump=0, bc=None):
        L = _lib.lib()
        self.mesh, self.order, self.quad, self.lump = mesh, int(order), quad, int(lump)
        self.dim = mesh.dim
        sig = np.ascontiguousarray(sigma_t, dtype=np.float64).reshape(-1, mesh.num_elements)
        self.G = sig.shape[0]
        self.Nw = quad.size
        self.n = (self.order + 1) ** self.dim
        self.ndof = mesh.num_elements * self.n
        self._keep = [np.ascontiguousarray(mesh.vertices, dtype=np.float64),
                      np.ascontiguousarray(mesh.elements, dtype=np.int32),
                      np.ascontiguousarray(mesh.boundary_faces, dtype=np.int32),
                      np.ascontiguousarray(mesh.boundary_attributes, dtype=np.int32),
                      np.ascontiguousarray(quad.omega, dtype=np.float64),
                      np.ascontiguousarray(quad.weights, dtype=np.float64), sig]
        v, e, bf, ba, om, w, s = self._keep
        md = MeshDesc(self.dim, v.shape[0], v.ctypes.data, e.shape[0], e.ctypes.data,
                      ba.shape[0], bf.ctypes.data, ba.ctypes.data)
        fd = FeDesc(self.order, 0, self.lump)
        qd = QuadDesc(self.dim, self.Nw, om.ctypes.data, w.ctypes.data)
        bcd = None
        self.has_reflective = bool(bc) and any(str(k).lower() == "reflective" for k in bc.values())
        if bc:
            kinds = {"inflow": 0, "reflective": 1}
            attrs = np.array(list(bc.keys()), dtype=np.int32)
            kd = np.array([kinds[str(k).lower()] for k in bc.values()], dtype=np.int32)
            self._keep += [attrs, kd]
            bcd = C.pointer(BcDesc(len(attrs), attrs.ctypes.data, kd.ctypes.data))
        h = C.c_void_p()
        st = L.allium_sweep_create(C.byref(md), C.byref(fd), C.byref(qd), self.G, s.ctypes.data, bcd, C.byref(h))
        check(st)
        self.h = h
        self.pbj = False
        self.num_pbj_sweeps = 1
        if torch is not None and torch.cuda.is_available():
            self.set_stream(torch.cuda.current_stream())
        psi_size, ndof, nlev = C.c_longlong(), C.c_longlong(), C.c_int()
        check(L.allium_sweep_sizes(self.h, C.byref(psi_size), C.byref(ndof), C.byref(nlev)), self.h)
        self.height = self.width = int(psi_size.value)
        self.num_levels = int(nlev.value)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            _lib.lib().allium_sweep_destroy(h)
            self.h = None

    # --- reference surface
    def Height(self):
        return self.height

    def Width(self):
        return self.width

    def set_stream(self, stream):
        ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else (stream or 0)
        check(_lib.lib().allium_sweep_set_stream(self.h, C.c_void_p(ptr)), self.h)

    def Mult(self, source, psi):
        """psi = L^{-1} source (FP64); source may be psi itself."""
        sp = _ptr(source, np.float64, self.width, "source")
        pp = _ptr(psi, np.float64, self.height, "psi")
        # With one GPU owning every cell, the parallel block Jacobi variant
        # (sweep.cpp:671-875) has no off-rank data to lag: any number of PBJ
        # sweeps gives the upwind result, so one sweep serves both modes.
        check(_lib.lib().allium_sweep_mult(self.h, C.c_void_p(sp), C.c_void_p(pp)), self.h)

    def MultF32(self, source, psi):
        """FP32 sweep (storage and local solves in FP32)."""
        check(_lib.lib().allium_sweep_mult_f32(self.h, C.c_void_p(_ptr(source, np.float32, self.width, "source")),
                                               C.c_void_p(_ptr(psi, np.float32, self.height, "psi"))), self.h)

    def SetFixup(self, kind, minimum=0.0):
        """Negative-flux fixup: None/0 off, "zero"/1, "zero_and_scale"/2 (src/fixup.cpp:3-57)."""
        kinds = {None: 0, "none": 0, "zero": 1, "zero_and_scale": 2}
        k = kinds[kind] if not isinstance(kind, int) else kind
        check(_lib.lib().allium_sweep_set_fixup(self.h, k, float(minimum)), self.h)

    def UseFixup(self, use=True, kind="zero_and_scale", minimum=0.0):
        self.SetFixup(kind if use else 0, minimum)

    def FixupCounts(self, reset=False):
        a, f = C.c_longlong(), C.c_longlong()
        check(_lib.lib().allium_sweep_fixup_counts(self.h, C.byref(a), C.byref(f), int(reset)), self.h)
        return a.value, f.value

    def SetSchedule(self, mode):
        """0: one launch per wavefront level (default); 1: one persistent dataflow launch per sweep."""
        check(_lib.lib().allium_sweep_set_schedule(self.h, int(mode)), self.h)

    def SetBlockSize(self, precision, threads):
        """Threads per block (32/64/128) of the FP64 (64) or FP32 (32) level kernels."""
        check(_lib.lib().allium_sweep_set_block_size(self.h, int(precision), int(threads)), self.h)

    def SetPipeline(self, chunks, streams, taper=0):
        """Direction slices (2..32), compute streams (1..4) and end-slice taper
        (0..3: first and last slices 1/2^taper of the others) of the
        pinned-host-buffer Mult."""
        check(_lib.lib().allium_sweep_set_pipeline(self.h, int(chunks), int(streams), int(taper)), self.h)

    def SetF32InverseLayout(self, entry_major):
        """Order of the FP32 inverse copy of the node-major FP32 sweep: 0 block per node-group, 1 entry-major."""
        check(_lib.lib().allium_sweep_set_f32_inverse_layout(self.h, int(entry_major)), self.h)

    def SetFactorCache(self, mode):
        """1: keep FP64 local-matrix inverses across Mults when memory allows (default); 0: off."""
        check(_lib.lib().allium_sweep_set_factor_cache(self.h, int(mode)), self.h)

    def MultF32Nodes(self, source, psi):
        """FP32 sweep on node-major device vectors v[((e*Nw + a)*G + g)*n + i]."""
        check(_lib.lib().allium_sweep_mult_f32_nodes(self.h, C.c_void_p(_ptr(source, np.float32, self.width, "source")),
                                                     C.c_void_p(_ptr(psi, np.float32, self.height, "psi"))), self.h)

    def ToNodeLayoutF32(self, psi, out):
        check(_lib.lib().allium_sweep_to_node_layout_f32(self.h, C.c_void_p(_ptr(psi, np.float64, self.width, "psi")),
                                                         C.c_void_p(_ptr(out, np.float32, self.width, "out"))), self.h)
        return out

    def FromNodeLayoutF32(self, v, psi):
        check(_lib.lib().allium_sweep_from_node_layout_f32(self.h, C.c_void_p(_ptr(v, np.float32, self.width, "v")),
                                                           C.c_void_p(_ptr(psi, np.float64, self.width, "psi"))), self.h)
        return psi

    # --- fused FP32 inner operator and the double-float residual (device tensors;
    # psi-sized vectors in the fused layout v[((g*Ne + e)*Nw + a)*n + i])
    def FusedMultF32(self, iso, source, psi, phi=None, phi_mode=0, acc=None):
        """psi = L^{-1} (iso + source) in FP32 with phi = D psi (phi_mode 1) or
        phi += D psi (2) in the same graph, summed in double-float, or phi = D psi
        summed in FP32 (3, for inner operators); acc = (hi, lo) double-float
        accumulator that psi is added to.  iso [G*Ndof] float32 per-cell source
        or None, source psi-sized float32 or None."""
        nd = self.G * self.ndof
        ip = _ptr(iso, np.float32, nd, "iso") if iso is not None else None
        sp = _ptr(source, np.float32, self.width, "source") if source is not None else None
        fp = _ptr(phi, np.float64, nd, "phi") if phi is not None else None
        hp = _ptr(acc[0], np.float32, self.width, "acc_hi") if acc is not None else None
        lp = _ptr(acc[1], np.float32, self.width, "acc_lo") if acc is not None else None
        check(_lib.lib().allium_sweep_fused_mult_f32(self.h, C.c_void_p(ip), C.c_void_p(sp),
                                                     C.c_void_p(_ptr(psi, np.float32, self.width, "psi")),
                                                     C.c_void_p(fp), int(phi_mode), C.c_void_p(hp), C.c_void_p(lp)),
              self.h)
        return psi

    def FusedLevels(self):
        """(number of levels, 1 if they are unit levels else 0) of the fused sweep's schedule."""
        n, u = C.c_int(), C.c_int()
        check(_lib.lib().allium_sweep_fused_levels(self.h, C.byref(n), C.byref(u)), self.h)
        return n.value, u.value

    def SetFusedPDL(self, on):
        """1: the fused sweep's level launches overlap (programmatic dependent launch); 0: plain order."""
        check(_lib.lib().allium_sweep_set_fused_pdl(self.h, int(on)), self.h)

    def SetLevelPDL(self, on):
        """1: the stored-inverse sweep's level launches overlap (programmatic dependent launch); 0: plain order."""
        check(_lib.lib().allium_sweep_set_level_pdl(self.h, int(on)), self.h)

    def IsotropicSource(self, sigma_s, phi, q_iso=None, out=None, out_hi=None, out_lo=None):
        """Per-cell source (sigma_s M phi)/sum(w) + q_iso in FP64, written as float32
        (out) and/or double-float (out_hi, out_lo).  sigma_s [G, Ne] numpy or
        float64 CUDA tensor, or None to reuse the last one; phi, q_iso float64
        CUDA tensors [G*Ndof] or None."""
        nd = self.G * self.ndof
        sp = None
        if sigma_s is not None:
            if torch is not None and isinstance(sigma_s, torch.Tensor):
                sp = _ptr(sigma_s, np.float64, self.G * self.mesh.num_elements, "sigma_s")
            else:
                sig = np.ascontiguousarray(sigma_s, dtype=np.float64).reshape(self.G, -1)
                self._sigma_s_keep = sig
                sp = sig.ctypes.data
        args = [sp, _ptr(phi, np.float64, nd, "phi") if phi is not None else None,
                _ptr(q_iso, np.float64, nd, "q_iso") if q_iso is not None else None,
                _ptr(out, np.float32, nd, "out") if out is not None else None,
                _ptr(out_hi, np.float32, nd, "out_hi") if out_hi is not None else None,
                _ptr(out_lo, np.float32, nd, "out_lo") if out_lo is not None else None]
        check(_lib.lib().allium_sweep_isotropic_source(self.h, *[C.c_void_p(a) for a in args]), self.h)

    def TransportResidualDF(self, iso_hi, iso_lo, psi_hi, psi_lo, r, q_hi=None, q_lo=None):
        """r = q + D^T S phi - L psi in double-float arithmetic, stored as float32."""
        nd = self.G * self.ndof
        W = self.width
        args = [_ptr(iso_hi, np.float32, nd, "iso_hi"), _ptr(iso_lo, np.float32, nd, "iso_lo"),
                _ptr(q_hi, np.float32, W, "q_hi") if q_hi is not None else None,
                _ptr(q_lo, np.float32, W, "q_lo") if q_lo is not None else None,
                _ptr(psi_hi, np.float32, W, "psi_hi"), _ptr(psi_lo, np.float32, W, "psi_lo"),
                _ptr(r, np.float32, W, "r")]
        check(_lib.lib().allium_sweep_transport_residual_df(self.h, *[C.c_void_p(a) for a in args]), self.h)
        return r

    def TransportResidualUpdateF32(self, iso, dpsi, r):
        """r += iso - L dpsi in FP32 (the residual after a small correction dpsi)."""
        W = self.width
        check(_lib.lib().allium_sweep_transport_residual_update_f32(
            self.h, C.c_void_p(_ptr(iso, np.float32, self.G * self.ndof, "iso")),
            C.c_void_p(_ptr(dpsi, np.float32, W, "dpsi")), C.c_void_p(_ptr(r, np.float32, W, "r"))), self.h)
        return r

    def MomentsDF(self, hi, lo, phi):
        """phi = D (hi + lo) for a fused-layout double-float psi, FP64 out."""
        check(_lib.lib().allium_sweep_moments_df(
            self.h, C.c_void_p(_ptr(hi, np.float32, self.width, "hi")),
            C.c_void_p(_ptr(lo, np.float32, self.width, "lo")),
            C.c_void_p(_ptr(phi, np.float64, self.G * self.ndof, "phi"))), self.h)
        return phi

    def ToFusedLayout(self, psi, hi, lo=None):
        """RIGHT float64 psi -> fused-layout float32 hi (and its remainder lo)."""
        check(_lib.lib().allium_sweep_to_fused_layout(
            self.h, C.c_void_p(_ptr(psi, np.float64, self.width, "psi")),
            C.c_void_p(_ptr(hi, np.float32, self.width, "hi")),
            C.c_void_p(_ptr(lo, np.float32, self.width, "lo") if lo is not None else None)), self.h)
        return hi

    def FromFusedLayout(self, hi, lo, psi):
        """fused-layout float32 hi (+ lo) -> RIGHT float64 psi."""
        check(_lib.lib().allium_sweep_from_fused_layout(
            self.h, C.c_void_p(_ptr(hi, np.float32, self.width, "hi")),
            C.c_void_p(_ptr(lo, np.float32, self.width, "lo") if lo is not None else None),
            C.c_void_p(_ptr(psi, np.float64, self.width, "psi"))), self.h)
        return psi

    RIGHT, LEFT = 0, 1

    def Relayout(self, x, x_layout, out, out_layout):
        """Copy a psi-sized float64 CUDA tensor between the RIGHT layout
        (i + Ndof (a + Nw g), the one every other call takes) and the LEFT
        layout (g + G (a + Nw i)) of src/tvector.hpp:47-53."""
        check(_lib.lib().allium_sweep_relayout(self.h, C.c_void_p(_ptr(x, np.float64, self.width, "x")), int(x_layout),
                                               C.c_void_p(_ptr(out, np.float64, self.width, "out")), int(out_layout)),
              self.h)
        return out

    def AssembleLocalMatrices(self, sigma_t=None):
        """Reassemble with new total cross sections [G, Ne] (numpy, or a float64
        CUDA tensor read in place on the device)."""
        if sigma_t is None:
            sigma_t = self._keep[6]
        if torch is not None and isinstance(sigma_t, torch.Tensor) and sigma_t.is_cuda:
            if sigma_t.dtype != torch.float64 or not sigma_t.is_contiguous() or sigma_t.numel() != self.G * self.mesh.num_elements:
                raise ValueError("sigma_t must be a contiguous float64 tensor of G * Ne entries")
            check(_lib.lib().allium_sweep_assemble(self.h, C.c_void_p(sigma_t.data_ptr())), self.h)
            return
        sig = np.ascontiguousarray(sigma_t, dtype=np.float64).reshape(self.G, -1)
        self._keep[6] = sig
        check(_lib.lib().allium_sweep_assemble(self.h, C.c_void_p(sig.ctypes.data)), self.h)

    def SetTimeAbsorption(self, tau):
        self.time_absorption = float(tau)
        check(_lib.lib().allium_sweep_set_time_absorption(self.h, float(tau)), self.h)

    def GetTimeAbsorption(self):
        return getattr(self, "time_absorption", 0.0)

    def UseParallelBlockJacobi(self, use=True):
        self.pbj = bool(use)

    def IsParallelBlockJacobi(self):
        return self.pbj

    def SetNumPBJSweeps(self, n):
        self.num_pbj_sweeps = int(n)

    def Exchange(self, psi):
        """PBJ ghost exchange; a single GPU owns every cell, so nothing moves."""
        return None

    def GetLumpingType(self):
        return self.lump

    def levels(self):
        lev = np.empty(self.mesh.num_elements * self.Nw, dtype=np.int32)
        check(_lib.lib().allium_sweep_levels(self.h, C.c_void_p(lev.ctypes.data)), self.h)
        return lev

    def synchronize(self):
        check(_lib.lib().allium_sweep_synchronize(self.h), self.h)


class AdvectionOperator:
    """Forward operator L sharing the sweep's matrices (src/sweep.hpp:155-166)."""

    def __init__(self, Linv: InverseAdvectionOperator):
        self.Linv = Linv
        self.height = self.width = Linv.height

    def Mult(self, x, y):
        L = self.Linv
        check(_lib.lib().allium_sweep_apply_L(L.h, C.c_void_p(_ptr(x, np.float64, L.width, "x")),
                                              C.c_void_p(_ptr(y, np.float64, L.height, "y"))), L.h)

    def ComputeBalance(self, psi):
        L = self.Linv
        out = np.zeros(1)
        check(_lib.lib().allium_sweep_balance(L.h, C.c_void_p(_ptr(psi, np.float64, L.width, "psi")),
                                              C.c_void_p(out.ctypes.data)), L.h)
        return float(out[0])


class DiscreteToMoment:
    """phi = D psi and its transposes (src/transport_op.cpp:3-89)."""

    def __init__(self, Linv: InverseAdvectionOperator, num_moments=1):
        if num_moments not in (1, Linv.dim + 1):
            raise ValueError("num_moments must be 1 or dim + 1")
        self.Linv = Linv
        self.num_moments = num_moments
        self.height = Linv.G * num_moments * Linv.ndof
        self.width = Linv.width

    def Mult(self, psi, phi):
        L = self.Linv
        check(_lib.lib().allium_sweep_moments(L.h, C.c_void_p(_ptr(psi, np.float64, self.width, "psi")),
                                              C.c_void_p(_ptr(phi, np.float64, self.height, "phi")),
                                              self.num_moments), L.h)

    def MultTranspose(self, phi, psi):
        self._transpose(phi, psi, 1.0, 0)

    def AddMultTranspose(self, phi, psi, alpha=1.0):
        self._transpose(phi, psi, alpha, 1)

    def _transpose(self, phi, psi, alpha, add):
        L = self.Linv
        check(_lib.lib().allium_sweep_moments_transpose(
            L.h, C.c_void_p(_ptr(phi, np.float64, self.height, "phi")),
            C.c_void_p(_ptr(psi, np.float64, self.width, "psi")), self.num_moments, float(alpha), int(add)), L.h)


def ScatteringSource(Linv: InverseAdvectionOperator, sigma_s, phi, q_fixed=None, out=None):
    """out = D^T (S phi) + q_fixed with S = sigma_s[G, Ne] x MassIntegrator matrix
    (the source-iteration update of transport_op.hpp:75-90)."""
    if out is None:
        out = np.empty(Linv.width)
    sig = np.ascontiguousarray(sigma_s, dtype=np.float64).reshape(Linv.G, -1)
    qp = _ptr(q_fixed, np.float64, Linv.width, "q_fixed") if q_fixed is not None else None
    check(_lib.lib().allium_sweep_scattering_source(
        Linv.h, C.c_void_p(sig.ctypes.data), C.c_void_p(_ptr(phi, np.float64, Linv.G * Linv.ndof, "phi")),
        C.c_void_p(qp), C.c_void_p(_ptr(out, np.float64, Linv.width, "out"))), Linv.h)
    return out


def ScatteringSourceF32(Linv: InverseAdvectionOperator, sigma_s, phi, q_fixed, out):
    """FP32 out = D^T (S phi) + q_fixed (S phi in FP64); device tensors only."""
    sig = np.ascontiguousarray(sigma_s, dtype=np.float64).reshape(Linv.G, -1)
    qp = _ptr(q_fixed, np.float32, Linv.width, "q_fixed") if q_fixed is not None else None
    check(_lib.lib().allium_sweep_scattering_source_f32(
        Linv.h, C.c_void_p(sig.ctypes.data), C.c_void_p(_ptr(phi, np.float64, Linv.G * Linv.ndof, "phi")),
        C.c_void_p(qp), C.c_void_p(_ptr(out, np.float32, Linv.width, "out"))), Linv.h)
    return out


def ScatteringSourceF32Nodes(Linv: InverseAdvectionOperator, sigma_s, phi, q_nodes, out):
    """Node-major FP32 out = D^T (S phi) + q_nodes; device tensors only."""
    sig = np.ascontiguousarray(sigma_s, dtype=np.float64).reshape(Linv.G, -1)
    qp = _ptr(q_nodes, np.float32, Linv.width, "q_nodes") if q_nodes is not None else None
    check(_lib.lib().allium_sweep_scattering_source_f32_nodes(
        Linv.h, C.c_void_p(sig.ctypes.data), C.c_void_p(_ptr(phi, np.float64, Linv.G * Linv.ndof, "phi")),
        C.c_void_p(qp), C.c_void_p(_ptr(out, np.float32, Linv.width, "out"))), Linv.h)
    return out


def MomentsF32Nodes(Linv: InverseAdvectionOperator, psi, phi):
    """FP64 zeroth moment of a node-major FP32 psi; device tensors only."""
    check(_lib.lib().allium_sweep_moments_f32_nodes(Linv.h, C.c_void_p(_ptr(psi, np.float32, Linv.width, "psi")),
                                                    C.c_void_p(_ptr(phi, np.float64, Linv.G * Linv.ndof, "phi"))), Linv.h)
    return phi


def MomentsF32(Linv: InverseAdvectionOperator, psi, phi):
    """FP64 zeroth moment of an FP32 psi; device tensors only."""
    check(_lib.lib().allium_sweep_moments_f32(Linv.h, C.c_void_p(_ptr(psi, np.float32, Linv.width, "psi")),
                                              C.c_void_p(_ptr(phi, np.float64, Linv.G * Linv.ndof, "phi"))), Linv.h)
    return phi


def FormTransportSource(Linv: InverseAdvectionOperator, q_cell=None, inflow=None, out=None):
    """Weak-form source for an isotropic density q_cell[G, Ne] and an isotropic
    inflow[G, num_attr] indexed by boundary attribute (vacuum where 0)."""
    L = _lib.lib()
    if out is None:
        out = np.empty(Linv.width)
    qp = inp = None
    nattr = 0
    keep = []
    if q_cell is not None:
        q = np.ascontiguousarray(q_cell, dtype=np.float64).reshape(Linv.G, -1)
        keep.append(q)
        qp = q.ctypes.data
    if inflow is not None:
        fin = np.ascontiguousarray(inflow, dtype=np.float64).reshape(Linv.G, -1)
        keep.append(fin)
        inp, nattr = fin.ctypes.data, fin.shape[1]
    check(L.allium_sweep_form_source(Linv.h, C.c_void_p(qp), C.c_void_p(inp), nattr,
                                     C.c_void_p(_ptr(out, np.float64, Linv.width, "source"))), Linv.h)
    return out


def SourcePoints(Linv: InverseAdvectionOperator):
    """Physical coordinates [Ne, P, dim] of the source's domain-rule points."""
    L = _lib.lib()
    npc = C.c_int()
    check(L.allium_sweep_source_points(Linv.h, C.byref(npc), None), Linv.h)
    out = np.empty((Linv.mesh.num_elements, npc.value, Linv.dim))
    check(L.allium_sweep_source_points(Linv.h, C.byref(npc), C.c_void_p(out.ctypes.data)), Linv.h)
    return out


def FormTransportSourceGeneral(Linv: InverseAdvectionOperator, q_fn=None, inflow_angular=None, out=None,
                               per_direction=False):
    """Weak-form source for a density evaluated at the domain-rule points:
    q_fn(x, g) -> [Ne, P] (x: [Ne, P, dim] coordinates), or with per_direction
    q_fn(x, omega, g) -> [Ne, P] for each direction omega; and a
    direction-dependent inflow_angular[G, Nw, num_attr] per boundary attribute."""
    L = _lib.lib()
    if out is None:
        out = np.empty(Linv.width)
    qp = inp = None
    nattr = 0
    keep = []
    if q_fn is not None:
        x = SourcePoints(Linv)
        shape = x.shape[:2]
        if per_direction:
            q = np.stack([np.stack([np.asarray(q_fn(x, Linv.quad.omega[a], g), dtype=np.float64).reshape(shape)
                                    for a in range(Linv.Nw)]) for g in range(Linv.G)])
        else:
            q = np.stack([np.asarray(q_fn(x, g), dtype=np.float64).reshape(shape) for g in range(Linv.G)])
        q = np.ascontiguousarray(q)
        keep.append(q)
        qp = q.ctypes.data
    if inflow_angular is not None:
        fin = np.ascontiguousarray(inflow_angular, dtype=np.float64).reshape(Linv.G, Linv.Nw, -1)
        keep.append(fin)
        inp, nattr = fin.ctypes.data, fin.shape[2]
    check(L.allium_sweep_form_source_general(Linv.h, C.c_void_p(qp), int(bool(per_direction)), C.c_void_p(inp), nattr,
                                             C.c_void_p(_ptr(out, np.float64, Linv.width, "source"))), Linv.h)
    return out


class TransportOperator:
    """I - D L^{-1} S D^T applied to phi (src/transport_op.hpp:9-35).  S is a
    callable phi -> S phi (the scattering mass), psi the work vector."""

    def __init__(self, D: DiscreteToMoment, Linv: InverseAdvectionOperator, S, psi):
        self.D, self.Linv, self.S, self.psi = D, Linv, S, psi

    def Mult(self, x, y):
        self.S(x, y)
        self.D.MultTranspose(y, self.psi)
        self.Linv.Mult(self.psi, self.psi)
        self.D.Mult(self.psi, y)
        y -= x
        y *= -1.0
