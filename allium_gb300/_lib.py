"""Loader for liballium_sweep.so (the CUDA product).  There is no fallback: if the
library cannot be built or loaded, or no GPU is present, calls raise."""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_lib = None


class AlliumError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"allium status {status}: {msg}")
        self.status = status


class MeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("num_vertices", C.c_int), ("vertices", C.c_void_p),
                ("num_elements", C.c_int), ("element_vertices", C.c_void_p),
                ("num_boundary_faces", C.c_int), ("boundary_face_vertices", C.c_void_p),
                ("boundary_attributes", C.c_void_p)]


class FeDesc(C.Structure):
    _fields_ = [("order", C.c_int), ("basis", C.c_int), ("lump", C.c_int)]


class QuadDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("num_angles", C.c_int), ("omega", C.c_void_p), ("weights", C.c_void_p)]


class BcDesc(C.Structure):
    _fields_ = [("num", C.c_int), ("attributes", C.c_void_p), ("kinds", C.c_void_p)]


EXPORTS = {
    "allium_sweep_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(FeDesc), C.POINTER(QuadDesc), C.c_int,
                                      C.c_void_p, C.POINTER(BcDesc), C.POINTER(C.c_void_p)]),
    "allium_sweep_destroy": (None, [C.c_void_p]),
    "allium_sweep_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "allium_sweep_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_int)]),
    "allium_sweep_assemble": (C.c_int, [C.c_void_p, C.c_void_p]),
    "allium_sweep_set_time_absorption": (C.c_int, [C.c_void_p, C.c_double]),
    "allium_sweep_mult": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_set_factor_cache": (C.c_int, [C.c_void_p, C.c_int]),
    "allium_sweep_set_schedule": (C.c_int, [C.c_void_p, C.c_int]),
    "allium_sweep_mult_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_set_fixup": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "allium_sweep_set_block_size": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "allium_sweep_set_pipeline": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "allium_sweep_set_f32_inverse_layout": (C.c_int, [C.c_void_p, C.c_int]),
    "allium_sweep_relayout": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "allium_sweep_fixup_counts": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.c_int]),
    "allium_sweep_apply_L": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_balance": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_balance_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_moments": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "allium_sweep_moments_transpose": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int]),
    "allium_sweep_form_source": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "allium_sweep_form_source_general": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
    "allium_sweep_source_points": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_scattering_source": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_moments_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_scattering_source_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_to_node_layout_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_from_node_layout_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_mult_f32_nodes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_scattering_source_f32_nodes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_moments_f32_nodes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_isotropic_source": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p]),
    "allium_sweep_fused_mult_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                              C.c_void_p, C.c_void_p]),
    "allium_sweep_fused_levels": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "allium_sweep_set_fused_pdl": (C.c_int, [C.c_void_p, C.c_int]),
    "allium_sweep_set_level_pdl": (C.c_int, [C.c_void_p, C.c_int]),
    "allium_sweep_transport_residual_df": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                     C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_moments_df": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_transport_residual_update_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_to_fused_layout": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_from_fused_layout": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_levels": (C.c_int, [C.c_void_p, C.c_void_p]),
    "allium_sweep_selftest_wait": (C.c_int, [C.c_void_p, C.c_int]),
    "allium_planck_spectrum": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_void_p]),
    "allium_sweep_planck_emission": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                               C.c_void_p]),
    "allium_sweep_energy_balance": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                              C.c_void_p, C.c_void_p]),
    "allium_sweep_block_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_double,
                                           C.c_int]),
    "allium_sweep_absorption": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int]),
    "allium_sweep_time_source": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "allium_sweep_powerlaw_opacity": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                                C.c_void_p]),
    "allium_sweep_dsa_setup": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double]),
    "allium_sweep_dsa_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_dsa_jacobi": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_sweep_dsa_blocks": (C.c_int, [C.c_void_p, C.c_void_p]),
    "allium_sweep_neighbours": (C.c_int, [C.c_void_p, C.c_void_p]),
    "allium_pair_aggregates": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_csr_spmv": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                  C.c_double, C.c_void_p]),
    "allium_mlp_gemm": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_longlong, C.c_void_p,
                                  C.c_longlong, C.c_longlong, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p,
                                  C.c_float, C.c_float, C.c_int, C.c_void_p]),
    "allium_mlp_relu_backward": (C.c_int, [C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_mlp_bias_grad": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_mlp_mse_grad": (C.c_int, [C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_mlp_adam": (C.c_int, [C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                  C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p]),
    "allium_mlp_to_bf16": (C.c_int, [C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p]),
    "allium_mlp_gemm_tc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong,
                                     C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_void_p, C.c_float,
                                     C.c_float, C.c_int, C.c_int, C.c_void_p]),
    "allium_mlp_transpose_bf16": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong,
                                            C.c_void_p]),
    "allium_mlp_status": (C.c_int, [C.c_void_p]),
    "allium_fp64_fma_probe": (C.c_int, [C.c_int, C.c_int, C.c_longlong, C.c_void_p, C.c_void_p]),
    "allium_sweep_synchronize": (C.c_int, [C.c_void_p]),
    "allium_sweep_last_error": (C.c_char_p, [C.c_void_p]),
    "allium_status_string": (C.c_char_p, [C.c_int]),
}


def path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Load (building first if needed) liballium_sweep.so and declare its ABI."""
    global _lib
    if _lib is None:
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError(f"{_build.LIB} is missing; run allium_gb300.build.build()")
        L = C.CDLL(_build.LIB)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, handle=None):
    if status != 0:
        L = lib()
        msg = L.allium_status_string(status).decode()
        if handle:
            detail = L.allium_sweep_last_error(handle)
            if detail:
                msg += f" ({detail.decode()})"
        raise AlliumError(status, msg)
