"""ctypes binding of the C ABI declared in ``include/montjoie_gb300.h``.

The shared library is built in-tree by ``montjoie_gb300.build``; there is no
fallback: if it is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

MJ_OK = 0
MJ_ERR_ARG = 1
MJ_ERR_CUDA = 2
MJ_ERR_STATE = 3
MJ_ERR_NONFINITE = 4
MJ_ERR_GEOMETRY = 5
MJ_ERR_NOMEM = 6
MJ_FP64 = 0
MJ_FP32 = 1

EXPORTED = [
    "mj_last_error", "mj_version", "mj_op_create", "mj_op_destroy", "mj_op_mltadd", "mj_op_mltadd_device",
    "mj_op_info", "mj_op_tuning", "mj_op_set_variant", "mj_kernel_launches", "mj_lf_create", "mj_lf_destroy", "mj_lf_init", "mj_lf_advance",
    "mj_lf_get_state", "mj_lf_run", "mj_lf_device_state", "mj_lf_profile", "mj_lf_set_graph", "mj_lf_set_scheme", "mj_lf_set_stream_gather", "mj_lf_set_stream", "mj_number_hex_mesh",
    "mj_geometry", "mj_lumped_mass", "mj_stiffness_mltadd_static",
    "mj_lfb_create", "mj_lfb_destroy", "mj_lfb_init", "mj_lfb_advance", "mj_lfb_get_state", "mj_lfb_info",
    "mj_op_set_element_scale", "mj_adj_create", "mj_adj_destroy", "mj_adj_forward", "mj_adj_backward",
    "mj_lfb_set_fused", "mj_lfb_step_info", "mj_lfb_profile", "mj_lfb_phase_ms", "mj_mb_create", "mj_mb_destroy", "mj_mb_advance", "mj_mb_info", "mj_mb_profile", "mj_mb_phase_ms", "mj_mb_tuning", "mj_mb_set_config",
]

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)
_VP = ctypes.c_void_p


class MeshDesc(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("n_elt", ctypes.c_int), ("n_dof", ctypes.c_int), ("nodle", _I)]


class GeomDesc(ctypes.Structure):
    _fields_ = [("factors", _D), ("gradphi", _D)]


class LfDesc(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double), ("mass", _D), ("inv_mass", _D),
        ("n_src", ctypes.c_int), ("src_idx", _I), ("src_val", _D),
        ("n_pulse", ctypes.c_int), ("pulse", _D),
        ("norm_weight", _D),
        ("n_rec", ctypes.c_int), ("n_rec_w", ctypes.c_int), ("rec_idx", _I), ("rec_w", _D),
    ]


class LfbDesc(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double), ("n_rhs", ctypes.c_int), ("mass", _D), ("inv_mass", _D),
        ("n_src", ctypes.c_int), ("src_idx", _I), ("src_rhs", _I), ("src_val", _D),
        ("n_pulse", ctypes.c_int), ("pulse", _D),
        ("n_rec", ctypes.c_int), ("n_rec_w", ctypes.c_int), ("rec_idx", _I), ("rec_w", _D),
    ]


class MontjoieError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads the product library (building it with nvcc when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"montjoie_gb300 native library not built: {path}")
        _build.build()
    L = ctypes.CDLL(path)
    L.mj_last_error.restype = ctypes.c_char_p
    L.mj_version.restype = ctypes.c_char_p
    L.mj_kernel_launches.restype = ctypes.c_uint64
    L.mj_op_create.argtypes = [ctypes.POINTER(MeshDesc), ctypes.POINTER(GeomDesc), ctypes.c_int, ctypes.POINTER(_VP)]
    L.mj_op_create_geometry.argtypes = [ctypes.POINTER(MeshDesc), _D, _D, ctypes.c_int, ctypes.POINTER(_VP)]
    L.mj_op_lumped_mass.argtypes = [_VP, _D, _D]
    L.mj_op_gaussian_source.argtypes = [_VP, _D, ctypes.c_double, ctypes.c_int, _I, _D, ctypes.POINTER(ctypes.c_int)]
    L.mj_op_power_iteration.argtypes = [_VP, _D, _D, ctypes.c_int, _D]
    L.mj_op_destroy.argtypes = [_VP]
    L.mj_op_mltadd.argtypes = [_VP, ctypes.c_double, _D, ctypes.c_double, _D]
    L.mj_op_mltadd_device.argtypes = [_VP, ctypes.c_double, _VP, ctypes.c_double, _VP, _VP]
    L.mj_op_info.argtypes = [_VP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                             ctypes.POINTER(ctypes.c_size_t)]
    L.mj_op_tuning.argtypes = [_VP] + [ctypes.POINTER(ctypes.c_int)] * 4 + [_D]
    L.mj_op_set_variant.argtypes = [_VP, ctypes.c_int, ctypes.c_int]
    L.mj_lf_create.argtypes = [_VP, ctypes.POINTER(LfDesc), ctypes.POINTER(_VP)]
    L.mj_lf_destroy.argtypes = [_VP]
    L.mj_lf_init.argtypes = [_VP, _D, _D]
    L.mj_lf_advance.argtypes = [_VP, ctypes.c_int, _D, _D, ctypes.c_int]
    L.mj_lf_get_state.argtypes = [_VP, _D, _D]
    L.mj_lf_run.argtypes = [_VP, _D, _D, ctypes.c_int, _D, _D, _D, ctypes.c_int]
    L.mj_lf_device_state.argtypes = [_VP, ctypes.POINTER(_VP), ctypes.POINTER(_VP), ctypes.POINTER(ctypes.c_int)]
    L.mj_lf_set_stream.argtypes = [_VP, _VP]
    L.mj_lf_set_graph.argtypes = [_VP, ctypes.c_int]
    L.mj_lf_set_scheme.argtypes = [_VP, ctypes.c_int, ctypes.c_int, _D]
    L.mj_lf_set_stream_gather.argtypes = [_VP, ctypes.c_int]
    L.mj_lf_set_norm_max.argtypes = [_VP, ctypes.c_double]
    L.mj_debug_set_wait_limits.argtypes = [ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong]
    L.mj_lf_profile.argtypes = [_VP, ctypes.c_int, _D, _D, ctypes.POINTER(ctypes.c_int)]
    L.mj_number_hex_mesh.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _I, ctypes.POINTER(ctypes.c_int)]
    L.mj_geometry.argtypes = [ctypes.c_int, ctypes.c_int, _D, _D, _D, _D, _D]
    L.mj_lumped_mass.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _D, _D, _D]
    L.mj_lfb_create.argtypes = [_VP, ctypes.POINTER(LfbDesc), ctypes.POINTER(_VP)]
    L.mj_lfb_destroy.argtypes = [_VP]
    L.mj_lfb_init.argtypes = [_VP, _D, _D]
    L.mj_lfb_advance.argtypes = [_VP, ctypes.c_int, _D, ctypes.c_int, ctypes.c_int]
    L.mj_lfb_get_state.argtypes = [_VP, _D, _D]
    L.mj_lfb_info.argtypes = [_VP] + [ctypes.POINTER(ctypes.c_int)] * 5
    L.mj_op_set_element_scale.argtypes = [_VP, _D]
    L.mj_adj_create.argtypes = [_VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_VP)]
    L.mj_adj_create_revolve.argtypes = [_VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_VP)]
    L.mj_adj_info.argtypes = [_VP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                              ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_size_t)]
    L.mj_revolve_schedule.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_longlong)]
    L.mj_adj_destroy.argtypes = [_VP]
    L.mj_adj_forward.argtypes = [_VP, _D]
    L.mj_adj_backward.argtypes = [_VP, _D, _D, _D]
    L.mj_lfb_set_fused.argtypes = [_VP, ctypes.c_int]
    L.mj_lfb_profile.argtypes = [_VP, ctypes.c_int]
    L.mj_lfb_phase_ms.argtypes = [_VP, _D]
    L.mj_lfb_step_info.argtypes = [_VP] + [ctypes.POINTER(ctypes.c_int)] * 4 + [_D]
    L.mj_lfb_set_step_variant.argtypes = [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.mj_mb_create.argtypes = [ctypes.c_int, ctypes.POINTER(_VP), ctypes.POINTER(_VP)]
    L.mj_mb_destroy.argtypes = [_VP]
    L.mj_mb_advance.argtypes = [_VP, ctypes.c_int, ctypes.c_int]
    L.mj_mb_info.argtypes = [_VP] + [ctypes.POINTER(ctypes.c_int)] * 6
    L.mj_mb_profile.argtypes = [_VP, ctypes.c_int]
    L.mj_mb_phase_ms.argtypes = [_VP, _D]
    L.mj_mb_tuning.argtypes = [_VP, ctypes.POINTER(ctypes.c_int), _D]
    L.mj_mb_set_config.argtypes = [_VP, ctypes.c_int]
    L.mj_mb_grouping.argtypes = [_VP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), _D]
    L.mj_mb_group_info.argtypes = [_VP, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 3 + [_D, _D]
    L.mj_mb_union_info.argtypes = [_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _D,
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.mj_stiffness_mltadd_static.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP, ctypes.c_double,
                                             _VP, ctypes.c_double, _VP, _VP]
    _lib = L
    return _lib


def check(code: int) -> None:
    if code != MJ_OK:
        msg = load().mj_last_error().decode(errors="replace")
        raise MontjoieError(code, msg)


def dptr(a):
    if a is None:
        return ctypes.cast(None, _D)
    assert a.dtype == np.float64 and a.flags.c_contiguous, "expected a contiguous float64 array"
    return a.ctypes.data_as(_D)


def iptr(a):
    if a is None:
        return ctypes.cast(None, _I)
    assert a.dtype == np.int32 and a.flags.c_contiguous, "expected a contiguous int32 array"
    return a.ctypes.data_as(_I)


def kernel_launches() -> int:
    return int(load().mj_kernel_launches())
