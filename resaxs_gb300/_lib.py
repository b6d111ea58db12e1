"""ctypes binding of librsx.so (the C ABI declared in include/rsx.h).

The library is the only compute path: if ``librsx.so`` is missing or cannot be
loaded, every call raises ``LibraryNotBuilt`` -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "librsx.so")

# resaxs::error codes (resaxslib/include/resaxs.hpp:212-220) and librsx extensions
RSX_OK = 0
RSX_INVALID_DEVICE = -1
RSX_ALG_NOT_INITIALIZED = -2
RSX_INVALID_ARG = -3
RSX_PROGRAM_NOT_LOADED = -4
RSX_ARGS_NOT_SET = -5
RSX_NO_INITIAL_CALC = -6
RSX_CUDA_ERROR = -100
RSX_OUT_OF_MEMORY = -101
RSX_TIMEOUT = -102
RSX_NOT_SUPPORTED = -103
RSX_INJECTED_FAULT = -104
RSX_PDB_FILE_NOT_FOUND = -1100


class LibraryNotBuilt(RuntimeError):
    pass


class ResaxsError(RuntimeError):
    """Mirror of resaxs::error: ``err()`` is the status code, str() the message."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg

    def err(self) -> int:
        return self.code


class DebyeOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("q_slab", ctypes.c_int), ("max_items", ctypes.c_int),
                ("force_general_q", ctypes.c_int), ("timing", ctypes.c_int),
                ("autotune", ctypes.c_int), ("no_pair_tables", ctypes.c_int),
                ("pairs_per_step", ctypes.c_int)]


_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_i = ctypes.c_int
_u = ctypes.c_uint
_st = ctypes.c_int

# (name, restype, argtypes) of every exported entry point
SIGNATURES = [
    ("rsx_version", ctypes.c_char_p, []),
    ("rsx_last_error", ctypes.c_char_p, []),
    ("rsx_launch_count", ctypes.c_ulonglong, []),
    ("rsx_debug_inject_fault", None, [_i, _i]),
    ("rsx_debug_layout", _st, [_f32p, _i, _i, _i, _i, ctypes.POINTER(_i), ctypes.POINTER(_i),
                               ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    ("rsx_calc_saxs_curve", None, [_f32p, _i, _f32p, _i, _f32p, _i, _f32p]),
    ("rsx_calc_saxs_curve_status", _st, [_f32p, _i, _f32p, _i, _f32p, _i, _f32p]),
    ("rsx_calc_saxs_curve_device_noalloc", _st, [_vp, _i, _vp, _i, _vp, _i, _vp, _vp]),
    ("rsx_debye_default_options", None, [ctypes.POINTER(DebyeOptions)]),
    ("rsx_autotune_clear", None, []),
    ("rsx_debye_create", _st, [_f32p, _i, _f32p, _i, _i, ctypes.POINTER(DebyeOptions),
                               ctypes.POINTER(_vp)]),
    ("rsx_debye_destroy", _st, [_vp]),
    ("rsx_debye_set_factors", _st, [_vp, _f32p, _i]),
    ("rsx_debye_set_water", _st, [_vp, ctypes.c_float, _i, _vp]),
    ("rsx_debye_calc", _st, [_vp, _f32p, _f32p]),
    ("rsx_debye_calc_shard", _st, [_vp, _f32p, _i, _i, _f64p]),
    ("rsx_debug_theta_level", _i, [_i, ctypes.c_double, ctypes.c_double]),
    ("rsx_debug_wide_plan", _st, [_i, _i, np.ctypeslib.ndpointer(np.int32)]),
    ("rsx_debug_chain_plan", _st, [_i, np.ctypeslib.ndpointer(np.int32)]),
    ("rsx_debug_shard_items", _st, [_f32p, _i, _i, _i, _i, np.ctypeslib.ndpointer(np.int32),
                                    _vp]),
    ("rsx_debug_autotune_lookup", _i, [ctypes.c_char_p, ctypes.POINTER(_i)]),
    ("rsx_debye_recalc_range", _st, [_vp, _f32p, _u, _u, _f32p]),
    ("rsx_debye_recalc_indices", _st, [_vp, _f32p, _u32p, _u, _f32p]),
    ("rsx_debye_commit", _st, [_vp]),
    ("rsx_debye_revert", _st, [_vp]),
    ("rsx_debye_curve_f64", _st, [_vp, _f64p]),
    ("rsx_debye_forward_resident", _st, [_vp]),
    ("rsx_debye_sync", _st, [_vp]),
    ("rsx_debye_stream", _vp, [_vp]),
    ("rsx_measure_fp32_fma_rate", _st, [_i, ctypes.POINTER(ctypes.c_double)]),
    ("rsx_debye_timing", _st, [_vp, ctypes.POINTER(ctypes.c_float),
                               ctypes.POINTER(ctypes.c_float)]),
    ("rsx_debye_backward", _st, [_vp, _f32p, _f32p]),
    ("rsx_debye_backward_f64", _st, [_vp, _f32p, _f64p]),
    ("rsx_debye_chi2_backward", _st, [_vp, _f32p, _f32p, ctypes.POINTER(ctypes.c_double),
                                      _vp]),
    ("rsx_debye_tile_shape", _st, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    ("rsx_debye_config", _st, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i),
                               ctypes.POINTER(_i)]),
    ("rsx_ff_type_count", _i, []),
    ("rsx_ff_water_index", _i, []),
    ("rsx_ff_atomic_table", _st, [_f32p, _i, ctypes.c_float, ctypes.c_float, _f32p]),
    ("rsx_ff_radii", _st, [_f32p]),
    ("rsx_ff_avg_radius", _st, [_f32p, _i, ctypes.POINTER(ctypes.c_float)]),
    ("rsx_pdb_count", _st, [ctypes.c_char_p, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    ("rsx_pdb_read", _st, [ctypes.c_char_p, _i, _f32p, _i, np.ctypeslib.ndpointer(np.int32), _i]),
    ("rsx_sasa_fibonacci_dots", _st, [_i, _f32p]),
    ("rsx_sasa_dodeca_icosa_dots", _st, [_f32p]),
    ("rsx_sasa_create", _st, [_i, _f32p, _i, ctypes.c_float, _i, ctypes.POINTER(_vp)]),
    ("rsx_sasa_sphere_dots", _st, [_i, ctypes.c_float, ctypes.c_float, ctypes.c_float, _f32p,
                              _i, ctypes.POINTER(_i)]),
    ("rsx_sasa_create_typed", _st, [_i, _f32p, _i, _i, _f32p, ctypes.c_float, _i,
                               ctypes.POINTER(_vp)]),
    ("rsx_sasa_counts_typed", _st, [_vp, _f32p, _u32p]),
    ("rsx_sasa_calc_typed", _st, [_vp, _f32p, _f32p]),
    ("rsx_sasa_destroy", _st, [_vp]),
    ("rsx_sasa_counts", _st, [_vp, _f32p, _f32p, _u32p]),
    ("rsx_sasa_calc", _st, [_vp, _f32p, _f32p, _f32p]),
    ("rsx_sasa_stats", _st, [_vp, ctypes.POINTER(ctypes.c_ulonglong),
                             ctypes.POINTER(ctypes.c_float)]),
    ("rsx_batch_create", _st, [_f32p, _i, _f32p, _i, np.ctypeslib.ndpointer(np.int32), _i,
                               ctypes.POINTER(DebyeOptions), ctypes.POINTER(_vp)]),
    ("rsx_batch_destroy", _st, [_vp]),
    ("rsx_batch_forward", _st, [_vp, _f32p, _f32p]),
    ("rsx_batch_set_targets", _st, [_vp, _f32p, _f32p]),
    ("rsx_batch_set_factors", _st, [_vp, _f32p, _i]),
    ("rsx_batch_set_water", _st, [_vp, ctypes.c_float, _i, _vp]),
    ("rsx_batch_forward_chi2_backward", _st, [_vp, _f32p, _vp, _vp, _vp]),
    ("rsx_batch_timing", _st, [_vp, ctypes.POINTER(ctypes.c_float)]),
    ("rsx_batch_config", _st, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i),
                               ctypes.POINTER(_i)]),
]

_lib = None


def lib():
    """Loads librsx.so once; raises LibraryNotBuilt when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LibraryNotBuilt(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
            "g.build()\"` (librsx has no CPU fallback)")
    try:
        L = ctypes.CDLL(LIB_PATH)
    except OSError as e:
        raise LibraryNotBuilt(f"cannot load {LIB_PATH}: {e}") from e
    for name, res, args in SIGNATURES:
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def exported_symbols():
    return [name for name, _, _ in SIGNATURES]


def check(status: int) -> None:
    if status != RSX_OK:
        raise ResaxsError(status, lib().rsx_last_error().decode(errors="replace"))


def last_error() -> str:
    return lib().rsx_last_error().decode(errors="replace")


def launch_count() -> int:
    return int(lib().rsx_launch_count())


def inject_fault(kind: int, nth: int) -> None:
    lib().rsx_debug_inject_fault(int(kind), int(nth))
