"""ctypes binding of libtomoj_gb300.so (declarations in include/tomoj_gb300.h).

The engine has no CPU fallback: if the library or a GPU is missing, the calls
raise.  Nothing here imports the oracle.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libtomoj_gb300.so")

TOMO_OK = 0
ERRORS = {
    -1: "TOMO_ERR_INVALID", -2: "TOMO_ERR_CUDA", -3: "TOMO_ERR_NOMEM", -4: "TOMO_ERR_STATE",
    -5: "TOMO_ERR_UNSUPPORTED", -6: "TOMO_ERR_CANCELLED", -7: "TOMO_ERR_DEVICE",
}
FILL_NONE, FILL_AVG, FILL_NAN = 0, 1, 2
WEIGHT_NONE, WEIGHT_RADERMACHER, WEIGHT_RAMP, WEIGHT_HAMMING_RAMP = 0, 1, 2, 3
PREC_FP32 = 0
PREC_BF16 = 1
PREC_FP16 = 2


class TomoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class NoMemoryError(TomoError):
    pass


class CancelledError(TomoError):
    pass


class UnsupportedError(TomoError):
    pass


class Geom(C.Structure):
    _fields_ = [("W", C.c_int32), ("H", C.c_int32), ("D", C.c_int32), ("w", C.c_int32), ("h", C.c_int32),
                ("nproj", C.c_int32), ("vol_center", C.c_double * 3), ("proj_center", C.c_double * 4),
                ("scale", C.c_double)]


class Params(C.Structure):
    _fields_ = [("positivity", C.c_int32), ("long_object", C.c_int32), ("fill", C.c_int32),
                ("normalize", C.c_int32), ("precision", C.c_int32), ("reserved", C.c_int32 * 3)]


_lib = None
_P = C.c_void_p
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)

# name -> (restype, argtypes); mirrors include/tomoj_gb300.h one to one.
SIGNATURES = {
    "tomo_abi_version": (C.c_int32, []),
    "tomo_last_error": (C.c_char_p, []),
    "tomo_set_memory_limit": (C.c_int32, [C.c_uint64]),
    "tomo_memory_in_use": (C.c_uint64, []),
    "tomo_device_memory": (C.c_int32, [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "tomo_kernel_launches": (C.c_uint64, []),
    "tomo_create": (C.c_int32, [C.POINTER(Geom), C.POINTER(Params), C.POINTER(_P)]),
    "tomo_destroy": (C.c_int32, [_P]),
    "tomo_set_stream": (C.c_int32, [_P, C.c_void_p]),
    "tomo_set_priority": (C.c_int32, [_P, C.c_int32]),
    "tomo_load_series": (C.c_int32, [_P, C.c_void_p, C.c_int32, _f64p, _f64p, _f64p]),
    "tomo_get_aligned": (C.c_int32, [_P, C.c_int32, _f32p]),
    "tomo_set_fill": (C.c_int32, [_P, C.c_int32]),
    "tomo_set_volume": (C.c_int32, [_P, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "tomo_get_volume": (C.c_int32, [_P, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "tomo_fill_volume": (C.c_int32, [_P, C.c_float]),
    "tomo_volume_device_ptr": (C.c_int32, [_P, C.POINTER(C.c_void_p)]),
    "tomo_share_volume": (C.c_int32, [_P, _P]),
    "tomo_add_projection": (C.c_int32, [_P, C.c_int32]),
    "tomo_clear_projections": (C.c_int32, [_P]),
    "tomo_project": (C.c_int32, [_P, C.c_int32, C.c_int32]),
    "tomo_project_and_difference": (C.c_int32, [_P, C.c_double, C.c_int32, C.c_int32, _f64p]),
    "tomo_backproject": (C.c_int32, [_P, C.c_int32, C.c_int32]),
    "tomo_start_iteration": (C.c_int32, [_P]),
    "tomo_end_iteration": (C.c_int32, [_P]),
    "tomo_get_projection": (C.c_int32, [_P, C.c_int32, _f32p]),
    "tomo_get_norm": (C.c_int32, [_P, C.c_int32, _f32p]),
    "tomo_get_difference": (C.c_int32, [_P, C.c_int32, _f32p]),
    "tomo_projection_count": (C.c_int32, [_P]),
    "tomo_set_row_streams": (C.c_int32, [_P, C.c_int32]),
    "tomo_set_positivity": (C.c_int32, [_P, C.c_int32]),
    "tomo_set_long_object": (C.c_int32, [_P, C.c_int32]),
    "tomo_set_scale": (C.c_int32, [_P, C.c_double]),
    "tomo_set_centers": (C.c_int32, [_P, _f64p, _f64p]),
    "tomo_set_weighting": (C.c_int32, [_P, C.c_int32, C.c_double, _f64p, _f64p]),
    "tomo_set_tvm": (C.c_int32, [_P, C.c_float, C.c_float, C.c_float, C.c_int32]),
    "tomo_set_fista": (C.c_int32, [_P, C.c_int32]),
    "tomo_set_bayesian": (C.c_int32, [_P, C.c_double, C.c_double, C.c_int32]),
    "tomo_set_bgart": (C.c_int32, [_P, C.c_double, C.c_int32, C.c_int32, C.c_double, C.c_int32]),
    "tomo_set_compressed_sensing": (C.c_int32, [_P, C.c_int32, C.c_double, C.c_double, C.c_double,
                                                C.POINTER(C.c_int32), C.c_int32]),
    "tomo_compressed_sensing_threshold": (C.c_int32, [_P, _f64p]),
    "tomo_run_wbp": (C.c_int32, [_P, C.c_int32, C.c_int32]),
    "tomo_run_ossart": (C.c_int32, [_P, C.c_int32, C.c_double, C.c_int32, C.c_uint64, C.c_int32, C.c_int32,
                                    C.c_int32, _f64p]),
    "tomo_first_index": (C.c_int32, [C.c_uint64, C.c_int32, C.c_int32]),
    "tomo_order": (C.c_int32, [_P, C.c_int32, _i32p]),
    "tomo_order_shuffle": (C.c_int32, [C.c_int32, _f64p, C.c_int32, _i32p]),
    "tomo_cancel": (C.c_int32, [_P]),
    "tomo_set_profiling": (C.c_int32, [_P, C.c_int32]),
    "tomo_profile_read": (C.c_int32, [_P, _f64p]),
    "tomo_set_tilts_per_cta": (C.c_int32, [_P, C.c_int32]),
    "tomo_set_bp_rows": (C.c_int32, [_P, C.c_int32]),
    "tomo_autotune": (C.c_int32, [_P, C.c_int32, C.c_int32, _f64p]),
    "tomo_debug_hold_first_copy": (C.c_int32, [_P, C.c_int32]),
    "tomo_batch_create": (C.c_int32, [C.POINTER(C.c_void_p)]),
    "tomo_batch_destroy": (C.c_int32, [C.c_void_p]),
    "tomo_batch_set": (C.c_int32, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int32]),
    "tomo_batch_set_priority": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tomo_batch_set_persistent": (C.c_int32, [C.c_void_p, C.c_int32]),
    "tomo_batch_set_stream": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tomo_batch_iteration": (C.c_int32, [C.c_void_p, _f64p, _i32p, _i32p, C.c_int32, _f64p]),
    "tomo_project_and_difference_noalloc": (C.c_int32, [C.POINTER(Geom), _f64p, _i32p, C.c_int32, C.c_double,
                                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                        C.c_void_p, _f64p, C.c_void_p]),
}


def load():
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with tomoj_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


OK = 0
ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_UNSUPPORTED, ERR_CANCELLED, ERR_DEVICE = -1, -2, -3, -4, -5, -6, -7


def check(rc: int) -> None:
    if rc != TOMO_OK:
        msg = load().tomo_last_error().decode(errors="replace")
        cls = {-3: NoMemoryError, -6: CancelledError, -5: UnsupportedError}.get(rc, TomoError)
        raise cls(rc, msg)


def ptr(a: np.ndarray, ct=C.c_float):
    return a.ctypes.data_as(C.POINTER(ct))


def make_geom(W, H, D, w, h, nproj, vol_center=None, proj_center=None, scale=1.0) -> Geom:
    g = Geom()
    g.W, g.H, g.D, g.w, g.h, g.nproj = W, H, D, w, h, nproj
    vc = vol_center if vol_center is not None else (math.nan,) * 3
    pc = proj_center if proj_center is not None else (math.nan,) * 4
    g.vol_center = (C.c_double * 3)(*vc)
    g.proj_center = (C.c_double * 4)(*pc)
    g.scale = scale
    return g


def precision_code(v) -> int:
    """PREC_* value of "fp32" / "bf16" / "fp16" (or of an int)."""
    if isinstance(v, str):
        names = {"fp32": PREC_FP32, "f32": PREC_FP32, "bf16": PREC_BF16, "fp16": PREC_FP16, "f16": PREC_FP16}
        if v.lower() not in names:
            raise ValueError(f"unknown precision {v!r}")
        return names[v.lower()]
    return int(v)


def make_params(positivity=False, long_object=False, fill=FILL_NAN, normalize=False, precision=PREC_FP32) -> Params:
    p = Params()
    p.positivity, p.long_object, p.fill, p.normalize, p.precision = (int(positivity), int(long_object), int(fill),
                                                                      int(normalize), int(precision))
    return p
