"""ctypes binding of libnumrs_gb300.so (the C ABI in include/numrs_gpu.h).

The library must be built (``numrs_gb300.build.build()``); importing the
package without it raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnumrs_gb300.so")

# Enumerations (must match include/numrs_gpu.h)
F32, F64, I32, I64 = 0, 1, 2, 3
OK = 0
ERR_INVALID, ERR_SHAPE, ERR_DTYPE, ERR_AXIS, ERR_EMPTY, ERR_STRIDE = -1, -2, -3, -4, -5, -6
ERR_CUDA, ERR_TIMEOUT, ERR_ALLOC, ERR_UNSUPPORTED, ERR_TOO_LARGE, ERR_IO = -7, -8, -9, -10, -11, -12
NPY_MAX_DIMS = 32
SUM, MEAN, MAX, MIN, PROD, VAR, STD, ARGMAX, ARGMIN = 0, 1, 2, 3, 4, 5, 6, 7, 8
AXIS_NONE = -(2 ** 63)
OP_INPUT, OP_SCALAR, OP_ADD, OP_SUB, OP_MUL, OP_DIV = 0, 1, 2, 3, 4, 5
OP_NEG, OP_ABS, OP_SQRT, OP_EXP, OP_LN, OP_MAX, OP_MIN = 6, 7, 8, 9, 10, 11, 12
GEMM_ACCUMULATE, GEMM_TRANS_A, GEMM_TRANS_B = 1, 2, 4
GEMM_AUTO, GEMM_DMMA, GEMM_SIMT, GEMM_GENERIC, GEMM_SIMT_SMALL = 0, 1, 2, 3, 4
PEAK_FP64_DMMA, PEAK_FP32_FMA = 0, 1
PLAN_F64_DMMA, PLAN_F64_OZAKI = 0, 1
PLAN_F32_FMA, PLAN_F32_OZAKI = 0, 1
RNG_UNIFORM, RNG_NORMAL, RNG_INT, RNG_OZAKI = 0, 1, 2, 3
TILE_VARIANTS = 6


class NpyInfo(C.Structure):
    """nrs_npy_info."""
    _fields_ = [("descr", C.c_char * 16), ("dtype", C.c_int), ("itemsize", C.c_int),
                ("fortran_order", C.c_int), ("ndim", C.c_int), ("shape", C.c_int64 * NPY_MAX_DIMS),
                ("data_offset", C.c_int64), ("nbytes", C.c_int64)]


class UfuncOp(C.Structure):
    _fields_ = [("code", C.c_int32), ("arg", C.c_int32), ("scalar", C.c_double)]


class OzakiInfo(C.Structure):
    _fields_ = [("slices", C.c_int32), ("products", C.c_int32), ("slice_bits", C.c_int32),
                ("k_chunk", C.c_int32), ("est_rel_error", C.c_double), ("spread", C.c_double)]


class PlanOptions(C.Structure):
    _fields_ = [("f64_mode", C.c_int32), ("f64_slices", C.c_int32), ("f64_digit_bits", C.c_int32),
                ("f32_mode", C.c_int32)]


class AutotuneReport(C.Structure):
    _fields_ = [("untuned_ms", C.c_double), ("isolated_ms", C.c_double), ("final_ms", C.c_double),
                ("ozaki_ms", C.c_double), ("buckets", C.c_int32), ("trials", C.c_int32),
                ("options", PlanOptions), ("ozaki_f32_ms", C.c_double)]


class GemmDesc(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("flags", C.c_uint32), ("m", C.c_int64), ("k", C.c_int64),
                ("n", C.c_int64), ("A", C.c_void_p), ("lda", C.c_int64), ("B", C.c_void_p),
                ("ldb", C.c_int64), ("C", C.c_void_p), ("ldc", C.c_int64)]


class RowReduceDesc(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("op", C.c_int32), ("len", C.c_int64), ("x", C.c_void_p),
                ("out", C.c_void_p)]


_lock = threading.Lock()
_lib = None

# (name, restype, argtypes) for every exported function.
_vp, _i, _i64, _u64, _d, _f, _sz, _u = (C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double,
                                        C.c_float, C.c_size_t, C.c_uint)
_u32 = C.c_uint32
_P64 = C.POINTER(C.c_int64)
SIGNATURES = {
    "nrs_abi_version": (_i, []),
    "nrs_status_string": (C.c_char_p, [_i]),
    "nrs_create": (_i, [_i, C.POINTER(_vp)]),
    "nrs_destroy": (_i, [_vp]),
    "nrs_set_stream": (_i, [_vp, _vp]),
    "nrs_use_own_stream": (_i, [_vp]),
    "nrs_get_stream": (_vp, [_vp]),
    "nrs_synchronize": (_i, [_vp]),
    "nrs_last_error": (C.c_char_p, [_vp]),
    "nrs_malloc": (_i, [_vp, _sz, C.POINTER(_vp)]),
    "nrs_free": (_i, [_vp, _vp]),
    "nrs_host_alloc": (_i, [_vp, _sz, C.POINTER(_vp)]),
    "nrs_host_free": (_i, [_vp, _vp]),
    "nrs_memcpy_h2d": (_i, [_vp, _vp, _vp, _sz]),
    "nrs_memcpy_d2h": (_i, [_vp, _vp, _vp, _sz]),
    "nrs_fill_random": (_i, [_vp, _i, _i, _u64, _i64, _d, _d, _vp]),
    "nrs_reduce": (_i, [_vp, _i, _i, _i, _P64, _P64, _i64, _i64, _vp, _vp]),
    "nrs_reduce_flat_noalloc": (_i, [_vp, _i, _i, _i64, _vp, _vp]),
    "nrs_ufunc": (_i, [_vp, _i, C.POINTER(UfuncOp), _i, _i, _P64, _i, C.POINTER(_vp), _P64, _vp, _P64]),
    "nrs_exp_affine": (_i, [_vp, _i, _i64, _vp, _d, _d, _vp]),
    "nrs_ufunc_reduce": (_i, [_vp, _i, _i, _i, _P64, _P64, _i64, _vp, _vp, _vp]),
    "nrs_npy_inspect": (_i, [_vp, C.c_char_p, _i64, C.POINTER(NpyInfo)]),
    "nrs_npz_locate": (_i, [_vp, C.c_char_p, C.c_char_p, C.POINTER(_i64), C.POINTER(_i64)]),
    "nrs_npy_read": (_i, [_vp, C.c_char_p, C.POINTER(NpyInfo), _vp, _i64]),
    "nrs_npy_write": (_i, [_vp, C.c_char_p, _i, _i, _P64, _vp]),
    "nrs_accumulate": (_i, [_vp, _i, _i, _i, _P64, _P64, _i64, _vp, _vp, _P64]),
    "nrs_gemm": (_i, [_vp, _i, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _u, _i]),
    "nrs_set_sm_budget": (_i, [_vp, _i]),
    "nrs_test_expire_next_wait": (_i, [_vp, _u32]),
    "nrs_probe_peak": (_i, [_vp, _i, C.POINTER(C.c_double)]),
    "nrs_gemm_ozaki": (_i, [_vp, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _u32, _i,
                            C.POINTER(OzakiInfo)]),
    "nrs_tuner_save": (_i, [_vp, C.c_char_p]),
    "nrs_tuner_load": (_i, [_vp, C.c_char_p]),
    "nrs_selector_save": (_i, [_vp, _vp, C.c_char_p]),
    "nrs_selector_load": (_i, [_vp, _vp, C.c_char_p]),
    "nrs_plan_autotune": (_i, [_vp, _i64, C.POINTER(GemmDesc), _i64, C.POINTER(RowReduceDesc),
                               C.POINTER(PlanOptions), _i, _i, C.POINTER(AutotuneReport)]),
    "nrs_plan_create_ex": (_i, [_vp, _i64, C.POINTER(GemmDesc), _i64, C.POINTER(RowReduceDesc),
                                C.POINTER(PlanOptions), C.POINTER(_vp)]),
    "nrs_plan_f64_info": (_i, [_vp, C.POINTER(_i64), C.POINTER(_i), C.POINTER(_i)]),
    "nrs_plan_f32_info": (_i, [_vp, C.POINTER(_i64), C.POINTER(_i), C.POINTER(_i)]),
    "nrs_gemm_ozaki_grouped": (_i, [_vp, _i64, C.POINTER(GemmDesc), _i, C.POINTER(_i), C.POINTER(OzakiInfo)]),
    "nrs_plan_create": (_i, [_vp, _i64, C.POINTER(GemmDesc), _i64, C.POINTER(RowReduceDesc),
                             C.POINTER(_vp)]),
    "nrs_plan_run": (_i, [_vp, _vp, _i]),
    "nrs_plan_stats": (_i, [_vp, _P64, _P64]),
    "nrs_plan_destroy": (_i, [_vp]),
    "nrs_tile_variant_info": (_i, [_i, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]),
    "nrs_tune_gemm": (_i, [_vp, _i, _i64, _i64, _i64, _u, _i64, _i, C.POINTER(_f), C.POINTER(_i)]),
    "nrs_tuner_set_selector": (_i, [_vp, _vp]),
    "nrs_tuner_set": (_i, [_vp, _i, _i64, _i64, _i64, _i]),
    "nrs_tuner_get": (_i, [_vp, _i, _i64, _i64, _i64]),
    "nrs_tuner_clear": (_i, [_vp]),
    "nrs_selector_create": (_i, [_vp, _i, _i, _i, _u64, C.POINTER(_vp)]),
    "nrs_selector_destroy": (_i, [_vp]),
    "nrs_selector_num_params": (_i64, [_vp]),
    "nrs_selector_get_params": (_i, [_vp, _vp, _vp]),
    "nrs_selector_set_params": (_i, [_vp, _vp, _vp]),
    "nrs_selector_forward_backward": (_i, [_vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, C.POINTER(_f)]),
    "nrs_selector_train": (_i, [_vp, _vp, _i64, _vp, _vp, _vp, _i, _i64, _f, _u64, C.POINTER(_f)]),
    "nrs_selector_predict": (_i, [_vp, _vp, _i64, _vp, _vp]),
}


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with numrs_gb300.build.build(); "
                    "there is no CPU fallback")
            lib = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name, None)
                if fn is None:
                    continue
                fn.restype, fn.argtypes = res, args
            _lib = lib
    return _lib


class NumRs2Error(RuntimeError):
    """Raised for a non-zero status (mirrors numrs2's NumRs2Error kinds)."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"[{status}] {message}")


class DimensionMismatch(NumRs2Error):
    pass


class ShapeMismatch(NumRs2Error):
    pass


class InvalidOperation(NumRs2Error):
    pass


class DeviceTimeout(NumRs2Error):
    pass


_KINDS = {ERR_AXIS: DimensionMismatch, ERR_SHAPE: ShapeMismatch, ERR_EMPTY: InvalidOperation,
          ERR_TIMEOUT: DeviceTimeout}


def check(status: int, handle=None) -> None:
    if status == OK:
        return
    lib = load()
    msg = lib.nrs_status_string(status).decode()
    if handle is not None:
        detail = lib.nrs_last_error(handle).decode()
        if detail:
            msg = f"{msg}: {detail}"
    raise _KINDS.get(status, NumRs2Error)(status, msg)


def i64_array(values):
    vals = [int(v) for v in values]
    arr = (C.c_int64 * max(1, len(vals)))(*vals)
    return arr
