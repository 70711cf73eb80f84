"""ctypes loader for liblofgb.so (the C ABI declared in include/lofgb.h).

The library is built in-tree by lofloat_gb300/build.py. There is no fallback:
if the library cannot be built or loaded, every op raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None


class LofgbFormat(C.Structure):
    """``lofgb_format`` (include/lofgb.h)."""
    _fields_ = [("bitwidth", C.c_int32), ("mantissa_bits", C.c_int32), ("bias", C.c_int32),
                ("inf_behavior", C.c_uint8), ("nan_behavior", C.c_uint8),
                ("signedness", C.c_uint8), ("reserved", C.c_uint8)]


class LofgbRoundTask(C.Structure):
    """``lofgb_round_task`` (include/lofgb.h)."""
    _fields_ = [("in_", C.c_void_p), ("out", C.c_void_p), ("n", C.c_int64), ("fmt", LofgbFormat),
                ("mode", C.c_int32), ("stoch_len", C.c_int32), ("scale", C.c_float),
                ("reserved", C.c_int32), ("seed", C.c_uint64), ("offset", C.c_uint64)]


class LofgbGemmTask(C.Structure):
    """``lofgb_gemm_task`` (include/lofgb.h)."""
    _fields_ = [("A", C.c_void_p), ("lda", C.c_int64), ("B", C.c_void_p), ("ldb", C.c_int64),
                ("D", C.c_void_p), ("ldd", C.c_int64), ("trans_a", C.c_int32),
                ("trans_b", C.c_int32), ("M", C.c_int32), ("N", C.c_int32), ("K", C.c_int32),
                ("accum_mant_bits", C.c_int32), ("alpha", C.c_float), ("chunk", C.c_int32)]


class LofgbCodecFormat(C.Structure):
    """``lofgb_codec_format`` (include/lofgb.h)."""
    _fields_ = [("fmt", LofgbFormat), ("inf_or", C.c_uint32), ("inf_match", C.c_uint32),
                ("pos_inf", C.c_uint32), ("neg_inf", C.c_uint32), ("qnan", C.c_uint32),
                ("snan", C.c_uint32), ("nan_kind", C.c_uint8), ("neg_to_nan", C.c_uint8),
                ("reserved", C.c_uint8 * 2)]


class LofgbConv2dShape(C.Structure):
    """``lofgb_conv2d_shape`` (include/lofgb.h)."""
    _fields_ = [(f, C.c_int32) for f in ("n", "c", "h", "w", "k", "r", "s", "pad_h", "pad_w",
                                         "stride_h", "stride_w", "dil_h", "dil_w")]


# (name, restype, argtypes) for every entry point of include/lofgb.h
_vp, _i64, _i32, _u64, _f32, _f64, _sz = (C.c_void_p, C.c_int64, C.c_int, C.c_uint64, C.c_float,
                                          C.c_double, C.c_size_t)
_FP = C.POINTER(LofgbFormat)
SIGNATURES = [
    ("lofgb_strerror", C.c_char_p, [_i32]),
    ("lofgb_last_error_detail", C.c_char_p, []),
    ("lofgb_version", _i32, []),
    ("lofgb_round_f32", _i32, [_vp, _vp, _i64, _FP, _i32, _i32, _f32, _u64, _u64, _vp]),
    ("lofgb_round_f64", _i32, [_vp, _vp, _i64, _FP, _i32, _i32, _f64, _u64, _u64, _vp]),
    ("lofgb_round_f16", _i32, [_vp, _vp, _i64, _FP, _i32, _i32, _f32, _u64, _u64, _vp]),
    ("lofgb_round_mantissa_f32", _i32, [_vp, _vp, _i64, _i32, _i32, _i32, _f32, _u64, _u64, _vp]),
    ("lofgb_round_mantissa_f64", _i32, [_vp, _vp, _i64, _i32, _i32, _i32, _f64, _u64, _u64, _vp]),
    ("lofgb_round_mantissa_f16", _i32, [_vp, _vp, _i64, _i32, _i32, _i32, _f32, _u64, _u64, _vp]),
    ("lofgb_mx_round_f32", _i32, [_vp, _vp, _i64, _i32, _FP, _FP, _i32, _i32, _i32, _u64, _u64,
                                  _vp]),
    ("lofgb_mx_round_bf16", _i32, [_vp, _vp, _i64, _i32, _FP, _FP, _i32, _i32, _i32, _u64, _u64,
                                   _vp]),
    ("lofgb_gemm_f32", _i32, [_vp, _i64, _i32, _vp, _i64, _i32, _vp, _i64, _i32, _i32, _i32,
                              _i32, _i32, _f32, _i32, _i32, _vp, _sz, _vp]),
    ("lofgb_gemm_tc_workspace_size", _sz, [_i32, _i32, _i32]),
    ("lofgb_gemm_batched_f32", _i32, [_vp, _i64, _i64, _i32, _vp, _i64, _i64, _i32, _vp, _i64, _i64,
                                      _i32, _i32, _i32, _i32, _i32, _i32, _f32, _i32, _i32, _vp,
                                      _sz, _vp]),
    ("lofgb_gemm_batched_tc_workspace_size", _sz, [_i32, _i32, _i32, _i32]),
    ("lofgb_gemm_accfmt_f32", _i32, [_vp, _i64, _i32, _vp, _i64, _i32, _vp, _i64, _i32, _i32, _i32,
                                     _FP, _f32, _i32, _i32, _vp, _sz, _vp]),
    ("lofgb_gemm_tc_noalloc_f32", _i32, [_vp, _i64, _i32, _vp, _i64, _i32, _vp, _i64, _i32, _i32,
                                         _i32, _i32, _f32, _i32, _vp]),
    ("lofgb_gemm_f64_ref", _i32, [_vp, _i64, _i32, _vp, _i64, _i32, _vp, _i64, _i32, _i32, _i32,
                                  _vp]),
    ("lofgb_gemm_grouped_workspace_size", _sz, [C.POINTER(LofgbGemmTask), _i32]),
    ("lofgb_gemm_grouped_table_size", _sz, [C.POINTER(LofgbGemmTask), _i32]),
    ("lofgb_gemm_grouped_prepare", _i32, [C.POINTER(LofgbGemmTask), _i32, _vp, _sz, _i32, _i32, _vp,
                                          _sz, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("lofgb_gemm_grouped_launch", _i32, [_vp, _i64, _i64, _i32, _vp]),
    ("lofgb_gemm_grouped_launch_w", _i32, [_vp, _i64, _i64, _i32, _i32, _vp]),
    ("lofgb_round_grouped_table_size", _sz, [_i32]),
    ("lofgb_round_grouped_prepare", _i32, [C.POINTER(LofgbRoundTask), _i32, _vp, _sz,
                                           C.POINTER(C.c_int64)]),
    ("lofgb_round_grouped_prepare_items", _i32, [C.POINTER(LofgbRoundTask), _i32, _vp, _sz, _i64,
                                                 C.POINTER(C.c_int64)]),
    ("lofgb_round_grouped_f32", _i32, [_vp, _i32, _i64, _vp]),
    ("lofgb_conv2d_out_size", _i32, [C.POINTER(LofgbConv2dShape), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]),
    ("lofgb_conv2d_workspace_size", _sz, [C.POINTER(LofgbConv2dShape), _i32, _i32]),
    ("lofgb_conv2d_f32", _i32, [_vp, _vp, _vp, C.POINTER(LofgbConv2dShape), _i32, _i32, _f32, _i32,
                                _i32, _i32, _vp, _sz, _vp]),
    ("lofgb_pwl_silu_f32", _i32, [_vp, _vp, _i64, _vp, _i32, _f32, _vp]),
    ("lofgb_pwl_silu_f64", _i32, [_vp, _vp, _i64, _vp, _i32, _f32, _vp]),
    ("lofgb_pwl_silu_f16", _i32, [_vp, _vp, _i64, _vp, _i32, _f32, _vp]),
    ("lofgb_bn_workspace_size", _sz, [_i64, _i64, _i64]),
    ("lofgb_bn_stats_f32", _i32, [_vp, _i64, _i64, _i64, _i32, _vp, _vp, _vp, _vp, _f32, _vp, _sz,
                                  _vp]),
    ("lofgb_bn_apply_f32", _i32, [_vp, _vp, _i64, _i64, _i64, _vp, _vp, _f32, _i32, _vp, _vp, _vp,
                                  _vp, _i32, _vp]),
    ("lofgb_gemm_tc_wait_selftest", _i32, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _sz, C.c_uint32,
                                           _vp]),
    ("lofgb_packed_size", _sz, [_i32, _i64]),
    ("lofgb_encode_f32", _i32, [_vp, _vp, _i64, C.POINTER(LofgbCodecFormat), _i32, _i32, _i32, _i32,
                                _u64, _u64, _vp]),
    ("lofgb_decode_f32", _i32, [_vp, _vp, _i64, C.POINTER(LofgbCodecFormat), _i32, _vp]),
    ("lofgb_mx_encode_f32", _i32, [_vp, _vp, _vp, _i64, _i32, C.POINTER(LofgbCodecFormat),
                                   C.POINTER(LofgbCodecFormat), _i32, _i32, _i32, _i32, _u64, _u64,
                                   _vp]),
    ("lofgb_mx_decode_f32", _i32, [_vp, _vp, _vp, _i64, _i32, C.POINTER(LofgbCodecFormat),
                                   C.POINTER(LofgbCodecFormat), _vp]),
]


class LofgbError(RuntimeError):
    def __init__(self, status: int, where: str):
        lib_ = _lib
        msg = lib_.lofgb_strerror(status).decode() if lib_ else str(status)
        detail = lib_.lofgb_last_error_detail().decode() if lib_ else ""
        super().__init__(f"{where}: {msg}" + (f" ({detail})" if detail else ""))
        self.status = status


def library_path() -> str:
    return _build.LIB


def lib():
    """Build (if stale) and load liblofgb.so."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = C.CDLL(path)
            for name, res, args in SIGNATURES:
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != 0:
        raise LofgbError(status, where)


def exported_symbols() -> list[str]:
    return [name for name, _, _ in SIGNATURES]
