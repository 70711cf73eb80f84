"""ctypes front-end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module. It loads ``oracle/_build/liblof_oracle.so`` (built by
``oracle/build_oracle.py``) and, when present, the reference shim
``oracle/_ref/libref_shim.so``. Arrays are numpy; f16 data travels as uint16
bit patterns.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle as _bo

_lib = None
_ref = None


class ConvShape(C.Structure):
    """Same layout as ``lofgb_conv2d_shape`` in include/lofgb.h."""
    _fields_ = [(f, C.c_int32) for f in ("n", "c", "h", "w", "k", "r", "s", "pad_h", "pad_w",
                                         "stride_h", "stride_w", "dil_h", "dil_w")]


class Format(C.Structure):
    """Same layout as ``lofgb_format`` in include/lofgb.h."""
    _fields_ = [("bitwidth", C.c_int32), ("mantissa_bits", C.c_int32), ("bias", C.c_int32),
                ("inf_behavior", C.c_uint8), ("nan_behavior", C.c_uint8),
                ("signedness", C.c_uint8), ("reserved", C.c_uint8)]


class CodecFormat(C.Structure):
    """Same layout as ``lofgb_codec_format`` in include/lofgb.h."""
    _fields_ = [("fmt", Format), ("inf_or", C.c_uint32), ("inf_match", C.c_uint32),
                ("pos_inf", C.c_uint32), ("neg_inf", C.c_uint32), ("qnan", C.c_uint32),
                ("snan", C.c_uint32), ("nan_kind", C.c_uint8), ("neg_to_nan", C.c_uint8),
                ("reserved", C.c_uint8 * 2)]


def fmt(bitwidth, mantissa_bits, bias, saturating=True, signed=True, nan_754=False) -> Format:
    return Format(bitwidth, mantissa_bits, bias, 1 if saturating else 0, 1 if nan_754 else 0,
                  0 if signed else 1, 0)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        path = _bo.build_oracle()
        L = C.CDLL(path)
        vp, i64, i32, u64, f32, f64 = C.c_void_p, C.c_int64, C.c_int, C.c_uint64, C.c_float, C.c_double
        P = C.POINTER(Format)
        L.orc_rng.restype = u64
        L.orc_rng.argtypes = [u64, u64]
        L.orc_rng_elem.restype = u64
        L.orc_rng_elem.argtypes = [u64, u64, C.c_int]
        L.orc_rng_lanes_log2.restype = C.c_int
        L.orc_rng_lanes_log2.argtypes = [C.c_int, C.c_int]
        for name, sc in (("orc_round_f32", f32), ("orc_round_f64", f64), ("orc_round_f16", f32)):
            getattr(L, name).argtypes = [vp, vp, i64, P, i32, i32, sc, u64, u64, i32]
        for name, sc in (("orc_round_mantissa_f32", f32), ("orc_round_mantissa_f64", f64),
                         ("orc_round_mantissa_f16", f32)):
            getattr(L, name).argtypes = [vp, vp, i64, i32, i32, i32, sc, u64, u64, i32]
        for name in ("orc_round_f32_bits", "orc_round_f64_bits", "orc_round_f16_bits"):
            getattr(L, name).argtypes = [vp, vp, i64, P, i32, i32, vp, vp]
        for name in ("orc_round_mantissa_f32_bits", "orc_round_mantissa_f64_bits",
                     "orc_round_mantissa_f16_bits"):
            getattr(L, name).argtypes = [vp, vp, i64, i32, i32, i32, vp, vp]
        L.orc_mx_round_f32.argtypes = [vp, vp, i64, i32, P, P, i32, i32, i32, u64, u64, i32, i32]
        L.orc_gemm_f32.argtypes = [vp, i64, i32, vp, i64, i32, vp, i64, i32, i32, i32, i32, f32, i32]
        L.orc_gemm_f32_rows.argtypes = [vp, i64, i32, vp, i64, i32, vp, i64, i32, i32, i32, i32,
                                        f32, i32, i32, i32]
        L.orc_gemm_chunked_f32.argtypes = [vp, i64, i32, vp, i64, i32, vp, i64, i32, i32, i32, i32,
                                           i32, f32, i32]
        L.orc_conv2d_f32.argtypes = [vp, vp, vp, C.POINTER(ConvShape), i32, f32, i32, i64, i64, i32]
        L.orc_pwl_silu_f32.argtypes = [vp, vp, i64, vp, i32, f32]
        CP = C.POINTER(CodecFormat)
        L.orc_codec_encode_rep.restype = C.c_uint32
        L.orc_codec_encode_rep.argtypes = [f32, CP, i32, i32, i32, u64, f64]
        L.orc_codec_decode_rep.restype = f32
        L.orc_codec_decode_rep.argtypes = [C.c_uint32, CP]
        L.orc_packed_size.restype = i64
        L.orc_packed_size.argtypes = [i32, i64]
        L.orc_encode_f32.argtypes = [vp, vp, i64, CP, i32, i32, i32, i32, u64, u64]
        L.orc_decode_f32.argtypes = [vp, vp, i64, CP, i32]
        L.orc_mx_encode_f32.argtypes = [vp, i64, i32, CP, CP, i32, i32, i32, i32, u64, u64, vp, vp]
        L.orc_gemm_accfmt_f32.argtypes = [vp, i64, i32, vp, i64, i32, vp, i64, i32, i32, i32, P,
                                          f32, i32]
        L.orc_rto_fma.restype = f32
        L.orc_rto_fma.argtypes = [f32, f32, f32]
        L.orc_max_threads.restype = i32
        L.orc_validate_format.argtypes = [P, i32]
        _lib = L
    return _lib


def ref():
    """The reference shim, or None when it is not built (no reference checkout)."""
    global _ref
    if _ref is None:
        path = _bo.build_ref() if os.path.exists(_bo.reference_src_dir()) else (
            _bo.REF_SO if os.path.exists(_bo.REF_SO) else None)
        if path is None:
            return None
        R = C.CDLL(path)
        vp, i64, i32, f32 = C.c_void_p, C.c_int64, C.c_int, C.c_float
        for name in ("ref_round_f32", "ref_round_f64"):
            getattr(R, name).argtypes = [vp, vp, i64, i32, i32, i32, i32, i32, i32, i32, i32, vp, vp, vp]
        for name in ("ref_round_mantissa_f32", "ref_round_mantissa_f64", "ref_round_mantissa_f16"):
            getattr(R, name).argtypes = [vp, vp, i64, i32, i32, i32, vp, vp, vp]
        R.ref_mx_round_f32.argtypes = [vp, vp, i64, i32] + [i32] * 13
        R.ref_gemm_f32.argtypes = [vp, vp, vp, i32, i32, i32, i32, f32]
        R.ref_encode_f32.argtypes = [vp, vp, i64, vp, i32, i32, i32, i32]
        R.ref_decode_f32.argtypes = [vp, vp, i64, vp, i32]
        R.ref_packed_size.restype = i64
        R.ref_packed_size.argtypes = [i32, i64]
        _ref = R
    return _ref


def _check(st):
    if st != 0:
        raise ValueError(f"oracle status {st}")


_DT = {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64", np.dtype(np.uint16): "f16"}


def rng(seed: int, idx: int) -> int:
    return lib().orc_rng(seed, idx)


def rng_lanes_log2(mode: int, stoch_len: int) -> int:
    return lib().orc_rng_lanes_log2(mode, stoch_len)


def rng_elem(seed: int, g: int, lg: int) -> int:
    """Random word of element g (lane g mod 2^lg of output g >> lg)."""
    return lib().orc_rng_elem(seed, g, lg)


def round(x: np.ndarray, f: Format, mode: int, stoch_len: int = 0, scale: float = 1.0,
          seed: int = 0, offset: int = 0, nthreads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    t = _DT[x.dtype]
    _check(getattr(lib(), f"orc_round_{t}")(_p(x), _p(out), x.size, C.byref(f), mode, stoch_len,
                                            scale, seed, offset, nthreads))
    return out


def round_mantissa(x: np.ndarray, mbits: int, mode: int, stoch_len: int = 0, scale: float = 1.0,
                   seed: int = 0, offset: int = 0, nthreads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    t = _DT[x.dtype]
    _check(getattr(lib(), f"orc_round_mantissa_{t}")(_p(x), _p(out), x.size, mbits, mode,
                                                     stoch_len, scale, seed, offset, nthreads))
    return out


def round_bits(x, f: Format | None, mode: int, stoch_len: int, rbits=None, usamp=None,
               mbits: int | None = None) -> np.ndarray:
    """Round with explicit per-element random words (golden pinning)."""
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    t = _DT[x.dtype]
    rb = None if rbits is None else np.ascontiguousarray(rbits, dtype=np.uint64)
    us = None if usamp is None else np.ascontiguousarray(usamp, dtype=np.float64)
    if f is not None:
        st = getattr(lib(), f"orc_round_{t}_bits")(_p(x), _p(out), x.size, C.byref(f), mode,
                                                   stoch_len, _p(rb), _p(us))
    else:
        st = getattr(lib(), f"orc_round_mantissa_{t}_bits")(_p(x), _p(out), x.size, mbits, mode,
                                                            stoch_len, _p(rb), _p(us))
    _check(st)
    return out


def mx_round(x: np.ndarray, block: int, ef: Format, sf: Format, mode: int = 0,
             scale_mode: int = 0, stoch_len: int = 0, seed: int = 0, offset: int = 0,
             scale_formula: int = 0, nthreads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    _check(lib().orc_mx_round_f32(_p(x), _p(out), x.size, block, C.byref(ef), C.byref(sf), mode,
                                  scale_mode, stoch_len, seed, offset, scale_formula, nthreads))
    return out


def _gemm_args(A, B, trans_a, trans_b):
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    M, K = (A.shape[1], A.shape[0]) if trans_a else A.shape
    Kb, N = (B.shape[1], B.shape[0]) if trans_b else B.shape
    assert K == Kb, "inner dimensions differ"
    return A, B, M, N, K


def gemm(A, B, mbits: int, alpha: float = 1.0, trans_a: int = 0, trans_b: int = 0,
         nthreads: int = 0) -> np.ndarray:
    """Bit-exact sequential-k emulated GEMM (A M×K or K×M when trans_a)."""
    A, B, M, N, K = _gemm_args(A, B, trans_a, trans_b)
    D = np.empty((M, N), np.float32)
    _check(lib().orc_gemm_f32(_p(A), A.shape[1], trans_a, _p(B), B.shape[1], trans_b, _p(D), N,
                              M, N, K, mbits, alpha, nthreads))
    return D


def gemm_rows(A, B, mbits: int, row0: int, rows: int, alpha: float = 1.0, trans_a: int = 0,
              trans_b: int = 0, nthreads: int = 0) -> np.ndarray:
    A, B, M, N, K = _gemm_args(A, B, trans_a, trans_b)
    D = np.zeros((M, N), np.float32)
    _check(lib().orc_gemm_f32_rows(_p(A), A.shape[1], trans_a, _p(B), B.shape[1], trans_b,
                                   _p(D), N, M, N, K, mbits, alpha, row0, rows, nthreads))
    return D[row0:row0 + rows]


def gemm_chunked(A, B, mbits: int, chunk: int, alpha: float = 1.0, trans_a: int = 0,
                 trans_b: int = 0, nthreads: int = 0) -> np.ndarray:
    A, B, M, N, K = _gemm_args(A, B, trans_a, trans_b)
    D = np.empty((M, N), np.float32)
    _check(lib().orc_gemm_chunked_f32(_p(A), A.shape[1], trans_a, _p(B), B.shape[1], trans_b,
                                      _p(D), N, M, N, K, mbits, chunk, alpha, nthreads))
    return D


def rto_fma(a: float, b: float, c: float) -> float:
    return lib().orc_rto_fma(a, b, c)


def max_threads() -> int:
    return lib().orc_max_threads()


CONV_ORDERS = {"crs": 0, "tiled8": 1}


def conv_out_size(h, w, r, s, stride=(1, 1), padding=(0, 0), dilation=(1, 1)):
    p = (h + 2 * padding[0] - dilation[0] * (r - 1) - 1) // stride[0] + 1
    q = (w + 2 * padding[1] - dilation[1] * (s - 1) - 1) // stride[1] + 1
    return p, q


def conv2d(x, w, mbits: int, stride=(1, 1), padding=(0, 0), dilation=(1, 1), alpha: float = 1.0,
           order: str = "crs", col0: int = 0, ncols: int = -1, nthreads: int = 0) -> np.ndarray:
    """Emulated-accumulation conv2d, NCHW x KCRS -> NKPQ (lofgb_conv2d_f32).
    With ncols >= 0 only output pixels [col0, col0 + ncols) of the flat (n, p, q)
    index are computed; the rest of the returned array is 0."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    w = np.ascontiguousarray(w, dtype=np.float32)
    n, c, h, wd = x.shape
    k, c2, r, s_ = w.shape
    assert c == c2
    sh = ConvShape(n, c, h, wd, k, r, s_, padding[0], padding[1], stride[0], stride[1],
                   dilation[0], dilation[1])
    p, q = conv_out_size(h, wd, r, s_, stride, padding, dilation)
    y = np.zeros((n, k, p, q), np.float32)
    _check(lib().orc_conv2d_f32(_p(x), _p(w), _p(y), C.byref(sh), mbits, alpha,
                                CONV_ORDERS[order], col0, ncols, nthreads))
    return y


def pwl_silu(x, lut, R: float) -> np.ndarray:
    """Piecewise-linear SiLU on float32 values (src/LoPy_bind.cpp:258-269)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    lut = np.ascontiguousarray(lut, dtype=np.float32)
    y = np.empty_like(x)
    _check(lib().orc_pwl_silu_f32(_p(x), _p(y), x.size, _p(lut), lut.size - 1, R))
    return y


# ---- storage codec ---------------------------------------------------------------
def codec_fmt(bitwidth, mantissa_bits, bias, saturating=True, signed=True, nan_754=False,
              inf_or=0, inf_match=0xFFFFFFFF, pos_inf=0, neg_inf=0, qnan=0, snan=0, nan_kind=0,
              neg_to_nan=False) -> CodecFormat:
    f = CodecFormat()
    f.fmt = fmt(bitwidth, mantissa_bits, bias, saturating, signed, nan_754)
    f.inf_or, f.inf_match, f.pos_inf, f.neg_inf = inf_or, inf_match, pos_inf, neg_inf
    f.qnan, f.snan, f.nan_kind, f.neg_to_nan = qnan, snan, nan_kind, int(neg_to_nan)
    return f


def codec_p3109(k, p, signed=True, saturating=True, bias=None, neg_to_nan=False) -> CodecFormat:
    """P3109 <k, p> with the reference's P_3109 checkers (src/lo_float.h:1679-1760)."""
    bias = (1 << (k - p - 1)) if bias is None else bias
    nan = (1 << (k - 1)) if signed else (1 << k) - 1
    if saturating:
        inf_or, inf_match, pos, neg = 0, 0xFFFFFFFF, ((1 << (k - 1)) - 1 if signed else (1 << k) - 2), \
            ((1 << k) - 1 if signed else 0)
    else:
        inf_or, inf_match = 1 << (k - 1), ((1 << k) - 1 if signed else (1 << k) - 2)
        pos, neg = ((1 << (k - 1)) - 1 if signed else (1 << k) - 2), ((1 << k) - 1 if signed else 0)
    return codec_fmt(k, p - 1, bias, saturating, signed, False, inf_or, inf_match, pos, neg, nan,
                     nan, 0, neg_to_nan)


def codec_ieee(bitwidth, mantissa_bits, bias, qnan, snan) -> CodecFormat:
    """IEEE-style format (FP16 / BF16 checkers, src/fp_tools.hpp:334-395):
    infinity = exponent all ones, mantissa 0; NaN = exponent all ones, mantissa != 0."""
    sign = 1 << (bitwidth - 1)
    expall = ((1 << (bitwidth - 1 - mantissa_bits)) - 1) << mantissa_bits
    return codec_fmt(bitwidth, mantissa_bits, bias, False, True, True, sign, sign | expall, expall,
                     sign | expall, qnan, snan, 1)


def codec_fields(f: CodecFormat) -> np.ndarray:
    """The int64 vector the reference shim's make_codec takes."""
    base = f.fmt
    return np.array([base.bitwidth, base.mantissa_bits, base.bias, base.inf_behavior,
                     base.nan_behavior, base.signedness, f.inf_or, f.inf_match, f.pos_inf,
                     f.neg_inf, f.qnan, f.snan, f.nan_kind, f.neg_to_nan], np.int64)


def packed_size(bitwidth: int, count: int) -> int:
    return int(lib().orc_packed_size(bitwidth, count))


def encode(x, f: CodecFormat, mode: int = 0, sat: int = 0, stoch_len: int = 0,
           reverse: int = 0, seed: int = 0, offset: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.zeros(packed_size(f.fmt.bitwidth, x.size), np.uint8)
    _check(lib().orc_encode_f32(_p(out), _p(x), x.size, C.byref(f), mode, sat, stoch_len, reverse,
                                seed, offset))
    return out


def mx_encode(x, block: int, ef: CodecFormat, sf: CodecFormat, mode: int = 0, scale_mode: int = 0,
              stoch_len: int = 0, sat: int = 1, seed: int = 0, offset: int = 0):
    """MX storage of x: (packed element codes, packed block-scale codes)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    nb = (x.size + block - 1) // block
    codes = np.zeros(packed_size(ef.fmt.bitwidth, x.size), np.uint8)
    scales = np.zeros(packed_size(sf.fmt.bitwidth, nb), np.uint8)
    _check(lib().orc_mx_encode_f32(_p(x), x.size, block, C.byref(ef), C.byref(sf), mode, scale_mode,
                                   stoch_len, sat, seed, offset, _p(codes), _p(scales)))
    return codes, scales


def decode(packed, count: int, f: CodecFormat, reverse: int = 0) -> np.ndarray:
    packed = np.ascontiguousarray(packed, dtype=np.uint8)
    out = np.empty(count, np.float32)
    _check(lib().orc_decode_f32(_p(out), _p(packed), count, C.byref(f), reverse))
    return out


def encode_rep(x: float, f: CodecFormat, mode: int = 0, sat: int = 0) -> int:
    return int(lib().orc_codec_encode_rep(x, C.byref(f), mode, sat, 0, 0, 0.0))


def decode_rep(rep: int, f: CodecFormat) -> float:
    return float(lib().orc_codec_decode_rep(rep, C.byref(f)))


def gemm_accfmt(A, B, f: Format, alpha: float = 1.0, trans_a: int = 0, trans_b: int = 0,
                nthreads: int = 0) -> np.ndarray:
    """Sequential-k emulated GEMM with the accumulator rounded into format f."""
    A, B, M, N, K = _gemm_args(A, B, trans_a, trans_b)
    D = np.empty((M, N), np.float32)
    _check(lib().orc_gemm_accfmt_f32(_p(A), A.shape[1], trans_a, _p(B), B.shape[1], trans_b,
                                     _p(D), N, M, N, K, C.byref(f), alpha, nthreads))
    return D
