"""Python surface of the GB300 kernels, mirroring the reference's compiled
module ``LoFloat.LoFloat`` (src/LoPy_bind.cpp:281-394): the enums,
``FloatFormatDescriptor``, ``virtual_round`` (mantissa and format overloads),
``virtual_mx_round`` and ``lof_gemm``. Every op runs through liblofgb.so on
the tensor's device, on torch's current stream, out of place.

Differences from the reference, all deliberate:
  * CPU tensors raise (the reference's CUDA build returns an uninitialised
    tensor for them, src/LoPy_bind.cpp:80-97, 140-154);
  * non-contiguous inputs are made contiguous first (the reference reads
    data_ptr() of whatever layout it is given);
  * stochastic modes draw from a counter-based generator keyed by
    (seed, offset) — ``set_seed`` plays the role of lo_float::set_seed
    (src/lo_float.h:58-62) and every stochastic call advances the offset by
    the number of elements it rounds.
"""
from __future__ import annotations

import ctypes as C
import enum
import threading

import numpy as np
import torch

from . import _native
from ._native import LofgbFormat, check


class Signedness(enum.IntEnum):
    Signed = 0
    Unsigned = 1


class InfBehavior(enum.IntEnum):
    Extended = 0
    Saturating = 1


class NaNBehavior(enum.IntEnum):
    _3109 = 0
    _754 = 1


class RoundingMode(enum.IntEnum):
    """Integer values follow src/fp_tools.hpp:13-28."""
    RoundToNearestEven = 0
    RoundTowardsZero = 1
    RoundAwayFromZero = 2
    StochasticRoundingA = 3
    RoundToNearestOdd = 4
    RoundDown = 5
    RoundUp = 6
    RoundTiesToAway = 7
    StochasticRoundingB = 8
    StochasticRoundingC = 9
    True_StochasticRounding = 10
    ProbabilisticRounding = 11
    RoundToOdd = 12
    RoundTiesTowardsZero = 13
    StochasticRoundingD = 14


STOCHASTIC_MODES = {3, 8, 9, 10, 11, 14}

# expose enum members at module level like pybind's export_values()
for _e in (Signedness, InfBehavior, RoundingMode, NaNBehavior):
    for _m in _e:
        globals().setdefault(_m.name, _m)


class FloatFormatDescriptor:
    """Runtime float format (src/LoPy_bind.cpp:45-68, bound at :315-327).

    The inf/NaN checkers are validated like the reference does (callable, with
    minNegInf/minPosInf, and qNanBitPattern or sNanBitPattern) and kept for
    callers that read them; the rounding path does not use them.
    """

    __slots__ = ("_total_bits", "_mantissa_bits", "_bias", "_inf", "_nan", "_sign",
                 "_is_inf", "_is_nan", "_c")

    def __init__(self, total_bits, mantissa_bits, bias, inf_behavior, nan_behavior, signedness,
                 is_inf_checker, is_nan_checker):
        if not callable(is_inf_checker):
            raise ValueError("inf_checker must be callable")
        if not hasattr(is_inf_checker, "minNegInf"):
            raise ValueError("inf_checker must have minNegInf()")
        if not hasattr(is_inf_checker, "minPosInf"):
            raise ValueError("inf_checker must have minPosInf()")
        if not callable(is_nan_checker):
            raise ValueError("nan_checker must be callable")
        if not (hasattr(is_nan_checker, "qNanBitPattern") or hasattr(is_nan_checker, "sNanBitPattern")):
            raise ValueError("nan_checker must have qNanBitPattern() or sNanBitPattern()")
        self._total_bits = int(total_bits)
        self._mantissa_bits = int(mantissa_bits)
        self._bias = int(bias)
        self._inf = InfBehavior(int(inf_behavior))
        self._nan = NaNBehavior(int(nan_behavior))
        self._sign = Signedness(int(signedness))
        self._is_inf = is_inf_checker
        self._is_nan = is_nan_checker
        self._c = LofgbFormat(self._total_bits, self._mantissa_bits, self._bias, int(self._inf),
                              int(self._nan), int(self._sign), 0)

    total_bits = property(lambda s: s._total_bits)
    mantissa_bits = property(lambda s: s._mantissa_bits)
    bias = property(lambda s: s._bias)
    inf_behavior = property(lambda s: s._inf)
    nan_behavior = property(lambda s: s._nan)
    signedness = property(lambda s: s._sign)
    is_inf_checker = property(lambda s: s._is_inf)
    is_nan_checker = property(lambda s: s._is_nan)

    @property
    def c_format(self) -> LofgbFormat:
        return self._c

    def __repr__(self):
        return (f"FloatFormatDescriptor(total_bits={self._total_bits}, mantissa_bits="
                f"{self._mantissa_bits}, bias={self._bias}, {self._inf.name}, {self._sign.name})")


# ---- stochastic-rounding generator state -----------------------------------
_rng_lock = threading.Lock()
_rng_state = {"seed": 12345, "offset": 0}


def set_seed(seed: int) -> None:
    """Seed the counter-based generator used by the stochastic modes."""
    with _rng_lock:
        _rng_state["seed"] = int(seed) & ((1 << 64) - 1)
        _rng_state["offset"] = 0


def get_rng_state() -> tuple[int, int]:
    with _rng_lock:
        return _rng_state["seed"], _rng_state["offset"]


def set_rng_state(seed: int, offset: int) -> None:
    with _rng_lock:
        _rng_state["seed"] = int(seed) & ((1 << 64) - 1)
        _rng_state["offset"] = int(offset)


def _take_counters(mode: int, n: int) -> tuple[int, int]:
    with _rng_lock:
        seed, off = _rng_state["seed"], _rng_state["offset"]
        if int(mode) in STOCHASTIC_MODES:
            _rng_state["offset"] = off + int(n)
        return seed, off


def _stream(t: torch.Tensor):
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _require_cuda(t: torch.Tensor, what: str) -> None:
    if not t.is_cuda:
        raise RuntimeError(f"{what}: liblofgb runs on CUDA tensors only (got {t.device})")


_ROUND_FNS = {torch.float32: ("lofgb_round_f32", "lofgb_round_mantissa_f32"),
              torch.float64: ("lofgb_round_f64", "lofgb_round_mantissa_f64"),
              torch.float16: ("lofgb_round_f16", "lofgb_round_mantissa_f16")}


def virtual_round(input: torch.Tensor, params, round_mode=RoundingMode.RoundToNearestEven,
                  stoch_len: int = 0, scale: float = 1.0, *, out: torch.Tensor | None = None,
                  seed: int | None = None, offset: int | None = None) -> torch.Tensor:
    """round(scale * input) to `params` (a FloatFormatDescriptor) or to an
    int number of mantissa bits — the two overloads of
    src/LoPy_bind.cpp:329-339. Returns a new tensor (or fills `out`)."""
    _require_cuda(input, "virtual_round")
    if input.dtype not in _ROUND_FNS:
        raise RuntimeError(f"virtual_round: unsupported dtype {input.dtype} "
                           "(float16, float32, float64)")
    x = input.contiguous()
    y = torch.empty_like(x) if out is None else out
    if y.shape != x.shape or y.dtype != x.dtype or not y.is_contiguous() or y.device != x.device:
        raise RuntimeError("virtual_round: out must be a contiguous tensor like input")
    n = x.numel()
    mode = int(round_mode)
    if seed is None:
        s, o = _take_counters(mode, n)
    else:
        s, o = int(seed), int(offset or 0)
    L = _native.lib()
    with torch.cuda.device(x.device):
        st = _stream(x)
        if isinstance(params, FloatFormatDescriptor):
            fn = getattr(L, _ROUND_FNS[x.dtype][0])
            check(fn(x.data_ptr(), y.data_ptr(), n, C.byref(params.c_format), mode, int(stoch_len),
                     float(scale), s, o, st), "virtual_round")
        elif isinstance(params, (int, np.integer)) and not isinstance(params, bool):
            fn = getattr(L, _ROUND_FNS[x.dtype][1])
            check(fn(x.data_ptr(), y.data_ptr(), n, int(params), mode, int(stoch_len), float(scale),
                     s, o, st), "virtual_round")
        else:
            raise TypeError("virtual_round: params must be a FloatFormatDescriptor or an int "
                            "number of mantissa bits")
    return y


def virtual_mx_round(input: torch.Tensor, block_size: int, element_format: FloatFormatDescriptor,
                     scale_format: FloatFormatDescriptor,
                     round_mode=RoundingMode.RoundToNearestEven,
                     scale_round_mode=RoundingMode.RoundToNearestEven, stoch_len: int = 0, *,
                     out: torch.Tensor | None = None, seed: int | None = None,
                     offset: int | None = None) -> torch.Tensor:
    """MX block fake-quantisation (src/LoPy_bind.cpp:165-217): contiguous blocks
    of `block_size`, one shared scale per block in `scale_format`, elements
    rounded into `element_format` and rescaled. float32 input (the reference's
    only type), or bfloat16 input rounded exactly as its float32 copy would
    be, without making it (lofgb_mx_round_bf16); the result is float32."""
    if input.dtype not in (torch.float32, torch.bfloat16):
        raise RuntimeError("virtual_mx_round: float32 or bfloat16 tensors only")
    if int(block_size) <= 0:
        raise RuntimeError("virtual_mx_round: block_size must be positive")
    _require_cuda(input, "virtual_mx_round")
    x = input.contiguous()
    y = torch.empty(x.shape, dtype=torch.float32, device=x.device) if out is None else out
    if y.shape != x.shape or y.dtype != torch.float32 or not y.is_contiguous() or y.device != x.device:
        raise RuntimeError("virtual_mx_round: out must be a contiguous float32 tensor of the input's shape")
    n = x.numel()
    mode = int(round_mode)
    if seed is None:
        s, o = _take_counters(mode, n)
    else:
        s, o = int(seed), int(offset or 0)
    fn = "lofgb_mx_round_bf16" if x.dtype == torch.bfloat16 else "lofgb_mx_round_f32"
    with torch.cuda.device(x.device):
        check(getattr(_native.lib(), fn)(
            x.data_ptr(), y.data_ptr(), n, int(block_size), C.byref(element_format.c_format),
            C.byref(scale_format.c_format), mode, int(scale_round_mode), int(stoch_len), s, o,
            _stream(x)), "virtual_mx_round")
    return y.view(input.shape)


def gemm_alpha(scale_a: float, scale_b: float) -> float:
    """alpha = 1/(scale_a*scale_b) in float32, 1 when the product is 0
    (src/cutlass_gemms.cuh:1784-1786, scales narrowed to float at
    src/Lof_kernel.cu:140-141)."""
    sa, sb = np.float32(scale_a), np.float32(scale_b)
    denom = np.float32(sa * sb)
    return 1.0 if denom == 0 else float(np.float32(1.0) / denom)


_ws_cache: dict = {}


def _tc_workspace(device: torch.device, M: int, N: int, K: int) -> torch.Tensor:
    return _workspace(device, int(_native.lib().lofgb_gemm_tc_workspace_size(M, N, K)))


def _workspace(device: torch.device, need: int) -> torch.Tensor:
    # one workspace per (device, stream): calls on one stream are ordered, so
    # reusing it is race-free; another stream gets its own
    key = (device, torch.cuda.current_stream(device).cuda_stream)
    buf = _ws_cache.get(key)
    if buf is None or buf.numel() < need:
        buf = torch.empty(max(need, 256), dtype=torch.uint8, device=device)
        _ws_cache[key] = buf
    return buf


def tc_device_status(device=None) -> int:
    """Status word the tensor-core GEMM left in its workspace on `device`
    (0, or LOFGB_ERR_TIMEOUT if a bounded device-side wait expired). Reads
    device memory, so it synchronises with the current stream."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    buf = _ws_cache.get((dev, torch.cuda.current_stream(dev).cuda_stream))
    if buf is None:
        return 0
    return int(buf[:4].view(torch.int32).item())


def gemm(A: torch.Tensor, B: torch.Tensor, accum_mant_bits: int, *, trans_a: bool = False,
         trans_b: bool = False, alpha: float = 1.0, variant: str = "plain", chunk: int = 32,
         out: torch.Tensor | None = None,
         accum_format: FloatFormatDescriptor | None = None) -> torch.Tensor:
    """Emulated-accumulation GEMM with explicit layouts.

    A is (M, K), or (K, M) when trans_a; B is (K, N), or (N, K) when trans_b;
    both contiguous float32 CUDA tensors. A leading batch dimension on either
    operand makes it a strided-batched GEMM (one launch; a 2-D operand, or a
    batch of 1, is shared by every product) with D of shape (batch, M, N).
    variant "plain" is bit-exact to the reference leaf; "tc" is the tcgen05
    chunked form. `accum_format` (2-D only) rounds the accumulator into a
    whole format instead of to `accum_mant_bits` mantissa bits
    (lofgb_gemm_accfmt_f32)."""
    for t, nm in ((A, "A"), (B, "B")):
        if t.dim() not in (2, 3):
            raise RuntimeError(f"lof_gemm: {nm} must be 2-D (or 3-D for a batch)")
        if t.dtype != torch.float32:
            raise RuntimeError("lof_gemm: only float32 inputs are supported")
        _require_cuda(t, "lof_gemm")
    batched = A.dim() == 3 or B.dim() == 3
    A = A.contiguous()
    B = B.contiguous()
    M, K = (A.shape[-1], A.shape[-2]) if trans_a else (A.shape[-2], A.shape[-1])
    Kb, N = (B.shape[-1], B.shape[-2]) if trans_b else (B.shape[-2], B.shape[-1])
    if K != Kb:
        raise RuntimeError(f"LoF_gemm: A.cols ({K}) != B.rows ({Kb})")
    ba = A.shape[0] if A.dim() == 3 else 1
    bb = B.shape[0] if B.dim() == 3 else 1
    if ba != bb and 1 not in (ba, bb):
        raise RuntimeError(f"lof_gemm: batch sizes differ ({ba} vs {bb})")
    batch = max(ba, bb)
    shape = (batch, M, N) if batched else (M, N)
    D = torch.empty(shape, dtype=torch.float32, device=A.device) if out is None else out
    if tuple(D.shape) != shape or not D.is_contiguous() or D.dtype != torch.float32:
        raise RuntimeError(f"lof_gemm: out must be a contiguous float32 {shape} tensor")
    v = {"plain": 0, "tc": 1}[variant]
    L = _native.lib()
    sa = A.shape[-2] * A.shape[-1] if ba > 1 else 0
    sb = B.shape[-2] * B.shape[-1] if bb > 1 else 0
    with torch.cuda.device(A.device):
        ws, wsb = None, 0
        if v == 1 and M and N and K:
            buf = _workspace(A.device, int(L.lofgb_gemm_batched_tc_workspace_size(M, N, K, batch)))
            ws, wsb = buf.data_ptr(), buf.numel()
        if accum_format is not None:
            if batched:
                raise RuntimeError("lof_gemm: accum_format takes 2-D operands")
            check(L.lofgb_gemm_accfmt_f32(A.data_ptr(), A.shape[-1], int(trans_a), B.data_ptr(),
                                          B.shape[-1], int(trans_b), D.data_ptr(), N, M, N, K,
                                          C.byref(accum_format.c_format), float(alpha), v,
                                          int(chunk), ws, wsb, _stream(A)), "lof_gemm")
            return D
        check(L.lofgb_gemm_batched_f32(A.data_ptr(), A.shape[-1], sa, int(trans_a), B.data_ptr(),
                                       B.shape[-1], sb, int(trans_b), D.data_ptr(), N, M * N, M,
                                       N, K, batch, int(accum_mant_bits),
                                       int(RoundingMode.RoundToNearestEven), float(alpha), v,
                                       int(chunk), ws, wsb, _stream(A)), "lof_gemm")
    return D


def lof_gemm(A: torch.Tensor, B: torch.Tensor, accum_mant_bits: int,
             round_mode=RoundingMode.RoundToNearestEven, stochastic_rounding_bits: int = 0,
             scale_a: float = 1.0, scale_b: float = 1.0) -> torch.Tensor:
    """Drop-in for the reference's lof_gemm (src/Lof_kernel.cu:96-154): D = (A @ B)
    / (scale_a*scale_b) with the accumulator re-rounded to `accum_mant_bits`
    after every multiply-add, bit-exact. Like the reference leaf, the
    accumulator always rounds to nearest even; `round_mode` and
    `stochastic_rounding_bits` are accepted and ignored
    (src/cutlass_gemms.cuh:122)."""
    del round_mode, stochastic_rounding_bits
    if A.dim() != 2 or B.dim() != 2:
        raise RuntimeError("LoF_gemm: A and B must be 2-D")
    return gemm(A, B, accum_mant_bits, alpha=gemm_alpha(scale_a, scale_b))


def gemm_f64_reference(A: torch.Tensor, B: torch.Tensor, *, trans_a: bool = False,
                       trans_b: bool = False) -> torch.Tensor:
    """FP64 GEMM of the FP32 operands on the GPU (the oracle for the tensor-core
    form's error statistics)."""
    A = A.contiguous()
    B = B.contiguous()
    M, K = (A.shape[1], A.shape[0]) if trans_a else (A.shape[0], A.shape[1])
    N = B.shape[0] if trans_b else B.shape[1]
    D = torch.empty((M, N), dtype=torch.float64, device=A.device)
    with torch.cuda.device(A.device):
        check(_native.lib().lofgb_gemm_f64_ref(A.data_ptr(), A.shape[1], int(trans_a), B.data_ptr(),
                                               B.shape[1], int(trans_b), D.data_ptr(), N, M, N, K,
                                               _stream(A)), "gemm_f64_reference")
    return D


# ---- conv2d -------------------------------------------------------------------
CONV_ORDERS = {"crs": 0, "tiled8": 1}


def conv2d_alpha(weight_scale: float, input_scale: float) -> float:
    """(float)(1.0 / (weight_scale * input_scale)) computed in double, 1 when the
    product is 0 (src/Lof_kernel.cu:203-206)."""
    denom = float(weight_scale) * float(input_scale)
    return 1.0 if denom == 0.0 else float(np.float32(1.0 / denom))


def _pair(v) -> tuple[int, int]:
    return (int(v[0]), int(v[1])) if isinstance(v, (tuple, list)) else (int(v), int(v))


def conv2d_shape(input_shape, weight_shape, stride=1, padding=0, dilation=1):
    """lofgb_conv2d_shape for an NCHW input and a KCRS weight."""
    sh, sw = _pair(stride)
    ph, pw = _pair(padding)
    dh, dw = _pair(dilation)
    n, c, h, w = (int(v) for v in input_shape)
    k, _, r, s_ = (int(v) for v in weight_shape)
    return _native.LofgbConv2dShape(n, c, h, w, k, r, s_, ph, pw, sh, sw, dh, dw)


def conv2d(input: torch.Tensor, weight: torch.Tensor, accum_mant_bits: int, *, stride=1,
           padding=0, dilation=1, alpha: float = 1.0, order: str = "crs",
           variant: str = "plain", chunk: int = 32,
           out: torch.Tensor | None = None) -> torch.Tensor:
    """Emulated-accumulation conv2d (cross-correlation, groups = 1) on NCHW
    input and KCRS weight, output NCHW. `order` picks the reduction order:
    "crs" (c, r, s — the im2col + lof_gemm path of LoF_Conv2d) or "tiled8"
    (8-channel tiles outer — lof_conv2d's implicit GEMM). variant "plain" is
    bit-exact; "tc" is the chunked tensor-core form."""
    for t, nm in ((input, "input"), (weight, "weight")):
        if t.dim() != 4:
            raise RuntimeError("LoF_conv2d: input and weight must be 4-D (NCHW / OIHW)")
        if t.dtype != torch.float32:
            raise RuntimeError("LoF_conv2d: only float32 inputs are supported")
        _require_cuda(t, "LoF_conv2d")
    if input.shape[1] != weight.shape[1]:
        raise RuntimeError(f"LoF_conv2d: input C_in ({input.shape[1]}) != weight C_in "
                           f"({weight.shape[1]})")
    x = input.contiguous()
    w = weight.contiguous()
    shape = conv2d_shape(x.shape, w.shape, stride, padding, dilation)
    L = _native.lib()
    P, Q = C.c_int32(), C.c_int32()
    check(L.lofgb_conv2d_out_size(C.byref(shape), C.byref(P), C.byref(Q)), "LoF_conv2d")
    oshape = (x.shape[0], w.shape[0], P.value, Q.value)
    y = torch.empty(oshape, dtype=torch.float32, device=x.device) if out is None else out
    if tuple(y.shape) != oshape or not y.is_contiguous() or y.dtype != torch.float32:
        raise RuntimeError(f"LoF_conv2d: out must be a contiguous float32 {oshape} tensor")
    o = CONV_ORDERS[order]
    v = {"plain": 0, "tc": 1}[variant]
    with torch.cuda.device(x.device):
        ws, wsb = None, 0
        if v == 1:
            buf = _workspace(x.device, int(L.lofgb_conv2d_workspace_size(C.byref(shape), o, v)))
            ws, wsb = buf.data_ptr(), buf.numel()
        check(L.lofgb_conv2d_f32(x.data_ptr(), w.data_ptr(), y.data_ptr(), C.byref(shape),
                                 int(accum_mant_bits), int(RoundingMode.RoundToNearestEven),
                                 float(alpha), o, v, int(chunk), ws, wsb, _stream(x)),
              "LoF_conv2d")
    return y


def lof_conv2d(input: torch.Tensor, weight: torch.Tensor, pad_h: int, pad_w: int, stride_h: int,
               stride_w: int, dilation_h: int, dilation_w: int, accum_mant_bits: int,
               round_mode=RoundingMode.RoundToNearestEven, stochastic_rounding_bits: int = 0,
               weight_scale: float = 1.0, input_scale: float = 1.0) -> torch.Tensor:
    """Drop-in for the reference's lof_conv2d (src/LoPy_bind.cpp:374-389 →
    src/Lof_kernel.cu:156-227): NCHW / OIHW float32 CUDA tensors, output NCHW
    divided by (weight_scale * input_scale), the accumulator re-rounded to
    `accum_mant_bits` after every multiply-add in the implicit GEMM's order,
    bit-exact. round_mode and stochastic_rounding_bits are accepted and
    ignored, as by the shared GEMM leaf."""
    del round_mode, stochastic_rounding_bits
    return conv2d(input, weight, accum_mant_bits, stride=(stride_h, stride_w),
                  padding=(pad_h, pad_w), dilation=(dilation_h, dilation_w),
                  alpha=conv2d_alpha(weight_scale, input_scale), order="tiled8")


# ---- piecewise-linear SiLU -------------------------------------------------------
_PWL_FNS = {torch.float32: "lofgb_pwl_silu_f32", torch.float64: "lofgb_pwl_silu_f64",
            torch.float16: "lofgb_pwl_silu_f16"}


def pwl_silu(input: torch.Tensor, lut: torch.Tensor, R: float, *,
             out: torch.Tensor | None = None) -> torch.Tensor:
    """Drop-in for the reference's pwl_silu (src/LoPy_bind.cpp:228-272): SiLU
    interpolated from `lut` (segments + 1 knots over [-R, R], segments a power
    of two in [2, 4096]), the relu asymptote outside [-R, R]. Returns a new
    tensor of the input's dtype (float16, float32 or float64)."""
    if lut.dim() != 1 or lut.numel() < 2:
        raise RuntimeError("pwl_silu: lut must be 1-D with >= 2 entries")
    if not float(R) > 0.0:
        raise RuntimeError("pwl_silu: R must be positive")
    _require_cuda(input, "pwl_silu")
    if input.dtype not in _PWL_FNS:
        raise RuntimeError(f"pwl_silu: unsupported dtype {input.dtype}")
    nseg = lut.numel() - 1
    if nseg < 2 or nseg > 4096 or nseg & (nseg - 1):
        raise RuntimeError(f"pwl_silu: lut length {nseg} is not a supported power of 2 in "
                           "[2, 4096]")
    x = input.contiguous()
    lut_f = lut.to(device=x.device, dtype=torch.float32).contiguous()
    y = torch.empty_like(x) if out is None else out
    if y.shape != x.shape or y.dtype != x.dtype or not y.is_contiguous() or y.device != x.device:
        raise RuntimeError("pwl_silu: out must be a contiguous tensor like input")
    with torch.cuda.device(x.device):
        check(getattr(_native.lib(), _PWL_FNS[x.dtype])(x.data_ptr(), y.data_ptr(), x.numel(),
                                                        lut_f.data_ptr(), nseg, float(R),
                                                        _stream(x)), "pwl_silu")
    return y


# ---- BatchNorm approximations (LoFloat/layers.py:805-1047) ------------------------
class BnStat(enum.IntEnum):
    MEAN_ABS_DEV = 0
    MAX_ABS_DEV = 1
    VARIANCE = 2


class BnNorm(enum.IntEnum):
    DIVIDE = 0
    FISR = 1
    PWL = 2


def _bn_view(x: torch.Tensor, what: str) -> tuple[torch.Tensor, int, int, int]:
    _require_cuda(x, what)
    if x.dim() < 2:
        raise RuntimeError(f"{what}: input must be (N, C, *)")
    if x.dtype != torch.float32:
        raise RuntimeError(f"{what}: float32 input required (got {x.dtype})")
    x = x.contiguous()
    n, c = x.shape[0], x.shape[1]
    inner = x.numel() // max(1, n * c)
    return x, n, c, inner


def _chan(t, c: int, dev, what: str):
    if t is None:
        return None
    t = t.detach()
    if t.numel() != c or t.dtype != torch.float32 or t.device != dev:
        raise RuntimeError(f"{what}: per-channel tensors must be float32 with {c} elements on {dev}")
    return t.contiguous()


def bn_stats(x: torch.Tensor, stat: BnStat, *, running_mean: torch.Tensor | None = None,
             running_dev: torch.Tensor | None = None, momentum: float = 0.1):
    """Per-channel FP32 mean and deviation statistic of x (N, C, *) in one or
    two passes (lofgb_bn_stats_f32). running_mean / running_dev, if given
    (float32, contiguous, C elements), are updated in place to
    r (1 - momentum) + momentum s."""
    x, n, c, inner = _bn_view(x, "bn_stats")
    L = _native.lib()
    mean = torch.empty(c, dtype=torch.float32, device=x.device)
    dev = torch.empty_like(mean)
    for r in (running_mean, running_dev):
        if r is not None and (r.numel() != c or r.dtype != torch.float32 or not r.is_contiguous()
                              or r.device != x.device):
            raise RuntimeError("bn_stats: running buffers must be contiguous float32 with C elements")
    with torch.cuda.device(x.device):
        ws = _workspace(x.device, int(L.lofgb_bn_workspace_size(n, c, inner)))
        check(L.lofgb_bn_stats_f32(x.data_ptr(), n, c, inner, int(stat), mean.data_ptr(),
                                   dev.data_ptr(),
                                   running_mean.data_ptr() if running_mean is not None else None,
                                   running_dev.data_ptr() if running_dev is not None else None,
                                   float(momentum), ws.data_ptr(), ws.numel(), _stream(x)),
              "bn_stats")
    return mean, dev


def bn_apply(x: torch.Tensor, mean: torch.Tensor, dev: torch.Tensor, eps: float, norm: BnNorm, *,
             scale: torch.Tensor | None = None, weight: torch.Tensor | None = None,
             bias: torch.Tensor | None = None, lut: torch.Tensor | None = None,
             out: torch.Tensor | None = None) -> torch.Tensor:
    """Fused normalise + scale + affine of x (N, C, *) with per-channel
    statistics (lofgb_bn_apply_f32)."""
    x, n, c, inner = _bn_view(x, "bn_apply")
    L = _native.lib()
    mean, dev = _chan(mean, c, x.device, "bn_apply"), _chan(dev, c, x.device, "bn_apply")
    scale, weight, bias = (_chan(t, c, x.device, "bn_apply") for t in (scale, weight, bias))
    if (weight is None) != (bias is None):
        raise RuntimeError("bn_apply: weight and bias go together")
    segs = 0
    if int(norm) == BnNorm.PWL:
        if lut is None or lut.dim() != 1 or lut.numel() < 2:
            raise RuntimeError("bn_apply: the PWL normaliser needs a 1-D table")
        lut = lut.detach().to(device=x.device, dtype=torch.float32).contiguous()
        segs = lut.numel() - 1
    y = torch.empty_like(x) if out is None else out
    if y.shape != x.shape or y.dtype != x.dtype or not y.is_contiguous() or y.device != x.device:
        raise RuntimeError("bn_apply: out must be a contiguous tensor like input")

    def ptr(t):
        return t.data_ptr() if t is not None else None
    with torch.cuda.device(x.device):
        check(L.lofgb_bn_apply_f32(x.data_ptr(), y.data_ptr(), n, c, inner, mean.data_ptr(),
                                   dev.data_ptr(), float(eps), int(norm), ptr(scale), ptr(weight),
                                   ptr(bias), ptr(lut), segs, _stream(x)), "bn_apply")
    return y


# ---- storage codec (src/lo_pack.hpp) ----------------------------------------------
class SaturationMode(enum.IntEnum):
    """Saturation_Mode (src/fp_tools.hpp:38-41): what an overflow encodes to."""
    OvfInf = 0
    SatFinite = 1
    SatPropagate = 2


_codec_cache: dict = {}


def codec_format(params: FloatFormatDescriptor, neg_to_nan: bool = False):
    """lofgb_codec_format for `params`: the checkers' predicates are evaluated
    over every code of the format (at most 2^16) and matched to the forms the
    kernels evaluate — IsInf(rep) <=> (rep | inf_or) == inf_match; IsNaN as a
    single pattern, the IEEE exponent-all-ones range, or never. Raises for a
    checker that fits neither (the reference's P3109, IEEE-style, OCP, E8M0
    and trivial checkers all fit). Cached per (format fields, checker
    objects, neg_to_nan): the scan costs about as much as a kernel launch."""
    key = (params.total_bits, params.mantissa_bits, params.bias, int(params.inf_behavior),
           int(params.nan_behavior), int(params.signedness), id(params.is_inf_checker),
           id(params.is_nan_checker), bool(neg_to_nan))
    hit = _codec_cache.get(key)
    if hit is None:
        # the checkers stay referenced with their entry, so their ids stay theirs
        hit = (_codec_format_scan(params, neg_to_nan), params.is_inf_checker, params.is_nan_checker)
        _codec_cache[key] = hit
    return hit[0]


def _codec_format_scan(params: FloatFormatDescriptor, neg_to_nan: bool):
    n, m = params.total_bits, params.mantissa_bits
    if not 1 <= n <= 16:
        raise RuntimeError(f"codec: bitwidth {n} outside [1, 16]")
    signed = params.signedness == Signedness.Signed
    codes = range(1 << n)
    inf_set = {r for r in codes if params.is_inf_checker(r)}
    nan_set = {r for r in codes if params.is_nan_checker(r)}
    sign = (1 << (n - 1)) if signed else 0
    inf_or, inf_match = 0, 0xFFFFFFFF
    if inf_set:
        for o in (0, sign, 1 << (n - 1)):
            t = min(inf_set) | o
            if {r for r in codes if (r | o) == t} == inf_set:
                inf_or, inf_match = o, t
                break
        else:
            raise RuntimeError("codec: the format's infinity checker has no supported form")
    qnan = int(params.is_nan_checker.qNanBitPattern()) if hasattr(params.is_nan_checker, "qNanBitPattern") \
        else int(params.is_nan_checker.sNanBitPattern())
    snan = int(params.is_nan_checker.sNanBitPattern()) if hasattr(params.is_nan_checker, "sNanBitPattern") \
        else qnan
    ebits = n - m - (1 if signed else 0)
    expall = ((1 << ebits) - 1) << m
    if not nan_set:
        kind = 2
    elif nan_set == {qnan}:
        kind = 0
    elif nan_set == {r for r in codes if (r & ~sign) > expall}:
        kind = 1
    else:
        raise RuntimeError("codec: the format's NaN checker has no supported form")
    f = _native.LofgbCodecFormat()
    f.fmt = params.c_format
    f.inf_or, f.inf_match = inf_or & 0xFFFFFFFF, inf_match & 0xFFFFFFFF
    f.pos_inf = int(params.is_inf_checker.minPosInf()) & 0xFFFFFFFF
    f.neg_inf = int(params.is_inf_checker.minNegInf()) & 0xFFFFFFFF
    f.qnan, f.snan, f.nan_kind, f.neg_to_nan = qnan, snan, kind, int(bool(neg_to_nan))
    return f


def packed_size(bitwidth: int, count: int) -> int:
    """Bytes `count` codes of `bitwidth` bits occupy (LoF_packed_size,
    src/lo_pack.hpp:374-377)."""
    return int(_native.lib().lofgb_packed_size(int(bitwidth), int(count)))


def lof_encode(input: torch.Tensor, params: FloatFormatDescriptor,
               round_mode=RoundingMode.RoundToNearestEven, saturation=SaturationMode.OvfInf,
               stoch_len: int = 0, *, reverse: bool = False, neg_to_nan: bool = False,
               out: torch.Tensor | None = None, seed: int | None = None,
               offset: int | None = None) -> torch.Tensor:
    """Round float32 values to `params` codes and pack them (LoF_encode_cuda,
    src/lo_pack.hpp:496-512). Returns a uint8 tensor of packed_size bytes."""
    if input.dtype != torch.float32:
        raise RuntimeError("lof_encode: float32 input only")
    _require_cuda(input, "lof_encode")
    x = input.contiguous()
    f = codec_format(params, neg_to_nan)
    nbytes = packed_size(params.total_bits, x.numel())
    y = torch.empty(nbytes, dtype=torch.uint8, device=x.device) if out is None else out
    if y.dtype != torch.uint8 or y.numel() < nbytes or not y.is_contiguous():
        raise RuntimeError(f"lof_encode: out must be a contiguous uint8 tensor of {nbytes} bytes")
    mode = int(round_mode)
    if seed is None:
        s, o = _take_counters(mode, x.numel())
    else:
        s, o = int(seed), int(offset or 0)
    with torch.cuda.device(x.device):
        check(_native.lib().lofgb_encode_f32(y.data_ptr(), x.data_ptr(), x.numel(), C.byref(f),
                                             mode, int(saturation), int(stoch_len), int(reverse),
                                             s, o, _stream(x)), "lof_encode")
    return y


def mx_encode(input: torch.Tensor, element_format: FloatFormatDescriptor,
              scale_format: FloatFormatDescriptor, round_mode=RoundingMode.RoundToNearestEven,
              scale_round_mode=RoundingMode.RoundToNearestEven,
              saturation=SaturationMode.SatFinite, stoch_len: int = 0, *, block_size: int = 32,
              seed: int | None = None, offset: int | None = None):
    """MX storage of a float32 tensor in one pass (lofgb_mx_encode_f32):
    returns (element codes, block-scale codes) as uint8 tensors — the MX
    block rounding's quotients as packed `element_format` codes (4, 6 or 8
    bits) and one `scale_format` code (8 bits, e.g. E8M0) per block of 32."""
    if input.dtype != torch.float32:
        raise RuntimeError("mx_encode: float32 input only")
    _require_cuda(input, "mx_encode")
    x = input.contiguous()
    ef, sf = codec_format(element_format), codec_format(scale_format)
    n = x.numel()
    codes = torch.empty(packed_size(element_format.total_bits, n), dtype=torch.uint8, device=x.device)
    scales = torch.empty((n + block_size - 1) // max(1, block_size), dtype=torch.uint8, device=x.device)
    mode = int(round_mode)
    if seed is None:
        s, o = _take_counters(mode, n)
    else:
        s, o = int(seed), int(offset or 0)
    with torch.cuda.device(x.device):
        check(_native.lib().lofgb_mx_encode_f32(x.data_ptr(), codes.data_ptr(), scales.data_ptr(), n,
                                                int(block_size), C.byref(ef), C.byref(sf), mode,
                                                int(scale_round_mode), int(saturation), int(stoch_len),
                                                s, o, _stream(x)), "mx_encode")
    return codes, scales


def mx_decode(codes: torch.Tensor, scales: torch.Tensor, count: int,
              element_format: FloatFormatDescriptor, scale_format: FloatFormatDescriptor, *,
              block_size: int = 32) -> torch.Tensor:
    """Values of MX storage: decoded element codes times their block's decoded
    scale (a float32 tensor of `count` values); one kernel
    (lofgb_mx_decode_f32) for blocks of 32, 4/6/8-bit element codes and
    8-bit scale codes, else the two codec decodes and the product."""
    if (block_size == 32 and element_format.total_bits in (4, 6, 8) and scale_format.total_bits == 8
            and codes.dtype == torch.uint8 and scales.dtype == torch.uint8 and codes.is_cuda
            and scales.is_cuda and codes.device == scales.device and count >= 0
            and codes.is_contiguous() and scales.is_contiguous() and codes.data_ptr() % 4 == 0):
        if codes.numel() < packed_size(element_format.total_bits, count) or scales.numel() < (count + 31) // 32:
            raise RuntimeError("mx_decode: codes or scales shorter than `count` values need")
        out = torch.empty(count, dtype=torch.float32, device=codes.device)
        if count == 0:
            return out
        ef, sf = codec_format(element_format), codec_format(scale_format)
        with torch.cuda.device(codes.device):
            check(_native.lib().lofgb_mx_decode_f32(codes.data_ptr(), scales.data_ptr(), out.data_ptr(),
                                                    count, 32, C.byref(ef), C.byref(sf),
                                                    _stream(codes)), "mx_decode")
        return out
    q = lof_decode(codes, count, element_format)
    nb = (count + block_size - 1) // block_size
    sc = lof_decode(scales, nb, scale_format)
    return (q.view(-1)[:count] * sc.repeat_interleave(block_size)[:count])


def lof_decode(packed: torch.Tensor, count: int, params: FloatFormatDescriptor, *,
               reverse: bool = False, out: torch.Tensor | None = None) -> torch.Tensor:
    """Unpack `count` codes of `params` and convert them to float32
    (LoF_decode_cuda, src/lo_pack.hpp:515-532)."""
    if packed.dtype != torch.uint8:
        raise RuntimeError("lof_decode: packed must be a uint8 tensor")
    _require_cuda(packed, "lof_decode")
    p = packed.contiguous()
    need = packed_size(params.total_bits, count)
    if p.numel() < need:
        raise RuntimeError(f"lof_decode: {count} codes need {need} bytes, got {p.numel()}")
    f = codec_format(params)
    y = torch.empty(int(count), dtype=torch.float32, device=p.device) if out is None else out
    if y.dtype != torch.float32 or y.numel() != count or not y.is_contiguous():
        raise RuntimeError("lof_decode: out must be a contiguous float32 tensor of count values")
    with torch.cuda.device(p.device):
        check(_native.lib().lofgb_decode_f32(y.data_ptr(), p.data_ptr(), int(count), C.byref(f),
                                             int(reverse), _stream(p)), "lof_decode")
    return y
