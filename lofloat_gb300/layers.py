"""Straight-through rounding functions and the LoFloat linear layer
(LoFloat/layers.py:8-57, 58-110, 121-168, 221-447), running on liblofgb.

Forward semantics match the reference. In addition, the GEMM is
differentiable here: ``LoFLinearFunction`` is a hand-written autograd
function whose backward uses a straight-through estimator for the rounding
and emulated-accumulation GEMMs for dX = dY·W_q and dW = dYᵀ·X_q, with dY
optionally stochastic-rounded to a gradient format first. The reference
defines no gradient through lof_gemm (its test states it is
non-differentiable, test/test_mx_round_py.py:57-58).
"""
from __future__ import annotations

import math

import torch
import torch.nn as nn

from . import binding as lof
from ._custom_ops import register_format
from .formats import create_e8m0_params, create_p3109_params
from .pwl import pwl_table
from .pwl import silu as pwl_silu_fn


class STERound(torch.autograd.Function):
    """round(scale * x) forward; ∂/∂x = scale (LoFloat/layers.py:8-31)."""

    @staticmethod
    def forward(ctx, tensor, params, rounding_mode=lof.RoundingMode.RoundToNearestEven, scale=1.0):
        ctx.scale = float(scale)
        if isinstance(params, int):
            return torch.ops.lofloat.virtual_round(tensor, params, int(rounding_mode), 0, float(scale))
        return lof.virtual_round(tensor, params, round_mode=rounding_mode, stoch_len=0,
                                 scale=float(scale))

    @staticmethod
    def backward(ctx, grad_output):
        if ctx.scale == 1.0:
            return grad_output, None, None, None
        return grad_output * ctx.scale, None, None, None


class STEMXRound(torch.autograd.Function):
    """MX fake-quantisation along the last axis; identity backward
    (LoFloat/layers.py:34-57)."""

    @staticmethod
    def forward(ctx, tensor, element_params, scale_params, block_size,
                rounding_mode=lof.RoundingMode.RoundToNearestEven):
        if isinstance(element_params, int):
            return torch.ops.lofloat.virtual_mx_round(
                tensor, int(block_size), element_params, scale_params, int(rounding_mode),
                int(lof.RoundingMode.RoundToNearestEven), 0)
        return lof.virtual_mx_round(tensor, int(block_size), element_params, scale_params,
                                    round_mode=rounding_mode)

    @staticmethod
    def backward(ctx, grad_output):
        return grad_output, None, None, None, None


class LoF_Quantize(nn.Module):
    """Fake-quantise a tensor per tensor or with MX block scaling
    (LoFloat/layers.py:58-104)."""

    def __init__(self, params, rounding_mode=None, scaling="per_tensor", mx_block_size=32,
                 scale_format=None):
        super().__init__()
        if scaling not in ("per_tensor", "mx"):
            raise ValueError(f"scaling must be 'per_tensor' or 'mx', got {scaling!r}")
        self.params = params
        self.rounding_mode = rounding_mode if rounding_mode is not None else lof.RoundingMode.RoundToNearestEven
        self.scaling = scaling
        self.mx_block_size = mx_block_size
        self.scale_format = scale_format if scale_format is not None else create_e8m0_params()

    def forward(self, x):
        if self.scaling == "mx":
            if x.shape[-1] % self.mx_block_size != 0:
                raise ValueError(f"mx scaling needs the last dim ({x.shape[-1]}) divisible by "
                                 f"mx_block_size ({self.mx_block_size})")
            return STEMXRound.apply(x, self.params, self.scale_format, self.mx_block_size,
                                    self.rounding_mode)
        return STERound.apply(x, self.params, self.rounding_mode)


def _quantize(self, tensor, params):
    """STE rounding of `tensor` to `params` under the owner's rounding_mode
    (LoFloat/layers.py:106-109); None leaves the tensor as is."""
    if params is None:
        return tensor
    return STERound.apply(tensor, params, self.rounding_mode)


def mantissa_quantize(tensor, mantissa_bits):
    """STE rounding to a signed, saturating P3109 format with 8 exponent bits
    and `mantissa_bits` stored mantissa bits (LoFloat/layers.py:111-114)."""
    if mantissa_bits is None:
        return tensor
    return STERound.apply(tensor, create_p3109_params(8 + mantissa_bits + 1, mantissa_bits + 1, True, True))


def exp_mant_quantize(tensor, exp_bits, mantissa_bits):
    """STE rounding to a signed, saturating P3109 format with `exp_bits`
    exponent and `mantissa_bits` stored mantissa bits
    (LoFloat/layers.py:116-119)."""
    if exp_bits is None or mantissa_bits is None:
        return tensor
    return STERound.apply(tensor, create_p3109_params(exp_bits + mantissa_bits + 1, mantissa_bits + 1,
                                                      True, True))


def _lof_gemm_2d(A, B, accum_mant_bits, gemm_round_mode, stochastic_rounding_bits, scale_a=1.0,
                 scale_b=1.0, variant="plain", chunk=32):
    """(..., M, K) x (..., K, N) -> (..., M, N) (LoFloat/layers.py:121-150), with
    the batch in one strided-batched launch instead of a Python loop of
    lof_gemm calls (same per-product bits). A B that is the transposed view of
    a contiguous (..., N, K) tensor — attention's K^T — is read in place."""
    del gemm_round_mode, stochastic_rounding_bits
    alpha = lof.gemm_alpha(scale_a, scale_b)
    if A.dim() == 2 and B.dim() == 2:
        return lof.gemm(A.contiguous(), B.contiguous(), accum_mant_bits, alpha=alpha,
                        variant=variant, chunk=chunk)
    batch_shape = A.shape[:-2]
    M, K = A.shape[-2], A.shape[-1]
    N = B.shape[-1]
    A_flat = A.reshape(-1, M, K).contiguous()
    Bt = B.transpose(-2, -1)
    if Bt.is_contiguous():
        B_flat, tb = Bt.reshape(-1, N, K), True
    else:
        B_flat, tb = B.reshape(-1, K, N).contiguous(), False
    out = lof.gemm(A_flat, B_flat, accum_mant_bits, trans_b=tb, alpha=alpha, variant=variant,
                   chunk=chunk)
    return out.reshape(*batch_shape, M, N)


def _lof_linear(x, weight, bias, accum_mant_bits, gemm_round_mode, stochastic_rounding_bits,
                scale_a=1.0, scale_b=1.0):
    """x (..., K) · weight (N, K)ᵀ through the emulated GEMM
    (LoFloat/layers.py:153-168). The weight is consumed in place as the
    transposed B operand — no transpose copy."""
    leading = x.shape[:-1]
    K = x.shape[-1]
    x2d = x.reshape(-1, K).contiguous()
    out = lof.gemm(x2d, weight.contiguous(), accum_mant_bits, trans_b=True,
                   alpha=lof.gemm_alpha(scale_a, scale_b))
    out = out.reshape(*leading, weight.shape[0])
    if bias is not None:
        out = out + bias
    return out


_TILED8 = {}


def _tiled8_order(c: int, rs: int, device) -> torch.Tensor:
    """The implicit-GEMM conv kernel's reduction order (csrc/conv.cu decode_t,
    LOFGB_CONV_TILED8: 8-channel tiles outer, then the kernel position r*S + s,
    then the channel within the tile; steps of channels past C skipped) as
    indices into the im2col reduction axis c * RS + rs."""
    key = (c, rs, str(device))
    if key not in _TILED8:
        perm = []
        for t in range((c + 7) // 8 * 8 * rs):
            ct, rem = divmod(t, 8 * rs)
            ch = ct * 8 + (rem & 7)
            if ch < c:
                perm.append(ch * rs + (rem >> 3))
        _TILED8[key] = torch.tensor(perm, dtype=torch.long, device=device)
    return _TILED8[key]


def _fwht(x: torch.Tensor, block_size=None) -> torch.Tensor:
    """Orthonormal Walsh–Hadamard transform along the last dim, optionally
    blockwise (same contract as LoFloat/layers.py:173-209)."""
    n = x.shape[-1]
    if block_size is None:
        block_size = n
    if block_size <= 0 or (block_size & (block_size - 1)) != 0:
        raise ValueError(f"block_size must be a power of 2, got {block_size}")
    if n % block_size != 0:
        raise ValueError(f"block_size {block_size} must divide last dim {n}")
    shape = x.shape
    y = x.reshape(-1, block_size)
    h = 1
    while h < block_size:
        y = y.view(-1, block_size // (2 * h), 2, h)
        y = torch.stack((y[:, :, 0, :] + y[:, :, 1, :], y[:, :, 0, :] - y[:, :, 1, :]), dim=2)
        y = y.reshape(-1, block_size)
        h *= 2
    return (y * (1.0 / math.sqrt(block_size))).view(shape)


class LinearConfig:
    """Numerics of one emulated linear layer (forward and backward)."""

    def __init__(self, act_format=None, weight_format=None, scale_format=None, mx_block=32,
                 round_mode=lof.RoundingMode.RoundToNearestEven, accum_mant_bits=10,
                 variant="plain", chunk=32, grad_format=None,
                 grad_round_mode=lof.RoundingMode.StochasticRoundingA, grad_stoch_len=8,
                 grad_variant=None, alpha=1.0, accum_format=None):
        self.act_format = act_format
        self.weight_format = weight_format
        self.scale_format = scale_format if scale_format is not None else create_e8m0_params()
        self.mx_block = mx_block
        self.round_mode = round_mode
        self.accum_mant_bits = accum_mant_bits
        self.variant = variant
        self.chunk = chunk
        self.grad_format = grad_format
        self.grad_round_mode = grad_round_mode
        self.grad_stoch_len = grad_stoch_len
        self.grad_variant = grad_variant or variant
        self.alpha = float(alpha)  # forward output scale: D = alpha * acc
        # a whole accumulator format (e.g. FP16-like 5e/10m) instead of
        # accum_mant_bits mantissa bits with FP32's exponent range
        self.accum_format = accum_format


def _mx(t, fmt, cfg):
    if fmt is None:
        return t.float().contiguous()
    return lof.virtual_mx_round(t.contiguous(), cfg.mx_block, fmt, cfg.scale_format,
                                round_mode=cfg.round_mode)


class LoFLinearFunction(torch.autograd.Function):
    """Y = alpha · MX(X) · MX(W)ᵀ with emulated accumulation; hand-written backward.

    forward:  X_q = MX(X), W_q = MX(W) along K; Y = gemm(X_q, W_q, trans_b, alpha)
    backward: dY_q = round(alpha·dY, grad_format, SR)   (or alpha·dY)
              dX = gemm(dY_q, W_q)               (M×N · N×K)
              dW = gemm(dY_q, X_q, trans_a)      (N×M · M×K)
              STE: ∂MX(t)/∂t = I
    Gradients come back in the dtype of X and W (e.g. bf16 master copies)."""

    @staticmethod
    def forward(ctx, x, w, cfg: LinearConfig):
        # MX rounding reads BF16 masters directly (no FP32 copy first)
        xq = _mx(x, cfg.act_format, cfg)
        wq = _mx(w, cfg.weight_format, cfg)
        y = lof.gemm(xq, wq, cfg.accum_mant_bits, trans_b=True, alpha=cfg.alpha, variant=cfg.variant,
                     chunk=cfg.chunk, accum_format=cfg.accum_format)
        ctx.save_for_backward(xq, wq)
        ctx.cfg = cfg
        ctx.dtypes = (x.dtype, w.dtype)
        return y

    @staticmethod
    def backward(ctx, dy):
        xq, wq = ctx.saved_tensors
        cfg = ctx.cfg
        dy = dy.float().contiguous()
        if cfg.grad_format is not None:
            # alpha rides in the rounding kernel's input scale: round(alpha * dY)
            dy = lof.virtual_round(dy, cfg.grad_format, round_mode=cfg.grad_round_mode,
                                   stoch_len=cfg.grad_stoch_len, scale=cfg.alpha)
        elif cfg.alpha != 1.0:
            dy = dy * cfg.alpha
        dx = dw = None
        if ctx.needs_input_grad[0]:
            dx = lof.gemm(dy, wq, cfg.accum_mant_bits, variant=cfg.grad_variant, chunk=cfg.chunk,
                          accum_format=cfg.accum_format)
            dx = dx.to(ctx.dtypes[0])
        if ctx.needs_input_grad[1]:
            dw = lof.gemm(dy, xq, cfg.accum_mant_bits, trans_a=True, variant=cfg.grad_variant,
                          chunk=cfg.chunk, accum_format=cfg.accum_format)
            dw = dw.to(ctx.dtypes[1])
        return dx, dw, None


def lof_linear(x, w, cfg: LinearConfig):
    """Differentiable emulated linear: x (..., K), w (N, K) -> (..., N)."""
    lead = x.shape[:-1]
    y = LoFLinearFunction.apply(x.reshape(-1, x.shape[-1]), w, cfg)
    return y.reshape(*lead, w.shape[0])


class LoF_Linear(nn.Module):
    """LoFloat linear layer with the reference's constructor
    (LoFloat/layers.py:221-447). Forward is the reference's; with
    ``differentiable=True`` (default) gradients flow through the emulated GEMM
    via LoFLinearFunction."""

    def __init__(self, in_features, out_features, act_params=None, weight_params=None, bias=True,
                 bias_params=None, act_exp=None, act_mant=None, weight_exp=None, weight_mant=None,
                 bias_exp=None, bias_mant=None, rounding_mode=None, act_scale_factor=1.0,
                 w_scale_factor=1.0, b_scale_factor=1.0, accum_mant_bits=23, gemm_round_mode=None,
                 stochastic_rounding_bits=0, hadamard_transform=False, hadamard_block_size=None,
                 scaling="per_tensor", mx_block_size=32, scale_format=None, differentiable=True,
                 grad_format=None, gemm_variant="plain", chunk=32):
        super().__init__()
        if scaling not in ("per_tensor", "mx"):
            raise ValueError(f"scaling must be 'per_tensor' or 'mx', got {scaling!r}")
        self.in_features = in_features
        self.out_features = out_features
        self.rounding_mode = rounding_mode if rounding_mode is not None else lof.RoundingMode.RoundToNearestEven
        self.act_scale_factor = act_scale_factor
        self.w_scale_factor = w_scale_factor
        self.b_scale_factor = b_scale_factor
        self.scaling = scaling
        self.mx_block_size = mx_block_size
        self.scale_format = scale_format if scale_format is not None else create_e8m0_params()
        if scaling == "mx" and in_features % mx_block_size != 0:
            raise ValueError(f"mx scaling needs in_features ({in_features}) divisible by "
                             f"mx_block_size ({mx_block_size})")
        self.accum_mant_bits = accum_mant_bits
        self.gemm_round_mode = gemm_round_mode if gemm_round_mode is not None else lof.RoundingMode.RoundToNearestEven
        self.stochastic_rounding_bits = stochastic_rounding_bits
        self.hadamard_transform = hadamard_transform
        self.hadamard_block_size = hadamard_block_size
        self.act_params = act_params if act_params is not None else create_p3109_params(
            act_exp + act_mant + 1, act_mant + 1, True, True)
        self.weight_params = weight_params if weight_params is not None else create_p3109_params(
            weight_exp + weight_mant + 1, weight_mant + 1, True, True)
        if bias_params is not None:
            self.bias_params = bias_params
        elif bias_exp is not None and bias_mant is not None:
            self.bias_params = create_p3109_params(bias_exp + bias_mant + 1, bias_mant + 1, True, True)
        else:
            self.bias_params = None
        self.differentiable = differentiable
        self.grad_format = grad_format
        self.gemm_variant = gemm_variant
        self.chunk = chunk
        self._act_fid = register_format(self.act_params)
        self._weight_fid = register_format(self.weight_params)
        self._bias_fid = register_format(self.bias_params) if self.bias_params is not None else None
        self.weight = nn.Parameter(torch.empty(out_features, in_features))
        if bias:
            self.bias = nn.Parameter(torch.zeros(out_features))
        else:
            self.register_parameter("bias", None)
        nn.init.kaiming_uniform_(self.weight)

    def _cfg(self, mx: bool) -> LinearConfig:
        return LinearConfig(act_format=self.act_params if mx else None,
                            weight_format=self.weight_params if mx else None,
                            scale_format=self.scale_format, mx_block=self.mx_block_size,
                            round_mode=self.rounding_mode, accum_mant_bits=self.accum_mant_bits,
                            variant=self.gemm_variant, chunk=self.chunk, grad_format=self.grad_format)

    def forward(self, x):
        if self.hadamard_transform:
            x = _fwht(x, block_size=self.hadamard_block_size)
        if self.scaling == "mx":
            if self.differentiable:
                out = lof_linear(x, self.weight, self._cfg(True))
            else:
                x_q = STEMXRound.apply(x, self.act_params, self.scale_format, self.mx_block_size,
                                       self.rounding_mode)
                w_q = STEMXRound.apply(self.weight, self.weight_params, self.scale_format,
                                       self.mx_block_size, self.rounding_mode)
                out = _lof_linear(x_q, w_q, None, self.accum_mant_bits, self.gemm_round_mode,
                                  self.stochastic_rounding_bits)
        else:
            x_q = STERound.apply(x, self._act_fid, int(self.rounding_mode), self.act_scale_factor)
            w_q = STERound.apply(self.weight, self._weight_fid, int(self.rounding_mode),
                                 self.w_scale_factor)
            if self.differentiable:
                cfg = self._cfg(False)
                cfg.alpha = lof.gemm_alpha(float(self.act_scale_factor), float(self.w_scale_factor))
                out = lof_linear(x_q, w_q, cfg)
            else:
                out = _lof_linear(x_q, w_q, None, self.accum_mant_bits, self.gemm_round_mode,
                                  self.stochastic_rounding_bits, scale_a=float(self.act_scale_factor),
                                  scale_b=float(self.w_scale_factor))
        if self.bias is not None:
            if self._bias_fid is not None:
                b_q = STERound.apply(self.bias, self._bias_fid, int(self.rounding_mode),
                                     self.b_scale_factor)
                if self.b_scale_factor != 1.0:
                    b_q = b_q / self.b_scale_factor
            else:
                b_q = self.bias
            out = out + b_q
        return out


# ---- convolution ---------------------------------------------------------------
class LoF_Conv2d(nn.Module):
    """Conv2d with fake-quantised activation, weight and bias and an emulated
    accumulator, with the reference's constructor and forward
    (LoFloat/layers.py:453-780).

    backend "im2col" (default) gives the bits of the reference's unfold +
    per-image lof_gemm path (layers.py:684-713) without materialising the
    unfolded input: the implicit-GEMM conv2d in (c, r, s) order. backend
    "cutlass" gives lof_conv2d's bits (layers.py:620-640; the implicit GEMM in
    8-channel-tile order). scaling "mx" MX-quantises the unfolded activation and
    the reshaped weight along the reduction axis (layers.py:643-676) and runs
    the emulated GEMM per image with the activation read as the transposed
    operand. `gemm_variant` "tc" selects the tensor-core form for the
    per-tensor paths. As in the reference, no gradient flows through the
    emulated accumulation."""

    @staticmethod
    def _resolve_params(exp, mant, params):
        if params is not None:
            return params
        if exp is not None and mant is not None:
            return create_p3109_params(exp + mant + 1, mant + 1)
        raise ValueError("Must provide either (exp, mant) or params for each tensor")

    def __init__(self, in_channels, out_channels, kernel_size, stride=1, padding=0, dilation=1,
                 groups=1, act_params=None, weight_params=None, bias=True, bias_params=None,
                 act_exp=None, act_mant=None, weight_exp=None, weight_mant=None, bias_exp=None,
                 bias_mant=None, rounding_mode=None, act_scale_factor=1.0, w_scale_factor=1.0,
                 b_scale_factor=1.0, accum_mant_bits=23, gemm_round_mode=None,
                 stochastic_rounding_bits=0, hadamard_transform=False, hadamard_block_size=None,
                 scaling="per_tensor", mx_block_size=32, scale_format=None, backend="im2col",
                 gemm_variant="plain", chunk=32):
        super().__init__()
        if scaling not in ("per_tensor", "mx"):
            raise ValueError(f"scaling must be 'per_tensor' or 'mx', got {scaling!r}")
        if backend not in ("im2col", "cutlass"):
            raise ValueError(f"backend must be 'im2col' or 'cutlass', got {backend!r}")
        self.backend = backend
        self.in_channels = in_channels
        self.out_channels = out_channels
        self.kernel_size = kernel_size if isinstance(kernel_size, tuple) else (kernel_size, kernel_size)
        self.stride = stride if isinstance(stride, tuple) else (stride, stride)
        self.padding = padding if isinstance(padding, tuple) else (padding, padding)
        self.dilation = dilation if isinstance(dilation, tuple) else (dilation, dilation)
        self.groups = groups
        self.rounding_mode = rounding_mode if rounding_mode is not None else lof.RoundingMode.RoundToNearestEven
        self.act_scale_factor = act_scale_factor
        self.w_scale_factor = w_scale_factor
        self.b_scale_factor = b_scale_factor
        self.accum_mant_bits = accum_mant_bits
        self.gemm_round_mode = gemm_round_mode if gemm_round_mode is not None else lof.RoundingMode.RoundToNearestEven
        self.stochastic_rounding_bits = stochastic_rounding_bits
        self.gemm_variant = gemm_variant
        self.chunk = chunk
        self.scaling = scaling
        self.mx_block_size = mx_block_size
        self.scale_format = scale_format if scale_format is not None else create_e8m0_params()
        if scaling == "mx":
            kh, kw = self.kernel_size
            if (in_channels // groups) * kh * kw % mx_block_size != 0:
                raise ValueError(
                    f"mx scaling needs the im2col K=(C_in/groups)*kH*kW="
                    f"{(in_channels // groups) * kh * kw} divisible by mx_block_size ({mx_block_size})")
        self.hadamard_transform = hadamard_transform
        self.hadamard_block_size = hadamard_block_size
        if hadamard_transform:
            cpg = in_channels // groups
            eff = hadamard_block_size if hadamard_block_size is not None else cpg
            if eff <= 0 or (eff & (eff - 1)) != 0:
                raise ValueError("hadamard_transform=True requires (hadamard_block_size or "
                                 f"in_channels//groups) to be a power of 2, got {eff}")
            if cpg % eff != 0:
                raise ValueError(f"hadamard_block_size={eff} must divide in_channels//groups={cpg}")
        self.act_params = act_params if act_params is not None else create_p3109_params(
            act_exp + act_mant + 1, act_mant + 1, True, True)
        self.weight_params = weight_params if weight_params is not None else create_p3109_params(
            weight_exp + weight_mant + 1, weight_mant + 1, True, True)
        self.bias_params = bias_params if bias_params is not None else create_p3109_params(
            bias_exp + bias_mant + 1, bias_mant + 1, True, True) if (
                bias_exp is not None and bias_mant is not None) else None
        self.weight = nn.Parameter(torch.empty(out_channels, in_channels // groups, *self.kernel_size))
        if bias:
            self.bias = nn.Parameter(torch.zeros(out_channels))
        else:
            self.register_parameter("bias", None)
        nn.init.kaiming_uniform_(self.weight)

    @classmethod
    def from_conv2d(cls, conv: nn.Conv2d, act_params, weight_params, bias_params=None,
                    rounding_mode=None, accum_mant_bits=23, gemm_round_mode=None,
                    stochastic_rounding_bits=0, hadamard_transform=False,
                    hadamard_block_size=None):
        layer = cls(conv.in_channels, conv.out_channels, conv.kernel_size, stride=conv.stride,
                    padding=conv.padding, dilation=conv.dilation, groups=conv.groups,
                    act_params=act_params, weight_params=weight_params,
                    bias=conv.bias is not None, bias_params=bias_params,
                    rounding_mode=rounding_mode, accum_mant_bits=accum_mant_bits,
                    gemm_round_mode=gemm_round_mode,
                    stochastic_rounding_bits=stochastic_rounding_bits,
                    hadamard_transform=hadamard_transform,
                    hadamard_block_size=hadamard_block_size)
        layer.weight = nn.Parameter(conv.weight.detach().clone())
        if conv.bias is not None:
            layer.bias = nn.Parameter(conv.bias.detach().clone())
        return layer

    def __deepcopy__(self, memo):
        new = LoF_Conv2d(
            self.in_channels, self.out_channels, self.kernel_size, stride=self.stride,
            padding=self.padding, dilation=self.dilation, groups=self.groups,
            act_params=self.act_params, weight_params=self.weight_params,
            bias=self.bias is not None, bias_params=self.bias_params,
            rounding_mode=self.rounding_mode, act_scale_factor=self.act_scale_factor,
            w_scale_factor=self.w_scale_factor, b_scale_factor=self.b_scale_factor,
            accum_mant_bits=self.accum_mant_bits, gemm_round_mode=self.gemm_round_mode,
            stochastic_rounding_bits=self.stochastic_rounding_bits,
            hadamard_transform=self.hadamard_transform,
            hadamard_block_size=self.hadamard_block_size, scaling=self.scaling,
            mx_block_size=self.mx_block_size, scale_format=self.scale_format,
            backend=self.backend, gemm_variant=self.gemm_variant, chunk=self.chunk)
        new.load_state_dict(self.state_dict())
        memo[id(self)] = new
        return new

    def _out_hw(self, h, w):
        kh, kw = self.kernel_size
        ho = (h + 2 * self.padding[0] - self.dilation[0] * (kh - 1) - 1) // self.stride[0] + 1
        wo = (w + 2 * self.padding[1] - self.dilation[1] * (kw - 1) - 1) // self.stride[1] + 1
        return ho, wo

    def _bias(self, out, scaled=True):
        if self.bias is None:
            return out
        if self.bias_params is None:
            return out + self.bias.view(1, -1, 1, 1)
        if scaled:
            b_q = STERound.apply(self.bias, self.bias_params, self.rounding_mode, self.b_scale_factor)
            if self.b_scale_factor != 1.0:
                b_q = b_q / self.b_scale_factor
        else:
            b_q = STERound.apply(self.bias, self.bias_params, self.rounding_mode)
        return out + b_q.view(1, -1, 1, 1)

    def forward(self, x):
        if self.hadamard_transform:
            if self.groups == 1:
                x = _fwht(x.movedim(1, -1).contiguous(), block_size=self.hadamard_block_size)
                x = x.movedim(-1, 1).contiguous()
            else:
                b, c, h, w = x.shape
                x = x.view(b, self.groups, c // self.groups, h, w).movedim(2, -1).contiguous()
                x = _fwht(x, block_size=self.hadamard_block_size)
                x = x.movedim(-1, 2).contiguous().view(b, c, h, w)

        cin, cout = self.in_channels // self.groups, self.out_channels // self.groups

        if self.scaling == "mx":
            # MX blocks along each group's im2col reduction (C_in/groups * kH * kW),
            # as the reference's im2col path defines them; one batched GEMM per
            # group. backend="cutlass" sums the same rounded values in the
            # implicit-GEMM kernel's reduction order (8-channel tiles, then
            # (r, s), then the channel in the tile), by permuting the reduction
            # axis before a sequential GEMM.
            b = x.shape[0]
            ho, wo = self._out_hw(x.shape[2], x.shape[3])
            outs = []
            for g in range(self.groups):
                xg = x if self.groups == 1 else x[:, g * cin:(g + 1) * cin]
                x_col = torch.nn.functional.unfold(xg, kernel_size=self.kernel_size,
                                                   dilation=self.dilation, padding=self.padding,
                                                   stride=self.stride)           # (B, K, L)
                x_lk = STEMXRound.apply(x_col.transpose(1, 2).contiguous(), self.act_params,
                                        self.scale_format, self.mx_block_size,
                                        self.rounding_mode)                      # (B, L, K)
                wg = self.weight if self.groups == 1 else self.weight[g * cout:(g + 1) * cout]
                w_col = STEMXRound.apply(wg.reshape(cout, -1), self.weight_params,
                                         self.scale_format, self.mx_block_size, self.rounding_mode)
                if self.backend == "cutlass":
                    perm = _tiled8_order(cin, self.kernel_size[0] * self.kernel_size[1], x.device)
                    x_lk = x_lk.index_select(2, perm).contiguous()
                    w_col = w_col.index_select(1, perm).contiguous()
                outs.append(lof.gemm(w_col, x_lk, self.accum_mant_bits, trans_b=True,
                                     variant=self.gemm_variant, chunk=self.chunk))   # (B, cout, L)
            out = outs[0] if self.groups == 1 else torch.cat(outs, dim=1)
            return self._bias(out.view(b, self.out_channels, ho, wo), scaled=False)

        if self.backend == "cutlass":
            x_q = STERound.apply(x, self.act_params, self.rounding_mode, self.act_scale_factor)
            w_q = STERound.apply(self.weight, self.weight_params, self.rounding_mode,
                                 self.w_scale_factor)

            def run(xx, ww):
                if self.gemm_variant == "plain":
                    return lof.lof_conv2d(xx, ww, self.padding[0], self.padding[1], self.stride[0],
                                          self.stride[1], self.dilation[0], self.dilation[1],
                                          self.accum_mant_bits, self.gemm_round_mode,
                                          self.stochastic_rounding_bits, float(self.w_scale_factor),
                                          float(self.act_scale_factor))
                return lof.conv2d(xx, ww, self.accum_mant_bits, stride=self.stride,
                                  padding=self.padding, dilation=self.dilation,
                                  alpha=lof.conv2d_alpha(self.w_scale_factor, self.act_scale_factor),
                                  order="tiled8", variant=self.gemm_variant, chunk=self.chunk)
            if self.groups == 1:
                out = run(x_q, w_q)
            else:   # each group is an independent convolution over its channels
                out = torch.cat([run(x_q[:, g * cin:(g + 1) * cin].contiguous(),
                                     w_q[g * cout:(g + 1) * cout].contiguous())
                                 for g in range(self.groups)], dim=1)
            return self._bias(out)

        x_q = STERound.apply(x, self.act_params, self.rounding_mode, self.act_scale_factor)
        w_q = STERound.apply(self.weight, self.weight_params, self.rounding_mode, self.w_scale_factor)
        # the im2col GEMM is W @ X_col: scale_a is the weight's, scale_b the activation's
        alpha = lof.gemm_alpha(float(self.w_scale_factor), float(self.act_scale_factor))
        conv = lambda xx, ww: lof.conv2d(  # noqa: E731
            xx, ww, self.accum_mant_bits, stride=self.stride, padding=self.padding,
            dilation=self.dilation, alpha=alpha, order="crs", variant=self.gemm_variant,
            chunk=self.chunk)
        if self.groups == 1:
            out = conv(x_q, w_q)
        else:
            out = torch.cat([conv(x_q[:, g * cin:(g + 1) * cin].contiguous(),
                                  w_q[g * cout:(g + 1) * cout].contiguous())
                             for g in range(self.groups)], dim=1)
        return self._bias(out)

    def set_mantissa(self, activ_mant, weight_mant, bias_mant):
        ae = self.act_params.total_bits - self.act_params.mantissa_bits - 1
        we = self.weight_params.total_bits - self.weight_params.mantissa_bits - 1
        be = self.bias_params.total_bits - self.bias_params.mantissa_bits - 1
        self.act_params = create_p3109_params(1 + ae + activ_mant, activ_mant + 1, True, True)
        self.weight_params = create_p3109_params(1 + we + weight_mant, weight_mant + 1, True, True)
        self.bias_params = create_p3109_params(1 + be + bias_mant, bias_mant + 1, True, True)

    def set_exponent(self, activ_exp, weight_exp, bias_exp):
        am, wm = self.act_params.mantissa_bits, self.weight_params.mantissa_bits
        bm = self.bias_params.mantissa_bits
        self.act_params = create_p3109_params(1 + activ_exp + am, am + 1, True, True)
        self.weight_params = create_p3109_params(1 + weight_exp + wm, wm + 1, True, True)
        self.bias_params = create_p3109_params(1 + bias_exp + bm, bm + 1, True, True)

    def set_exponentbias(self, activ_expbias, weight_expbias, bias_expbias):
        self.act_params = create_p3109_params(self.act_params.total_bits,
                                              self.act_params.mantissa_bits, True, True,
                                              activ_expbias)
        self.weight_params = create_p3109_params(self.weight_params.total_bits,
                                                 self.weight_params.mantissa_bits, True, True,
                                                 weight_expbias)
        self.bias_params = create_p3109_params(self.bias_params.total_bits,
                                               self.bias_params.mantissa_bits, True, True,
                                               bias_expbias)

    def set_saturation_mode(self, activ_sat, weight_sat, bias_sat):
        self.act_params = create_p3109_params(self.act_params.total_bits,
                                              self.act_params.mantissa_bits, True, activ_sat)
        self.weight_params = create_p3109_params(self.weight_params.total_bits,
                                                 self.weight_params.mantissa_bits, True, weight_sat)
        self.bias_params = create_p3109_params(self.bias_params.total_bits,
                                               self.bias_params.mantissa_bits, True, bias_sat)

    def set_accumulation_precision(self, accum_mant_bits):
        self.accum_mant_bits = accum_mant_bits

    def extra_repr(self):
        def em(p):
            return (p.mantissa_bits, p.total_bits - p.mantissa_bits - 1) if p is not None else (None, None)
        (am, ae), (wm, we), (bm, be) = em(self.act_params), em(self.weight_params), em(self.bias_params)
        return (f"in_channels={self.in_channels}, out_channels={self.out_channels}, "
                f"kernel_size={self.kernel_size}, stride={self.stride}, padding={self.padding}, "
                f"dilation={self.dilation}, groups={self.groups}, bias={self.bias is not None}, "
                f"act_mantissa={am}, act_exponent={ae}, weight_mantissa={wm}, "
                f"weight_exponent={we}, bias_mantissa={bm}, bias_exponent={be}, "
                f"accum_mant_bits={self.accum_mant_bits}, "
                f"hadamard_transform={self.hadamard_transform}, "
                f"hadamard_block_size={self.hadamard_block_size}")


# ---- piecewise-linear SiLU -------------------------------------------------------
class _PWLSiLUApprox(torch.autograd.Function):
    """pwl_silu forward (one read, one write); backward is the analytic SiLU
    derivative s·(1 + x·(1 − s)), s = sigmoid(x) (LoFloat/layers.py:1050-1069)."""

    @staticmethod
    def forward(ctx, x, lut, R):
        ctx.save_for_backward(x)
        return lof.pwl_silu(x, lut, float(R))

    @staticmethod
    def backward(ctx, grad_output):
        (x,) = ctx.saved_tensors
        s = torch.sigmoid(x)
        return grad_output * (s * (1 + x * (1 - s))), None, None


class PWLSiLU(nn.Module):
    """SiLU from a piecewise-linear table of 2^lut_bits uniform segments on
    [-R, R], relu outside (LoFloat/layers.py:1072-1146), run by the
    pwl_silu kernel (one read, one write); backward is the analytic SiLU
    derivative. The table is built by pwl.pwl_table ('uniform', 'midpoint'
    or 'minimax'). The kernel holds tables of up to 4096 segments
    (lut_bits <= 12); `use_ext` is accepted for the reference's signature,
    and there is no other path."""

    def __init__(self, R=8.0, lut_bits=4, lut_method="minimax", use_ext=True):
        super().__init__()
        self.R = float(R)
        self.lut_bits = lut_bits
        self.lut_size = 1 << lut_bits
        if self.lut_size % 2 != 0:
            raise ValueError("lut_size must be even so x=0 is a knot.")
        if self.lut_size > 4096:
            raise ValueError(f"lut_bits {lut_bits}: the pwl_silu kernel holds at most 4096 segments")
        self.use_ext = True
        self.register_buffer("lut", torch.empty(self.lut_size + 1))
        self.init_lut(lut_method)

    def init_lut(self, method="minimax"):
        self.lut.copy_(pwl_table(pwl_silu_fn, -self.R, self.R, self.lut_size, method, self.lut.dtype))
        self.lut_method = method

    def forward(self, x):
        return _PWLSiLUApprox.apply(x, self.lut, self.R)


# ---- attention -------------------------------------------------------------------
class LoF_MultiHeadAttention(nn.Module):
    """Multi-head attention whose four projections and two attention products
    run on the emulated-accumulation GEMM, with the reference's constructor and
    forward (LoFloat/layers.py:1152-1410). Inputs are batch-first (B, T, E).
    The score product Q·Kᵀ and the context product P·V are strided-batched
    launches over all (batch, head) pairs, Kᵀ read in place; softmax, masks and
    dropout are torch ops as in the reference. `gemm_variant` "tc" moves every
    product to the tensor-core form."""

    def __init__(self, embed_dim, num_heads, act_params=None, weight_params=None, bias=True,
                 bias_params=None, act_exp=None, act_mant=None, weight_exp=None, weight_mant=None,
                 bias_exp=None, bias_mant=None, rounding_mode=None, dropout=0.0,
                 accum_mant_bits=23, gemm_round_mode=None, stochastic_rounding_bits=0,
                 scaling="per_tensor", mx_block_size=32, scale_format=None,
                 gemm_variant="plain", chunk=32):
        super().__init__()
        assert embed_dim % num_heads == 0, "embed_dim must be divisible by num_heads"
        if scaling not in ("per_tensor", "mx"):
            raise ValueError(f"scaling must be 'per_tensor' or 'mx', got {scaling!r}")
        self.embed_dim = embed_dim
        self.num_heads = num_heads
        self.head_dim = embed_dim // num_heads
        self.scale = self.head_dim ** -0.5
        self.dropout = dropout
        self.rounding_mode = rounding_mode if rounding_mode is not None else lof.RoundingMode.RoundToNearestEven
        self.scaling = scaling
        self.mx_block_size = mx_block_size
        self.scale_format = scale_format if scale_format is not None else create_e8m0_params()
        if scaling == "mx" and embed_dim % mx_block_size != 0:
            raise ValueError(f"mx scaling needs embed_dim ({embed_dim}) divisible by "
                             f"mx_block_size ({mx_block_size})")
        self.accum_mant_bits = accum_mant_bits
        self.gemm_round_mode = gemm_round_mode if gemm_round_mode is not None else lof.RoundingMode.RoundToNearestEven
        self.stochastic_rounding_bits = stochastic_rounding_bits
        self.gemm_variant = gemm_variant
        self.chunk = chunk
        self.act_params = act_params if act_params is not None else create_p3109_params(
            act_exp + act_mant + 1, act_mant + 1, True, True)
        self.weight_params = weight_params if weight_params is not None else create_p3109_params(
            weight_exp + weight_mant + 1, weight_mant + 1, True, True)
        self.bias_params = bias_params if bias_params is not None else create_p3109_params(
            bias_exp + bias_mant + 1, bias_mant + 1, True, True) if (
                bias_exp is not None and bias_mant is not None) else None
        for nm in ("q", "k", "v", "out"):
            self.register_parameter(f"{nm}_weight", nn.Parameter(torch.empty(embed_dim, embed_dim)))
            if bias:
                self.register_parameter(f"{nm}_bias", nn.Parameter(torch.zeros(embed_dim)))
            else:
                self.register_parameter(f"{nm}_bias", None)
        self._reset_parameters()

    def _reset_parameters(self):
        for w in (self.q_weight, self.k_weight, self.v_weight, self.out_weight):
            nn.init.xavier_uniform_(w)

    @classmethod
    def from_mha(cls, mha: nn.MultiheadAttention, act_params, weight_params, bias_params=None,
                 rounding_mode=None, accum_mant_bits=23, gemm_round_mode=None,
                 stochastic_rounding_bits=0):
        layer = cls(mha.embed_dim, mha.num_heads, act_params=act_params,
                    weight_params=weight_params, bias=mha.in_proj_bias is not None,
                    bias_params=bias_params, rounding_mode=rounding_mode, dropout=mha.dropout,
                    accum_mant_bits=accum_mant_bits, gemm_round_mode=gemm_round_mode,
                    stochastic_rounding_bits=stochastic_rounding_bits)
        e = mha.embed_dim
        w = mha.in_proj_weight.data
        dev = w.device

        def q(t, p):  # rounding runs on the GPU; the result goes back to t's device
            return layer._quantize(t.detach().clone().to("cuda"), p).to(t.device)

        layer.q_weight = nn.Parameter(q(w[:e], layer.weight_params))
        layer.k_weight = nn.Parameter(q(w[e:2 * e], layer.weight_params))
        layer.v_weight = nn.Parameter(q(w[2 * e:], layer.weight_params))
        layer.out_weight = nn.Parameter(q(mha.out_proj.weight.data, layer.weight_params))
        if mha.in_proj_bias is not None:
            b = mha.in_proj_bias.data
            layer.q_bias = nn.Parameter(q(b[:e], layer.bias_params))
            layer.k_bias = nn.Parameter(q(b[e:2 * e], layer.bias_params))
            layer.v_bias = nn.Parameter(q(b[2 * e:], layer.bias_params))
            layer.out_bias = nn.Parameter(q(mha.out_proj.bias.data, layer.bias_params))
        return layer.to(dev)

    def __deepcopy__(self, memo):
        new = LoF_MultiHeadAttention(
            self.embed_dim, self.num_heads, act_params=self.act_params,
            weight_params=self.weight_params, bias=self.q_bias is not None,
            bias_params=self.bias_params, rounding_mode=self.rounding_mode, dropout=self.dropout,
            accum_mant_bits=self.accum_mant_bits, gemm_round_mode=self.gemm_round_mode,
            stochastic_rounding_bits=self.stochastic_rounding_bits, scaling=self.scaling,
            mx_block_size=self.mx_block_size, scale_format=self.scale_format,
            gemm_variant=self.gemm_variant, chunk=self.chunk)
        new.load_state_dict(self.state_dict())
        memo[id(self)] = new
        return new

    def _quantize(self, tensor, params):
        if params is None:
            return tensor
        if self.scaling == "mx":
            if tensor.shape[-1] % self.mx_block_size != 0:
                raise ValueError(f"mx scaling needs the last dim ({tensor.shape[-1]}) divisible by "
                                 f"mx_block_size ({self.mx_block_size})")
            return STEMXRound.apply(tensor, params, self.scale_format, self.mx_block_size,
                                    self.rounding_mode)
        return STERound.apply(tensor, params, self.rounding_mode)

    def _linear(self, x, w, b):
        leading, k = x.shape[:-1], x.shape[-1]
        out = lof.gemm(x.reshape(-1, k).contiguous(), w.contiguous(), self.accum_mant_bits,
                       trans_b=True, variant=self.gemm_variant, chunk=self.chunk)
        out = out.reshape(*leading, w.shape[0])
        return out + b if b is not None else out

    def forward(self, query, key, value, attn_mask=None, key_padding_mask=None,
                need_weights=False):
        bsz, t, e = query.shape
        s_len = key.shape[1]
        query = self._quantize(query, self.act_params)
        key = self._quantize(key, self.act_params)
        value = self._quantize(value, self.act_params)
        wq, wk, wv, wo = (self._quantize(w, self.weight_params)
                          for w in (self.q_weight, self.k_weight, self.v_weight, self.out_weight))
        bq, bk, bv, bo = (self._quantize(b, self.bias_params) if b is not None else None
                          for b in (self.q_bias, self.k_bias, self.v_bias, self.out_bias))
        h, d = self.num_heads, self.head_dim
        q = self._linear(query, wq, bq).view(bsz, t, h, d).transpose(1, 2)
        k = self._linear(key, wk, bk).view(bsz, s_len, h, d).transpose(1, 2)
        v = self._linear(value, wv, bv).view(bsz, s_len, h, d).transpose(1, 2)
        attn = _lof_gemm_2d(q, k.transpose(-2, -1), self.accum_mant_bits, self.gemm_round_mode,
                            self.stochastic_rounding_bits, variant=self.gemm_variant,
                            chunk=self.chunk) * self.scale
        if attn_mask is not None:
            attn = attn + attn_mask
        if key_padding_mask is not None:
            attn = attn.masked_fill(key_padding_mask.unsqueeze(1).unsqueeze(2), float("-inf"))
        attn = torch.softmax(attn, dim=-1)
        if self.training and self.dropout > 0.0:
            attn = torch.nn.functional.dropout(attn, p=self.dropout)
        out = _lof_gemm_2d(attn, v, self.accum_mant_bits, self.gemm_round_mode,
                           self.stochastic_rounding_bits, variant=self.gemm_variant,
                           chunk=self.chunk)
        out = out.transpose(1, 2).contiguous().view(bsz, t, e)
        out = self._linear(out, wo, bo)
        return (out, attn) if need_weights else (out, None)

    def set_accumulation_precision(self, accum_mant_bits):
        self.accum_mant_bits = accum_mant_bits

    def extra_repr(self):
        return (f"embed_dim={self.embed_dim}, num_heads={self.num_heads}, "
                f"head_dim={self.head_dim}, dropout={self.dropout}, "
                f"bias={self.q_bias is not None}, accum_mant_bits={self.accum_mant_bits}")
