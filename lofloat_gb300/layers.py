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


def _lof_gemm_2d(A, B, accum_mant_bits, gemm_round_mode, stochastic_rounding_bits, scale_a=1.0,
                 scale_b=1.0):
    """(..., M, K) x (..., K, N) -> (..., M, N) (LoFloat/layers.py:121-150)."""
    if A.dim() == 2 and B.dim() == 2:
        return lof.lof_gemm(A.contiguous(), B.contiguous(), accum_mant_bits, gemm_round_mode,
                            stochastic_rounding_bits, scale_a, scale_b)
    batch_shape = A.shape[:-2]
    M, K = A.shape[-2], A.shape[-1]
    N = B.shape[-1]
    A_flat = A.reshape(-1, M, K).contiguous()
    B_flat = B.reshape(-1, K, N).contiguous()
    out = torch.stack([lof.lof_gemm(A_flat[i], B_flat[i], accum_mant_bits, gemm_round_mode,
                                    stochastic_rounding_bits, scale_a, scale_b)
                       for i in range(A_flat.shape[0])])
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
                 grad_variant=None, alpha=1.0):
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


def _mx(t, fmt, cfg):
    if fmt is None:
        return t.contiguous()
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
        x32 = x.float()
        w32 = w.float()
        xq = _mx(x32, cfg.act_format, cfg)
        wq = _mx(w32, cfg.weight_format, cfg)
        y = lof.gemm(xq, wq, cfg.accum_mant_bits, trans_b=True, alpha=cfg.alpha, variant=cfg.variant,
                     chunk=cfg.chunk)
        ctx.save_for_backward(xq, wq)
        ctx.cfg = cfg
        ctx.dtypes = (x.dtype, w.dtype)
        return y

    @staticmethod
    def backward(ctx, dy):
        xq, wq = ctx.saved_tensors
        cfg = ctx.cfg
        dy = dy.float().contiguous()
        if cfg.alpha != 1.0:
            dy = dy * cfg.alpha
        if cfg.grad_format is not None:
            dy = lof.virtual_round(dy, cfg.grad_format, round_mode=cfg.grad_round_mode,
                                   stoch_len=cfg.grad_stoch_len)
        dx = dw = None
        if ctx.needs_input_grad[0]:
            dx = lof.gemm(dy, wq, cfg.accum_mant_bits, variant=cfg.grad_variant, chunk=cfg.chunk)
            dx = dx.to(ctx.dtypes[0])
        if ctx.needs_input_grad[1]:
            dw = lof.gemm(dy, xq, cfg.accum_mant_bits, trans_a=True, variant=cfg.grad_variant,
                          chunk=cfg.chunk)
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
