"""BatchNorm variants with cheap normaliser approximations
(LoFloat/layers.py:805-1047): L1 (mean absolute deviation), L-infinity
(max absolute deviation), FISR (bit-trick inverse square root with two
Newton steps) and PWL (piecewise-linear table for 1/sqrt on the mantissa).

The forward runs on two kernels (csrc/norms.cu): the per-channel
statistics (one pass for the variance variants, two for the deviation ones,
with the running averages updated in the same launch) and one fused
normalise + scale + affine pass. Modules, buffers and arguments are the
reference's. The backward gives the gradient of the reference's own
formulation (autograd through its FP32 chain, including the approximate
normalisers): it recomputes that chain with torch ops from the saved input,
which costs about what the reference's forward did; the forward, the part a
model runs at inference, has no such pass.
"""
from __future__ import annotations

import math

import torch
import torch.nn as nn

from . import binding as lof
from .pwl import inv_sqrt, pwl_table

_MAGIC = 0x5F3759DF
_INV_SQRT2 = 0.7071067811865476


def _scale_buffer(scale, num_features):
    """Per-channel scale: a number, or a tensor of 1 or num_features values."""
    if not isinstance(scale, torch.Tensor):
        return torch.full((num_features,), float(scale))
    flat = scale.detach().float().reshape(-1)
    if flat.numel() == 1:
        return flat.expand(num_features).clone()
    if flat.numel() != num_features:
        raise ValueError(f"scale must hold 1 or {num_features} values (one per channel), "
                         f"not {flat.numel()}")
    return flat.clone()


# ---- the reference's formulation, for the backward pass --------------------------
def _fisr_chain(v):
    half = v * 0.5
    y = (_MAGIC - (v.detach().contiguous().view(torch.int32) >> 1)).view(torch.float32)
    for _ in range(2):
        y = y * (1.5 - half * y * y)
    return y


def _pwl_chain(v, lut):
    n = lut.numel() - 1
    m, e = torch.frexp(v)
    u = (m * 2.0 - 1.0) * n
    i = u.detach().floor().long().clamp(0, n - 1)
    frac = u - i.to(v.dtype)
    r = lut[i] + frac * (lut[i + 1] - lut[i])
    e = e - 1
    sc = torch.ldexp(torch.ones_like(v), -torch.div(e, 2, rounding_mode="floor"))
    return r * torch.where(e % 2 != 0, sc * _INV_SQRT2, sc)


def _chain(kind, x, weight, bias, scale, eps, lut, stats):
    """Output of the reference's op chain for x (N, C, *); stats = None
    recomputes the batch statistics (training), else (mean, dev) buffers."""
    dims = [0] + list(range(2, x.dim()))
    shape = [1, -1] + [1] * (x.dim() - 2)
    if stats is None:
        mean = x.mean(dim=dims)
        xc = x - mean.view(shape)
        if kind == "l1":
            dev = xc.abs().mean(dim=dims)
        elif kind == "linf":
            dev = xc.abs().amax(dim=dims)
        else:
            dev = x.var(dim=dims, unbiased=False)
    else:
        mean, dev = stats
        xc = x - mean.view(shape)
    if kind in ("l1", "linf"):
        out = xc / (dev.view(shape) + eps) * scale.view(shape)
    else:
        r = _fisr_chain(dev + eps) if kind == "fisr" else _pwl_chain(dev + eps, lut)
        out = xc * r.view(shape)
    if weight is not None:
        out = out * weight.view(shape) + bias.view(shape)
    return out


class _BatchNormFn(torch.autograd.Function):
    """Forward: the two kernels. Backward: autograd through the reference's
    chain, recomputed from the saved input."""

    @staticmethod
    def forward(ctx, x, weight, bias, mod, training):
        kind = mod._kind
        xf = x.float().contiguous()
        if training:
            rdev = getattr(mod, mod._dev_buffer)
            mean, dev = lof.bn_stats(xf, mod._stat, running_mean=mod.running_mean,
                                     running_dev=rdev, momentum=mod.momentum)
        else:
            mean, dev = mod.running_mean, getattr(mod, mod._dev_buffer)
        y = lof.bn_apply(xf, mean, dev, mod.eps, mod._norm, scale=getattr(mod, "scale", None)
                         if kind in ("l1", "linf") else None,
                         weight=weight, bias=bias, lut=getattr(mod, "lut", None))
        ctx.kind, ctx.eps, ctx.training = kind, mod.eps, training
        ctx.scale = getattr(mod, "scale", None)
        ctx.lut = getattr(mod, "lut", None)
        ctx.stats = None if training else (mean.detach().clone(), dev.detach().clone())
        ctx.save_for_backward(x, weight, bias)
        return y.to(x.dtype)

    @staticmethod
    def backward(ctx, gy):
        x, weight, bias = ctx.saved_tensors
        with torch.enable_grad():
            xs = x.detach().float().requires_grad_(ctx.needs_input_grad[0])
            ws = weight.detach().requires_grad_(ctx.needs_input_grad[1]) if weight is not None else None
            bs = bias.detach().requires_grad_(ctx.needs_input_grad[2]) if bias is not None else None
            out = _chain(ctx.kind, xs, ws, bs, ctx.scale, ctx.eps, ctx.lut, ctx.stats)
            wrt = [t for t in (xs, ws, bs) if t is not None and t.requires_grad]
            grads = iter(torch.autograd.grad(out, wrt, gy.float()) if wrt else ())
        gx = next(grads).to(x.dtype) if xs.requires_grad else None
        gw = next(grads) if ws is not None and ws.requires_grad else None
        gb = next(grads) if bs is not None and bs.requires_grad else None
        return gx, gw, gb, None, None


class _BatchNormBase(nn.Module):
    _kind = ""
    _stat = lof.BnStat.VARIANCE
    _norm = lof.BnNorm.DIVIDE
    _dev_buffer = "running_var"
    _tracks_batches = True

    def __init__(self, num_features, eps, momentum, affine):
        super().__init__()
        self.num_features = num_features
        self.eps = eps
        self.momentum = momentum
        self.affine = affine
        if affine:
            self.weight = nn.Parameter(torch.ones(num_features))
            self.bias = nn.Parameter(torch.zeros(num_features))
        else:
            self.register_parameter("weight", None)
            self.register_parameter("bias", None)
        self.register_buffer("running_mean", torch.zeros(num_features))
        self.register_buffer(self._dev_buffer, torch.ones(num_features))
        if self._tracks_batches:
            self.register_buffer("num_batches_tracked", torch.tensor(0, dtype=torch.long))

    def forward(self, x):
        if self.training and self._tracks_batches:
            with torch.no_grad():
                self.num_batches_tracked += 1
        return _BatchNormFn.apply(x, self.weight, self.bias, self, self.training)


class L1BatchNorm(_BatchNormBase):
    """(x - mean) / (mean |x - mean| + eps) * scale, scale sqrt(2/pi) by
    default (the Gaussian ratio of std to mean absolute deviation)."""
    _kind, _stat, _norm, _dev_buffer = "l1", lof.BnStat.MEAN_ABS_DEV, lof.BnNorm.DIVIDE, "running_mad"

    def __init__(self, num_features, eps=1e-5, momentum=0.1, affine=True,
                 scale=math.sqrt(2 / math.pi)):
        super().__init__(num_features, eps, momentum, affine)
        self.register_buffer("scale", _scale_buffer(scale, num_features))


class LinfBatchNorm(_BatchNormBase):
    """(x - mean) / (max |x - mean| + eps) * scale (scale 1 by default)."""
    _kind, _stat, _norm, _dev_buffer = "linf", lof.BnStat.MAX_ABS_DEV, lof.BnNorm.DIVIDE, "running_maxdev"
    _tracks_batches = False

    def __init__(self, num_features, eps=1e-5, momentum=0.1, affine=True, scale=1.0):
        super().__init__(num_features, eps, momentum, affine)
        self.register_buffer("scale", _scale_buffer(scale, num_features))


class FISRBatchNorm(_BatchNormBase):
    """Variance normalisation with the bit-trick inverse square root:
    y0 = bits(0x5F3759DF - (bits(v) >> 1)), then two Newton steps
    y <- y (1.5 - v/2 y^2)."""
    _kind, _norm = "fisr", lof.BnNorm.FISR
    MAGIC = _MAGIC

    def __init__(self, num_features, eps=1e-5, momentum=0.1, affine=True):
        super().__init__(num_features, eps, momentum, affine)

    @staticmethod
    def _fast_rsqrt(v):
        return _fisr_chain(v.to(torch.float32)).to(v.dtype)


class PWLBatchNorm(_BatchNormBase):
    """Variance normalisation with 1/sqrt from a piecewise-linear table over
    the mantissa: var + eps = m 2^e with m in [1, 2); 1/sqrt(m) interpolated
    from 2^lut_bits uniform segments ('uniform', 'midpoint' or 'minimax'
    knot values), times 2^(-e/2) (and 1/sqrt(2) for odd e)."""
    _kind, _norm = "pwl", lof.BnNorm.PWL
    INV_SQRT2 = _INV_SQRT2

    def __init__(self, num_features, eps=1e-5, momentum=0.1, affine=True, lut_bits=4,
                 lut_method="minimax"):
        super().__init__(num_features, eps, momentum, affine)
        self.lut_bits = lut_bits
        self.lut_size = 1 << lut_bits
        self.register_buffer("lut", torch.empty(self.lut_size + 1))
        self.init_lut(lut_method)

    def init_lut(self, method="minimax"):
        self.lut.copy_(pwl_table(inv_sqrt, 1.0, 2.0, self.lut_size, method, self.lut.dtype))
        self.lut_method = method

    def _rsqrt_pwl(self, v):
        return _pwl_chain(v, self.lut)
