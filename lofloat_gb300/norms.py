"""BatchNorm variants with cheap normaliser approximations
(LoFloat/layers.py:805-1047): L1 (mean absolute deviation), L-infinity
(max absolute deviation), FISR (bit-trick inverse square root with two
Newton steps) and PWL (piecewise-linear table for 1/sqrt on the mantissa).

In the reference these are compositions of torch ops, not kernels; they are
kept as such here (same statistics, buffers, momentum updates and affine
step), so they run on any device torch supports.
"""
from __future__ import annotations

import math

import torch
import torch.nn as nn

from .pwl import inv_sqrt, pwl_table


def _scale_buffer(scale, num_features):
    if isinstance(scale, torch.Tensor):
        s = scale.detach().float().reshape(-1)
        if s.numel() == 1:
            return torch.full((num_features,), s.item())
        if s.numel() != num_features:
            raise ValueError(f"scale tensor must have 1 or {num_features} elements; got {s.numel()}")
        return s.clone()
    return torch.full((num_features,), float(scale))


class _BatchNormBase(nn.Module):
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

    @staticmethod
    def _dims(x):
        return [0] + list(range(2, x.dim())), [1, -1] + [1] * (x.dim() - 2)

    def _track(self, name, value):
        buf = getattr(self, name)
        buf.mul_(1 - self.momentum).add_(value.detach(), alpha=self.momentum)

    def _affine(self, out, view):
        if self.affine:
            out = out * self.weight.view(view) + self.bias.view(view)
        return out


class L1BatchNorm(_BatchNormBase):
    """(x - mean) / (mean |x - mean| + eps) * scale, scale sqrt(2/pi) by
    default (the Gaussian ratio of std to mean absolute deviation)."""

    def __init__(self, num_features, eps=1e-5, momentum=0.1, affine=True,
                 scale=math.sqrt(2 / math.pi)):
        super().__init__(num_features, eps, momentum, affine)
        self.register_buffer("running_mad", torch.ones(num_features))
        self.register_buffer("num_batches_tracked", torch.tensor(0, dtype=torch.long))
        self.register_buffer("scale", _scale_buffer(scale, num_features))

    def forward(self, x):
        dims, view = self._dims(x)
        if self.training:
            mean = x.mean(dim=dims)
            xc = x - mean.view(view)
            mad = xc.abs().mean(dim=dims)
            with torch.no_grad():
                self.num_batches_tracked += 1
                self._track("running_mean", mean)
                self._track("running_mad", mad)
        else:
            mean, mad = self.running_mean, self.running_mad
            xc = x - mean.view(view)
        out = xc / (mad.view(view) + self.eps) * self.scale.view(view)
        return self._affine(out, view)


class LinfBatchNorm(_BatchNormBase):
    """(x - mean) / (max |x - mean| + eps) * scale (scale 1 by default)."""

    def __init__(self, num_features, eps=1e-5, momentum=0.1, affine=True, scale=1.0):
        super().__init__(num_features, eps, momentum, affine)
        self.register_buffer("running_maxdev", torch.ones(num_features))
        self.register_buffer("scale", _scale_buffer(scale, num_features))

    def forward(self, x):
        dims, view = self._dims(x)
        if self.training:
            mean = x.mean(dim=dims)
            xc = x - mean.view(view)
            maxdev = xc.abs().amax(dim=dims)
            with torch.no_grad():
                self._track("running_mean", mean)
                self._track("running_maxdev", maxdev)
        else:
            mean, maxdev = self.running_mean, self.running_maxdev
            xc = x - mean.view(view)
        out = xc / (maxdev.view(view) + self.eps) * self.scale.view(view)
        return self._affine(out, view)


class FISRBatchNorm(_BatchNormBase):
    """Variance normalisation with the bit-trick inverse square root:
    y0 = bits(0x5F3759DF - (bits(v) >> 1)), then two Newton steps
    y <- y (1.5 - v/2 y^2). FP32 bit manipulation."""

    MAGIC = 0x5F3759DF

    def __init__(self, num_features, eps=1e-5, momentum=0.1, affine=True):
        super().__init__(num_features, eps, momentum, affine)
        self.register_buffer("running_var", torch.ones(num_features))
        self.register_buffer("num_batches_tracked", torch.tensor(0, dtype=torch.long))

    @staticmethod
    def _fast_rsqrt(v):
        v32 = v.to(torch.float32).contiguous()
        half = v32 * 0.5
        y = (FISRBatchNorm.MAGIC - (v32.view(torch.int32) >> 1)).view(torch.float32).clone()
        y = y * (1.5 - half * y * y)
        y = y * (1.5 - half * y * y)
        return y.to(v.dtype)

    def forward(self, x):
        dims, view = self._dims(x)
        if self.training:
            mean = x.mean(dim=dims)
            var = x.var(dim=dims, unbiased=False)
            with torch.no_grad():
                self.num_batches_tracked += 1
                self._track("running_mean", mean)
                self._track("running_var", var)
        else:
            mean, var = self.running_mean, self.running_var
        out = (x - mean.view(view)) * self._fast_rsqrt(var + self.eps).view(view)
        return self._affine(out, view)


class PWLBatchNorm(_BatchNormBase):
    """Variance normalisation with 1/sqrt from a piecewise-linear table over
    the mantissa: var + eps = m 2^e with m in [1, 2); 1/sqrt(m) interpolated
    from 2^lut_bits uniform segments ('uniform', 'midpoint' or 'minimax'
    knot values), times 2^(-e/2) (and 1/sqrt(2) for odd e)."""

    INV_SQRT2 = 0.7071067811865476

    def __init__(self, num_features, eps=1e-5, momentum=0.1, affine=True, lut_bits=4,
                 lut_method="minimax"):
        super().__init__(num_features, eps, momentum, affine)
        self.lut_bits = lut_bits
        self.lut_size = 1 << lut_bits
        self.register_buffer("running_var", torch.ones(num_features))
        self.register_buffer("num_batches_tracked", torch.tensor(0, dtype=torch.long))
        self.register_buffer("lut", torch.empty(self.lut_size + 1))
        self.init_lut(lut_method)

    def init_lut(self, method="minimax"):
        self.lut.copy_(pwl_table(inv_sqrt, 1.0, 2.0, self.lut_size, method, self.lut.dtype))
        self.lut_method = method

    def _rsqrt_pwl(self, v):
        m, e = torch.frexp(v)
        m = m * 2.0
        e = e - 1
        u = (m - 1.0) * self.lut_size
        idx = u.floor().long().clamp(0, self.lut_size - 1)
        frac = u - idx.to(v.dtype)
        f, g = self.lut[idx], self.lut[idx + 1]
        r = f + frac * (g - f)
        eh = torch.div(e, 2, rounding_mode="floor")
        scale = torch.ldexp(torch.ones_like(v), -eh)
        scale = torch.where(e % 2 != 0, scale * self.INV_SQRT2, scale)
        return r * scale

    def forward(self, x):
        dims, view = self._dims(x)
        if self.training:
            mean = x.mean(dim=dims)
            var = x.var(dim=dims, unbiased=False)
            with torch.no_grad():
                self.num_batches_tracked += 1
                self._track("running_mean", mean)
                self._track("running_var", var)
        else:
            mean, var = self.running_mean, self.running_var
        out = (x - mean.view(view)) * self._rsqrt_pwl(var + self.eps).view(view)
        return self._affine(out, view)
