"""Knot tables of the piecewise-linear approximations (PWL SiLU and the PWL
inverse square root of PWLBatchNorm).

A table holds the values at the n + 1 uniform knots x_0..x_n of [lo, hi]
(n segments) between which the kernels interpolate linearly. Three
constructions, as LoFloat defines them (LoFloat/layers.py:1089-1113 for SiLU,
:985-1006 for 1/sqrt):

  uniform   the function at the knots, T_i = f(x_i);
  midpoint  the end knots keep f, interior knot i takes f at the midpoint
            of the segment before it, T_i = f((x_(i-1) + x_i) / 2);
  minimax   with d_j = f(m_j) - (f(x_j) + f(x_(j+1))) / 2 the gap between
            the function and the chord at the middle m_j of segment j, each
            knot moves by the mean of the half-gaps of the segments that meet
            there: T_i = f(x_i) + (d_(i-1) + d_i) / 4 inside, and by half the
            gap of its only segment at the ends, so that every chord splits
            its segment's error evenly.

Everything is computed with torch in the table's dtype (float32 by default),
in an order whose every rounding matches LoFloat's, so the tables are the
same numbers as the reference layers'.
"""
from __future__ import annotations

from typing import Callable

import torch
import torch.nn.functional as F

METHODS = ("uniform", "midpoint", "minimax")


def pwl_table(f: Callable[[torch.Tensor], torch.Tensor], lo: float, hi: float, segments: int,
              method: str = "minimax", dtype: torch.dtype = torch.float32) -> torch.Tensor:
    """segments + 1 knot values of f over [lo, hi] by `method` (see above)."""
    if method not in METHODS:
        raise ValueError(f"Unknown lut_method {method!r}")
    x = torch.linspace(lo, hi, segments + 1, dtype=dtype)
    fx = f(x)
    if method == "uniform":
        return fx.clone()
    mid = (x[:-1] + x[1:]) * 0.5
    fm = f(mid)
    if method == "midpoint":
        # knot i (0 < i < n) moves to the value at the middle of segment i - 1
        return torch.cat([fx[:1], fm[:-1], fx[-1:]])
    gap = fm - (fx[:-1] + fx[1:]) * 0.5
    # interior knots: the two adjacent gaps over 4; the zero padding makes
    # the ends gap / 4, which doubles (exactly) to gap / 2
    corr = (F.pad(gap, (1, 0)) + F.pad(gap, (0, 1))) / 4
    corr[0] = corr[0] * 2
    corr[-1] = corr[-1] * 2
    return fx + corr


def silu(x: torch.Tensor) -> torch.Tensor:
    return x * torch.sigmoid(x)


def inv_sqrt(x: torch.Tensor) -> torch.Tensor:
    return 1.0 / x.sqrt()
