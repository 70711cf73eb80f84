"""The BatchNorm approximations (LoFloat/layers.py:805-1047) are torch
compositions in the reference and here; checked on CPU against the formulas
they implement."""
import math

import torch

import lofloat_gb300 as lg


def _x():
    g = torch.Generator().manual_seed(0)
    return torch.randn(16, 6, 5, 5, generator=g) * 3 + 1


def test_l1_and_linf_normalise_by_deviation():
    x = _x()
    for cls, stat in ((lg.L1BatchNorm, lambda d: d.abs().mean(dim=(0, 2, 3))),
                      (lg.LinfBatchNorm, lambda d: d.abs().amax(dim=(0, 2, 3)))):
        bn = cls(6)
        y = bn(x)
        mean = x.mean(dim=(0, 2, 3))
        d = x - mean.view(1, -1, 1, 1)
        want = d / (stat(d).view(1, -1, 1, 1) + bn.eps) * bn.scale.view(1, -1, 1, 1)
        assert torch.allclose(y, want, rtol=1e-6, atol=1e-6)
        assert torch.allclose(bn.running_mean, 0.1 * mean, rtol=1e-5, atol=1e-6)
        bn.eval()
        y2 = bn(x)
        assert y2.shape == x.shape
    assert abs(lg.L1BatchNorm(3).scale[0].item() - math.sqrt(2 / math.pi)) < 1e-7


def test_fisr_and_pwl_rsqrt_accuracy():
    v = torch.logspace(-6, 6, 2001)
    fisr = lg.FISRBatchNorm._fast_rsqrt(v)
    assert ((fisr * v.sqrt() - 1).abs().max() < 1e-5)
    pwl = lg.PWLBatchNorm(4, lut_bits=6)
    r = pwl._rsqrt_pwl(v)
    assert ((r * v.sqrt() - 1).abs().max() < 2e-4)
    # the "midpoint" table shifts interior knots to segment midpoints, a coarser fit
    for method, tol in (("uniform", 1e-3), ("midpoint", 2e-2), ("minimax", 1e-3)):
        p = lg.PWLBatchNorm(4, lut_bits=4, lut_method=method)
        assert ((p._rsqrt_pwl(v) * v.sqrt() - 1).abs().max() < tol)


def test_variance_variants_match_batchnorm():
    x = _x()
    ref = torch.nn.BatchNorm2d(6, affine=False)
    want = ref(x)
    for cls in (lg.FISRBatchNorm, lg.PWLBatchNorm):
        bn = cls(6, affine=False)
        y = bn(x)
        assert (y - want).abs().max() < 5e-3 * want.abs().max()
        assert int(bn.num_batches_tracked) == 1
