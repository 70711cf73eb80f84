"""The reference's STE quantisation helpers (LoFloat/layers.py:106-119):
forward = virtual_round into the P3109 format they build, backward = the
identity."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import same_bits
from gpu_util import from_gpu, ofmt
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_mantissa_and_exp_mant_quantize():
    rng = np.random.default_rng(4)
    x = (rng.standard_normal(5000) * 2.0 ** rng.integers(-30, 31, 5000)).astype(np.float32)
    xg = torch.from_numpy(x).cuda().requires_grad_(True)
    y = lg.mantissa_quantize(xg, 10)
    want = O.round(x, ofmt(lg.create_p3109_params(19, 11, True, True)), 0)
    assert same_bits(from_gpu(y.detach()), want)
    y.sum().backward()
    assert torch.all(xg.grad == 1)
    z = lg.exp_mant_quantize(xg.detach(), 4, 3)
    assert same_bits(from_gpu(z), O.round(x, ofmt(lg.create_p3109_params(8, 4, True, True)), 0))
    assert lg.mantissa_quantize(xg, None) is xg and lg.exp_mant_quantize(xg, None, 3) is xg


def test_owner_quantize_uses_rounding_mode():
    class Owner:
        rounding_mode = lg.RoundingMode.RoundTowardsZero

    x = torch.randn(4096, device="cuda") * 7
    p = lg.create_p3109_params(8, 4)
    got = lg._quantize(Owner(), x, p)
    want = lg.virtual_round(x, p, round_mode=lg.RoundingMode.RoundTowardsZero)
    assert torch.equal(got.view(torch.int32), want.view(torch.int32))
    assert lg._quantize(Owner(), x, None) is x
