"""Streaming kernels are launched with programmatic dependent launch: each
waits for the previous kernel in the stream before touching memory. Chains
of back-to-back in-place launches (each reading what the one before wrote)
must give the results of running the steps one at a time."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import same_bits
from gpu_util import from_gpu, ofmt
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _x(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(n) * 2.0 ** rng.integers(-12, 13, n)).astype(np.float32)


def test_in_place_round_chain():
    fmts = [lg.create_p3109_params(8, 4), lg.create_p3109_params(8, 3), lg.create_p3109_params(6, 3),
            lg.create_half_params()]
    x = _x((1 << 22) + 3, 1)
    y = torch.from_numpy(x).cuda()
    for i in range(12):                      # no synchronisation inside the chain
        lg.virtual_round(y, fmts[i % 4], round_mode=(0, 3)[i % 2], stoch_len=6, seed=i, offset=0, out=y)
    got = from_gpu(y)
    want = x.copy()
    for i in range(12):
        want = O.round(want, ofmt(fmts[i % 4]), (0, 3)[i % 2], 6, seed=i, offset=0)
    assert same_bits(got, want)


def test_mx_then_round_then_codec_chain():
    e4m3, e8 = lg.create_p3109_params(8, 4), lg.create_e8m0_params()
    x = _x(1 << 21, 2).reshape(1024, 2048)
    xg = torch.from_numpy(x).cuda()
    a = lg.virtual_mx_round(xg, 32, e4m3, e8)
    lg.virtual_round(a, 5, out=a)            # in place, right behind the MX kernel
    packed = lg.lof_encode(a, e4m3)
    back = lg.lof_decode(packed, a.numel(), e4m3).reshape(a.shape)
    lg.virtual_mx_round(back, 32, e4m3, e8, out=back)
    ef, sf = O.fmt(8, 3, 8), O.fmt(8, 0, 127, saturating=False, signed=False)
    w = O.mx_round(x.reshape(-1), 32, ef, sf)
    w = O.round_mantissa(w, 5, 0)
    f = O.codec_p3109(8, 4)
    w = O.decode(O.encode(w, f), w.size, f)
    w = O.mx_round(w, 32, ef, sf)
    assert same_bits(from_gpu(back).reshape(-1), w)
