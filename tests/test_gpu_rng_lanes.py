"""The random stream of the stochastic modes on the GPU: element g reads lane
g mod 2^lg of SplitMix64 output g >> lg, with lanes of 8, 16, 32 or 64 bits
by what the mode reads. Every lane width, unaligned stream offsets, every
source type, MX elements and codec encodes agree bit for bit with the oracle,
and a stream split at any point reproduces the single call."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import same_bits
from gpu_util import from_gpu, ofmt, to_gpu
from oracle import oracle as O
from test_gpu_codec import gpu_encode

pytestmark = pytest.mark.gpu

SR_A, SR_B, SR_C, TRUE_SR, PROB, SR_D = 3, 8, 9, 10, 11, 14


def _desc(bw, m, bias):
    return lg.FloatFormatDescriptor(bw, m, bias, lg.InfBehavior.Saturating, lg.NaNBehavior._3109,
                                    lg.Signedness.Signed, lg.formats.P3109_InfChecker(bw),
                                    lg.formats.P3109_NaNChecker(bw))


def _x(n, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(n) * 2.0 ** rng.integers(-6, 7, n)).astype(dtype)


@pytest.mark.parametrize("mode,ln", [(SR_A, 1), (SR_A, 8), (SR_A, 12), (SR_A, 16), (SR_A, 20),
                                     (SR_A, 31), (SR_A, 32), (SR_A, 40), (SR_B, 8), (SR_B, 13),
                                     (SR_C, 8), (SR_C, 24), (SR_D, 7), (SR_D, 8), (SR_D, 16),
                                     (SR_D, 31), (PROB, 0), (TRUE_SR, 0)])
@pytest.mark.parametrize("offset", [0, 1, 2, 3, 6, 1 << 33])
def test_f32_lanes_vs_oracle(mode, ln, offset):
    assert O.rng_lanes_log2(mode, ln) in (0, 1, 2, 3)
    desc = _desc(8, 3, 7)
    x = _x(4099, mode * 100 + ln)
    got = from_gpu(lg.virtual_round(to_gpu(x), desc, round_mode=mode, stoch_len=ln, seed=17,
                                    offset=offset))
    want = O.round(x, ofmt(desc), mode, ln, seed=17, offset=offset)
    assert same_bits(got, want)


@pytest.mark.parametrize("mode,ln", [(SR_A, 8), (SR_A, 30), (SR_A, 45), (SR_D, 20), (TRUE_SR, 0)])
@pytest.mark.parametrize("offset", [0, 3])
def test_f64_f16_lanes_vs_oracle(mode, ln, offset):
    desc = _desc(8, 3, 7)
    x64 = _x(2051, ln, np.float64)
    got = from_gpu(lg.virtual_round(to_gpu(x64), desc, round_mode=mode, stoch_len=ln, seed=5,
                                    offset=offset))
    assert same_bits(got, O.round(x64, ofmt(desc), mode, ln, seed=5, offset=offset))
    if ln <= 10:
        x16 = _x(2051, ln + 1, np.float16)
        h = lg.virtual_round(torch.from_numpy(x16).cuda(), desc, round_mode=mode, stoch_len=ln,
                             seed=5, offset=offset).cpu().numpy()
        want = O.round(x16.view(np.uint16), ofmt(desc), mode, ln, seed=5, offset=offset)
        assert np.array_equal(h.view(np.uint16), want)


@pytest.mark.parametrize("mode,ln", [(SR_A, 8), (SR_A, 12), (SR_A, 20), (SR_D, 8)])
def test_split_stream_equals_one_call(mode, ln):
    desc = _desc(8, 3, 7)
    x = _x(10_000, 3)
    xg = to_gpu(x)
    full = from_gpu(lg.virtual_round(xg, desc, round_mode=mode, stoch_len=ln, seed=9, offset=0))
    cuts = [0, 1, 3, 6, 10, 17, 4099, 10_000]
    parts = [from_gpu(lg.virtual_round(xg[a:b].clone(), desc, round_mode=mode, stoch_len=ln,
                                       seed=9, offset=a)) for a, b in zip(cuts, cuts[1:])]
    assert same_bits(full, np.concatenate(parts))


@pytest.mark.parametrize("ln,offset", [(8, 0), (8, 5), (12, 2), (20, 0)])
def test_mx_elements_lanes_vs_oracle(ln, offset):
    e4m3, e8 = lg.create_p3109_params(8, 4), lg.create_e8m0_params()
    x = _x(64 * 96, ln).reshape(64, 96)
    got = from_gpu(lg.virtual_mx_round(to_gpu(x), 32, e4m3, e8, round_mode=SR_A, stoch_len=ln,
                                       seed=21, offset=offset))
    ef, sf = O.fmt(8, 3, 8), O.fmt(8, 0, 127, saturating=False, signed=False)
    want = O.mx_round(x.reshape(-1), 32, ef, sf, mode=SR_A, stoch_len=ln, seed=21,
                      offset=offset).reshape(64, 96)
    assert same_bits(got, want)


@pytest.mark.parametrize("ln,offset", [(8, 0), (8, 7), (16, 1)])
def test_codec_encode_lanes_vs_oracle(ln, offset):
    f = O.codec_p3109(8, 4)
    x = _x(5000, ln)
    got = gpu_encode(x, f, mode=SR_A, stoch_len=ln, seed=13, offset=offset)
    want = O.encode(x, f, mode=SR_A, stoch_len=ln, seed=13, offset=offset)
    assert np.array_equal(got, want)
