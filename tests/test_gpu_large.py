"""Maximum sizes: more than 2^31 elements through the rounding and MX entry
points (64-bit indexing end to end), checked on sampled positions against
the oracle — the head, the tail across the 2^31 boundary, and random
positions."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import same_bits
from oracle import oracle as O

pytestmark = pytest.mark.gpu

N = (1 << 31) + 4099  # not a multiple of the vector width or of a warp tile


def _sample_idx(n, rng):
    return np.unique(np.concatenate([np.arange(0, 4096), np.arange((1 << 31) - 4096, n),
                                     rng.integers(0, n, 8192)]))


@pytest.fixture(scope="module")
def big():
    g = torch.Generator(device="cuda").manual_seed(11)
    x = torch.randn(N, device="cuda", generator=g)
    x.mul_(torch.exp2(torch.randint(-20, 21, (N,), device="cuda", generator=g, dtype=torch.int8).float()))
    yield x
    del x
    torch.cuda.empty_cache()


@pytest.mark.parametrize("mode,ln", [(0, 0), (3, 8), (12, 0)])
def test_round_beyond_2_31(big, mode, ln):
    e4m3 = lg.create_p3109_params(8, 4)
    y = lg.virtual_round(big, e4m3, round_mode=mode, stoch_len=ln, seed=5, offset=7)
    idx = _sample_idx(N, np.random.default_rng(mode))
    it = torch.from_numpy(idx).cuda()
    xs = big[it].cpu().numpy()
    got = y[it].cpu().numpy()
    del y
    f = O.fmt(8, 3, 8)
    # stochastic modes draw R from (seed, offset + global index): the oracle
    # rounds each sampled element with its own index's random lane
    if mode == 3:
        lgl = O.rng_lanes_log2(mode, ln)
        rbits = np.array([O.rng_elem(5, 7 + int(i), lgl) for i in idx], np.uint64)
        want = O.round_bits(xs, f, mode, ln, rbits=rbits)
    else:
        want = O.round(xs, f, mode, ln)
    assert same_bits(got, want)


def test_mx_beyond_2_31(big):
    e4m3 = lg.create_p3109_params(8, 4)
    e8 = lg.create_e8m0_params()
    n = N - (N % 32) + 16  # a ragged last block
    x = big[:n]
    y = lg.virtual_mx_round(x, 32, e4m3, e8)
    rng = np.random.default_rng(1)
    blocks = np.unique(np.concatenate([np.arange(0, 64), np.arange(n // 32 - 64, (n + 31) // 32),
                                       rng.integers(0, n // 32, 512)]))
    ef, sf = O.fmt(8, 3, 8), O.fmt(8, 0, 127, saturating=False, signed=False)
    for b in blocks:
        lo, hi = int(b) * 32, min(int(b) * 32 + 32, n)
        xs = x[lo:hi].cpu().numpy()
        want = O.mx_round(xs, 32, ef, sf)
        assert same_bits(y[lo:hi].cpu().numpy(), want), b
    del y


def test_codec_beyond_2_31(big):
    """8-bit codes: byte i is element i's code, so sampled bytes check directly."""
    e4m3 = lg.create_p3109_params(8, 4)
    packed = lg.lof_encode(big, e4m3)
    assert packed.numel() == N
    idx = _sample_idx(N, np.random.default_rng(2))
    it = torch.from_numpy(idx).cuda()
    xs = big[it].cpu().numpy()
    got = packed[it].cpu().numpy()
    f = O.codec_p3109(8, 4)
    want = np.array([O.encode_rep(float(v), f) for v in xs], np.uint32).astype(np.uint8)
    assert np.array_equal(got, want)
    back = lg.lof_decode(packed, N, e4m3)
    del packed
    assert same_bits(back[it].cpu().numpy(), O.decode(want, want.size, f))
    del back
