"""MX storage in one pass (lofgb_mx_encode_f32): element codes and E8M0 block
scales against the oracle's composition of the MX block loop and the storage
codec (orc_mx_encode_f32), byte for byte; and the decoded storage against the
MX rounding's output wherever the quotient is a value of the element format."""
import ctypes as C

import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from gpu_util import mx_matrix_data, from_gpu, to_gpu
from lofloat_gb300 import _native
from oracle import oracle as O

pytestmark = pytest.mark.gpu

E8M0_O = O.codec_fmt(8, 0, 127, True, False, False, 0, 0xFFFFFFFF, 0, 0, 0xFF, 0xFF, 0, False)


def _native_fmt(f):
    return _native.LofgbCodecFormat.from_buffer_copy(bytes(f))


def _gpu_mx_encode(x, ef, mode=0, sat=1, ln=0, seed=0, offset=0, skew=0):
    """through the C ABI; skew shifts the input and outputs off alignment"""
    n = x.size
    xt = torch.zeros(n + skew, device="cuda")
    xt[skew:] = to_gpu(x)
    cb = O.packed_size(ef.fmt.bitwidth, n)
    nb = (n + 31) // 32
    codes = torch.zeros(cb + skew, dtype=torch.uint8, device="cuda")
    scales = torch.zeros(nb + skew, dtype=torch.uint8, device="cuda")
    nf, sf = _native_fmt(ef), _native_fmt(E8M0_O)
    L = _native.lib()
    st = L.lofgb_mx_encode_f32(xt[skew:].data_ptr(), codes[skew:].data_ptr(), scales[skew:].data_ptr(),
                               n, 32, C.byref(nf), C.byref(sf), mode, 0, sat, ln, seed, offset,
                               torch.cuda.current_stream().cuda_stream)
    assert st == 0, L.lofgb_last_error_detail().decode()
    return from_gpu(codes[skew:]), from_gpu(scales[skew:])


FORMATS = [("e2m1", O.codec_p3109(4, 2)), ("fp6_e3m2", O.codec_p3109(6, 3)),
           ("fp6_e2m3", O.codec_p3109(6, 4)), ("e4m3", O.codec_p3109(8, 4)),
           ("e5m2", O.codec_p3109(8, 3))]


@pytest.mark.parametrize("name,ef", FORMATS)
@pytest.mark.parametrize("n", [32 * 4096, 32 * 77 + 13, 5, 128 * 3 + 31])
@pytest.mark.parametrize("sat", [0, 1])
def test_against_oracle(name, ef, n, sat):
    rng = np.random.default_rng(n + sat)
    x = (rng.standard_normal(n) * np.exp2(rng.integers(-8, 9, n))).astype(np.float32)
    x[rng.random(n) < 0.01] *= 4096.0
    if n > 64:
        x[32:64] = 0.0                      # an all-zero block: scale 0, codes of +0
    got_c, got_s = _gpu_mx_encode(x, ef, sat=sat)
    want_c, want_s = O.mx_encode(x, 32, ef, E8M0_O, sat=sat)
    assert np.array_equal(got_c, want_c), np.count_nonzero(got_c != want_c)
    assert np.array_equal(got_s, want_s)


SPECIAL_FORMATS = FORMATS + [("e4m3_unsigned", O.codec_p3109(8, 4, signed=False)),
                             ("fp6_unsigned", O.codec_p3109(6, 3, signed=False)),
                             ("e4m3_nonsat", O.codec_p3109(8, 4, saturating=False)),
                             ("e5m2_nonsat", O.codec_p3109(8, 3, saturating=False))]


@pytest.mark.parametrize("name,ef", SPECIAL_FORMATS)
@pytest.mark.parametrize("sat", [0, 1, 2])
def test_specials_signs_and_formats(name, ef, sat):
    """Infinities, NaNs of both signs and with payloads, -0 and overflowing
    values inside otherwise ordinary blocks; signed, unsigned and
    non-saturating element formats, every saturation mode. Saturating
    formats under RNE encode quotients without rounding them first except in
    warps that hold an infinity or NaN; the others round first."""
    rng = np.random.default_rng(len(name) * 7 + sat)
    n = 32 * 512 + 19
    x = (rng.standard_normal(n) * np.exp2(rng.integers(-10, 11, n))).astype(np.float32)
    specials = np.array([0x7F800000, 0xFF800000, 0x7FC00000, 0xFFC00000, 0x7F800001, 0xFFFFFFFF,
                         0x80000000, 0x7F7FFFFF, 0xFF7FFFFF], np.uint32).view(np.float32)
    idx = rng.choice(n, 60, replace=False)
    x[idx] = specials[rng.integers(0, specials.size, idx.size)]
    x[-7:] = -x[-7:]
    got_c, got_s = _gpu_mx_encode(x, ef, sat=sat)
    want_c, want_s = O.mx_encode(x, 32, ef, E8M0_O, sat=sat)
    assert np.array_equal(got_s, want_s)
    assert np.array_equal(got_c, want_c), np.count_nonzero(got_c != want_c)


@pytest.mark.parametrize("skew", [1, 2, 3])
@pytest.mark.parametrize("mode,ln", [(0, 0), (3, 8), (1, 0)])
def test_modes_and_misaligned_buffers(skew, mode, ln):
    ef = O.codec_p3109(8, 4)
    rng = np.random.default_rng(skew * 10 + mode)
    x = rng.standard_normal(32 * 300 + 7).astype(np.float32)
    got = _gpu_mx_encode(x, ef, mode=mode, ln=ln, seed=9, offset=33, skew=skew)
    want = O.mx_encode(x, 32, ef, E8M0_O, mode=mode, stoch_len=ln, seed=9, offset=33)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_mx_8192x8192_storage_against_oracle_and_mx_round():
    """The 8192 x 8192 matrix (N(0,1), 1 % outliers x 2^12): the GPU's element
    codes and E8M0 scales equal the oracle's byte for byte over the whole
    matrix; and decode(codes) * scale equals the MX-E4M3 rounding wherever
    the rounding's quotient is an E4M3 value (equal values: P3109 formats
    have no -0, their sign-only code being NaN, so -0 is stored as +0).
    Elsewhere — about 4 % of this matrix's quotients overflow E4M3 and pass
    through the rounding unrounded — storage holds the largest finite code
    (SatFinite): the decoded value is that code's value times the block
    scale, with the rounding's sign and a smaller magnitude."""
    x = mx_matrix_data()
    xg = to_gpu(x)
    e4m3, e8 = lg.create_p3109_params(8, 4), lg.create_e8m0_params()
    codes, scales = lg.mx_encode(xg, e4m3, e8)
    ef = O.codec_p3109(8, 4)
    want_c, want_s = O.mx_encode(x.reshape(-1), 32, ef, E8M0_O, sat=1)
    got_c, got_s = from_gpu(codes), from_gpu(scales)
    assert np.array_equal(got_s, want_s), np.count_nonzero(got_s != want_s)
    assert np.array_equal(got_c, want_c), np.count_nonzero(got_c != want_c)
    n = x.size
    q = O.decode(got_c, n, ef)
    sc = O.decode(got_s, n // 32, E8M0_O)
    back = (q * np.repeat(sc, 32)).reshape(-1, 32)
    ref = from_gpu(lg.virtual_mx_round(xg, 32, e4m3, e8)).reshape(-1, 32)
    every = O.decode(np.arange(256, dtype=np.uint8), 256, ef)
    top = np.float32(np.abs(every[np.isfinite(every)]).max())
    diff = back != ref
    assert diff.mean() < 0.06
    bd, rd = back[diff], ref[diff]
    assert np.array_equal(np.abs(bd), (top * np.repeat(sc, 32).reshape(-1, 32))[diff])
    assert np.all(np.abs(rd) > np.abs(bd)) and np.all(np.sign(rd) == np.sign(bd))


def _composed_decode(codes, scales, n, ef_desc, sf_desc):
    q = lg.lof_decode(codes, n, ef_desc)
    sc = lg.lof_decode(scales, (n + 31) // 32, sf_desc)
    return q.view(-1)[:n] * sc.repeat_interleave(32)[:n]


@pytest.mark.parametrize("bits,p,signed", [(4, 2, True), (6, 3, True), (6, 4, True), (8, 4, True),
                                           (8, 3, True), (8, 4, False), (6, 3, False)])
@pytest.mark.parametrize("n", [32 * 4096, 32 * 77 + 13, 5, 128 * 3 + 31, 1000])
def test_mx_decode_kernel_equals_composition(bits, p, signed, n):
    """lofgb_mx_decode_f32 (one kernel) against the two codec decodes and the
    FP32 product, bit for bit, on storage with specials and all-zero blocks."""
    rng = np.random.default_rng(bits * 100 + n)
    x = (rng.standard_normal(n) * np.exp2(rng.integers(-12, 13, n))).astype(np.float32)
    if n > 70:
        x[32:64] = 0.0
        x[rng.integers(0, n, 3)] = np.array([np.inf, np.nan, -np.inf], np.float32)
    ef = lg.create_p3109_params(bits, p, signed)
    e8 = lg.create_e8m0_params()
    codes, scales = lg.mx_encode(to_gpu(x), ef, e8)
    got = lg.mx_decode(codes, scales, n, ef, e8)
    want = _composed_decode(codes, scales, n, ef, e8)
    assert got.shape == (n,)
    assert np.array_equal(from_gpu(got).view(np.uint32), from_gpu(want).view(np.uint32)), \
        int((from_gpu(got).view(np.uint32) != from_gpu(want).view(np.uint32)).sum())


def test_mx_decode_argument_checks():
    L = _native.lib()
    ef, sf = _native_fmt(O.codec_p3109(8, 4)), _native_fmt(E8M0_O)
    c = torch.zeros(64, dtype=torch.uint8, device="cuda")
    s = torch.zeros(2, dtype=torch.uint8, device="cuda")
    d = torch.zeros(64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert L.lofgb_mx_decode_f32(c.data_ptr(), s.data_ptr(), d.data_ptr(), 64, 16, C.byref(ef),
                                 C.byref(sf), st) == -5
    assert L.lofgb_mx_decode_f32(c.data_ptr(), s.data_ptr(), d.data_ptr() + 4, 64, 32, C.byref(ef),
                                 C.byref(sf), st) == -2
    assert L.lofgb_mx_decode_f32(c.data_ptr(), s.data_ptr(), d.data_ptr(), 64, 32, C.byref(ef),
                                 C.byref(sf), st) == 0
