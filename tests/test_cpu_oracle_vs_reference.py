"""The oracle against the compiled reference, live, on fresh random inputs.

The committed golden vectors pin the oracle on fixed cases everywhere. Where
the reference sources are present, `oracle/build_oracle.py` also compiles the
reference's own scalar code into `oracle/_ref/libref_shim.so`; these tests
feed it and the oracle new seeded inputs (random bit patterns, so NaNs,
infinities, subnormals and overflow included) and require the same bits, for
every deterministic mode, on formats beyond the golden set (every P3109
<k,p> with k = 3..8, both overflow behaviours, signed and unsigned), for
f64 sources and every f16 bit pattern, and for the codec's bytes (modes,
saturation modes, both byte orders) and decoded values.
They skip where the shim is not built (no reference checkout).
"""
import ctypes as C

import numpy as np
import pytest

O = pytest.importorskip("oracle.oracle")

DETERMINISTIC = (0, 1, 2, 4, 5, 6, 7, 12, 13)


@pytest.fixture(scope="module")
def R():
    r = O.ref()
    if r is None:
        pytest.skip("reference shim not built (no reference checkout)")
    return r


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _bits_f32(n, seed):
    rng = np.random.default_rng(seed)
    b = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    x = b.view(np.float32).copy()
    # half of them in a range where most formats round rather than overflow
    k = n // 2
    x[:k] = (rng.standard_normal(k) * np.exp2(rng.integers(-30, 30, k))).astype(np.float32)
    return x


FORMATS = [(k, p - 1, 1 << (k - p - 1), sat, signed)
           for k in range(3, 9) for p in range(1, k) for sat in (True, False)
           for signed in (True, False) if not (signed and k - (p - 1) - 1 < 1)]


@pytest.mark.parametrize("f", FORMATS, ids=lambda f: "k%d_m%d_b%d_%s_%s" % (
    f[0], f[1], f[2], "sat" if f[3] else "ext", "s" if f[4] else "u"))
def test_format_rounding_matches_reference(R, f):
    x = _bits_f32(4096, hash(f) & 0xFFFF)
    of = O.fmt(f[0], f[1], f[2], saturating=f[3], signed=f[4])
    for mode in DETERMINISTIC:
        y = np.empty_like(x)
        R.ref_round_f32(_p(x), _p(y), x.size, f[0], f[1], f[2], int(f[3]), 0,
                        0 if f[4] else 1, mode, 0, None, None, None)
        got = O.round(x, of, mode)
        same = (got.view(np.uint32) == y.view(np.uint32)) | (np.isnan(got) & np.isnan(y))
        assert np.all(same), (f, mode, x[~same][:4], got[~same][:4], y[~same][:4])


@pytest.mark.parametrize("mbits", [0, 1, 3, 7, 10, 15, 22])
def test_mantissa_rounding_matches_reference(R, mbits):
    x = _bits_f32(1 << 14, 1000 + mbits)
    for mode in DETERMINISTIC:
        y = np.empty_like(x)
        R.ref_round_mantissa_f32(_p(x), _p(y), x.size, mbits, mode, 0, None, None, None)
        got = O.round_mantissa(x, mbits, mode)
        assert np.array_equal(got.view(np.uint32), y.view(np.uint32)), (mbits, mode)


@pytest.mark.parametrize("block", [8, 32, 128])
def test_mx_matches_reference(R, block):
    rng = np.random.default_rng(block)
    n = 5003
    x = (rng.standard_normal(n) * np.exp2(rng.integers(-12, 12, n))).astype(np.float32)
    for ef in ((8, 3, 7), (8, 2, 15), (4, 1, 1), (6, 2, 3)):
        for mode in (0, 1, 5, 6):
            y = np.empty_like(x)
            R.ref_mx_round_f32(_p(x), _p(y), n, block, ef[0], ef[1], ef[2], 1, 0,
                               8, 0, 127, 0, 1, mode, 0, 0)
            got = O.mx_round(x, block, O.fmt(*ef), O.fmt(8, 0, 127, saturating=False,
                                                          signed=False), mode=mode)
            assert np.array_equal(got.view(np.uint32), y.view(np.uint32)), (ef, mode)


@pytest.mark.parametrize("mbits", [3, 7, 10, 15])
def test_gemm_matches_reference(R, mbits):
    rng = np.random.default_rng(mbits)
    M, N, K = 24, 20, 70
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    D = np.empty((M, N), np.float32)
    R.ref_gemm_f32(_p(A), _p(B), _p(D), M, N, K, mbits, C.c_float(0.5))
    assert np.array_equal(O.gemm(A, B, mbits, alpha=0.5).view(np.uint32), D.view(np.uint32))


F64_FORMATS = [(8, 3, 7, True, True), (16, 10, 15, False, True), (16, 7, 127, True, True),
               (32, 23, 127, False, True), (40, 30, 255, True, True), (8, 2, 16, False, False)]


@pytest.mark.parametrize("f", F64_FORMATS, ids=str)
def test_f64_format_rounding_matches_reference(R, f):
    rng = np.random.default_rng(f[0] * 100 + f[1])
    n = 4096
    x = rng.integers(0, 1 << 64, n, dtype=np.uint64).view(np.float64).copy()
    x[: n // 2] = rng.standard_normal(n // 2) * np.exp2(rng.integers(-300, 300, n // 2))
    of = O.fmt(f[0], f[1], f[2], saturating=f[3], signed=f[4])
    for mode in DETERMINISTIC:
        y = np.empty_like(x)
        R.ref_round_f64(_p(x), _p(y), n, f[0], f[1], f[2], int(f[3]), 0, 0 if f[4] else 1,
                        mode, 0, None, None, None)
        got = O.round(x, of, mode)
        same = (got.view(np.uint64) == y.view(np.uint64)) | (np.isnan(got) & np.isnan(y))
        assert np.all(same), (f, mode)


@pytest.mark.parametrize("t,mbits", [("f64", m) for m in (0, 10, 30, 51)] +
                         [("f16", m) for m in (0, 2, 5, 9)])
def test_f64_f16_mantissa_rounding_matches_reference(R, t, mbits):
    rng = np.random.default_rng(mbits)
    if t == "f64":
        x = rng.integers(0, 1 << 64, 1 << 13, dtype=np.uint64).view(np.float64).copy()
        view = np.uint64
    else:
        x = np.arange(1 << 16, dtype=np.uint16)  # every f16 bit pattern
        view = np.uint16
    for mode in DETERMINISTIC:
        y = np.empty_like(x)
        getattr(R, f"ref_round_mantissa_{t}")(_p(x), _p(y), x.size, mbits, mode, 0,
                                              None, None, None)
        got = O.round_mantissa(x, mbits, mode)
        assert np.array_equal(got.view(view), y.view(view)), (t, mbits, mode)


@pytest.mark.parametrize("k,p,sat", [(k, p, s) for k in range(3, 9) for p in range(1, k)
                                     for s in (True, False)])
def test_codec_matches_reference(R, k, p, sat):
    f = O.codec_p3109(k, p, saturating=sat)
    cf = O.codec_fields(f)
    rng = np.random.default_rng(k * 10 + p)
    x = _bits_f32(1001, k * 10 + p)
    x[:500] = (rng.standard_normal(500) * np.exp2(rng.integers(-12, 12, 500))).astype(np.float32)
    size = int(R.ref_packed_size(k, x.size))
    assert size == O.packed_size(k, x.size)
    for mode in (0, 1, 5, 6, 12):
        for s in (0, 1, 2):
            for rev in (0, 1):
                buf = np.zeros(size, np.uint8)
                R.ref_encode_f32(_p(buf), _p(x), x.size, _p(cf), mode, s, 0, rev)
                assert np.array_equal(O.encode(x, f, mode=mode, sat=s, reverse=rev), buf), \
                    (mode, s, rev)
    raw = rng.integers(0, 256, size, dtype=np.uint8)
    for rev in (0, 1):
        dec = np.empty(x.size, np.float32)
        R.ref_decode_f32(_p(dec), _p(raw), x.size, _p(cf), rev)
        got = O.decode(raw, x.size, f, reverse=rev)
        same = (got.view(np.uint32) == dec.view(np.uint32)) | (np.isnan(got) & np.isnan(dec))
        assert np.all(same), rev


STOCH = (3, 8, 9, 10, 11, 14)
LEN_MODES = (3, 8, 9, 14)


@pytest.mark.parametrize("f", [(8, 3, 7, True, True), (8, 2, 15, True, True),
                               (6, 2, 3, False, True), (16, 10, 15, False, True),
                               (16, 7, 127, False, True)], ids=str)
def test_stochastic_formulas_match_reference(R, f):
    """The reference's host stochastic rounding re-seeds its generator per
    call, so the shim seeds it per element and reports the draw each element
    consumed; fed those same bits, the oracle must give the same results."""
    rng = np.random.default_rng(f[0] * 7 + f[1])
    n = 4096
    x = (rng.standard_normal(n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    of = O.fmt(f[0], f[1], f[2], saturating=f[3], signed=f[4])
    for mode in STOCH:
        ln = min(8, 23 - f[1]) if mode in LEN_MODES else 0
        seeds = rng.integers(1, 2 ** 32 - 1, n, dtype=np.uint32)
        rb = np.zeros(n, np.uint64)
        us = np.zeros(n, np.float64)
        y = np.empty_like(x)
        R.ref_round_f32(_p(x), _p(y), n, f[0], f[1], f[2], int(f[3]), 0, 0 if f[4] else 1,
                        mode, ln, _p(seeds), _p(rb), _p(us))
        assert rb.any() or us.any()  # the draws were recorded
        got = O.round_bits(x, of, mode, ln, rbits=rb, usamp=us)
        assert np.array_equal(got.view(np.uint32), y.view(np.uint32)), (f, mode)
