"""Properties of the oracle, as the reference's own test programs check them.

The golden vectors pin the oracle to the compiled reference on fixed cases;
these tests check the properties that the reference's tests assert on random
and constructed inputs, with expectations built independently here from the
bit pattern (truncate, step one grid point):

* `test/test_virtual_round.cu:178-227`: directed modes are one-sided and
  within one grid step; nearest modes are within half a step
  (inputs u·2^[-20,20] as `rnd32_wide`, `:93-98`; mantissa widths 7/10/15,
  `:687-689`);
* `:233-307`: exact ties go to even (RNE), to odd (RNO), away from zero (RTA);
* `:312-360`: stochastic modes with len 8 give RD or RU;
* `test/test_prob_round.cpp`: P(up) within 0.02 of its expectation;
* `test/test_virtual_mx_round_cuda.cu:155-172`: an all-zero block gives 0,
  not NaN; `:94`: lengths with a trailing partial block;
* `test/test_mx_round_py.py:33-38`: exactly representable blocks come back
  unchanged;
* `test/test_virtual_mx_round.cpp` (P3109 <l,p> sweep, l = 2..8): the block
  scale is the nearer E8M0 power of two of amax/pmn, and every element over
  that scale is the element format's rounding of x/scale;
* `test/test_blis_lof_accum.cpp:126-235`: the emulated GEMM within
  γ_K·|A||B| of the FP64 product, measurably less accurate than FP32, and
  exact where every partial sum is representable;
* `test/test_pack.cpp`: packed byte counts from an lcm formula, every code of
  the small P3109 formats round-tripping through the packed form in both
  byte orders with a partial group, and float round trips equal to the
  format's rounding;
* `test/test_sat_mode.cpp:70-140`: the codec's three saturation modes on
  over-range and infinite inputs;
* `test/test_rounding_modes.cpp` (P3109 formats, down into the subnormals):
  format rounding lands on the codec's decoded grid, RD/RU bracket x with
  no grid value between them, and tiny values round away to denorm_min;
* `test/stoch_expect_test.cpp`: stochastic rounding unbiased in the mean;
* the PWL SiLU kernel's definition (`src/Lof_kernel.cu:231-257`; the
  reference has no test of it): relu outside [-R, R], the table at the knots,
  linear interpolation between them.
"""
import numpy as np
import pytest

O = pytest.importorskip("oracle.oracle")

RNE, RTZ, RAFZ, SRA, RNO, RD, RU, RTA, SRB, SRC, TSR, PROB, RTO, RTTZ, SRD = range(15)


def wide_inputs(n, seed):
    """u·2^e with u uniform in [1, 2) (random sign) and e in [-20, 20]."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(1.0, 2.0, n) * rng.choice([-1.0, 1.0], n)
    return (u * np.exp2(rng.integers(-20, 21, n))).astype(np.float32)


def neighbours(x, mbits):
    """(toward-zero, away-from-zero) grid neighbours at `mbits` fraction bits,
    as f32, and whether x is already on the grid."""
    b = x.view(np.uint32)
    sign = b & np.uint32(0x80000000)
    mag = b & np.uint32(0x7FFFFFFF)
    step = np.uint32(1 << (23 - mbits))
    tz = mag & ~np.uint32(step - 1)
    exact = tz == mag
    az = np.where(exact, tz, tz + step)
    return (tz | sign).view(np.float32), (az | sign).view(np.float32), exact


def kept_lsb(y, mbits):
    return (y.view(np.uint32) >> np.uint32(23 - mbits)) & np.uint32(1)


@pytest.mark.parametrize("mbits", [7, 10, 15])
def test_directed_and_nearest_bounds(mbits):
    x = wide_inputs(1 << 16, 100 + mbits)
    tz, az, exact = neighbours(x, mbits)
    neg = x < 0
    rd = np.where(neg, az, tz)
    ru = np.where(neg, tz, az)
    eq = lambda a, b: np.array_equal(a.view(np.uint32), b.view(np.uint32))  # noqa: E731
    assert eq(O.round_mantissa(x, mbits, RTZ), tz)
    assert eq(O.round_mantissa(x, mbits, RAFZ), az)
    assert eq(O.round_mantissa(x, mbits, RD), rd)
    assert eq(O.round_mantissa(x, mbits, RU), ru)
    # round to odd: exact stays, otherwise the neighbour with the odd last bit
    rto = np.where(exact, x, np.where(kept_lsb(tz, mbits) == 1, tz, az))
    assert eq(O.round_mantissa(x, mbits, RTO), rto)
    # nearest modes: within half a step, and the nearer neighbour off ties
    x64 = x.astype(np.float64)
    dz, da = np.abs(x64 - tz), np.abs(az.astype(np.float64) - x64)
    half = (az.astype(np.float64) - tz.astype(np.float64)) / 2
    for mode in (RNE, RNO, RTA, RTTZ):
        y = O.round_mantissa(x, mbits, mode)
        assert np.all(np.abs(y.astype(np.float64) - x64) <= np.abs(half) + 0.0)
        off_tie = dz != da
        nearer = np.where(dz < da, tz, az)
        assert eq(y[off_tie], nearer[off_tie]), mode


@pytest.mark.parametrize("mbits", [7, 10, 15])
def test_exact_ties(mbits):
    rng = np.random.default_rng(7 + mbits)
    n = 4096
    exp = rng.integers(100, 160, n).astype(np.uint32)
    frac = rng.integers(0, 1 << mbits, n).astype(np.uint32)
    drop = 23 - mbits
    # kept bits, then exactly half a step below them: a tie
    bits = (exp << np.uint32(23)) | (frac << np.uint32(drop)) | np.uint32(1 << (drop - 1))
    bits |= rng.choice(np.array([0, 0x80000000], np.uint32), n)
    x = bits.view(np.float32)
    tz, az, _ = neighbours(x, mbits)
    eq = lambda a, b: np.array_equal(a.view(np.uint32), b.view(np.uint32))  # noqa: E731
    even = np.where(kept_lsb(tz, mbits) == 0, tz, az)
    odd = np.where(kept_lsb(tz, mbits) == 1, tz, az)
    assert eq(O.round_mantissa(x, mbits, RNE), even)
    assert eq(O.round_mantissa(x, mbits, RNO), odd)
    assert eq(O.round_mantissa(x, mbits, RTA), az)
    assert eq(O.round_mantissa(x, mbits, RTTZ), tz)


@pytest.mark.parametrize("mode", [SRA, SRB, SRC, SRD, TSR, PROB])
def test_stochastic_gives_a_neighbour(mode):
    mbits = 10
    x = wide_inputs(1 << 15, 31)
    tz, az, exact = neighbours(x, mbits)
    y = O.round_mantissa(x, mbits, mode, stoch_len=8, seed=5)
    yb, tb, ab = (v.view(np.uint32) for v in (y, tz, az))
    inexact = ~exact
    assert np.all((yb[inexact] == tb[inexact]) | (yb[inexact] == ab[inexact]))
    if mode in (SRA, SRB, TSR, PROB):
        assert np.array_equal(yb[exact], x.view(np.uint32)[exact])


@pytest.mark.parametrize("mode", [SRA, TSR])
def test_probability_of_rounding_up(mode):
    # 1.0 plus five 10-bit steps plus a tail of 80/256 of a step (13 dropped bits)
    mbits, n = 10, 200_000
    b = np.uint32(0x3F800000 + 5 * (1 << 13) + (80 << 5))
    x = np.full(n, b, np.uint32).view(np.float32)
    tz, az, _ = neighbours(x, mbits)
    y = O.round_mantissa(x, mbits, mode, stoch_len=8, seed=123)
    up = np.mean(y.view(np.uint32) == az.view(np.uint32))
    assert np.all((y == tz) | (y == az))
    assert abs(up - 80 / 256) < 0.02


E4M3 = (8, 3, 7)
E8M0 = dict(saturating=False, signed=False)


def test_mx_all_zero_block_is_zero():
    x = np.zeros(96, np.float32)
    x[32:64] = np.linspace(-3, 3, 32, dtype=np.float32)
    y = O.mx_round(x, 32, O.fmt(*E4M3), O.fmt(8, 0, 127, **E8M0))
    assert not np.any(np.isnan(y))
    assert np.all(y[:32].view(np.uint32) == 0) and np.all(y[64:].view(np.uint32) == 0)


@pytest.mark.parametrize("block", [8, 16, 32, 64, 128, 256])
def test_mx_trailing_partial_block_equals_zero_padding(block):
    ef, sf = O.fmt(*E4M3), O.fmt(8, 0, 127, **E8M0)
    rng = np.random.default_rng(block)
    for n in (block, 3 * block, 3 * block + 1, 1000, 4096, 5003):
        x = rng.standard_normal(n).astype(np.float32)
        pad = -(-n // block) * block
        xp = np.zeros(pad, np.float32)
        xp[:n] = x
        y = O.mx_round(x, block, ef, sf)
        yp = O.mx_round(xp, block, ef, sf)
        assert np.array_equal(y.view(np.uint32), yp[:n].view(np.uint32)), n


def test_mx_representable_blocks_round_trip():
    # E4M3 (8,3,7) grid values, each block holding the format's largest value
    # 1.875·2^8 scaled by a power of two, so that the E8M0 scale is exact
    ef, sf = O.fmt(*E4M3), O.fmt(8, 0, 127, **E8M0)
    rng = np.random.default_rng(3)
    nblk, block = 64, 32
    m = rng.integers(0, 8, (nblk, block))
    e = rng.integers(-6, 9, (nblk, block))
    m[e == 8] = np.minimum(m[e == 8], 7)
    v = (1 + m / 8.0) * np.exp2(e) * rng.choice([-1.0, 1.0], (nblk, block))
    v[:, 0] = 1.875 * 256.0
    k = rng.integers(-20, 21, (nblk, 1))
    x = (v * np.exp2(k)).astype(np.float32).reshape(-1)
    for mode in (RNE, RTZ, RD, RU):
        y = O.mx_round(x, block, ef, sf, mode=mode)
        assert np.array_equal(y.view(np.uint32), x.view(np.uint32)), mode


def _nearer_pow2(q):
    """The nearer of the two powers of two around q > 0 (None on an exact tie)."""
    lo = np.float32(2.0) ** np.floor(np.log2(np.float64(q)))
    lo = np.float32(lo)
    if q == lo:
        return lo
    hi = np.float32(lo * 2)
    if q - lo == hi - q:
        return None
    return lo if q - lo < hi - q else hi


@pytest.mark.parametrize("l", range(2, 9))
def test_mx_p3109_sweep_scale_and_elements(l):
    """test/test_virtual_mx_round.cpp's P3109 <l,p> sweep (l = 2..8,
    p = 1..l-1): the block scale is the nearer E8M0 power of two of
    amax·(1/pmn), and each element, divided by that scale, is the element
    format's own rounding of x/scale."""
    sf = O.fmt(8, 0, 127, **E8M0)
    rng = np.random.default_rng(40 + l)
    nblk, block = 16, 32
    x = (rng.standard_normal((nblk, block))
         * np.exp2(rng.integers(-8, 9, (nblk, 1)))).astype(np.float32)
    for p in range(1, l):
        bias = 1 << (l - p - 1)
        ef = O.fmt(l, p - 1, bias)
        me = (1 << (l - (p - 1) - 1)) - 1 - bias
        pmn = np.float32(np.ldexp(1.0, me) * (2.0 - np.ldexp(1.0, -(p - 1))))
        inv = np.float32(1.0) / pmn
        for mode in (RNE, RTZ, RD, RU, RAFZ):
            y = O.mx_round(x.reshape(-1), block, ef, sf, mode=mode).reshape(nblk, block)
            for b in range(nblk):
                amax = np.float32(np.max(np.abs(x[b])))
                s = _nearer_pow2(np.float32(amax * inv))
                if s is None:
                    continue
                z = O.round((x[b] / s).astype(np.float32), ef, mode)
                got = (y[b] / s).astype(np.float32)
                assert np.array_equal(got.view(np.uint32), z.view(np.uint32)), (l, p, mode, b)


def test_gemm_accumulation_bound_grid_and_exact_case():
    """test/test_blis_lof_accum.cpp on the emulated GEMM: error within
    γ_K·|A||B| of the FP64 product with a 10-bit accumulator (part 1); the
    low-precision accumulator is engaged, far less accurate than FP32 and
    every output on its grid (part 2); products whose partial sums are all
    representable give the exact result (part 3)."""
    rng = np.random.default_rng(13)
    M, N, K, mbits = 32, 32, 64, 10
    A = (rng.random((M, K)) - 0.5).astype(np.float32)
    B = (rng.random((K, N)) - 0.5).astype(np.float32)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    absab = np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64))
    keps = K * 2.0 ** -mbits
    gamma = keps / (1 - keps)
    D = O.gemm(A, B, mbits)
    err = np.abs(D.astype(np.float64) - exact)
    assert np.all(err <= gamma * absab)
    err32 = np.abs((A @ B).astype(np.float64) - exact).max()
    assert err.max() > 50 * err32 and err.max() > 1e-4
    low = D.view(np.uint32) & np.uint32((1 << (23 - mbits)) - 1)
    assert np.all(low == 0)
    # small integers: every partial sum is an integer below 2^11, exact at 10 bits
    Ai = rng.integers(-3, 4, (M, K)).astype(np.float32)
    Bi = rng.integers(-3, 4, (K, N)).astype(np.float32)
    Di = O.gemm(Ai, Bi, mbits)
    assert np.array_equal(Di, (Ai.astype(np.float64) @ Bi.astype(np.float64)).astype(np.float32))


def _group(n):
    """Codes per group and bytes per group: lcm(n, 8) bits up to 8-bit codes,
    lcm(n, 16) above, computed here independently of the codec."""
    from math import lcm
    bits = lcm(n, 8 if n <= 8 else 16)
    return bits // n, bits // 8


def test_codec_packed_sizes():
    """test/test_pack.cpp:31-38: byte counts against an lcm formula."""
    for n in range(1, 17):
        gc, gb = _group(n)
        for count in list(range(0, 70)) + [1000, 4097]:
            assert O.packed_size(n, count) == -(-count // gc) * gb, (n, count)


P3109_SMALL = [(k, p, sat) for k in range(3, 9) for p in range(1, k) for sat in (True, False)]


@pytest.mark.parametrize("k,p,sat", P3109_SMALL)
def test_codec_every_rep_round_trips(k, p, sat):
    """test/test_pack.cpp:7-12: decode then encode gives back every non-NaN
    code, through the packed form in both byte orders and with a partial
    group at the end."""
    f = O.codec_p3109(k, p, saturating=sat)
    reps = np.arange(1 << k)
    vals = np.array([O.decode_rep(int(r), f) for r in reps], np.float32)
    finite = ~np.isnan(vals)
    back = np.array([O.encode_rep(float(v), f) for v in vals[finite]])
    assert np.array_equal(back, reps[finite])
    assert np.isnan(O.decode_rep(O.encode_rep(float("nan"), f), f))
    gc, _ = _group(k)
    x = vals[finite]
    x = np.concatenate([x, x[: gc + 1]]) if gc > 1 else x
    for rev in (0, 1):
        packed = O.encode(x, f, reverse=rev)
        assert np.array_equal(O.decode(packed, x.size, f, reverse=rev).view(np.uint32),
                              x.view(np.uint32))
    if gc > 1:
        assert not np.array_equal(O.encode(x, f, reverse=0), O.encode(x, f, reverse=1))


@pytest.mark.parametrize("k,p", [(8, 4), (8, 3), (6, 3), (4, 2)])
def test_codec_float_round_trip_is_the_format_rounding(k, p):
    """test/test_pack.cpp:141-170: floats from -8 to 8 in steps of 1/8 (and
    ±0) encode and decode to the format's own rounding of them, within its
    finite range."""
    f = O.codec_p3109(k, p)
    ef = O.fmt(k, p - 1, 1 << (k - p - 1))
    x = np.concatenate([np.arange(-64, 65) / 8.0, [0.0, -0.0]]).astype(np.float32)
    top = max(O.decode_rep(r, f) for r in range(1 << (k - 1)) if not np.isnan(O.decode_rep(r, f)))
    x = x[np.abs(x) <= top]
    dec = O.decode(O.encode(x, f), x.size, f)
    want = O.round(x, ef, RNE)
    # P3109 has a single zero: -0 encodes to the zero code
    want[want == 0] = 0.0
    dec[dec == 0] = 0.0
    assert np.array_equal(dec.view(np.uint32), want.view(np.uint32))


OVF_INF, SAT_FINITE, SAT_PROPAGATE = 0, 1, 2


@pytest.mark.parametrize("k,p,sat", P3109_SMALL)
def test_codec_saturation_modes(k, p, sat):
    """test/test_sat_mode.cpp:70-140 on the codec: finite over-range inputs
    clamp to ±max-finite under SatFinite and SatPropagate and become ±inf
    under OvfInf where the format has an infinity; infinite inputs clamp under
    SatFinite and stay infinite under OvfInf and SatPropagate; 1.0 is the
    same under all three."""
    f = O.codec_p3109(k, p, saturating=sat)
    vals = np.array([O.decode_rep(r, f) for r in range(1 << k)])
    maxf = vals[np.isfinite(vals)].max()
    if not maxf > 0:
        pytest.skip("no finite nonzero value in this format")
    has_inf = bool(np.isinf(vals).any())
    rt = lambda x, s: O.decode_rep(O.encode_rep(x, f, RNE, s), f)  # noqa: E731
    for sign in (1.0, -1.0):
        for m in (2.0, 8.0, 137.0, 1e6):
            x = float(np.float32(sign * maxf * m))
            assert rt(x, SAT_FINITE) == sign * maxf
            assert rt(x, SAT_PROPAGATE) == sign * maxf
            assert rt(x, OVF_INF) == (sign * np.inf if has_inf else sign * maxf)
        xi = sign * np.inf
        assert rt(xi, SAT_FINITE) == sign * maxf
        for s in (OVF_INF, SAT_PROPAGATE):
            assert rt(xi, s) == (xi if has_inf else sign * maxf)
    if 1.0 <= maxf:
        assert rt(1.0, OVF_INF) == rt(1.0, SAT_FINITE) == rt(1.0, SAT_PROPAGATE) == 1.0


@pytest.mark.parametrize("k,p,sat", [(k, p, s) for k in range(4, 9) for p in range(2, k)
                                     for s in (True, False)])
def test_format_rounding_brackets_on_the_decoded_grid(k, p, sat):
    """test/test_rounding_modes.cpp's bounds on the format overload, with the
    grid taken from the codec's decoded values of the same format: every
    result lies on that grid; RD and RU bracket x with no grid value between
    them; RTZ/RAFZ are the neighbours toward/away from zero; nearest modes
    return the nearer neighbour off ties; a tiny nonzero value rounds away
    from zero to ±denorm_min, never to 0."""
    f = O.codec_p3109(k, p, saturating=sat)
    ef = O.fmt(k, p - 1, 1 << (k - p - 1), saturating=sat)
    vals = np.array([O.decode_rep(r, f) for r in range(1 << k)], np.float64)
    grid = np.unique(np.concatenate([vals[np.isfinite(vals)], [0.0]]))
    maxf, dmin = grid.max(), grid[grid > 0].min()
    rng = np.random.default_rng(k * 100 + p)
    mag = np.exp2(rng.uniform(np.log2(dmin) - 2, np.log2(maxf), 4096))
    x = (mag * rng.choice([-1.0, 1.0], mag.size)).astype(np.float32)
    x = x[np.abs(x) <= maxf]
    x64 = x.astype(np.float64)
    idx = np.searchsorted(grid, x64, side="right") - 1
    on = grid[idx] == x64
    lo = grid[idx]
    hi = np.where(on, lo, grid[np.minimum(idx + 1, grid.size - 1)])
    res = {m: O.round(x, ef, m).astype(np.float64) for m in (RNE, RTZ, RAFZ, RD, RU, RNO, RTA)}
    for m, y in res.items():
        assert np.all(np.isin(np.abs(y), grid)), m
        assert np.all(y[on] == x64[on]), m
    assert np.all(res[RD] == lo) and np.all(res[RU] == hi)
    toward = np.where(x64 < 0, hi, lo)
    away = np.where(x64 < 0, lo, hi)
    assert np.all(res[RTZ] == toward) and np.all(res[RAFZ] == away)
    dl, dh = x64 - lo, hi - x64
    off_tie = dl != dh
    nearer = np.where(dl < dh, lo, hi)
    for m in (RNE, RNO, RTA):
        assert np.all(res[m][off_tie] == nearer[off_tie]), m
    tiny = np.array([dmin / 3, -dmin / 3], np.float32)
    assert np.array_equal(O.round(tiny, ef, RAFZ).astype(np.float64), [dmin, -dmin])
    assert np.all(O.round(tiny, ef, RTZ) == 0)


@pytest.mark.parametrize("mode,ln", [(TSR, 0), (SRA, 13), (SRB, 13)])
def test_stochastic_rounding_is_unbiased(mode, ln):
    """test/stoch_expect_test.cpp's concern: stochastic rounding is unbiased.
    With as many random bits as dropped bits (13 at 10 mantissa bits; True-SR
    draws a double), the mean over many independent draws of each value is
    the value itself, within six standard errors."""
    mbits, reps = 10, 20000
    x = wide_inputs(64, 77)
    xs = np.repeat(x, reps)
    y = O.round_mantissa(xs, mbits, mode, stoch_len=ln, seed=9).astype(np.float64)
    tz, az, _ = neighbours(x, mbits)
    step = np.abs(az.astype(np.float64) - tz.astype(np.float64))
    mean = y.reshape(64, reps).mean(axis=1)
    tol = 6 * 0.5 * step / np.sqrt(reps) + 1e-30
    assert np.all(np.abs(mean - x.astype(np.float64)) <= tol)


@pytest.mark.parametrize("nseg,R", [(16, 4.0), (64, 8.0), (256, 8.0)])
def test_pwl_silu_knots_interpolation_and_asymptote(nseg, R):
    """The PWL SiLU of `src/Lof_kernel.cu:231-257`: outside [-R, R] the relu
    asymptote exactly; at every knot but the last the table value exactly;
    between knots the linear interpolation of the two neighbouring knots,
    within one float32 ulp of it evaluated in FP64 from the kernel's own
    float32 steps."""
    knots = np.linspace(-R, R, nseg + 1)
    lut = (knots / (1 + np.exp(-knots))).astype(np.float32)
    rng = np.random.default_rng(nseg)
    out = np.concatenate([rng.uniform(R, 4 * R, 500), -rng.uniform(R, 4 * R, 500)])
    out = out.astype(np.float32)
    out = out[np.abs(out) > R]
    assert np.array_equal(O.pwl_silu(out, lut, R), np.where(out > 0, out, 0).astype(np.float32))
    kx = knots[:-1].astype(np.float32)
    assert np.array_equal(O.pwl_silu(kx, lut, R), lut[:-1])
    x = rng.uniform(-R, R, 20000).astype(np.float32)
    inv = np.float32(nseg) / np.float32(2 * R)
    u = ((x + np.float32(R)) * inv).astype(np.float32)
    i = np.minimum(u.astype(np.int64), nseg - 1)
    frac = (u - i.astype(np.float32)).astype(np.float32)
    d = (lut[i + 1] - lut[i]).astype(np.float32)
    want = frac.astype(np.float64) * d + lut[i]
    got = O.pwl_silu(x, lut, R).astype(np.float64)
    ulp = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(got - want) <= ulp)


def test_mx_encode_composes_mx_round_and_codec():
    """orc_mx_encode_f32: scale codes are the codec's codes of the MX scales,
    and decoded elements times decoded scales give the MX rounding wherever
    the rounded quotient is a value of the element format."""
    rng = np.random.default_rng(21)
    x = (rng.standard_normal(32 * 200 + 9) * np.exp2(rng.integers(-6, 7, 32 * 200 + 9))).astype(np.float32)
    e8 = O.codec_fmt(8, 0, 127, True, False, False, 0, 0xFFFFFFFF, 0, 0, 0xFF, 0xFF, 0, False)
    ef = O.codec_p3109(8, 4)
    codes, scales = O.mx_encode(x, 32, ef, e8)
    assert codes.size == x.size and scales.size == (x.size + 31) // 32
    q = O.decode(codes, x.size, ef)
    sc = O.decode(scales, scales.size, e8)
    back = q * np.repeat(sc, 32)[: x.size]
    ref = O.mx_round(x, 32, O.fmt(8, 3, 8), O.fmt(8, 0, 127, saturating=False, signed=False))
    every = O.decode(np.arange(256, dtype=np.uint8), 256, ef)
    top = np.float32(np.abs(every[np.isfinite(every)]).max())
    diff = back != ref
    assert diff.mean() < 0.08
    assert np.array_equal(np.abs(back[diff]), (top * np.repeat(sc, 32)[: x.size])[diff])


@pytest.mark.parametrize("k,p", [(8, 4), (8, 3), (6, 3), (6, 2), (4, 2)])
@pytest.mark.parametrize("signed", [True, False])
def test_codec_rne_of_rounded_equals_codec_rne_saturating(k, p, signed):
    """For a saturating format under RNE, the codec's code of virtual_round(w)
    equals the codec's code of w itself for every finite w (same grid; the
    rounding returns an overflowing input unchanged and the codec saturates
    it). The MX storage encode relies on this to encode MX quotients without
    rounding them first; NaN quotients, where it fails for unsigned formats
    (the sign decides the code), take the rounding path."""
    rng = np.random.default_rng(k * 10 + p + signed)
    ef = O.codec_p3109(k, p, signed=signed)
    n = 1 << 18
    e = rng.integers(127 - ef.fmt.bias - 30, 127 + (1 << (k - p)) - ef.fmt.bias + 4, n)
    sh = rng.integers(0, 24, n)
    m = rng.integers(0, 1 << 23, n)
    kind = rng.integers(0, 4, n)
    low = np.where(kind == 0, 0, np.where(kind == 1, 1 << np.maximum(sh - 1, 0),
                                          np.where(kind == 2, (1 << sh) - 1, m & ((1 << sh) - 1))))
    mm = (((m >> sh) << sh) | low) & 0x7FFFFF
    s = rng.integers(0, 2, n).astype(np.uint32) << 31
    w = (s | (e.astype(np.uint32) << 23) | mm.astype(np.uint32)).view(np.float32)
    w = np.concatenate([w, np.array([0.0, -0.0, np.inf, -np.inf], np.float32)])
    for sat in (0, 1, 2):
        assert np.array_equal(O.encode(w, ef, 0, sat), O.encode(O.round(w, ef.fmt, 0), ef, 0, sat))
