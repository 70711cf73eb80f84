"""GPU parity of MX block rounding against the golden vectors and the oracle.
Bit-exact; NaN outputs match as a class (payloads of IEEE arithmetic on NaN
differ between host and GPU)."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import cases, fmt_tuple, same_bits_nan_class
from gpu_util import mx_matrix_data, from_gpu, mismatch_report, ofmt, to_gpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _desc(t):
    bw, m, bias, sat, signed = t
    return lg.FloatFormatDescriptor(bw, m, bias,
                                    lg.InfBehavior.Saturating if sat else lg.InfBehavior.Extended,
                                    lg.NaNBehavior._3109,
                                    lg.Signedness.Signed if signed else lg.Signedness.Unsigned,
                                    lg.formats.P3109_InfChecker(bw), lg.formats.P3109_NaNChecker(bw))


E2M1, E4M3, E5M2 = (4, 1, 1, True, True), (8, 3, 7, True, True), (8, 2, 15, True, True)
E8M0 = (8, 0, 127, False, False)


@pytest.mark.parametrize("cname,rec", list(cases("mx")), ids=lambda v: v if isinstance(v, str) else "")
def test_golden_mx(cname, rec):
    bs, mode, _ = (int(v) for v in rec["case"])
    ef, sf = _desc(fmt_tuple(rec["ef"])), _desc(fmt_tuple(rec["sf"]))
    x = rec["x"]
    got = from_gpu(lg.virtual_mx_round(to_gpu(x), bs, ef, sf, round_mode=mode))
    ok, bad = same_bits_nan_class(got, rec["y"])
    assert ok, (cname, mismatch_report(x, got, rec["y"]))


@pytest.mark.parametrize("elem", [E2M1, E4M3, E5M2])
def test_mx_8192x8192_full_size(elem):
    """8192x8192 N(0,1) with 1% outliers x2^12, blocks of 32 along rows, E8M0
    scale, RNE: bit-exact against the oracle at full size."""
    x = mx_matrix_data()
    ef, sf = _desc(elem), _desc(E8M0)
    got = from_gpu(lg.virtual_mx_round(to_gpu(x), 32, ef, sf))
    want = O.mx_round(x, 32, ofmt(ef), ofmt(sf))
    ok, bad = same_bits_nan_class(got, want)
    assert ok, mismatch_report(x, got, want)
    # the block max of an E8M0-scaled E4M3 block is exactly representable or passed through
    assert got.shape == x.shape


@pytest.mark.parametrize("bs", [8, 16, 32, 64, 128, 256])
@pytest.mark.parametrize("n", [1, 7, 255, 1000, 5003, 65536 + 13])
@pytest.mark.parametrize("mode", [0, 1, 5, 6, 12])
def test_block_sizes_lengths_modes(bs, n, mode):
    rng = np.random.default_rng(bs * 7919 + n)
    x = (rng.standard_normal(n) * 2.0 ** rng.integers(-12, 13, n)).astype(np.float32)
    ef, sf = _desc(E4M3), _desc(E8M0)
    got = from_gpu(lg.virtual_mx_round(to_gpu(x), bs, ef, sf, round_mode=mode))
    want = O.mx_round(x, bs, ofmt(ef), ofmt(sf), mode=mode)
    ok, _ = same_bits_nan_class(got, want)
    assert ok, mismatch_report(x, got, want)


@pytest.mark.parametrize("mode,len_", [(3, 8), (8, 4), (9, 6), (10, 0), (11, 0), (14, 5)])
def test_stochastic_elements(mode, len_):
    rng = np.random.default_rng(mode)
    x = rng.standard_normal(70_001).astype(np.float32)
    ef, sf = _desc(E5M2), _desc(E8M0)
    got = from_gpu(lg.virtual_mx_round(to_gpu(x), 32, ef, sf, round_mode=mode, stoch_len=len_,
                                       seed=77, offset=1000))
    want = O.mx_round(x, 32, ofmt(ef), ofmt(sf), mode=mode, stoch_len=len_, seed=77, offset=1000)
    ok, _ = same_bits_nan_class(got, want)
    assert ok, mismatch_report(x, got, want)


@pytest.mark.parametrize("smode", [1, 2, 5, 6, 10, 11, 12])
def test_scale_modes_and_scale_formats(smode):
    rng = np.random.default_rng(smode)
    x = (rng.standard_normal(40_000) * 2.0 ** rng.integers(-20, 20, 40_000)).astype(np.float32)
    for sfmt in (E8M0, (8, 2, 15, True, True), (6, 1, 7, False, True)):
        ef, sf = _desc(E4M3), _desc(sfmt)
        got = from_gpu(lg.virtual_mx_round(to_gpu(x), 64, ef, sf, scale_round_mode=smode, seed=3,
                                           offset=0))
        want = O.mx_round(x, 64, ofmt(ef), ofmt(sf), scale_mode=smode, seed=3, offset=0)
        ok, _ = same_bits_nan_class(got, want)
        assert ok, (sfmt, mismatch_report(x, got, want))


def test_special_values_and_zero_blocks():
    x = np.zeros(32 * 6, np.float32)
    x[32:64] = np.linspace(-3, 3, 32)
    x[70] = np.inf
    x[100] = np.nan
    x[130] = -np.inf
    x[160:192] = 1e-40  # FP32 subnormals
    ef, sf = _desc(E4M3), _desc(E8M0)
    got = from_gpu(lg.virtual_mx_round(to_gpu(x), 32, ef, sf))
    want = O.mx_round(x, 32, ofmt(ef), ofmt(sf))
    ok, _ = same_bits_nan_class(got, want)
    assert ok, mismatch_report(x, got, want)
    assert np.all(got[:32] == 0) and np.all(np.signbit(got[:32]) == False)  # noqa: E712


def test_misaligned_and_inplace():
    rng = np.random.default_rng(5)
    x = rng.standard_normal(4099).astype(np.float32)
    ef, sf = _desc(E4M3), _desc(E8M0)
    xg = to_gpu(x)
    got = from_gpu(lg.virtual_mx_round(xg[1:], 32, ef, sf))
    ok, _ = same_bits_nan_class(got, O.mx_round(x[1:], 32, ofmt(ef), ofmt(sf)))
    assert ok
    y = xg.clone()
    lg.virtual_mx_round(y, 32, ef, sf, out=y)
    ok, _ = same_bits_nan_class(from_gpu(y), O.mx_round(x, 32, ofmt(ef), ofmt(sf)))
    assert ok


def test_exact_block_roundtrip_and_errors():
    """An exactly representable block with amax = max normal keeps every value
    (the reference's test/test_mx_round_py.py:33-38 with the bias-8 format)."""
    e4m3 = lg.create_p3109_params(8, 4, True, True)  # 3 mantissa bits, bias 8, max 240
    maxn = 240.0
    exact = torch.tensor([[maxn, maxn / 2, -maxn / 4, 1.0, 0.5, -2.0, 8.0, 0.0] * 4], device="cuda")
    y = lg.virtual_mx_round(exact, 32, e4m3, lg.create_e8m0_params())
    assert torch.equal(y, exact)
    with pytest.raises(RuntimeError):
        lg.virtual_mx_round(exact.double(), 32, e4m3, lg.create_e8m0_params())
    with pytest.raises(RuntimeError):
        lg.virtual_mx_round(exact, 48, e4m3, lg.create_e8m0_params())
    with pytest.raises(RuntimeError):
        lg.virtual_mx_round(exact, 0, e4m3, lg.create_e8m0_params())


@pytest.mark.parametrize("bs", [8, 32, 64, 256])
@pytest.mark.parametrize("mode", [0, 1, 3])
@pytest.mark.parametrize("skew", [0, 1, 2])
def test_bf16_source_equals_fp32_copy(bs, mode, skew):
    """lofgb_mx_round_bf16 on BF16 bit patterns equals lofgb_mx_round_f32 on the
    same values widened to FP32, bit for bit: every block size class, a
    deterministic and a stochastic mode, and inputs offset by 0, 2 or 4
    bytes (vector and scalar paths), with a ragged last block."""
    g = torch.Generator(device="cuda").manual_seed(bs * 10 + mode)
    n = 40 * bs + 5
    base = (torch.randn(n + skew, device="cuda", generator=g) *
            torch.exp2(torch.randint(-12, 13, (n + skew,), device="cuda", generator=g).float()))
    xb = base.bfloat16()[skew:]
    e4m3, e8 = lg.create_p3109_params(8, 4), lg.create_e8m0_params()
    got = lg.virtual_mx_round(xb, bs, e4m3, e8, round_mode=mode, stoch_len=8 if mode == 3 else 0,
                              seed=3, offset=11)
    want = lg.virtual_mx_round(xb.float(), bs, e4m3, e8, round_mode=mode,
                               stoch_len=8 if mode == 3 else 0, seed=3, offset=11)
    assert got.dtype == torch.float32
    assert torch.equal(got.view(torch.int32), want.view(torch.int32))


def test_bf16_source_linear_operands():
    """The linear layer's MX-E4M3 rounding of BF16 masters (8192 x 4096) read
    directly equals rounding the FP32 copy."""
    g = torch.Generator(device="cuda").manual_seed(4)
    X = torch.randn(8192, 4096, device="cuda", generator=g).bfloat16()
    e4m3, e8 = lg.create_p3109_params(8, 4), lg.create_e8m0_params()
    assert torch.equal(lg.virtual_mx_round(X, 32, e4m3, e8), lg.virtual_mx_round(X.float(), 32, e4m3, e8))
