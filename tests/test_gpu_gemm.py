"""GPU parity of the emulated-accumulation GEMM: the CUDA-core form is
bit-exact against the golden vectors and the oracle (sequential k, RNE
accumulator, device round-to-odd FMA); NaN outputs match as a class."""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from golden_io import cases, same_bits, same_bits_nan_class
from gpu_util import from_gpu, mismatch_report, to_gpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cname,rec", list(cases("gemm")), ids=lambda v: v if isinstance(v, str) else "")
def test_golden_gemm(cname, rec):
    A, B = rec["A"], rec["B"]
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), int(rec["mbits"]), alpha=float(rec["alpha"])))
    assert same_bits(got, rec["D"]), (cname, mismatch_report(got, got, rec["D"]))


def _mx_e4m3(x):
    return O.mx_round(x, 32, O.fmt(8, 3, 7), O.fmt(8, 0, 127, saturating=False, signed=False)).reshape(x.shape)


@pytest.mark.parametrize("ta", [0, 1])
@pytest.mark.parametrize("tb", [0, 1])
@pytest.mark.parametrize("mbits", [7, 10, 12, 23])
def test_layouts_vs_oracle(ta, tb, mbits):
    rng = np.random.default_rng(ta * 2 + tb + mbits * 4)
    M, N, K = 200, 136, 300
    A = rng.standard_normal((K, M) if ta else (M, K)).astype(np.float32)
    B = rng.standard_normal((N, K) if tb else (K, N)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), mbits, trans_a=bool(ta), trans_b=bool(tb)))
    want = O.gemm(A, B, mbits, trans_a=ta, trans_b=tb)
    assert same_bits(got, want), mismatch_report(got, got, want)


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 7, 3), (5, 1, 17), (129, 257, 33), (64, 64, 1),
                                   (3, 300, 16), (130, 2, 1000)])
def test_shapes_and_tails(shape):
    M, N, K = shape
    rng = np.random.default_rng(M * N + K)
    A = _mx_e4m3(rng.standard_normal((M, K)).astype(np.float32)) if K % 32 == 0 else \
        rng.standard_normal((M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), 10))
    want = O.gemm(A, B, 10)
    assert same_bits(got, want), mismatch_report(got, got, want)


@pytest.mark.parametrize("shape", [(2600, 2200, 40), (1000, 700, 64)])
def test_whole_and_half_tiles(shape):
    """378 tiles of 128 x 128 (more than one wave: whole tiles) and 48 tiles
    (fewer than the GPU holds at once: 64-row half tiles), ragged M and N
    edges in both; every output equals the oracle's bits."""
    M, N, K = shape
    rng = np.random.default_rng(11)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), 10))
    want = O.gemm(A, B, 10)
    assert same_bits(got, want), mismatch_report(got, got, want)


def test_special_values():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((40, 64)).astype(np.float32)
    B = rng.standard_normal((64, 24)).astype(np.float32)
    A[3, 5] = np.nan
    A[7, 9] = np.inf
    B[11, 2] = -np.inf
    A[9, :] = 3.0e38  # overflow in the accumulator
    A[12, :] = 1e-42  # subnormal products
    A[13, :32] = -A[13, 32:]  # cancellation
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), 10))
    want = O.gemm(A, B, 10)
    ok, _ = same_bits_nan_class(got, want)
    assert ok, mismatch_report(got, got, want)


def test_alpha_and_dropin_signature():
    rng = np.random.default_rng(4)
    A = rng.standard_normal((64, 96)).astype(np.float32)
    B = rng.standard_normal((96, 48)).astype(np.float32)
    Ag, Bg = to_gpu(A), to_gpu(B)
    got = from_gpu(lg.lof_gemm(Ag, Bg, 10, lg.RoundingMode.RoundTowardsZero, 5, scale_a=0.5, scale_b=4.0))
    alpha = lg.gemm_alpha(0.5, 4.0)
    assert same_bits(got, O.gemm(A, B, 10, alpha=alpha))
    got_op = from_gpu(torch.ops.lofloat.lof_gemm(Ag, Bg, 10, 0, 0, 0.5, 4.0))
    assert same_bits(got_op, got)
    zero_scale = from_gpu(lg.lof_gemm(Ag, Bg, 10, scale_a=0.0, scale_b=3.0))
    assert same_bits(zero_scale, O.gemm(A, B, 10, alpha=1.0))
    with pytest.raises(RuntimeError):
        lg.lof_gemm(Ag, to_gpu(B[:50]), 10)
    with pytest.raises(RuntimeError):
        lg.lof_gemm(Ag.double(), Bg.double(), 10)
    with pytest.raises(RuntimeError):
        lg.lof_gemm(Ag.cpu(), Bg.cpu(), 10)


def test_gemm_4096_sample_rows():
    """M=N=K=4096, MX-E4M3 operands, 10-bit accumulator: 32 sampled rows of the
    full-size GPU output are bit-exact against the oracle, and the whole
    output agrees with an FP64 GEMM to the accumulator's precision."""
    g = torch.Generator().manual_seed(3)
    A = torch.randn(4096, 4096, generator=g).numpy()
    B = torch.randn(4096, 4096, generator=g).numpy()
    Aq = _mx_e4m3(A)
    Bq = np.ascontiguousarray(_mx_e4m3(np.ascontiguousarray(B.T)).T)  # blocks along K
    Ag, Bg = to_gpu(Aq), to_gpu(Bq)
    D = lg.gemm(Ag, Bg, 10)
    Dh = from_gpu(D)
    rows = np.random.default_rng(0).choice(4096, 32, replace=False)
    for r in rows:
        want = O.gemm_rows(Aq, Bq, 10, int(r), 1)
        assert same_bits(Dh[r:r + 1], want), f"row {r}"
    ref = lg.gemm_f64_reference(Ag, Bg)
    rel = ((D.double() - ref).abs() / ref.abs().clamp_min(1e-3 * ref.abs().mean())).mean().item()
    assert rel < 5e-2


def _half_fmt():
    return O.fmt(16, 10, 15, saturating=False)


@pytest.mark.parametrize("fmt_t", [(16, 10, 15, False), (8, 2, 15, True), (19, 10, 127, False),
                                   (12, 6, 15, False)])
@pytest.mark.parametrize("tb", [0, 1])
def test_format_accumulator_vs_oracle(fmt_t, tb):
    """Accumulator rounded into a whole format after every MAC (the FP16-like
    5e/10m accumulator and others, incl. one outside the float-rounding
    path): bit-exact to the oracle, overflow and underflow included."""
    bw, m, bias, sat = fmt_t
    rng = np.random.default_rng(bw * 100 + m + tb)
    M, N, K = 96, 80, 200
    A = (rng.standard_normal((M, K)) * 2.0 ** rng.integers(-12, 9, (M, K))).astype(np.float32)
    B = rng.standard_normal((N, K) if tb else (K, N)).astype(np.float32)
    desc = lg.FloatFormatDescriptor(bw, m, bias, lg.InfBehavior.Saturating if sat else lg.InfBehavior.Extended,
                                    lg.NaNBehavior._754, lg.Signedness.Signed,
                                    lg.formats.P3109_InfChecker(bw), lg.formats.P3109_NaNChecker(bw))
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), 10, trans_b=bool(tb), alpha=0.5, accum_format=desc))
    want = O.gemm_accfmt(A, B, O.fmt(bw, m, bias, saturating=sat), alpha=0.5, trans_b=tb)
    ok, _ = same_bits_nan_class(got, want)
    assert ok, mismatch_report(got, got, want)


def test_format_accumulator_tc():
    rng = np.random.default_rng(5)
    A = _mx_e4m3(rng.standard_normal((256, 512)).astype(np.float32))
    B = _mx_e4m3(rng.standard_normal((192, 512)).astype(np.float32))
    half = lg.create_half_params()
    Ag, Bg = to_gpu(A), to_gpu(B)
    tc = from_gpu(lg.gemm(Ag, Bg, 10, trans_b=True, variant="tc", chunk=64, accum_format=half))
    plain = from_gpu(lg.gemm(Ag, Bg, 10, trans_b=True, accum_format=half))
    ref = from_gpu(lg.gemm_f64_reference(Ag, Bg, trans_b=True))
    scale = np.abs(ref).mean()
    assert np.abs(tc - ref).max() / scale <= 1.5 * np.abs(plain - ref).max() / scale + 1e-3
    # exact small integers: both forms exact within FP16's range
    Ai = rng.integers(-3, 4, (64, 128)).astype(np.float32)
    Bi = rng.integers(-3, 4, (128, 48)).astype(np.float32)
    tci = from_gpu(lg.gemm(to_gpu(Ai), to_gpu(Bi), 10, variant="tc", accum_format=half))
    assert np.array_equal(tci, (Ai.astype(np.float64) @ Bi).astype(np.float32))
    # overflow of the FP16 range: the extended format's +inf
    big = np.full((4, 64), 3000.0, np.float32)  # 64 * 3000 > 65504
    ob = from_gpu(lg.gemm(to_gpu(big), to_gpu(np.ones((64, 4), np.float32)), 10, accum_format=half))
    assert np.all(np.isinf(ob))
    assert lg.binding.tc_device_status() == 0
