"""The tcgen05 chunked emulated-accumulation GEMM. Not bit-exact by design
(each k-chunk is summed in FP32 by the tensor cores before it is folded into
the emulated accumulator); checked against

  * the CPU chunked model with exact chunk sums (same fold, same chunks):
    results agree to within one accumulator ulp, mostly exactly;
  * the FP64 oracle GEMM: error of the order of the accumulator's precision;
  * exactly representable inputs: identical to the bit-exact CUDA-core form.
"""
import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from gpu_util import from_gpu, to_gpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _err_units(got, want, A, B, mbits, ta=0, tb=0):
    """|got - want| in units of 2^-mbits * (|A| @ |B|): the size of one
    accumulator ulp at the largest magnitude any partial sum can reach. A
    rounding flipped at an intermediate step costs at most a few such units,
    however much the final value cancels."""
    Ad = np.abs(A.astype(np.float64))
    Bd = np.abs(B.astype(np.float64))
    S = (Ad.T if ta else Ad) @ (Bd.T if tb else Bd)
    return np.abs(got.astype(np.float64) - want.astype(np.float64)) / (np.exp2(-mbits) * np.maximum(S, 1e-30))


def _status_ok():
    torch.cuda.synchronize()
    assert lg.binding.tc_device_status("cuda:0") == 0


@pytest.mark.parametrize("shape", [(128, 128, 64), (256, 256, 256), (200, 136, 300), (1, 1, 1),
                                   (129, 257, 33), (384, 128, 1000)])
@pytest.mark.parametrize("chunk", [32, 64])
def test_vs_chunked_model(shape, chunk):
    M, N, K = shape
    rng = np.random.default_rng(M + N + K + chunk)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), 10, variant="tc", chunk=chunk))
    _status_ok()
    want = O.gemm_chunked(A, B, 10, chunk)
    d = _err_units(got, want, A, B, 10)
    # a chunk sum off by ~2^-17 relative (BF16 hi/lo split, FP32 sums) moves a
    # 10-bit rounding only rarely, and each flip costs about one unit
    assert np.all(d <= 4.0), d.max()
    assert np.mean(d > 0) < 0.25


@pytest.mark.parametrize("ta", [0, 1])
@pytest.mark.parametrize("tb", [0, 1])
def test_layouts(ta, tb):
    M, N, K = 160, 192, 320
    rng = np.random.default_rng(ta * 2 + tb)
    A = rng.standard_normal((K, M) if ta else (M, K)).astype(np.float32)
    B = rng.standard_normal((N, K) if tb else (K, N)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), 12, trans_a=bool(ta), trans_b=bool(tb),
                           variant="tc", chunk=32))
    _status_ok()
    want = O.gemm_chunked(A, B, 12, 32, trans_a=ta, trans_b=tb)
    assert np.all(_err_units(got, want, A, B, 12, ta, tb) <= 4.0)


@pytest.mark.parametrize("chunk", [16, 48, 128, 256])
@pytest.mark.parametrize("mbits", [7, 23])
def test_chunks_and_widths(chunk, mbits):
    M, N, K = 128, 256, 512
    rng = np.random.default_rng(chunk + mbits)
    A = rng.uniform(-1, 1, (M, K)).astype(np.float32)
    B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), mbits, variant="tc", chunk=chunk, alpha=0.5))
    _status_ok()
    want = O.gemm_chunked(A, B, mbits, chunk, alpha=0.5)
    if mbits < 23:
        assert np.all(_err_units(got, want, A, B, mbits) <= 4.0)
    else:  # no accumulator rounding: only the FP32 chunk sums differ
        assert np.allclose(got, want, rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("chunk", [16, 32, 64])
@pytest.mark.parametrize("mbits", [5, 10, 14])
def test_exact_chunk_sums_bitexact(chunk, mbits):
    """A holds integers that need the hi+lo split, B integers exact in BF16, so
    every product and every chunk sum is exact in FP32 whatever order the
    tensor cores add in: the chunked form must then equal the CPU chunked
    model bit for bit (same chunks, same round-to-odd fold, same RNE)."""
    rng = np.random.default_rng(chunk * 100 + mbits)
    M, N, K = 160, 200, 512
    A = rng.integers(-600, 601, (M, K)).astype(np.float32)
    B = rng.integers(-100, 101, (K, N)).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), mbits, variant="tc", chunk=chunk))
    _status_ok()
    want = O.gemm_chunked(A, B, mbits, chunk)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        np.count_nonzero(got.view(np.uint32) != want.view(np.uint32))


@pytest.mark.parametrize("scale_a,scale_b", [(2.0**-70, 2.0**-40), (2.0**55, 2.0**45), (1.0, 1.0)])
@pytest.mark.parametrize("mbits", [5, 14])
def test_fold_choice_by_exponent_range(scale_a, scale_b, mbits):
    """The epilogue folds on the FMA pipe only when the operands' exponent
    ranges rule out subnormal and overflowing partial sums, and with the
    integer rounding otherwise. Tiny operands (partial sums down to 2^-110,
    whose smallest multiple would be subnormal), huge operands (partial sums
    near 2^125, where the FMA-pipe rounding would overflow) and plain ones:
    exact chunk sums, so every case must equal the CPU chunked model bit for
    bit."""
    rng = np.random.default_rng(mbits + int(np.log2(scale_a)) + 200)
    M, N, K = 128, 160, 512
    A = (rng.integers(-600, 601, (M, K)) * scale_a).astype(np.float32)
    B = (rng.integers(-100, 101, (K, N)) * scale_b).astype(np.float32)
    got = from_gpu(lg.gemm(to_gpu(A), to_gpu(B), mbits, variant="tc", chunk=64))
    _status_ok()
    want = O.gemm_chunked(A, B, mbits, 64)
    assert np.all(np.isfinite(want))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        np.count_nonzero(got.view(np.uint32) != want.view(np.uint32))


def test_exact_inputs_match_plain():
    """Small integers: every partial sum is exact, so all accumulation orders
    agree (the reference's exact-input check, test/test_blis_lof_accum.cpp:200-235)."""
    rng = np.random.default_rng(0)
    A = rng.integers(-3, 4, (256, 512)).astype(np.float32)
    B = rng.integers(-3, 4, (512, 128)).astype(np.float32)
    tc = lg.gemm(to_gpu(A), to_gpu(B), 23, variant="tc", chunk=32)
    pl = lg.gemm(to_gpu(A), to_gpu(B), 23)
    _status_ok()
    assert torch.equal(tc, pl)
    assert np.array_equal(from_gpu(tc), (A.astype(np.float64) @ B).astype(np.float32))


def test_gemm_4096_error_vs_fp64():
    """M=N=K=4096, MX-E4M3 operands along K, 10-bit accumulator, chunk 32:
    the error against the FP64 oracle is of the accumulator's order and
    close to the bit-exact CUDA-core form's."""
    g = torch.Generator().manual_seed(3)
    A = torch.randn(4096, 4096, generator=g).cuda()
    Bt = torch.randn(4096, 4096, generator=g).cuda()
    e4m3 = lg.create_p3109_params(8, 4)
    e8 = lg.create_e8m0_params()
    Aq = lg.virtual_mx_round(A, 32, e4m3, e8)
    Btq = lg.virtual_mx_round(Bt, 32, e4m3, e8)
    tc = lg.gemm(Aq, Btq, 10, trans_b=True, variant="tc", chunk=32)
    pl = lg.gemm(Aq, Btq, 10, trans_b=True)
    _status_ok()
    ref = lg.gemm_f64_reference(Aq, Btq, trans_b=True)
    big = ref.abs() > 1e-2 * ref.abs().mean()
    rel_tc = ((tc.double() - ref).abs() / ref.abs())[big]
    rel_pl = ((pl.double() - ref).abs() / ref.abs())[big]
    assert rel_tc.mean().item() < 2 * rel_pl.mean().item() + 1e-3
    assert rel_tc.mean().item() < 2e-2


@pytest.mark.parametrize("extra", ["none", "a", "b", "ab"])
def test_lo_tiles_left_out_bit_identical(extra):
    """Operands exact in BF16 have all-zero lo parts, and the GEMM then
    neither loads their lo tiles nor issues their MMAs (one MMA per k step
    instead of three, a deeper stage ring). One extra row of A (column of B)
    holding a value that BF16 does not hold turns that operand's lo MMAs back
    on; the outputs of every other row and column must not change by a bit,
    since the MMAs left out add only zero products."""
    g = torch.Generator(device="cuda").manual_seed(71)
    M, N, K = 300, 260, 1000
    A = torch.randn(M + 1, K, generator=g, device="cuda").bfloat16().float()
    B = torch.randn(K, N + 1, generator=g, device="cuda").bfloat16().float()
    base = lg.gemm(A[:M].contiguous(), B[:, :N].contiguous(), 10, variant="tc", chunk=32)
    _status_ok()
    A2, B2 = A.clone(), B.clone()
    if "a" in extra:
        A2[M, 7] = 1.0 + 2.0**-12
    if "b" in extra:
        B2[11, N] = -3.0 - 2.0**-11
    full = lg.gemm(A2, B2, 10, variant="tc", chunk=32)
    _status_ok()
    assert torch.equal(full[:M, :N], base)
    # the extra row / column itself against the CPU chunked model
    Ah, Bh, Dh = from_gpu(A2), from_gpu(B2), from_gpu(full)
    want = O.gemm_chunked(Ah[M:], Bh, 10, 32)
    assert np.all(_err_units(Dh[M:], want, Ah[M:], Bh, 10) <= 4.0)


@pytest.mark.parametrize("shape", [(256, 512, 256), (200, 300, 300), (129, 257, 33), (384, 640, 1000)])
@pytest.mark.parametrize("chunk", [32, 64])
def test_wide_tile(shape, chunk, monkeypatch):
    """The 128 x 256 output tile (LOFGB_TC_TILE_N=256; the launch picks it for
    large GEMMs): one MMA covers 256 columns and the epilogue folds 64-column
    slices in 8-column pieces. Against the CPU chunked model with the usual
    bound, and bit-identical to the 128 x 128 tile (every output sees the
    same chunk sums)."""
    M, N, K = shape
    rng = np.random.default_rng(M * 3 + N + K + chunk)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    monkeypatch.setenv("LOFGB_TC_TILE_N", "256")
    wide = lg.gemm(to_gpu(A), to_gpu(B), 10, variant="tc", chunk=chunk)
    _status_ok()
    monkeypatch.setenv("LOFGB_TC_TILE_N", "128")
    narrow = lg.gemm(to_gpu(A), to_gpu(B), 10, variant="tc", chunk=chunk)
    _status_ok()
    got = from_gpu(wide)
    d = _err_units(got, O.gemm_chunked(A, B, 10, chunk), A, B, 10)
    assert np.all(d <= 4.0), d.max()
    assert torch.equal(wide, narrow)


def test_wide_tile_batched_and_exact(monkeypatch):
    """Strided batch through the wide tile (a B box that runs past one batch
    entry's rows reads the next entry's, for columns that are not stored)
    and exactly representable inputs equal to the CUDA-core form."""
    monkeypatch.setenv("LOFGB_TC_TILE_N", "256")
    rng = np.random.default_rng(17)
    A = rng.integers(-3, 4, (3, 130, 200)).astype(np.float32)
    B = rng.integers(-3, 4, (3, 200, 300)).astype(np.float32)
    tc = lg.gemm(to_gpu(A), to_gpu(B), 23, variant="tc", chunk=32)
    _status_ok()
    pl = lg.gemm(to_gpu(A), to_gpu(B), 23)
    assert torch.equal(tc, pl)


def test_workspace_errors():
    A = torch.randn(64, 64, device="cuda")
    L = lg._native.lib()
    need = L.lofgb_gemm_tc_workspace_size(64, 64, 64)
    assert need > 0
    D = torch.empty(64, 64, device="cuda")
    st = L.lofgb_gemm_f32(A.data_ptr(), 64, 0, A.data_ptr(), 64, 0, D.data_ptr(), 64, 64, 64, 64, 10,
                          0, 1.0, 1, 32, None, 0, None)
    assert st == -9


@pytest.mark.parametrize("exact", [False, True])
def test_bounded_wait_runs_out_and_the_next_launch_is_clean(exact):
    """The wait self-test: every CTA's first pipeline stage is withheld (no
    copy issued, no fault), so the MMA warp's 1 ms wait runs out; the kernel
    must record LOFGB_ERR_TIMEOUT, drain, free its tensor memory and return.
    The next ordinary launch on the same stream then gives the same bits as
    before and a clean status. Operands with and without lo parts (three
    stages of four tiles, six stages of two)."""
    rng = np.random.default_rng(9)
    M, N, K = 256, 384, 512
    A = to_gpu(rng.standard_normal((M, K)).astype(np.float32))
    B = to_gpu(rng.standard_normal((K, N)).astype(np.float32))
    if exact:
        A, B = A.bfloat16().float(), B.bfloat16().float()
    before = lg.gemm(A, B, 10, variant="tc", chunk=32)
    _status_ok()
    L = lg._native.lib()
    ws = torch.zeros(L.lofgb_gemm_tc_workspace_size(M, N, K), dtype=torch.uint8, device="cuda")
    D = torch.empty(M, N, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = L.lofgb_gemm_tc_wait_selftest(A.data_ptr(), B.data_ptr(), D.data_ptr(), M, N, K,
                                       ws.data_ptr(), ws.numel(), 1000, stream)
    assert st == 0, L.lofgb_last_error_detail().decode()
    torch.cuda.synchronize()
    assert int(ws[:4].view(torch.int32).item()) == -10   # LOFGB_ERR_TIMEOUT
    after = lg.gemm(A, B, 10, variant="tc", chunk=32)
    _status_ok()
    assert torch.equal(after, before)
    assert L.lofgb_gemm_tc_wait_selftest(A.data_ptr(), B.data_ptr(), D.data_ptr(), M, N, K,
                                         ws.data_ptr(), ws.numel(), 10, stream) == -2
