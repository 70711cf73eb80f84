"""Parity at the benchmark workloads' own sizes.

  * the 4096^3 emulated GEMM (MX-E4M3 operands, 10-bit accumulator,
    CUDA-core form): 256 rows (16 blocks of 16 spread over M) bit-exact
    against the oracle, and the whole output bit-identical to the transposed
    problem D^T = B^T A^T, which reads the operands through the other
    loaders and tiles (every output is the same sequence of products, and
    a*b = b*a exactly);
  * the differentiable linear layer (X 8192x4096, W 4096x4096, BF16
    masters, MX-E4M3, FP16-like 5e/10m accumulator in 64-element chunks,
    dY stochastic-rounded to E5M2): output and gradients at full size against
    the FP64 surrogate (autograd through the rounded operands), with stated
    bounds;
  * the grouped rounding (512 tensors, each its own format and mode, one grouped
    launch): every tensor against the oracle — whole tensors up to 2^20
    elements, head, tail and 16 random windows of 4096 beyond;
  * the grouped GEMMs (64 GEMMs of 256..4096, one grouped tensor-core launch):
    sampled rows of every GEMM against the CPU chunked model, within the
    tensor-core tests' bound.
"""
import numpy as np
import pytest
import torch

import bench
import lofloat_gb300 as lg
from golden_io import same_bits
from gpu_util import from_gpu
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _err_units(got, want, Arows, B, mbits):
    """|got - want| in accumulator ulps at the largest partial sum (as
    test_gpu_tc): 2^-mbits * (|A| @ |B|)."""
    S = np.abs(Arows.astype(np.float64)) @ np.abs(B.astype(np.float64))
    return np.abs(got.astype(np.float64) - want.astype(np.float64)) / (np.exp2(-mbits) * np.maximum(S, 1e-30))


def test_gemm_4096_plain_256_rows_and_transposed_full_output():
    g = torch.Generator().manual_seed(3)
    A = torch.randn(4096, 4096, generator=g).cuda()
    Bt = torch.randn(4096, 4096, generator=g).cuda()
    e4m3, e8 = lg.create_p3109_params(8, 4), lg.create_e8m0_params()
    Aq = lg.virtual_mx_round(A, 32, e4m3, e8)
    Btq = lg.virtual_mx_round(Bt, 32, e4m3, e8)   # rows of B^T: blocks along K
    D = lg.gemm(Aq, Btq, 10, trans_b=True)
    Dt = lg.gemm(Btq, Aq, 10, trans_b=True)       # (B^T)(A^T) = D^T
    torch.cuda.synchronize()
    assert torch.equal(D, Dt.t()), int((D != Dt.t()).sum())
    Ah, Bh, Dh = from_gpu(Aq), from_gpu(Btq), from_gpu(D)
    for blk in range(16):
        r0 = blk * 256 + (blk * 37) % 240
        want = O.gemm_rows(Ah, Bh, 10, r0, 16, trans_b=1)
        assert same_bits(Dh[r0:r0 + 16], want), f"rows {r0}..{r0 + 15}"


def test_linear_8192x4096x4096_against_fp64():
    g = torch.Generator(device="cuda").manual_seed(4)
    X = torch.randn(8192, 4096, device="cuda", generator=g).bfloat16().requires_grad_(True)
    W = (torch.randn(4096, 4096, device="cuda", generator=g) * 0.02).bfloat16().requires_grad_(True)
    e4m3 = bench.fmt_desc(lg, 8, 3, 7)
    e5m2 = bench.fmt_desc(lg, 8, 2, 15)
    cfg = lg.LinearConfig(act_format=e4m3, weight_format=e4m3, accum_mant_bits=10, variant="tc",
                          chunk=64, grad_format=e5m2, grad_stoch_len=8,
                          accum_format=lg.create_half_params())
    lg.set_seed(0)
    y = lg.lof_linear(X, W, cfg)
    (y * y).sum().backward()
    xq = lg.virtual_mx_round(X.detach().float(), 32, e4m3, cfg.scale_format).double()
    wq = lg.virtual_mx_round(W.detach().float(), 32, e4m3, cfg.scale_format).double()
    y64 = xq @ wq.T
    dy = 2 * y64
    gx, gw = dy @ wq, dy.T @ xq
    rel = lambda a, b: ((a.double() - b).norm() / b.norm()).item()  # noqa: E731
    # forward: FP16-like accumulator (10 mantissa bits, 2^-11 per rounding)
    # folded 64 times over K = 4096
    assert rel(y, y64) < 1e-2
    # backward: dY rounded to E5M2 by SR-A (2 mantissa bits, ~2^-3 relative
    # noise per element, unbiased) dominates; measured about 0.05 / 0.04
    assert rel(X.grad, gx) < 0.08
    assert rel(W.grad, gw) < 0.07
    assert torch.isfinite(X.grad).all() and torch.isfinite(W.grad).all()


@pytest.fixture(scope="module")
def grouped_workloads():
    dev = torch.device("cuda", 0)
    gr, specs, rng, g = bench.grouped_round_case(torch, lg, dev, item=1 << 16)
    gr()
    torch.cuda.synchronize()
    yield gr, specs, rng, g
    del gr
    torch.cuda.empty_cache()


def _windows(n, rng):
    if n <= 1 << 20:
        return [(0, n)]
    starts = [0, n - 4096] + [int(v) for v in rng.integers(0, n - 4096, 16)]
    return [(s, s + 4096) for s in starts]


def test_grouped_rounding_512_tensors_every_tensor(grouped_workloads):
    gr, specs, _, _ = grouped_workloads
    wrng = np.random.default_rng(55)
    checked = 0
    for i, sp in enumerate(specs):
        x, y = gr.ins[i], gr.outs[i]
        f = O.fmt(1 + sp["exp"] + sp["mant"], sp["mant"], (1 << (sp["exp"] - 1)) - 1,
                  saturating=sp["saturating"])
        for a, b in _windows(x.numel(), wrng):
            xs = x[a:b].cpu().numpy()
            want = O.round(xs, f, sp["mode"], sp["stoch_len"], seed=sp["seed"], offset=a)
            got = y[a:b].cpu().numpy()
            assert same_bits(got, want), f"tensor {i} ({x.numel()} elements) window {a}"
            checked += b - a
    assert len(specs) == 512 and checked > 10_000_000


def test_grouped_gemms_64_every_task(grouped_workloads):
    _, _, rng, g = grouped_workloads
    dev = torch.device("cuda", 0)
    tasks = bench.grouped_gemm_case(torch, lg, dev, rng, g)
    gg = lg.GroupedGemm(tasks, schedule="lpt_snake")
    gg()
    torch.cuda.synchronize()
    assert gg.status() == 0
    srng = np.random.default_rng(5)
    for i, t in enumerate(tasks):
        M, N = t["D"].shape
        rows = np.sort(srng.choice(M, 3, replace=False))
        A = t["A"].cpu().numpy()
        Bt = t["B"].cpu().numpy()
        B = np.ascontiguousarray(Bt.T)
        D = t["D"].cpu().numpy()
        mb = t["accum_mant_bits"]
        for r in rows:
            want = O.gemm_chunked(A[r:r + 1], B, mb, t["chunk"])
            d = _err_units(D[r:r + 1], want, A[r:r + 1], B, mb)
            assert np.all(d <= 4.0), (i, int(r), float(d.max()))
            assert np.mean(d > 0) < 0.25, (i, int(r))
