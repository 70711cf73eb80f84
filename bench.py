"""Benchmark of the LoFloat emulation hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline (one step): MX block rounding of an 8192x8192 FP32 matrix (N(0,1)
with 1% outliers scaled by 2^12, seed 2), blocks of 32 along rows with an E8M0
scale, to E2M1, E4M3 and E5M2 in turn under RNE — 3 launches, 8 algorithmic
bytes per element each. `value` is GB/s with inputs resident in HBM (the
256 MiB input is larger than L2, so no flush is needed between steps);
`e2e` is the same metric through the public API with host buffers (pinned
input copied in, each result copied out, every step).

The line also carries the other workloads as secondary numbers: plain
rounding of 2^24 FP32 to E4M3 (RNE and SR-A), and the 4096^3 emulated GEMM
(CUDA-core bit-exact form and tensor-core chunked form with its FP64-oracle
error).

--impl reference times the reference algorithm on the host cores (the C
oracle, a restatement of the reference's scalar code, with all threads) on
the same workload: the whole matrix, three formats, every step. The
reference's own host code is compiled only where its sources are present
(x86, for the parity tests), so the timed CPU implementation is the port.

With N > 1 (torchrun) every rank runs an independent replica of the workload
on its own GPU (weak scaling, no data-path collective); timing is the max
over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MX_ROWS = MX_COLS = 8192
MX_BLOCK = 32
MX_BYTES = MX_ROWS * MX_COLS * 8  # per format: 4 B read + 4 B write per element
ELEM_FORMATS = {"e2m1": (4, 1, 1), "e4m3": (8, 3, 7), "e5m2": (8, 2, 15)}
C1_N = 1 << 24
GEMM_N = 4096
# the headline line's metric and workload, the same in both arms
METRIC = "MX block rounding throughput (8 B/elem); secondary: emulated-accum GEMM TFLOP/s"
WORKLOAD = ("MX round 8192x8192 f32, block 32 along rows, E8M0 scale, "
            "E2M1/E4M3/E5M2 in turn, RNE")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-secondary", action="store_true", help="headline workload only")
    ap.add_argument("--only", default=None,
                    choices=["mx", "round_rne", "round_sr", "gemm_plain", "gemm_tc", "conv_plain",
                             "conv_tc", "pwl", "encode", "decode", "encode_fp6", "decode_fp6",
                             "grouped_round", "bn_train", "bn_eval", "mx_encode"],
                    help="run one workload's kernel warmup+steps times and exit (for ncu captures)")
    ap.add_argument("--size", default="full", choices=["full", "small"],
                    help="with --only: full-size workload or a small case (GEMM 1024^3)")
    return ap.parse_args()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic(name: str):
    """dram bytes per launch recorded from an ncu capture in profiles/."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as fh:
            m = re.search(r"dram_bytes_per_launch\s*=\s*([0-9.eE+]+)", fh.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", f"lofgb_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                f = [v.strip() for v in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(dist, seconds, device):
    """Every rank's timings replaced by the slowest rank's, element by element
    (one all-reduce of a float64 vector on `device`: the rank's GPU under
    NCCL, the CPU under gloo)."""
    import torch
    t = torch.tensor(list(seconds), device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def whole_job_gbs(world, steps, step_bytes, seconds):
    """Whole-job throughput of `world` replicas that each processed `steps`
    steps of `step_bytes` algorithmic bytes in `seconds` (the max over ranks)."""
    return world * steps * step_bytes / seconds / 1e9


def mx_matrix_input(torch, dev):
    g = torch.Generator().manual_seed(2)
    x = torch.randn(MX_ROWS * MX_COLS, generator=g, dtype=torch.float32)
    mask = torch.rand(MX_ROWS * MX_COLS, generator=g) < 0.01
    x[mask] *= 4096.0
    return x.reshape(MX_ROWS, MX_COLS)


def fmt_desc(lg, bw, m, bias, sat=True, signed=True):
    return lg.FloatFormatDescriptor(bw, m, bias,
                                    lg.InfBehavior.Saturating if sat else lg.InfBehavior.Extended,
                                    lg.NaNBehavior._754,
                                    lg.Signedness.Signed if signed else lg.Signedness.Unsigned,
                                    lg.formats.P3109_InfChecker(bw), lg.formats.P3109_NaNChecker(bw))


# ---------------------------------------------------------------------------
# reference arm: the reference algorithm on the host cores
# ---------------------------------------------------------------------------
def run_reference(args, world, rank):
    if rank != 0:
        return
    import torch  # noqa: F401  (same environment as our arm)

    from oracle import oracle as O
    threads = O.max_threads()
    # the whole 8192 x 8192 matrix per format per step: the same work as our arm
    sample = mx_matrix_input(torch, None).reshape(-1).numpy()
    sf = O.fmt(8, 0, 127, saturating=False, signed=False)
    efs = [O.fmt(*v) for v in ELEM_FORMATS.values()]

    def step():
        for ef in efs:
            O.mx_round(sample, MX_BLOCK, ef, sf, nthreads=threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    gbs = args.steps * len(efs) * sample.size * 8 / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": gbs,
            "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD},
            "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": threads, "kind": "port",
                             "sample": "MX rounding of all 2^26 elements, 3 formats, every step"},
            "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def cpu_baseline_sample():
    """The oracle on a bounded sample of the headline workload (all threads)."""
    import torch

    from oracle import oracle as O
    threads = O.max_threads()
    x = mx_matrix_input(torch, None).reshape(-1).numpy()[: 1 << 22]
    sf = O.fmt(8, 0, 127, saturating=False, signed=False)
    efs = [O.fmt(*v) for v in ELEM_FORMATS.values()]
    O.mx_round(x, MX_BLOCK, efs[1], sf, nthreads=threads)
    reps, t0 = 0, time.perf_counter()
    while True:
        for ef in efs:
            O.mx_round(x, MX_BLOCK, ef, sf, nthreads=threads)
        reps += 1
        if time.perf_counter() - t0 > 10.0:
            break
    dt = time.perf_counter() - t0
    # single-thread figure on a smaller sample (about 3 s)
    x1 = x[: 1 << 19]
    reps1, t1 = 0, time.perf_counter()
    while True:
        for ef in efs:
            O.mx_round(x1, MX_BLOCK, ef, sf, nthreads=1)
        reps1 += 1
        if time.perf_counter() - t1 > 3.0:
            break
    dt1 = time.perf_counter() - t1
    return {"value": reps * len(efs) * x.size * 8 / dt / 1e9, "unit": "GB/s", "cores": threads,
            "kind": "port",
            "sample": f"MX rounding of 2^22 of the 2^26 config elements, 3 formats x {reps} reps",
            "single_thread": {"value": reps1 * len(efs) * x1.size * 8 / dt1 / 1e9, "unit": "GB/s",
                              "sample": f"2^19 elements, 3 formats x {reps1} reps"}}


def time_events(torch, fn, reps, stream):
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    for i in range(reps):
        starts[i].record(stream)
        fn()
        ends[i].record(stream)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def time_batched(torch, fn, stream, per_batch=10, batches=5):
    """Median per-launch time (ms) of `per_batch` back-to-back calls between
    two events, over `batches` batches (no event between two launches)."""
    return statistics.median(m / per_batch for m in
                             time_events(torch, lambda: [fn() for _ in range(per_batch)], batches, stream))


def secondary(torch, lg, dev, peaks):
    """Plain rounding of 2^24 FP32 values to E4M3 and the 4096^3 emulated GEMMs."""
    out = {}
    stream = torch.cuda.current_stream(dev)
    g = torch.Generator().manual_seed(0)
    x = (torch.randn(C1_N, generator=g) * torch.exp2(torch.randint(-20, 21, (C1_N,), generator=g).float()))
    xg = x.to(dev)
    yg = torch.empty_like(xg)
    e4m3 = fmt_desc(lg, 8, 3, 7)
    # the 2^24-element config is 128 MiB of traffic, about the size of L2:
    # launches cycle over four input/output pairs (512 MiB), so every launch
    # reads an input that is no longer in L2; 20 back-to-back launches
    # between two events, median of 5 such batches
    xs = [xg] + [xg.clone() for _ in range(3)]
    ys = [yg] + [torch.empty_like(xg) for _ in range(3)]
    for name, mode, ln in (("rne", 0, 0), ("sr_a", 3, 8)):
        def batch(mode=mode, ln=ln):
            for i in range(20):
                lg.virtual_round(xs[i % 4], e4m3, round_mode=mode, stoch_len=ln, seed=1, offset=0,
                                 out=ys[i % 4])
        batch()
        ms = [m / 20 for m in time_events(torch, batch, 5, stream)]
        gbs = C1_N * 8 / (statistics.median(ms) * 1e-3) / 1e9
        out[f"round_2^24_e4m3_{name}_GBs"] = round(gbs, 1)
        out[f"round_2^24_e4m3_{name}_frac_hbm"] = round(gbs / peaks["hbm_gbs"], 4)
    out["round_2^24_l2"] = "launches cycle over four 2^24-element input/output pairs (512 MiB)"
    del xs, ys
    # GEMM 4096^3, MX-E4M3 operands along K, 10-bit accumulator
    g = torch.Generator().manual_seed(3)
    A = torch.randn(GEMM_N, GEMM_N, generator=g).to(dev)
    Bt = torch.randn(GEMM_N, GEMM_N, generator=g).to(dev)
    e8 = lg.create_e8m0_params()
    Aq = lg.virtual_mx_round(A, 32, e4m3, e8)
    Btq = lg.virtual_mx_round(Bt, 32, e4m3, e8)  # rows of B^T = columns of B: blocks along K
    flops = 2.0 * GEMM_N ** 3
    D = torch.empty(GEMM_N, GEMM_N, device=dev)
    fn = lambda: lg.gemm(Aq, Btq, 10, trans_b=True, out=D)  # noqa: E731
    fn()
    ms = time_events(torch, fn, 3, stream)
    plain = flops / (statistics.median(ms) * 1e-3) / 1e12
    out["gemm_4096_plain_TFLOPs"] = round(plain, 3)
    out["gemm_4096_plain_ms"] = round(statistics.median(ms), 3)
    try:
        Dt = torch.empty_like(D)
        fn = lambda: lg.gemm(Aq, Btq, 10, trans_b=True, variant="tc", chunk=32, out=Dt)  # noqa: E731
        fn()
        ms = time_events(torch, fn, 5, stream)
        tc = flops / (statistics.median(ms) * 1e-3) / 1e12
        ref = lg.gemm_f64_reference(Aq, Btq, trans_b=True)
        den = ref.abs().clamp_min(1e-30)
        rel_tc = (Dt.double() - ref).abs() / den
        rel_pl = (D.double() - ref).abs() / den
        big = ref.abs() > 1e-2 * ref.abs().mean()
        out.update({
            "gemm_4096_tc_TFLOPs": round(tc, 2), "gemm_4096_tc_ms": round(statistics.median(ms), 3),
            "gemm_tc_over_plain": round(tc / plain, 2),
            "gemm_tc_frac_bf16_peak": round(tc / peaks["bf16_tflops"], 4),
            "gemm_tc_err_vs_fp64": {"max_rel": float(rel_tc[big].max()), "mean_rel": float(rel_tc[big].mean())},
            "gemm_plain_err_vs_fp64": {"max_rel": float(rel_pl[big].max()), "mean_rel": float(rel_pl[big].mean())},
            "gemm_err_note": "relative error over outputs with |ref| > 1% of mean |ref|",
        })
    except Exception as e:  # tensor-core form unavailable: report why
        out["gemm_tc_unavailable"] = str(e)[:200]
    del A, Bt, Aq, Btq, D
    out.update(linear_fwd_bwd(torch, lg, dev))
    out.update(grouped_workloads(torch, lg, dev))
    out.update(conv_workloads(torch, lg, dev, peaks))
    return out


CONV_SHAPE = (32, 256, 14, 14, 256, 3, 3)  # N, C, H, W, K, R, S; stride 1, pad 1


def conv_data(torch, lg, dev, shape=CONV_SHAPE):
    n, c, h, w, k, r, s_ = shape
    g = torch.Generator(device=dev).manual_seed(6)
    e4m3 = fmt_desc(lg, 8, 3, 7)
    x = lg.virtual_round(torch.randn(n, c, h, w, device=dev, generator=g), e4m3)
    wt = lg.virtual_round(torch.randn(k, c, r, s_, device=dev, generator=g) * 0.05, e4m3)
    return x, wt


def conv_workloads(torch, lg, dev, peaks):
    """Emulated-accumulation conv2d on a ResNet stage-4 layer: N=32, C=K=256,
    14x14, 3x3, pad 1, E4M3-rounded activations and weights, 10-bit
    accumulator; lof_conv2d's order (8-channel tiles) on the CUDA cores and on
    the tensor cores (chunk 32). Then PWL SiLU over 2^26 FP32 values (16
    segments on [-8, 8])."""
    out = {}
    stream = torch.cuda.current_stream(dev)
    x, wt = conv_data(torch, lg, dev)
    n, c, h, w, k, r, s_ = CONV_SHAPE
    flops = 2.0 * n * k * h * w * c * r * s_
    y = torch.empty(n, k, h, w, device=dev)
    for variant in ("plain", "tc"):
        fn = lambda: lg.conv2d(x, wt, 10, padding=1, order="tiled8", variant=variant, out=y)  # noqa: E731
        fn()
        ms = statistics.median(time_events(torch, fn, 5, stream))
        out[f"conv_resnet_{variant}_TFLOPs"] = round(flops / ms / 1e9, 2)
        out[f"conv_resnet_{variant}_ms"] = round(ms, 3)
    out["conv_tc_over_plain"] = round(out["conv_resnet_tc_TFLOPs"] / out["conv_resnet_plain_TFLOPs"], 2)
    del x, wt, y
    m = lg.PWLSiLU(R=8.0, lut_bits=4)
    lut = m.lut.to(dev)
    g = torch.Generator(device=dev).manual_seed(7)
    xs = torch.randn(1 << 26, device=dev, generator=g) * 4
    ys = torch.empty_like(xs)
    fn = lambda: lg.pwl_silu(xs, lut, 8.0, out=ys)  # noqa: E731
    for _ in range(3):
        fn()
    ms = time_batched(torch, fn, stream)
    gbs = (1 << 26) * 8 / (ms * 1e-3) / 1e9
    out["pwl_silu_2^26_GBs"] = round(gbs, 1)
    out["pwl_silu_2^26_frac_hbm"] = round(gbs / peaks["hbm_gbs"], 4)
    del xs, ys
    out.update(codec_workloads(torch, lg, dev, peaks))
    out.update(bn_workloads(torch, lg, dev, peaks))
    return out


BN_SHAPE = (32, 256, 56, 56)


def bn_workloads(torch, lg, dev, peaks):
    """BatchNorm approximations on an NCHW 32x256x56x56 FP32 activation
    (103 MB): training-mode forward (statistics + fused normalise/affine) of
    each variant, and the eval-mode forward (normalise/affine only). GB/s at
    8 B per element (one read and one write: the least any implementation
    moves); the statistics passes read the input again, mostly from L2."""
    out = {}
    stream = torch.cuda.current_stream(dev)
    g = torch.Generator(device=dev).manual_seed(9)
    x = torch.randn(*BN_SHAPE, device=dev, generator=g) * 2 + 0.5
    nbytes = x.numel() * 8
    for name, cls in (("l1", lg.L1BatchNorm), ("linf", lg.LinfBatchNorm), ("fisr", lg.FISRBatchNorm),
                      ("pwl", lg.PWLBatchNorm)):
        m = cls(BN_SHAPE[1]).to(dev)
        for mode in ("train", "eval"):
            m.train(mode == "train")
            graph = graph_of(torch, lambda: m(x))
            ms = time_batched(torch, graph.replay, stream)
            gbs = nbytes / (ms * 1e-3) / 1e9
            out[f"bn_{name}_{mode}_GBs"] = round(gbs, 1)
            out[f"bn_{name}_{mode}_frac_hbm"] = round(gbs / peaks["hbm_gbs"], 4)
    out["bn_note"] = ("NCHW 32x256x56x56 f32; 8 B/elem; train = statistics + normalise; "
                      "module forward captured in a CUDA graph, replays timed")
    return out


def graph_of(torch, fn):
    """fn's launches (under no_grad) captured in a CUDA graph, after three
    warm-up calls on the capture stream."""
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.no_grad(), torch.cuda.stream(side):
        for _ in range(3):
            fn()
    torch.cuda.current_stream().wait_stream(side)
    g = torch.cuda.CUDAGraph()
    with torch.no_grad(), torch.cuda.graph(g):
        fn()
    return g


def codec_workloads(torch, lg, dev, peaks):
    """Storage codec over 2^26 FP32 values (N(0,1) * 2^U{-20..20}): encode to
    packed E4M3 (8-bit) and P3109<6,3> (6-bit) codes and decode back, GB/s at
    4 + n/8 bytes per value."""
    out = {}
    stream = torch.cuda.current_stream(dev)
    n = 1 << 26
    g = torch.Generator(device=dev).manual_seed(8)
    x = torch.randn(n, device=dev, generator=g) * torch.exp2(
        torch.randint(-20, 21, (n,), device=dev, generator=g).float())
    y = torch.empty_like(x)
    for name, fmt in (("e4m3", lg.create_p3109_params(8, 4)), ("p3109_6p3", lg.create_p3109_params(6, 3))):
        bits = fmt.total_bits
        packed = torch.empty(lg.packed_size(bits, n), dtype=torch.uint8, device=dev)
        enc = lambda: lg.lof_encode(x, fmt, out=packed)  # noqa: E731
        dec = lambda: lg.lof_decode(packed, n, fmt, out=y)  # noqa: E731
        for fn, tag in ((enc, "encode"), (dec, "decode")):
            for _ in range(3):
                fn()
            ms = time_batched(torch, fn, stream)
            gbs = n * (4 + bits / 8) / (ms * 1e-3) / 1e9
            out[f"codec_{tag}_{name}_2^26_GBs"] = round(gbs, 1)
            out[f"codec_{tag}_{name}_2^26_frac_hbm"] = round(gbs / peaks["hbm_gbs"], 4)
    # MX storage of the 8192 x 8192 matrix in one pass: E4M3 / FP6 element codes
    # and E8M0 block scales (4 B read, bits/8 + 1/32 B written per value)
    del x, y
    xm = mx_matrix_input(torch, None).to(dev)
    e8 = lg.create_e8m0_params()
    for name, fmt in (("e4m3", lg.create_p3109_params(8, 4)), ("p3109_6p3", lg.create_p3109_params(6, 3))):
        fn = lambda: lg.mx_encode(xm, fmt, e8)  # noqa: E731
        for _ in range(3):
            fn()
        ms = time_batched(torch, fn, stream)
        nbytes = xm.numel() * (4 + fmt.total_bits / 8 + 1 / 32)
        out[f"mx_encode_{name}_8192^2_GBs"] = round(nbytes / (ms * 1e-3) / 1e9, 1)
        out[f"mx_encode_{name}_8192^2_frac_hbm"] = round(nbytes / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"], 4)
        # and back: element codes times block scales, one kernel
        codes, scales = fn()
        dec = lambda: lg.mx_decode(codes, scales, xm.numel(), fmt, e8)  # noqa: E731
        for _ in range(3):
            dec()
        ms = time_batched(torch, dec, stream)
        out[f"mx_decode_{name}_8192^2_GBs"] = round(nbytes / (ms * 1e-3) / 1e9, 1)
        out[f"mx_decode_{name}_8192^2_frac_hbm"] = round(nbytes / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"], 4)
    return out


def linear_fwd_bwd(torch, lg, dev):
    """Differentiable LoFloat linear layer, forward + backward: X 8192x4096 and
    W 4096x4096 BF16 masters (N(0,1), N(0,0.02), seed 4), MX-E4M3 along K,
    FP16-like (5 exponent, 10 mantissa bits) emulated accumulator in 64-element
    chunks on the tensor cores,
    loss = sum(Y^2), dY stochastic-rounded to E5M2; three 8192x4096x4096 GEMMs."""
    g = torch.Generator(device=dev).manual_seed(4)
    X = torch.randn(8192, 4096, device=dev, generator=g).bfloat16().requires_grad_(True)
    W = (torch.randn(4096, 4096, device=dev, generator=g) * 0.02).bfloat16().requires_grad_(True)
    e4m3 = fmt_desc(lg, 8, 3, 7)
    cfg = lg.LinearConfig(act_format=e4m3, weight_format=e4m3, accum_mant_bits=10, variant="tc",
                          chunk=64, grad_format=fmt_desc(lg, 8, 2, 15), grad_stoch_len=8,
                          accum_format=lg.create_half_params())

    def step():
        X.grad = W.grad = None
        y = lg.lof_linear(X, W, cfg)
        (y * y).sum().backward()

    for _ in range(2):
        step()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    s.record()
    for _ in range(reps):
        step()
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / reps
    flops = 3 * 2.0 * 8192 * 4096 * 4096
    # gradient error against autograd through STE MX rounding and FP64 GEMMs
    lg.set_seed(0)
    step()
    xq = lg.virtual_mx_round(X.detach().float(), 32, e4m3, cfg.scale_format).double()
    wq = lg.virtual_mx_round(W.detach().float(), 32, e4m3, cfg.scale_format).double()
    y = xq @ wq.T
    dy = 2 * y
    gx, gw = dy @ wq, dy.T @ xq
    rel_x = ((X.grad.double() - gx).norm() / gx.norm()).item()
    rel_w = ((W.grad.double() - gw).norm() / gw.norm()).item()
    return {"linear_fwd_bwd_ms": round(ms, 3), "linear_fwd_bwd_TFLOPs": round(flops / ms / 1e9, 2),
            "linear_grad_rel_err_vs_fp64": {"dX": rel_x, "dW": rel_w,
                                             "note": "dY rounded to E5M2 by SR-A: ~2^-3 noise"}}


def grouped_round_case(torch, lg, dev, item="auto"):
    """Grouped rounding: 512 FP32 tensors, each with its own format and mode
    (seed 5). Returns the grouped launch, the per-tensor specs (exp and
    mantissa bits, saturation, mode, stoch_len, seed) and the two generators,
    which the grouped GEMMs continue."""
    rng = np.random.default_rng(5)
    g = torch.Generator(device=dev).manual_seed(5)
    ins, outs, fmts, modes, lens, seeds, specs = [], [], [], [], [], [], []
    for i in range(512):
        n = int(2 ** rng.uniform(10, 24))
        x = torch.randn(n, device=dev, generator=g) * float(2 ** rng.uniform(-10, 10))
        ins.append(x)
        outs.append(torch.empty_like(x))
        e, m = int(rng.integers(2, 9)), int(rng.integers(1, 11))
        sat = bool(rng.integers(0, 2))
        fmts.append(lg.make_format(e, m, saturating=sat))
        modes.append(int(rng.choice([0, 1, 12, 3])))
        lens.append(8 if modes[-1] == 3 else 0)
        seeds.append(int(rng.integers(0, 2**62)))
        specs.append(dict(exp=e, mant=m, saturating=sat, mode=modes[-1], stoch_len=lens[-1],
                          seed=seeds[-1]))
    gr = lg.GroupedRound(ins, outs, fmts, modes, stoch_lens=lens, seeds=seeds, item=item)
    return gr, specs, rng, g


def grouped_gemm_case(torch, lg, dev, rng, g):
    """Grouped GEMMs: 64 emulated GEMMs, M, N, K in {256..4096 step 256},
    MX-E4M3 operands (B given transposed, blocks along K), accumulator bits
    7-12, chunk 32; continues the grouped rounding's generators."""
    e4m3 = fmt_desc(lg, 8, 3, 7)
    e8 = lg.create_e8m0_params()
    tasks = []
    for i in range(64):
        M, N, K = (int(v) for v in rng.integers(1, 17, 3) * 256)
        A = lg.virtual_mx_round(torch.randn(M, K, device=dev, generator=g), 32, e4m3, e8)
        Bt = lg.virtual_mx_round(torch.randn(N, K, device=dev, generator=g), 32, e4m3, e8)
        tasks.append(dict(A=A, B=Bt, D=torch.empty(M, N, device=dev), trans_b=1,
                          accum_mant_bits=int(rng.integers(7, 13)), chunk=32))
    return tasks


def grouped_workloads(torch, lg, dev):
    """The grouped workloads. Rounding: 512 FP32 tensors, n ~ 2^U(10,24), values
    N(0,1)*2^U(-10,10), each with its own format (exp 2-8, mant 1-10, bias
    2^(e-1)-1, saturating or not) and mode (RNE/RTZ/RTO/SR-A), seed 5: one
    grouped launch replayed from a CUDA graph. GEMMs: 64 emulated GEMMs,
    M,N,K in {256..4096 step 256}, MX-E4M3 operands, accumulator bits 7-12,
    one grouped tensor-core launch with the autotuned schedule, from a graph."""
    out = {}
    gr, _, rng, g = grouped_round_case(torch, lg, dev)
    gr.capture()
    for _ in range(3):
        gr.replay()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(10):
        gr.replay()
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / 10
    out["grouped_round_512_GBs"] = round(gr.bytes / ms / 1e6, 1)
    out["grouped_round_512_elements"] = int(gr.bytes // 8)
    out["grouped_round_512_item"] = gr.item
    out["grouped_round_512_tuning_ms"] = {str(k): v for k, v in gr.tuning_ms.items()}
    del gr
    torch.cuda.empty_cache()
    tasks = grouped_gemm_case(torch, lg, dev, rng, g)
    gg = lg.GroupedGemm(tasks, schedule="auto")
    gg.capture()
    for _ in range(2):
        gg.replay()
    torch.cuda.synchronize()
    s.record()
    for _ in range(5):
        gg.replay()
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / 5
    out["grouped_gemm_64_TFLOPs"] = round(gg.flops / ms / 1e9, 2)
    out["grouped_gemm_64_ms"] = round(ms, 3)
    out["grouped_gemm_64_schedule"] = gg.schedule
    out["grouped_gemm_64_tuning_ms"] = gg.tuning["ms"] if gg.tuning else None
    out["grouped_gemm_status"] = gg.status()
    return out


def bind_gpu_local_numa(local):
    """Restrict this process to the host CPUs of the GPU's NUMA node (the
    node sysfs records for the GPU's PCI device), so that pinned host buffers
    allocated next live next to the GPU. Returns what was done and the CPU
    set to restore once the buffers exist."""
    try:
        bus = subprocess.run(["nvidia-smi", "-i", str(local), "--query-gpu=pci.bus_id",
                              "--format=csv,noheader"], capture_output=True, text=True,
                             timeout=30).stdout.strip().lower()
        # sysfs names the device with a 4-digit domain
        dom, rest = bus.split(":", 1)
        path = f"/sys/bus/pci/devices/{int(dom, 16):04x}:{rest}/numa_node"
        node = int(open(path).read().strip())
        if node < 0:
            return {"node": None, "note": "no NUMA node recorded for the GPU"}
        cpus = set()
        for part in open(f"/sys/devices/system/node/node{node}/cpulist").read().strip().split(","):
            a, _, b = part.partition("-")
            cpus.update(range(int(a), int(b or a) + 1))
        before = os.sched_getaffinity(0)
        cpus &= before
        if not cpus:
            return {"node": node, "note": "no allowed CPU on the GPU's node"}
        os.sched_setaffinity(0, cpus)
        return {"node": node, "cpus": len(cpus), "restore": before}
    except (OSError, ValueError, subprocess.SubprocessError) as e:
        return {"node": None, "note": str(e)[:120]}


def link_bandwidth(torch, xh, yh, xd, yd, stream, s_out):
    """Host<->device copy rates of the e2e buffers, measured apart from the
    e2e loop: one 256 MiB pinned host-to-device copy, one device-to-host copy,
    and two device-to-host copies in flight on two streams. The e2e step
    moves 1x in and 3x out, with the input copy overlapping the outputs, so
    its ceiling is the step's algorithmic bytes over the slower direction.
    Each rate is the best of three batches of five copies: the host memory
    and link are shared with other jobs, and one slow batch would understate
    the ceiling the e2e loop can reach."""
    nbytes = xh.numel() * 4

    def timed(fn, reps=5, batches=3):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(batches):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b) / 1e3 / reps)
        return best

    t_h2d = timed(lambda: xd[0].copy_(xh, non_blocking=True))
    t_d2h = timed(lambda: yh[0].copy_(yd[0], non_blocking=True))

    def two_d2h():
        ev = torch.cuda.Event()
        ev.record(stream)
        for i, so in enumerate(s_out):
            so.wait_event(ev)
            with torch.cuda.stream(so):
                yh[i].copy_(yd[i], non_blocking=True)
        for so in s_out:
            stream.wait_stream(so)
    t_d2h2 = timed(two_d2h)
    h2d, d2h, d2h2 = nbytes / t_h2d / 1e9, nbytes / t_d2h / 1e9, 2 * nbytes / t_d2h2 / 1e9
    # one e2e step: 3 formats x 8 algorithmic B/elem = 6 x nbytes; its copies
    # take at least the slower of nbytes in and 3 x nbytes out
    t_copy = max(nbytes / (h2d * 1e9), 3 * nbytes / (max(d2h, d2h2) * 1e9))
    return {"h2d_gbs": round(h2d, 1), "d2h_gbs": round(d2h, 1), "d2h_two_streams_gbs": round(d2h2, 1),
            "e2e_ceiling_gbs": round(6 * nbytes / t_copy / 1e9, 1),
            "note": "ceiling = 3 x 8 B/elem over the slower of 1 x 4 B/elem in and 3 x 4 B/elem out"}


def run_ours(args, world, rank, local):
    import torch

    import lofloat_gb300 as lg
    from lofloat_gb300 import _native

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    peaks, peak_src = measured_peaks()
    x_host = mx_matrix_input(torch, None)
    x = x_host.to(dev)
    y = torch.empty_like(x)
    e8 = lg.create_e8m0_params()
    efs = [fmt_desc(lg, *v) for v in ELEM_FORMATS.values()]
    stream = torch.cuda.current_stream(dev)
    _native.lib()

    # one step: the three element formats in turn, back to back (no events
    # between the launches, which would stop a launch from overlapping the
    # tail of the one before it)
    def step():
        for ef in efs:
            lg.virtual_mx_round(x, MX_BLOCK, ef, e8, out=y)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    elapsed = t0.elapsed_time(t1) / 1e3
    # the timed region holds only mx_kernel launches: their average duration
    per_launch = elapsed / (args.steps * len(efs))

    # end to end through the public API with host buffers: every step copies
    # its input from pinned host memory, rounds it to the three formats and
    # copies the three results back to pinned host memory. Consecutive steps
    # overlap: input copies run on their own stream into two device buffers,
    # result copies alternate over two streams (two copy engines device to
    # host), the roundings stay on the timed stream; events order the reuse
    # of every device buffer.
    numa = bind_gpu_local_numa(local)
    xh = x_host.pin_memory()
    yh = [torch.empty_like(xh).pin_memory() for _ in efs]
    if "restore" in numa:  # pages are placed; the CPU baseline later uses every core
        os.sched_setaffinity(0, numa.pop("restore"))
    s_in = torch.cuda.Stream(dev)
    s_out = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    xd = [torch.empty(xh.shape, dtype=xh.dtype, device=dev) for _ in range(2)]
    yd = [torch.empty(xh.shape, dtype=xh.dtype, device=dev) for _ in efs]
    e2e = {"k": 0, "out_done": [None] * len(efs), "used": [None, None]}

    def e2e_step():
        k = e2e["k"]
        e2e["k"] += 1
        buf = xd[k % 2]
        with torch.cuda.stream(s_in):
            if e2e["used"][k % 2] is not None:
                s_in.wait_event(e2e["used"][k % 2])
            buf.copy_(xh, non_blocking=True)
            ev_in = torch.cuda.Event()
            ev_in.record(s_in)
        stream.wait_event(ev_in)
        for i, ef in enumerate(efs):
            if e2e["out_done"][i] is not None:
                stream.wait_event(e2e["out_done"][i])
            lg.virtual_mx_round(buf, MX_BLOCK, ef, e8, out=yd[i])
            ev_c = torch.cuda.Event()
            ev_c.record(stream)
            so = s_out[i % 2]
            so.wait_event(ev_c)
            with torch.cuda.stream(so):
                yh[i].copy_(yd[i], non_blocking=True)
                ev_o = torch.cuda.Event()
                ev_o.record(so)
            e2e["out_done"][i] = ev_o
        ev_u = torch.cuda.Event()
        ev_u.record(stream)
        e2e["used"][k % 2] = ev_u

    def e2e_join():
        for ev in e2e["out_done"]:
            stream.wait_event(ev)

    for _ in range(2):
        e2e_step()
    e2e_join()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_steps = max(3, min(args.steps, 10))
    e0.record(stream)
    s_in.wait_event(e0)
    for _ in range(e2e_steps):
        e2e_step()
    e2e_join()
    e1.record(stream)
    torch.cuda.synchronize()
    # the host copies hold the device results (checked outside the timed region)
    for i, ef in enumerate(efs):
        if not torch.equal(yh[i].to(dev), lg.virtual_mx_round(xd[0], MX_BLOCK, ef, e8)):
            raise RuntimeError(f"end-to-end result {i} differs from the device result")
    e2e_s = e0.elapsed_time(e1) / 1e3
    clk = clocks.stop()
    link = link_bandwidth(torch, xh, yh, xd, yd, stream, s_out)
    link["numa"] = numa

    if dist:
        elapsed, e2e_s = max_over_ranks(dist, [elapsed, e2e_s], dev)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    step_bytes = len(efs) * MX_BYTES
    value = whole_job_gbs(world, args.steps, step_bytes, elapsed)
    achieved = MX_BYTES / per_launch / 1e9
    traffic = profile_traffic("mx_kernel_8192x8192.md")
    line = {
        "metric": METRIC,
        "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": round(elapsed / args.steps * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded N(0,1), 1% outliers x2^12)",
        "config": {"workload": WORKLOAD,
                   "l2": "input 256 MiB > 129 MB L2; no flush", "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": traffic, "peak_source": f"{peak_src} hbm_gbs",
                     "kernel": "mx_kernel<32,RNE,RNE>", "algorithmic_bytes_per_launch": MX_BYTES},
        "e2e": {"value": round(whole_job_gbs(world, e2e_steps, step_bytes, e2e_s), 2), "unit": "GB/s",
                "h2d_bytes_per_step": MX_ROWS * MX_COLS * 4,
                "d2h_bytes_per_step": len(efs) * MX_ROWS * MX_COLS * 4,
                "api": "lofloat_gb300.virtual_mx_round (C ABI lofgb_mx_round_f32)",
                "link": link},
        "gpu_launches": args.steps * len(efs),
        "clocks": clk,
    }
    if not args.no_secondary:
        line["secondary"] = secondary(torch, lg, dev, peaks)
    if world == 1:
        line["cpu_baseline"] = cpu_baseline_sample()
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_only(args):
    """One workload, warmup + steps launches, timed with CUDA events; the
    command ncu captures (python bench.py --only <w> --steps K --warmup W)."""
    import torch

    import lofloat_gb300 as lg
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    e4m3 = fmt_desc(lg, 8, 3, 7)
    e8 = lg.create_e8m0_params()
    if args.only == "mx":
        x = mx_matrix_input(torch, None).to(dev)
        y = torch.empty_like(x)
        fn = lambda: lg.virtual_mx_round(x, MX_BLOCK, e4m3, e8, out=y)  # noqa: E731
        work, unit = MX_BYTES, "GB/s"
    elif args.only in ("round_rne", "round_sr"):
        g = torch.Generator().manual_seed(0)
        n = C1_N * 2  # 2^25 elements: 128 MiB in + 128 MiB out, above L2
        x = (torch.randn(n, generator=g) * torch.exp2(torch.randint(-20, 21, (n,), generator=g).float())).to(dev)
        y = torch.empty_like(x)
        mode, ln = (0, 0) if args.only == "round_rne" else (3, 8)
        fn = lambda: lg.virtual_round(x, e4m3, round_mode=mode, stoch_len=ln, seed=1, offset=0, out=y)  # noqa: E731
        work, unit = n * 8, "GB/s"
    elif args.only in ("conv_plain", "conv_tc"):
        shape = CONV_SHAPE if args.size == "full" else (4, 64, 14, 14, 64, 3, 3)
        x, wt = conv_data(torch, lg, dev, shape)
        n, c, h, w, k, r, s_ = shape
        y = torch.empty(n, k, h, w, device=dev)
        variant = args.only.split("_")[1]
        fn = lambda: lg.conv2d(x, wt, 10, padding=1, order="tiled8", variant=variant, out=y)  # noqa: E731
        work, unit = 2.0 * n * k * h * w * c * r * s_, "TFLOP/s"
    elif args.only == "pwl":
        xs = torch.randn(1 << 26, device=dev) * 4
        lut = lg.PWLSiLU(R=8.0, lut_bits=4).lut.to(dev)
        ys = torch.empty_like(xs)
        fn = lambda: lg.pwl_silu(xs, lut, 8.0, out=ys)  # noqa: E731
        work, unit = (1 << 26) * 8, "GB/s"
    elif args.only in ("encode", "decode", "encode_fp6", "decode_fp6"):
        n = 1 << 26
        x = (torch.randn(n, device=dev) * torch.exp2(torch.randint(-20, 21, (n,), device=dev).float()))
        bits = 6 if args.only.endswith("fp6") else 8
        fmt = lg.create_p3109_params(bits, 3 if bits == 6 else 4)
        packed = lg.lof_encode(x, fmt)
        y = torch.empty_like(x)
        fn = (lambda: lg.lof_encode(x, fmt, out=packed)) if args.only.startswith("encode") else \
            (lambda: lg.lof_decode(packed, n, fmt, out=y))  # noqa: E731
        work, unit = n * (4 + bits / 8), "GB/s"
    elif args.only == "mx_encode":
        x = mx_matrix_input(torch, None).to(dev)
        fn = lambda: lg.mx_encode(x, e4m3, e8)  # noqa: E731
        work, unit = x.numel() * (4 + 1 + 1 / 32), "GB/s"
    elif args.only in ("bn_train", "bn_eval"):
        x = torch.randn(*BN_SHAPE, device=dev) * 2 + 0.5
        m = lg.L1BatchNorm(BN_SHAPE[1]).to(dev).train(args.only == "bn_train")
        fn = graph_of(torch, lambda: m(x)).replay
        work, unit = x.numel() * 8, "GB/s"
    elif args.only == "grouped_round":
        gr = grouped_round_case(torch, lg, dev)[0]
        fn = gr
        work, unit = gr.bytes, "GB/s"
    else:
        n = GEMM_N if args.size == "full" else 1024
        g = torch.Generator().manual_seed(3)
        A = lg.virtual_mx_round(torch.randn(n, n, generator=g).to(dev), 32, e4m3, e8)
        Bt = lg.virtual_mx_round(torch.randn(n, n, generator=g).to(dev), 32, e4m3, e8)
        D = torch.empty(n, n, device=dev)
        variant = "plain" if args.only == "gemm_plain" else "tc"
        fn = lambda: lg.gemm(A, Bt, 10, trans_b=True, variant=variant, chunk=32, out=D)  # noqa: E731
        work, unit = 2.0 * n ** 3, "TFLOP/s"
    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    ms = time_events(torch, fn, args.steps, stream)
    med = statistics.median(ms) * 1e-3
    rate = work / med / (1e12 if unit == "TFLOP/s" else 1e9)
    print(json.dumps({"only": args.only, "size": args.size, "median_ms": med * 1e3,
                      "value": rate, "unit": unit, "launches": args.warmup + args.steps}), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.only:
        run_only(args)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
