"""Generate the golden vectors in tests/golden/ from the reference's own code.

Run in a checkout that has the reference sources (default /root/reference,
override with LOFGB_REFERENCE):

    python tests/golden/make_golden.py

It builds oracle/_ref/libref_shim.so (oracle/ref_shim.cpp compiled against the
reference headers, see oracle/build_oracle.py), feeds it seeded synthetic
inputs plus hand-built edge values, and writes compressed .npz fixtures and
MANIFEST.json (sha256 of every fixture). The fixtures are then committed; the
tests read only the fixtures, never the reference.

Stochastic cases seed the reference's host RNG per element
(lo_float::set_seed) and record the draw it consumed, so the oracle can be
fed the same random bits.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

MODES = list(range(15))
STOCH = {3: "SR_A", 8: "SR_B", 9: "SR_C", 10: "TRUE_SR", 11: "PROB", 14: "SR_D"}
LEN_MODES = {3, 8, 9, 14}  # modes whose draw width is stoch_len

# (bitwidth, mantissa_bits, bias, saturating, signed)
F32_FORMATS = {
    "e4m3": (8, 3, 7, True, True),
    "e5m2": (8, 2, 15, True, True),
    "e2m1": (4, 1, 1, True, True),
    "e8m0": (8, 0, 127, False, False),
    "p3109_8p4": (8, 3, 8, True, True),          # create_p3109_params(8, 4)
    "p3109_8p3_u_ext": (8, 2, 16, False, False),  # create_p3109_params(8, 3, False, False)
    "e4m3_ext": (8, 3, 7, False, True),
    "e3m4_ext": (8, 4, 3, False, True),
    "half": (16, 10, 15, False, True),           # create_half_params()
    "bf16": (16, 7, 127, False, True),
    "single": (32, 23, 127, False, True),        # create_single_params()
}
F64_FORMATS = {
    "e4m3": (8, 3, 7, True, True),
    "half": (16, 10, 15, False, True),
    "bf16": (16, 7, 127, True, True),
    "single": (32, 23, 127, False, True),
    "e9m30": (40, 30, 255, True, True),
    "double": (64, 52, 1023, False, True),
}

P = C.c_void_p


def p(a):
    return a.ctypes.data_as(P) if a is not None else None


def f32_bits(u):
    return np.asarray(u, np.uint32).view(np.float32)


def f64_bits(u):
    return np.asarray(u, np.uint64).view(np.float64)


def consts(f):
    bw, m, bias, sat, signed = f
    e = bw - m - (1 if signed else 0)
    to_max = (1 << e) - 1 - bias
    to_min = 1 - bias
    tiny = float(np.float32(2.0 ** to_min * 2.0 ** (-m)))
    return m, to_max, to_min, tiny


def inputs_f32(rng, f, n=512):
    m, to_max, to_min, tiny = consts(f)
    d = 23 - m
    vals = []
    # values of the 2^24-element rounding workload: N(0,1)*2^U{-20..20}
    vals += list((rng.standard_normal(200) * 2.0 ** rng.integers(-20, 21, 200)).astype(np.float32))
    # values across the format's exponent range and just outside it
    lo, hi = max(to_min - m - 3, -149), min(to_max + 3, 127)
    e = rng.integers(lo, hi + 1, 120)
    vals += list((np.sign(rng.standard_normal(120)) * (1 + rng.random(120)) * 2.0 ** e).astype(np.float32))
    # exact ties at the format's precision (normal range), and one ulp either side
    if d > 0:
        for _ in range(40):
            ee = int(rng.integers(max(to_min, -126), min(to_max, 127) + 1))
            b = np.array(np.float32((1 + rng.random()) * 2.0 ** ee)).view(np.uint32)
            b = (b & ~np.uint32((1 << d) - 1)) | np.uint32(1 << (d - 1))
            s = np.uint32(0x80000000) if rng.random() < 0.5 else np.uint32(0)
            vals += list(f32_bits([b | s, (b + 1) | s, (b - 1) | s]))
    # boundaries around the smallest subnormal and the largest finite
    for t in (tiny, tiny * 0.5, tiny * 0.75, tiny * 1.5, tiny * 2.5, tiny * 3):
        vals += [np.float32(t), -np.float32(t)]
    tb = np.array(np.float32(tiny * 0.5)).view(np.uint32)
    if tb > 1:
        vals += list(f32_bits([tb - 1, tb + 1]))
    if to_max < 128:
        mx = np.float32((2 - 2.0 ** -m) * 2.0 ** to_max) if to_max < 128 else np.float32(np.inf)
        if np.isfinite(mx):
            mb = np.array(mx).view(np.uint32)
            vals += list(f32_bits([mb, mb + 1, mb + (1 << max(d - 1, 0)), mb - 1]))
            vals += [-mx, mx * 1.25, -mx * 1.25]
    # specials
    vals += list(f32_bits([0, 0x80000000, 1, 0x80000001, 0x00800000, 0x80800000, 0x7F7FFFFF,
                           0xFF7FFFFF, 0x7F800000, 0xFF800000, 0x7FC00000, 0xFFC00000,
                           0x7F800001, 0x7FFFFFFF, 0x007FFFFF, 0x00400000]))
    # FP32 subnormal inputs
    vals += list(f32_bits(rng.integers(1, 1 << 23, 24, dtype=np.uint32) |
                          (rng.integers(0, 2, 24, dtype=np.uint32) << 31)))
    arr = np.array(vals, np.float32)
    if arr.size < n:
        extra = (rng.standard_normal(n - arr.size) * 2.0 ** rng.integers(-20, 21, n - arr.size))
        arr = np.concatenate([arr, extra.astype(np.float32)])
    return arr[:n].copy()


def inputs_f64(rng, f, n=512):
    m, to_max, to_min, tiny = consts(f)
    base = inputs_f32(rng, f, n // 2).astype(np.float64)
    vals = list(base)
    vals += list(rng.standard_normal(60) * 2.0 ** rng.integers(-300, 300, 60))
    d = 52 - m
    if d > 0:
        for _ in range(30):
            ee = int(rng.integers(max(to_min, -1022), min(to_max, 1023) + 1))
            b = np.array((1 + rng.random()) * 2.0 ** ee).view(np.uint64)
            b = (b & ~np.uint64((1 << d) - 1)) | np.uint64(1 << (d - 1))
            vals += list(f64_bits([b, b + np.uint64(1), b - np.uint64(1)]))
    vals += list(f64_bits([0, 1 << 63, 1, (1 << 63) | 1, 0x0010000000000000, 0x7FEFFFFFFFFFFFFF,
                           0x7FF0000000000000, 0xFFF0000000000000, 0x7FF8000000000000,
                           0x7FF0000000000001, 0x000FFFFFFFFFFFFF]))
    vals += [tiny * (1 - 2.0 ** -30), tiny * (1 + 2.0 ** -30), tiny * 0.5 * (1 + 2.0 ** -40),
             tiny * 0.5 * (1 - 2.0 ** -40)]
    arr = np.array(vals, np.float64)
    if arr.size < n:
        arr = np.concatenate([arr, rng.standard_normal(n - arr.size)])
    return arr[:n].copy()


def inputs_f16(rng, n=512):
    v = rng.integers(0, 1 << 16, n - 16, dtype=np.uint16)
    sp = np.array([0, 0x8000, 1, 0x8001, 0x03FF, 0x0400, 0x7BFF, 0xFBFF, 0x7C00, 0xFC00, 0x7E00,
                   0x7C01, 0x3C00, 0x3C01, 0x3E00, 0x4100], np.uint16)
    return np.concatenate([sp, v])


def stoch_len_for(mode, min_shift):
    if mode not in LEN_MODES:
        return 0
    return int(max(1, min(8, min_shift)))


def min_shift_fmt(f, src_m):
    """Smallest RoundMantissa shift the format overload can hit (normal path d,
    or 1 in the subnormal branch when d == 0)."""
    m = f[1]
    d = src_m - m
    return d if d > 0 else 1


def gen_round(R, rng, out):
    # f32 format overload
    for name, f in F32_FORMATS.items():
        x = inputs_f32(rng, f)
        rec = {"x": x}
        for mode in MODES:
            ln = stoch_len_for(mode, min_shift_fmt(f, 23))
            y = np.empty_like(x)
            seeds = rb = us = None
            if mode in STOCH:
                seeds = rng.integers(1, 2**32 - 1, x.size, dtype=np.uint32)
                rb = np.zeros(x.size, np.uint64)
                us = np.zeros(x.size, np.float64)
            R.ref_round_f32(p(x), p(y), x.size, f[0], f[1], f[2], int(f[3]), 0, 0 if f[4] else 1,
                            mode, ln, p(seeds), p(rb), p(us))
            rec[f"y{mode}"] = y
            rec[f"len{mode}"] = np.int32(ln)
            if mode in STOCH:
                rec[f"r{mode}"] = rb
                rec[f"u{mode}"] = us
        rec["fmt"] = np.array(f, np.int64)
        out[f"round_f32_{name}"] = rec
    # f64 format overload
    for name, f in F64_FORMATS.items():
        x = inputs_f64(rng, f)
        rec = {"x": x}
        for mode in MODES:
            ln = stoch_len_for(mode, min_shift_fmt(f, 52))
            y = np.empty_like(x)
            seeds = rb = us = None
            if mode in STOCH:
                seeds = rng.integers(1, 2**32 - 1, x.size, dtype=np.uint32)
                rb = np.zeros(x.size, np.uint64)
                us = np.zeros(x.size, np.float64)
            if mode == 9:
                # the reference computes the SR-C addend in 32-bit unsigned
                # (src/lo_float.h:809-810); on 64-bit sources the shift reaches
                # 32 in the normal or subnormal branch, which is undefined
                continue
            R.ref_round_f64(p(x), p(y), x.size, f[0], f[1], f[2], int(f[3]), 0, 0 if f[4] else 1,
                            mode, ln, p(seeds), p(rb), p(us))
            rec[f"y{mode}"] = y
            rec[f"len{mode}"] = np.int32(ln)
            if mode in STOCH:
                rec[f"r{mode}"] = rb
                rec[f"u{mode}"] = us
        rec["fmt"] = np.array(f, np.int64)
        out[f"round_f64_{name}"] = rec
    # mantissa overload
    for t, ms, src_m in (("f32", (0, 3, 7, 10, 22, 23), 23), ("f64", (10, 23, 40, 52), 52),
                         ("f16", (3, 7, 10), 10)):
        for mb in ms:
            if t == "f32":
                x = inputs_f32(rng, (32, mb, 127, False, True))
            elif t == "f64":
                x = inputs_f64(rng, (64, mb, 1023, False, True))
            else:
                x = inputs_f16(rng)
            ro = src_m - mb
            rec = {"x": x}
            for mode in MODES:
                if ro == 0 and mode in (3, 7, 14):
                    continue  # reference shifts by a negative count here (undefined)
                ln = stoch_len_for(mode, ro) if ro > 0 else 0
                if mode == 9 and t == "f64" and ro - ln + 1 >= 32:
                    continue
                y = np.empty_like(x)
                seeds = rb = us = None
                if mode in STOCH:
                    seeds = rng.integers(1, 2**32 - 1, x.size, dtype=np.uint32)
                    rb = np.zeros(x.size, np.uint64)
                    us = np.zeros(x.size, np.float64)
                getattr(R, f"ref_round_mantissa_{t}")(p(x), p(y), x.size, mb, mode, ln, p(seeds),
                                                      p(rb), p(us))
                rec[f"y{mode}"] = y
                rec[f"len{mode}"] = np.int32(ln)
                if mode in STOCH:
                    rec[f"r{mode}"] = rb
                    rec[f"u{mode}"] = us
            rec["mbits"] = np.int32(mb)
            out[f"mant_{t}_m{mb}"] = rec


MX_CASES = [
    # (block, elem, scale, mode) — the combinations of
    # test/test_virtual_mx_round_cuda.cu:139-152 plus the E2M1 / E4M3 / E5M2
    # formats of the 8192 x 8192 MX rounding workload
    (32, "e4m3", "e8m0", 0), (8, "e4m3", "e8m0", 5), (16, "e5m2", "e8m0", 6),
    (128, "e4m3", "e8m0", 0), (64, "e4m3", "e5m2s", 1), (128, "e5m2", "e8m0", 0),
    (256, "e4m3", "e8m0", 5), (256, "e5m2", "e8m0", 0), (32, "e2m1", "e8m0", 0),
    (32, "e5m2", "e8m0", 0),
]
MX_FMTS = {"e4m3": (8, 3, 7, True, True), "e5m2": (8, 2, 15, True, True),
           "e2m1": (4, 1, 1, True, True), "e8m0": (8, 0, 127, False, False),
           "e5m2s": (8, 2, 15, True, True)}


def rnd_wide(rng, n):
    u = (rng.random(n) + 1e-7).astype(np.float32)
    e = rng.integers(-10, 11, n)
    s = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    return (s * np.ldexp(u, e)).astype(np.float32)


def gen_mx(R, rng, out):
    for (bs, en, sn, mode) in MX_CASES:
        ef, sf = MX_FMTS[en], MX_FMTS[sn]
        for n in (bs, 3 * bs + 1, 1000, 5003):
            x = rnd_wide(rng, n)
            if n == 5003:
                x[:bs] = 0.0  # an all-zero block must give zeros, not NaN
                x[bs + 3] = np.inf
                x[2 * bs + 1] = np.nan
            rec = {"x": x, "case": np.array([bs, mode, 0], np.int64),
                   "ef": np.array(ef, np.int64), "sf": np.array(sf, np.int64)}
            ys = []
            for formula in (0, 1):
                y = np.empty_like(x)
                R.ref_mx_round_f32(p(x), p(y), n, bs, ef[0], ef[1], ef[2], int(ef[3]),
                                   0 if ef[4] else 1, sf[0], sf[1], sf[2], int(sf[3]),
                                   0 if sf[4] else 1, mode, 0, formula)
                ys.append(y)
            rec["y"] = ys[0]  # GPU scale expression amax * (1/pmn)
            # elements where the CPU expression amax / pmn gives a different result
            rec["cpu_formula_diff"] = np.int64(np.sum(ys[0].view(np.uint32) != ys[1].view(np.uint32)))
            out[f"mx_b{bs}_{en}_{sn}_m{mode}_n{n}"] = rec
    # the 8192 x 8192 workload's distribution: N(0,1) with 1% outliers scaled
    # by 2^12, blocks of 32, on 16384 values
    x = rng.standard_normal(16384).astype(np.float32)
    x[rng.random(16384) < 0.01] *= 4096.0
    for en in ("e2m1", "e4m3", "e5m2"):
        ef, sf = MX_FMTS[en], MX_FMTS["e8m0"]
        rec = {"x": x, "case": np.array([32, 0, 0], np.int64), "ef": np.array(ef, np.int64),
               "sf": np.array(sf, np.int64)}
        ys = []
        for formula in (0, 1):
            y = np.empty_like(x)
            R.ref_mx_round_f32(p(x), p(y), x.size, 32, ef[0], ef[1], ef[2], int(ef[3]), 0,
                               sf[0], sf[1], sf[2], int(sf[3]), 1, 0, 0, formula)
            ys.append(y)
        rec["y"] = ys[0]
        rec["cpu_formula_diff"] = np.int64(np.sum(ys[0].view(np.uint32) != ys[1].view(np.uint32)))
        out[f"mx_outliers_{en}"] = rec


def gen_gemm(R, rng, out):
    e4m3, e8m0 = O.fmt(8, 3, 7), O.fmt(8, 0, 127, saturating=False, signed=False)
    cases = []
    # MX-E4M3 operands along K (the 4096^3 GEMM workload's scheme), 10-bit accumulator
    A = O.mx_round(rng.standard_normal((24, 256)).astype(np.float32), 32, e4m3, e8m0)
    Bt = O.mx_round(rng.standard_normal((20, 256)).astype(np.float32), 32, e4m3, e8m0)
    cases.append(("mx_e4m3_m10", A, np.ascontiguousarray(Bt.T), 10, 1.0))
    # U(-1,1) operands as in test/gemm_test.cu:233-248, several accumulator widths
    A = rng.uniform(-1, 1, (13, 97)).astype(np.float32)
    B = rng.uniform(-1, 1, (97, 11)).astype(np.float32)
    for mb in (7, 12, 23):
        cases.append((f"unif_m{mb}", A, B, mb, 1.0))
    cases.append(("unif_m10_alpha", A, B, 10, float(np.float32(1.0) / (np.float32(0.5) * np.float32(3.0)))))
    # exactly representable small integers: result independent of accumulation
    A = rng.integers(-4, 5, (8, 64)).astype(np.float32)
    B = rng.integers(-4, 5, (64, 8)).astype(np.float32)
    cases.append(("exact_ints_m10", A, B, 10, 1.0))
    # cancellation to exact zero (signed-zero behaviour of the device leaf)
    A = np.array([[1.0, -1.0, 2.0, -2.0], [0.0, -0.0, 0.0, -0.0]], np.float32)
    B = np.array([[1.0, -1.0], [1.0, -1.0], [1.0, 0.0], [1.0, -0.0]], np.float32)
    cases.append(("signed_zero_m10", A, B, 10, 1.0))
    for name, A, B, mb, alpha in cases:
        M, K = A.shape
        N = B.shape[1]
        D = np.empty((M, N), np.float32)
        R.ref_gemm_f32(p(A), p(B), p(D), M, N, K, mb, alpha)
        out[f"gemm_{name}"] = {"A": A, "B": B, "D": D, "mbits": np.int32(mb),
                               "alpha": np.float32(alpha)}


CODEC_FORMATS = {
    # P3109 <k, p> with the reference's P_3109 checkers
    "p3109_8_4": dict(kind="p3109", k=8, p=4),
    "p3109_8_4_ext": dict(kind="p3109", k=8, p=4, saturating=False),
    "p3109_8_3": dict(kind="p3109", k=8, p=3),
    "p3109_7_3": dict(kind="p3109", k=7, p=3),
    "p3109_6_3": dict(kind="p3109", k=6, p=3),
    "p3109_5_2_ext": dict(kind="p3109", k=5, p=2, saturating=False),
    "p3109_4_2": dict(kind="p3109", k=4, p=2),
    "p3109_3_2": dict(kind="p3109", k=3, p=2),
    "p3109_2_1": dict(kind="p3109", k=2, p=1),
    "p3109_8_4_unsigned": dict(kind="p3109", k=8, p=4, signed=False),
    "p3109_8_4_unsigned_ext_negnan": dict(kind="p3109", k=8, p=4, signed=False, saturating=False,
                                          neg_to_nan=True),
    "p3109_10_4": dict(kind="p3109", k=10, p=4),
    "p3109_12_6_ext": dict(kind="p3109", k=12, p=6, saturating=False),
    "p3109_16_9": dict(kind="p3109", k=16, p=9),
    # IEEE-style checkers (src/fp_tools.hpp:334-395)
    "fp16": dict(kind="ieee", bw=16, m=10, bias=15, qnan=0x7E00, snan=0x7C01),
    "bf16": dict(kind="ieee", bw=16, m=7, bias=127, qnan=0x7FC0, snan=0x7F81),
    # OCP E8M0 (src/lo_float.h:1773-1790) and a format without specials
    "e8m0": dict(kind="raw", args=(8, 0, 127, True, False, False, 0, 0xFFFFFFFF, 0, 0, 0xFF, 0xFF, 0, False)),
    "nospecial_9_3": dict(kind="raw", args=(9, 3, 200, True, True, False, 0, 0xFFFFFFFF, 0, 0, 0, 0, 2, False)),
}
CODEC_DET_MODES = [0, 1, 2, 4, 5, 6, 7, 12, 13]


def codec_format(spec):
    if spec["kind"] == "p3109":
        return O.codec_p3109(spec["k"], spec["p"], signed=spec.get("signed", True),
                             saturating=spec.get("saturating", True),
                             neg_to_nan=spec.get("neg_to_nan", False))
    if spec["kind"] == "ieee":
        return O.codec_ieee(spec["bw"], spec["m"], spec["bias"], spec["qnan"], spec["snan"])
    return O.codec_fmt(*spec["args"])


def codec_probes(f, rng):
    """Every finite value of the format, its float neighbours and midpoints,
    specials, FP32 subnormals and wide random values."""
    n = f.fmt.bitwidth
    vals = np.array([O.decode_rep(r, f) for r in range(1 << n)], np.float32)
    fin = np.unique(vals[np.isfinite(vals)])
    if fin.size > 600:
        fin = fin[np.linspace(0, fin.size - 1, 600).astype(int)]
    parts = [fin, np.nextafter(fin, np.float32(np.inf)), np.nextafter(fin, np.float32(-np.inf)),
             (0.5 * (fin[1:].astype(np.float64) + fin[:-1])).astype(np.float32),
             np.array([0.0, -0.0, 1e30, -1e30, np.inf, -np.inf, np.nan, -np.nan, 1e-40, -1e-40,
                       1.4e-45, 3e38, -3e38, 2.0 ** -126, 2.0 ** -127], np.float32),
             (rng.standard_normal(800) * 2.0 ** rng.integers(-40, 40, 800)).astype(np.float32)]
    return np.concatenate(parts).astype(np.float32)


def gen_codec(R, rng, out):
    """convert_float_to_rep / convert_rep_to_float and the packing of
    src/lo_pack.hpp, run through the reference's LoF_encode / LoF_decode."""
    for name, spec in CODEC_FORMATS.items():
        f = codec_format(spec)
        cf = O.codec_fields(f)
        n = f.fmt.bitwidth
        x = codec_probes(f, rng)
        rec = {"fields": cf, "x": x}
        for mode in CODEC_DET_MODES:
            for sat in ((0, 1, 2) if mode == 0 else (0,)):
                for rev in ((0, 1) if mode == 0 else (0,)):
                    buf = np.zeros(int(R.ref_packed_size(n, x.size)), np.uint8)
                    R.ref_encode_f32(p(buf), p(x), x.size, p(cf), mode, sat, 0, rev)
                    rec[f"enc_m{mode}_s{sat}_r{rev}"] = buf
        raw = rng.integers(0, 256, int(R.ref_packed_size(n, 2048)), dtype=np.uint8)
        rec["raw"] = raw
        for rev in (0, 1):
            dec = np.empty(2048, np.float32)
            R.ref_decode_f32(p(dec), p(raw), 2048, p(cf), rev)
            rec[f"dec_r{rev}"] = dec
        out[f"codec_{name}"] = rec


def main():
    R = O.ref()
    if R is None:
        raise SystemExit("reference sources not found; set LOFGB_REFERENCE")
    rng = np.random.default_rng(20261203)
    out = {}
    gen_round(R, rng, out)
    gen_mx(R, rng, out)
    gen_gemm(R, rng, out)
    gen_codec(R, np.random.default_rng(20261204), out)
    groups = {"round": {}, "mant": {}, "mx": {}, "gemm": {}, "codec": {}}
    for k, v in out.items():
        groups[k.split("_")[0]][k] = v
    manifest = {"generator": "python tests/golden/make_golden.py",
                "reference": "SudhanvaKulkarni123/LoFloat src/lo_float.h scalar virtual_round, "
                             "src/lo_pack.hpp codec (via oracle/ref_shim.cpp)", "files": {}}
    for g, cases in groups.items():
        flat = {}
        for cname, rec in cases.items():
            for k, v in rec.items():
                flat[f"{cname}__{k}"] = np.asarray(v)
        path = os.path.join(HERE, f"golden_{g}.npz")
        np.savez_compressed(path, **flat)
        with open(path, "rb") as fh:
            sha = hashlib.sha256(fh.read()).hexdigest()
        manifest["files"][os.path.basename(path)] = {"sha256": sha, "cases": sorted(cases)}
        print(path, len(cases), "cases", os.path.getsize(path), "bytes")
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
