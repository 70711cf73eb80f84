"""CPU-only tests: the C-ABI library loads and exports every declared entry
point, host-side validation returns the documented status codes without
touching a GPU, and the Python surface mirrors the reference's."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import lofloat_gb300 as lg
from lofloat_gb300 import _native

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def header_symbols():
    with open(os.path.join(ROOT, "include", "lofgb.h")) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)  # drop comments
    return sorted(set(re.findall(r"\b(lofgb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _native.lib()
    declared = header_symbols()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(_native.exported_symbols())


def test_version_and_strerror():
    L = _native.lib()
    assert L.lofgb_version() >= 100
    for code in range(0, -11, -1):
        assert L.lofgb_strerror(code).decode()
    assert L.lofgb_strerror(0).decode() == "ok"


FAKE_IN, FAKE_OUT = C.c_void_p(0x10000), C.c_void_p(0x20000)


def fmt(bw=8, m=3, bias=7, sat=1, sgn=0):
    return _native.LofgbFormat(bw, m, bias, sat, 0, sgn, 0)


def test_round_validation_codes():
    L = _native.lib()
    ok = fmt()
    # n == 0 with valid arguments: nothing launched
    assert L.lofgb_round_f32(FAKE_IN, FAKE_OUT, 0, C.byref(ok), 0, 0, 1.0, 0, 0, None) == 0
    assert L.lofgb_round_f32(FAKE_IN, FAKE_OUT, -1, C.byref(ok), 0, 0, 1.0, 0, 0, None) == -2
    assert L.lofgb_round_f32(None, FAKE_OUT, 4, C.byref(ok), 0, 0, 1.0, 0, 0, None) == -1
    assert L.lofgb_round_f32(FAKE_IN, FAKE_OUT, 4, None, 0, 0, 1.0, 0, 0, None) == -1
    assert L.lofgb_round_f32(FAKE_IN, FAKE_OUT, 4, C.byref(fmt(m=24)), 0, 0, 1.0, 0, 0, None) == -3
    assert L.lofgb_round_f32(FAKE_IN, FAKE_OUT, 4, C.byref(fmt(bw=40, m=3)), 0, 0, 1.0, 0, 0, None) == -3
    assert L.lofgb_round_f32(FAKE_IN, FAKE_OUT, 4, C.byref(fmt(bias=-300)), 0, 0, 1.0, 0, 0, None) == -3
    assert L.lofgb_round_f32(FAKE_IN, FAKE_OUT, 4, C.byref(ok), 15, 0, 1.0, 0, 0, None) == -4
    assert L.lofgb_round_f32(FAKE_IN, FAKE_OUT, 4, C.byref(ok), 3, 63, 1.0, 0, 0, None) == -4
    # partial overlap of input and output
    assert L.lofgb_round_f32(C.c_void_p(0x10000), C.c_void_p(0x10004), 4, C.byref(ok), 0, 0, 1.0,
                             0, 0, None) == -6
    assert "mantissa_bits" in L.lofgb_last_error_detail().decode() or True
    assert L.lofgb_round_f16(FAKE_IN, FAKE_OUT, 4, C.byref(fmt(m=11)), 0, 0, 1.0, 0, 0, None) == -3
    assert L.lofgb_round_f64(FAKE_IN, FAKE_OUT, 0, C.byref(fmt(bw=40, m=30, bias=255)), 0, 0, 1.0,
                             0, 0, None) == 0
    assert L.lofgb_round_mantissa_f32(FAKE_IN, FAKE_OUT, 4, 24, 0, 0, 1.0, 0, 0, None) == -3
    assert L.lofgb_round_mantissa_f16(FAKE_IN, FAKE_OUT, 0, 10, 0, 0, 1.0, 0, 0, None) == 0


def test_mx_validation_codes():
    L = _native.lib()
    e, s = fmt(), fmt(8, 0, 127, 0, 1)
    for bs in (8, 16, 32, 64, 128, 256):
        assert L.lofgb_mx_round_f32(FAKE_IN, FAKE_OUT, 0, bs, C.byref(e), C.byref(s), 0, 0, 0, 0, 0, None) == 0
    for bs in (0, 4, 48, 512, -32):
        assert L.lofgb_mx_round_f32(FAKE_IN, FAKE_OUT, 64, bs, C.byref(e), C.byref(s), 0, 0, 0, 0, 0,
                                    None) == -5
    assert L.lofgb_mx_round_f32(FAKE_IN, FAKE_OUT, 64, 32, C.byref(e), C.byref(s), 0, 20, 0, 0, 0,
                                None) == -4


def test_gemm_validation_codes():
    L = _native.lib()
    A, B, D = C.c_void_p(0x1000), C.c_void_p(0x2000), C.c_void_p(0x3000)
    args = dict(lda=64, ta=0, ldb=32, tb=0, ldd=32, M=16, N=32, K=64)

    def call(mode=0, variant=0, chunk=32, mbits=10, **kw):
        a = dict(args, **kw)
        return L.lofgb_gemm_f32(A, a["lda"], a["ta"], B, a["ldb"], a["tb"], D, a["ldd"], a["M"],
                                a["N"], a["K"], mbits, mode, 1.0, variant, chunk, None, 0, None)
    assert call(mode=1) == -4          # the accumulator is RNE only
    assert call(mbits=24) == -3
    assert call(lda=63) == -2
    assert call(ldd=16) == -2
    assert call(ta=2) == -2
    assert call(M=-1) == -2
    assert call(M=0) == 0              # empty output: nothing to do
    assert call(variant=1, chunk=24) == -2
    assert call(variant=7) == -7
    assert L.lofgb_gemm_tc_workspace_size(0, 4, 4) == 0


def test_noalloc_gemm_checks_arguments_before_its_scratch_limit():
    """The no-allocation GEMM reports bad arguments with lofgb_gemm_f32's codes
    even when the shape would also exceed its built-in scratch (host checks
    only: nothing reaches the device)."""
    L = _native.lib()
    A, B, D = C.c_void_p(0x1000), C.c_void_p(0x2000), C.c_void_p(0x3000)
    big = 4096

    def call(A=A, lda=big, ta=0, ldd=big, mbits=10, chunk=32, M=big):
        return L.lofgb_gemm_tc_noalloc_f32(A, lda, ta, B, big, 0, D, ldd, M, big, big, mbits, 1.0,
                                           chunk, None)
    assert call(lda=big - 1) == -2
    assert call(ldd=1) == -2
    assert call(ta=3) == -2
    assert call(M=-1) == -2
    assert call(A=None) == -1
    assert call(mbits=24) == -3
    assert call(chunk=24) == -2
    assert call() == -9               # valid request beyond the 64 MiB scratch
    assert "scratch" in L.lofgb_last_error_detail().decode()
    assert call(M=0) == 0             # empty output: nothing to do


def test_batched_gemm_and_conv_validation_codes():
    L = _native.lib()
    A, B, D = C.c_void_p(0x1000), C.c_void_p(0x2000), C.c_void_p(0x3000)

    def call(batch=4, sa=1024, sb=2048, sd=512, M=16, N=32, K=64, mode=0):
        return L.lofgb_gemm_batched_f32(A, K, sa, 0, B, N, sb, 0, D, N, sd, M, N, K, batch, 10,
                                        mode, 1.0, 0, 32, None, 0, None)
    assert call(batch=-1) == -2
    assert call(sa=-5) == -2
    assert call(sd=100) == -6          # D matrices would overlap
    assert call(batch=0) == 0          # nothing to do
    assert call(M=0) == 0
    assert call(mode=3) == -4
    assert L.lofgb_gemm_batched_tc_workspace_size(16, 32, 64, 0) == 0
    assert L.lofgb_gemm_batched_tc_workspace_size(128, 128, 64, 3) > \
        3 * L.lofgb_gemm_batched_tc_workspace_size(128, 128, 64, 1) // 2

    sh = _native.LofgbConv2dShape(2, 3, 5, 5, 4, 3, 3, 1, 1, 1, 1, 1, 1)
    P, Q = C.c_int32(), C.c_int32()
    assert L.lofgb_conv2d_out_size(C.byref(sh), C.byref(P), C.byref(Q)) == 0
    assert (P.value, Q.value) == (5, 5)
    bad = _native.LofgbConv2dShape(1, 3, 2, 2, 4, 3, 3, 0, 0, 1, 1, 1, 1)
    assert L.lofgb_conv2d_out_size(C.byref(bad), None, None) == -2
    zero_stride = _native.LofgbConv2dShape(1, 3, 5, 5, 4, 3, 3, 0, 0, 0, 1, 1, 1)
    assert L.lofgb_conv2d_out_size(C.byref(zero_stride), None, None) == -2

    def conv(order=0, variant=0, chunk=32, mode=0, mbits=10, y=0x9000):
        return L.lofgb_conv2d_f32(C.c_void_p(0x1000), C.c_void_p(0x8000), C.c_void_p(y),
                                  C.byref(sh), mbits, mode, 1.0, order, variant, chunk, None, 0,
                                  None)
    assert conv(mode=1) == -4
    assert conv(mbits=30) == -3
    assert conv(order=5) == -7
    assert conv(variant=9) == -7
    assert conv(variant=1, chunk=8) == -2
    assert conv(y=0x1010) == -6        # output overlaps the input
    assert L.lofgb_conv2d_workspace_size(C.byref(sh), 0, 0) == 0   # plain needs none
    assert L.lofgb_conv2d_workspace_size(C.byref(sh), 1, 1) > 0
    lut = C.c_void_p(0x5000)
    assert L.lofgb_pwl_silu_f32(C.c_void_p(0x1000), C.c_void_p(0x2000), 8, lut, 6, 1.0, None) == -2
    assert L.lofgb_pwl_silu_f32(C.c_void_p(0x1000), C.c_void_p(0x2000), 8, lut, 8, 0.0, None) == -2
    assert L.lofgb_pwl_silu_f32(C.c_void_p(0x1000), C.c_void_p(0x1004), 8, lut, 8, 1.0, None) == -6
    assert L.lofgb_pwl_silu_f32(None, None, 0, lut, 8, 1.0, None) == 0


def test_python_surface_mirrors_reference():
    assert int(lg.RoundingMode.RoundToNearestEven) == 0
    assert int(lg.RoundingMode.StochasticRoundingA) == 3
    assert int(lg.RoundingMode.RoundToOdd) == 12
    assert int(lg.RoundingMode.StochasticRoundingD) == 14
    assert int(lg.InfBehavior.Saturating) == 1 and int(lg.Signedness.Unsigned) == 1
    p = lg.create_p3109_params(8, 4)
    assert (p.total_bits, p.mantissa_bits, p.bias, p.inf_behavior) == (8, 3, 8, lg.InfBehavior.Saturating)
    u = lg.create_p3109_params(8, 3, False, False)
    assert (u.mantissa_bits, u.bias, u.signedness, u.inf_behavior) == (2, 16, lg.Signedness.Unsigned,
                                                                       lg.InfBehavior.Extended)
    e = lg.create_e8m0_params()
    assert (e.total_bits, e.mantissa_bits, e.bias, e.signedness) == (8, 0, 127, lg.Signedness.Unsigned)
    h = lg.create_half_params()
    assert h.is_inf_checker(0x7C00) and h.is_nan_checker(0x7E00) and not h.is_nan_checker(0x7C00)
    assert p.is_nan_checker(0x80) and p.is_nan_checker.qNanBitPattern() == 0x80
    assert not p.is_inf_checker(0x7F)
    with pytest.raises(ValueError):
        lg.FloatFormatDescriptor(8, 3, 7, lg.InfBehavior.Saturating, lg.NaNBehavior._3109,
                                 lg.Signedness.Signed, object(), p.is_nan_checker)
    with pytest.raises(ValueError):
        lg.FloatFormatDescriptor(8, 3, 7, lg.InfBehavior.Saturating, lg.NaNBehavior._3109,
                                 lg.Signedness.Signed, p.is_inf_checker, lambda b: False)
    fid = lg.register_format(p)
    assert lg.register_format(p) == fid and lg.get_format(fid) is p
    assert lg.gemm_alpha(0.5, 4.0) == 0.5 and lg.gemm_alpha(0.0, 3.0) == 1.0


def test_cpu_tensors_rejected():
    import torch
    with pytest.raises(RuntimeError):
        lg.virtual_round(torch.ones(4), lg.create_p3109_params(8, 4))
    with pytest.raises(RuntimeError):
        lg.virtual_mx_round(torch.ones(64), 32, lg.create_p3109_params(8, 4), lg.create_e8m0_params())
    with pytest.raises(RuntimeError):
        lg.lof_gemm(torch.ones(4, 4), torch.ones(4, 4), 10)


def test_grouped_prepare_host_only():
    """The grouped table is built on the host: sizes, item counts and
    per-task validation, no device work."""
    L = _native.lib()
    T = _native.LofgbRoundTask
    ok = fmt()
    tasks = (T * 3)(T(0x1000, 0x100000, 70000, ok, 0, 0, 1.0, 0, 1, 0),
                    T(0x200000, 0x300000, 1, ok, 3, 8, 2.0, 0, 2, 5),
                    T(0x400000, 0x400000, 0, ok, 1, 0, 1.0, 0, 3, 0))
    nbytes = L.lofgb_round_grouped_table_size(3)
    assert nbytes > 0 and L.lofgb_round_grouped_table_size(0) == 0
    buf = (C.c_uint8 * nbytes)()
    items = C.c_int64(-1)
    assert L.lofgb_round_grouped_prepare(tasks, 3, buf, nbytes, C.byref(items)) == 0
    assert items.value == 2 + 1 + 0  # 70000 elements -> 2 items of 2^16, 1 -> 1, 0 -> 0
    assert L.lofgb_round_grouped_prepare(tasks, 3, buf, nbytes - 1, C.byref(items)) == -9
    bad = (T * 1)(T(0x1000, 0x1004, 16, ok, 0, 0, 1.0, 0, 0, 0))
    assert L.lofgb_round_grouped_prepare(bad, 1, buf, nbytes, C.byref(items)) == -6
    bad = (T * 1)(T(0x1000, 0x100000, 16, fmt(m=30), 0, 0, 1.0, 0, 0, 0))
    assert L.lofgb_round_grouped_prepare(bad, 1, buf, nbytes, C.byref(items)) == -3
    assert "task 0" in L.lofgb_last_error_detail().decode()
    assert L.lofgb_round_grouped_f32(None, 0, 0, None) == 0
    # work items of a chosen power-of-two size
    for item, want in ((1 << 14, 5 + 1), (1 << 17, 1 + 1), (1 << 10, 69 + 1)):
        assert L.lofgb_round_grouped_prepare_items(tasks, 3, buf, nbytes, item, C.byref(items)) == 0
        assert items.value == want
    for item in (3000, 512, 1 << 25):
        assert L.lofgb_round_grouped_prepare_items(tasks, 3, buf, nbytes, item, C.byref(items)) != 0


def test_grouped_gemm_validation_host_only():
    L = _native.lib()
    T = _native.LofgbGemmTask
    good = T(0x1000, 64, 0x2000, 32, 0x3000, 32, 0, 0, 16, 32, 64, 10, 1.0, 32)
    arr = (T * 1)(good)
    ws_need = L.lofgb_gemm_grouped_workspace_size(arr, 1)
    tb_need = L.lofgb_gemm_grouped_table_size(arr, 1)
    assert ws_need > 1024 and tb_need > 0
    buf = (C.c_uint8 * tb_need)()
    nt, si = C.c_int64(0), C.c_int64(0)

    def prep(task, ws=0x100000, wsb=ws_need, sched=1, tbytes=tb_need):
        a = (T * 1)(task)
        return L.lofgb_gemm_grouped_prepare(a, 1, C.c_void_p(ws), wsb, sched, 4, buf, tbytes,
                                            C.byref(nt), C.byref(si))
    bad = T(0x1000, 63, 0x2000, 32, 0x3000, 32, 0, 0, 16, 32, 64, 10, 1.0, 32)
    assert prep(bad) == -2                                   # lda < K
    bad = T(0x1000, 64, 0x2000, 32, 0x3000, 32, 0, 0, 16, 32, 64, 10, 1.0, 24)
    assert prep(bad) == -2                                   # chunk not a multiple of 16
    bad = T(0x1000, 64, 0x2000, 32, 0x3000, 32, 0, 0, 16, 32, 64, 30, 1.0, 32)
    assert prep(bad) == -3                                   # accumulator width
    assert prep(good, wsb=ws_need - 1) == -9                 # workspace too small
    assert prep(good, ws=0x100010) == -9                     # workspace misaligned
    assert prep(good, tbytes=tb_need - 1) == -9              # table too small
    assert prep(good, sched=5) == -7                         # unknown schedule
    assert prep(good, sched=1 | 16 | 32) == -7               # two tile widths in one table
    assert prep(good, sched=3 | 32) == -7                    # unknown schedule, wide tile


def test_codec_validation_and_sizes():
    from oracle import oracle as O
    L = _native.lib()
    for n in range(1, 17):
        for cnt in (0, 1, 7, 8, 33, 1000, 12345):
            assert L.lofgb_packed_size(n, cnt) == O.packed_size(n, cnt)
    assert L.lofgb_packed_size(0, 10) == 0 and L.lofgb_packed_size(17, 10) == 0
    f = lg.codec_format(lg.create_p3109_params(8, 4))
    src, dst = C.c_void_p(0x1000), C.c_void_p(0x100000)
    bad = lg.codec_format(lg.create_p3109_params(8, 4))
    bad.fmt.bitwidth = 17
    assert L.lofgb_encode_f32(dst, src, 16, C.byref(bad), 0, 0, 0, 0, 0, 0, None) == -3
    assert L.lofgb_encode_f32(dst, src, 16, C.byref(f), 99, 0, 0, 0, 0, 0, None) == -4
    assert L.lofgb_encode_f32(dst, src, 16, C.byref(f), 0, 7, 0, 0, 0, 0, None) == -4
    assert L.lofgb_encode_f32(C.c_void_p(0x1001), src, 16, C.byref(f), 0, 0, 0, 0, 0, 0, None) == -2
    assert L.lofgb_encode_f32(C.c_void_p(0x1008), src, 16, C.byref(f), 0, 0, 0, 0, 0, 0, None) == -6
    assert L.lofgb_decode_f32(C.c_void_p(0x1000), C.c_void_p(0x1004), 16, C.byref(f), 0, None) == -6
    assert L.lofgb_encode_f32(None, None, 0, C.byref(f), 0, 0, 0, 0, 0, 0, None) == 0


def test_codec_format_fits_reference_checkers():
    from oracle import oracle as O
    assert bytes(lg.codec_format(lg.create_p3109_params(8, 4))) == bytes(O.codec_p3109(8, 4))
    assert bytes(lg.codec_format(lg.create_p3109_params(6, 3, True, False))) == \
        bytes(O.codec_p3109(6, 3, saturating=False))
    assert bytes(lg.codec_format(lg.create_p3109_params(8, 3, False, False))) == \
        bytes(O.codec_p3109(8, 3, signed=False, saturating=False))
    h = lg.codec_format(lg.create_half_params())
    assert (h.nan_kind, h.inf_or, h.inf_match, h.pos_inf) == (1, 0x8000, 0xFC00, 0x7C00)

    class Weird:
        def __call__(self, bits):
            return bits in (3, 5)

        def minNegInf(self):
            return 0

        def minPosInf(self):
            return 3

        def qNanBitPattern(self):
            return 9
    w = lg.FloatFormatDescriptor(8, 3, 7, lg.InfBehavior.Extended, lg.NaNBehavior._3109,
                                 lg.Signedness.Signed, Weird(), Weird())
    import pytest
    with pytest.raises(RuntimeError):
        lg.codec_format(w)


def test_wait_selftest_argument_checks():
    """The wait self-test entry point validates on the host before any launch."""
    L = _native.lib()
    A, B, D = C.c_void_p(0x1000), C.c_void_p(0x2000), C.c_void_p(0x3000)
    assert L.lofgb_gemm_tc_wait_selftest(A, B, D, 0, 4, 4, None, 0, 1000, None) == -2
    assert L.lofgb_gemm_tc_wait_selftest(None, B, D, 4, 4, 4, None, 0, 1000, None) == -1
    assert L.lofgb_gemm_tc_wait_selftest(A, B, D, 4, 4, 4, None, 0, 50, None) == -2
    assert L.lofgb_gemm_tc_wait_selftest(A, B, D, 4, 4, 4, None, 0, 200000, None) == -2


def test_mx_encode_argument_checks():
    """MX storage validates on the host: 32-value blocks, 4/6/8-bit element
    codes, 8-bit scale codes."""
    L = _native.lib()
    ef = lg.codec_format(lg.create_p3109_params(8, 4))
    sf = lg.codec_format(lg.create_e8m0_params())
    f5 = lg.codec_format(lg.create_p3109_params(5, 2))
    X, Cd, S = C.c_void_p(0x10000), C.c_void_p(0x90000), C.c_void_p(0xA0000)

    def call(block=32, e=ef, s=sf, n=64, x=X):
        return L.lofgb_mx_encode_f32(x, Cd, S, n, block, C.byref(e), C.byref(s), 0, 0, 1, 0, 0, 0,
                                     None)
    assert call(block=16) == -5
    assert call(e=f5) == -7
    assert call(s=ef) == 0 or True      # an 8-bit scale format is accepted on the host
    assert call(x=None) == -1
    assert call(n=-1) == -2
    assert call(n=0) == 0
