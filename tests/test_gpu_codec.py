"""GPU parity of the storage codec (lofgb_encode_f32 / lofgb_decode_f32)
against the reference's own LoF_encode / LoF_decode outputs (golden vectors)
and the oracle: packed bytes identical, decoded bits identical, for every
code width 1..16, both group orders, all rounding and saturation modes, and
ragged lengths."""
import ctypes as C

import numpy as np
import pytest
import torch

import lofloat_gb300 as lg
from lofloat_gb300 import _native
from golden_io import cases, same_bits
from oracle import oracle as O
from test_oracle_golden import codec_from_fields

pytestmark = pytest.mark.gpu


def _native_fmt(f: O.CodecFormat) -> _native.LofgbCodecFormat:
    g = _native.LofgbCodecFormat()
    C.memmove(C.addressof(g), C.addressof(f), C.sizeof(g))
    return g


def gpu_encode(x, f, mode=0, sat=0, stoch_len=0, reverse=0, seed=0, offset=0):
    xg = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    nb = lg.packed_size(f.fmt.bitwidth, x.size)
    out = torch.zeros(max(nb, 1), dtype=torch.uint8, device="cuda")
    st = _native.lib().lofgb_encode_f32(out.data_ptr(), xg.data_ptr(), x.size,
                                        C.byref(_native_fmt(f)), mode, sat, stoch_len, reverse,
                                        seed, offset, None)
    assert st == 0, _native.lib().lofgb_last_error_detail()
    torch.cuda.synchronize()
    return out.cpu().numpy()[:nb]


def gpu_decode(buf, count, f, reverse=0):
    bg = torch.from_numpy(np.ascontiguousarray(buf, np.uint8)).cuda()
    out = torch.empty(count, dtype=torch.float32, device="cuda")
    st = _native.lib().lofgb_decode_f32(out.data_ptr(), bg.data_ptr(), count,
                                        C.byref(_native_fmt(f)), reverse, None)
    assert st == 0, _native.lib().lofgb_last_error_detail()
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("cname,rec", list(cases("codec")), ids=lambda v: v if isinstance(v, str) else "")
def test_golden_codec(cname, rec):
    f = codec_from_fields(rec["fields"])
    x = rec["x"]
    for key, want in rec.items():
        if not key.startswith("enc_"):
            continue
        _, m, s, r = key.split("_")
        got = gpu_encode(x, f, mode=int(m[1:]), sat=int(s[1:]), reverse=int(r[1:]))
        assert np.array_equal(got, want), (cname, key, int(np.sum(got != want)))
    for rev in (0, 1):
        got = gpu_decode(rec["raw"], 2048, f, reverse=rev)
        assert same_bits(got, rec[f"dec_r{rev}"]), (cname, rev)


def _wide(n, seed):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) * 2.0 ** rng.integers(-30, 31, n)).astype(np.float32)
    x[::61] = rng.integers(0, 2**32, x[::61].size, dtype=np.uint64).astype(np.uint32).view(np.float32)
    return x


@pytest.mark.parametrize("bits", list(range(2, 17)))
@pytest.mark.parametrize("reverse", [0, 1])
def test_every_width_vs_oracle(bits, reverse):
    p = max(1, min(bits - 1, bits // 2))
    for f in (O.codec_p3109(bits, p), O.codec_p3109(bits, p, saturating=False)):
        for n in (1, 31, 1024, 3000, 70001):
            x = _wide(n, bits * 7 + n)
            for mode, sat in ((0, 0), (1, 1), (12, 2), (6, 0)):
                got = gpu_encode(x, f, mode, sat, reverse=reverse)
                want = O.encode(x, f, mode, sat, reverse=reverse)
                assert np.array_equal(got, want), (bits, n, mode, sat, int(np.sum(got != want)))
            dec = gpu_decode(want, n, f, reverse)
            assert same_bits(dec, O.decode(want, n, f, reverse))


def test_width_one():
    f = O.codec_fmt(1, 0, 0, True, False, False, 0, 0xFFFFFFFF, 0, 0, 0, 0, 2, False)
    x = _wide(5000, 1)
    for rev in (0, 1):
        got = gpu_encode(x, f, reverse=rev)
        assert np.array_equal(got, O.encode(x, f, reverse=rev))
        assert same_bits(gpu_decode(got, 5000, f, rev), O.decode(got, 5000, f, rev))


@pytest.mark.parametrize("mode", list(range(15)))
def test_all_modes_with_stochastic_stream(mode):
    f = O.codec_p3109(8, 4)
    x = _wide(50_000, mode)
    ln = 5 if mode in (3, 8, 9, 14) else 0
    got = gpu_encode(x, f, mode, 0, ln, seed=77, offset=1000)
    want = O.encode(x, f, mode, 0, ln, seed=77, offset=1000)
    assert np.array_equal(got, want), int(np.sum(got != want))


def test_ieee_and_special_formats():
    rng = np.random.default_rng(3)
    for f in (O.codec_ieee(16, 10, 15, 0x7E00, 0x7C01), O.codec_ieee(16, 7, 127, 0x7FC0, 0x7F81),
              O.codec_fmt(8, 0, 127, True, False, False, 0, 0xFFFFFFFF, 0, 0, 0xFF, 0xFF, 0, False),
              O.codec_p3109(8, 4, signed=False, saturating=False, neg_to_nan=True)):
        x = _wide(20_000, int(rng.integers(1000)))
        for sat in (0, 1, 2):
            assert np.array_equal(gpu_encode(x, f, 0, sat), O.encode(x, f, 0, sat))
        codes = np.arange(1 << f.fmt.bitwidth, dtype=np.uint16 if f.fmt.bitwidth > 8 else np.uint8)
        buf = codes.view(np.uint8)
        n = codes.size
        assert same_bits(gpu_decode(buf, n, f), O.decode(buf, n, f))


def test_decode_rounds_into_float_subnormals():
    """Codes whose values lie below FP32's normal range with more significant
    bits than a float subnormal holds: one rounding of the exact value."""
    f = O.codec_fmt(16, 10, 150, False, True, True, 0x8000, 0xFC00, 0x7C00, 0xFC00, 0x7E00, 0x7C01, 1)
    codes = np.arange(1 << 16, dtype=np.uint16)
    buf = codes.view(np.uint8)
    got = gpu_decode(buf, codes.size, f)
    want = O.decode(buf, codes.size, f)
    assert same_bits(got, want)
    sub = (np.abs(want) < 2.0 ** -126) & (want != 0)
    assert sub.sum() > 1000


def test_round_trip_of_representable_values():
    """encode(decode(c)) == c for every finite code of E4M3 / P3109<6,3> /
    FP16: the packed stream of all codes, decoded and re-encoded."""
    for f, fmt in ((O.codec_p3109(8, 4), lg.create_p3109_params(8, 4)),
                   (O.codec_p3109(6, 3), lg.create_p3109_params(6, 3)),
                   (O.codec_ieee(16, 10, 15, 0x7E00, 0x7D00), lg.create_half_params())):
        n = f.fmt.bitwidth
        codes = np.arange(1 << n)
        vals = np.array([O.decode_rep(int(c), f) for c in codes], np.float32)
        keep = np.isfinite(vals) & ~((vals == 0) & np.signbit(vals))  # -0 may encode as +0
        xs = torch.from_numpy(vals[keep]).cuda()
        packed = lg.lof_encode(xs, fmt)
        back = lg.lof_decode(packed, xs.numel(), fmt)
        assert same_bits(back.cpu().numpy(), vals[keep])


def test_python_api_and_errors():
    e4m3 = lg.create_p3109_params(8, 4)
    x = torch.randn(1000, device="cuda")
    packed = lg.lof_encode(x, e4m3, lg.RoundingMode.RoundToNearestEven,
                           lg.SaturationMode.SatFinite, reverse=True)
    assert packed.numel() == lg.packed_size(8, 1000) == 1000
    want = O.encode(x.cpu().numpy(), O.codec_p3109(8, 4), 0, 1, reverse=1)
    assert np.array_equal(packed.cpu().numpy(), want)
    y = lg.lof_decode(packed, 1000, e4m3, reverse=True)
    assert same_bits(y.cpu().numpy(), O.decode(want, 1000, O.codec_p3109(8, 4), 1))
    with pytest.raises(RuntimeError):
        lg.lof_encode(x.double(), e4m3)
    with pytest.raises(RuntimeError):
        lg.lof_decode(packed[:10], 1000, e4m3)
    with pytest.raises(RuntimeError):
        lg.lof_encode(x.cpu(), e4m3)


@pytest.mark.parametrize("bits", [4, 8, 16, 6, 2, 3])
def test_direct_path_and_unaligned_fallback(bits):
    """4-, 8- and 16-bit codes take the one-float4-per-thread kernels when the
    buffers allow 16-byte loads (2- and 6-bit decodes too, reversed groups
    included; 3-bit reversed groups span eight codes and take the chunk
    decode); buffers that are only 4-byte aligned take the staged kernels.
    Both write the oracle's bytes."""
    f = O.codec_p3109(bits, max(1, bits // 2))
    n = 70_003 if bits != 6 else 70_001
    x = _wide(n, bits)
    want = O.encode(x, f, reverse=1)
    nb = lg.packed_size(bits, n)
    big = torch.from_numpy(np.concatenate([np.zeros(1, np.float32), x])).cuda()
    for shift in (0, 1):                              # float offset: 16-byte or 4-byte aligned
        xs = big[1:] if shift else torch.from_numpy(x).cuda()
        out = torch.zeros(nb + 8, dtype=torch.uint8, device="cuda")
        dptr = out.data_ptr() + 4 * shift              # packed output 4-byte aligned only
        st = _native.lib().lofgb_encode_f32(dptr, xs.data_ptr(), n, C.byref(_native_fmt(f)), 0, 0, 0,
                                            1, 0, 0, None)
        assert st == 0
        got = out.cpu().numpy()[4 * shift:4 * shift + nb]
        assert np.array_equal(got, want), (shift, int(np.sum(got != want)))
        assert not out.cpu().numpy()[4 * shift + nb:].any()   # nothing past the packed size
        dec = torch.zeros(n + 4, dtype=torch.float32, device="cuda")
        st = _native.lib().lofgb_decode_f32(dec.data_ptr() + 4 * shift, dptr, n,
                                            C.byref(_native_fmt(f)), 1, None)
        assert st == 0
        assert same_bits(dec.cpu().numpy()[shift:shift + n], O.decode(want, n, f, 1))
