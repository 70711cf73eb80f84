"""Pin the CPU oracle against golden vectors made by the reference's own
scalar functions (tests/golden/make_golden.py). Bit-exact, every case."""
import numpy as np
import pytest

from golden_io import cases, fmt_tuple, manifest, same_bits, verify_sha
from oracle import oracle as O

STOCH = {3, 8, 9, 10, 11, 14}


def test_manifest_hashes():
    for name in manifest()["files"]:
        assert verify_sha(name), name


def _diff(x, got, want):
    u = {2: np.uint16, 4: np.uint32, 8: np.uint64}[x.dtype.itemsize]
    idx = np.nonzero(got.view(u) != want.view(u))[0][:5]
    return [(x[i], got[i], want[i]) for i in idx]


def _fmt(a):
    bw, m, bias, sat, signed = fmt_tuple(a)
    return O.fmt(bw, m, bias, saturating=sat, signed=signed)


@pytest.mark.parametrize("cname,rec", list(cases("round")), ids=lambda v: v if isinstance(v, str) else "")
def test_round_format_overload(cname, rec):
    f = _fmt(rec["fmt"])
    x = rec["x"]
    for key in rec:
        if not key.startswith("y"):
            continue
        mode = int(key[1:])
        ln = int(rec[f"len{mode}"])
        rb = rec.get(f"r{mode}")
        us = rec.get(f"u{mode}")
        got = O.round_bits(x, f, mode, ln, rbits=rb, usamp=us if mode == 10 else None)
        assert same_bits(got, rec[key]), (cname, mode, _diff(x, got, rec[key]))


@pytest.mark.parametrize("cname,rec", list(cases("mant")), ids=lambda v: v if isinstance(v, str) else "")
def test_round_mantissa_overload(cname, rec):
    x = rec["x"]
    mb = int(rec["mbits"])
    for key in rec:
        if not key.startswith("y"):
            continue
        mode = int(key[1:])
        ln = int(rec[f"len{mode}"])
        got = O.round_bits(x, None, mode, ln, rbits=rec.get(f"r{mode}"),
                           usamp=rec.get(f"u{mode}") if mode == 10 else None, mbits=mb)
        assert same_bits(got, rec[key]), (cname, mode)


@pytest.mark.parametrize("cname,rec", list(cases("mx")), ids=lambda v: v if isinstance(v, str) else "")
def test_mx(cname, rec):
    bs, mode, _ = (int(v) for v in rec["case"])
    got = O.mx_round(rec["x"], bs, _fmt(rec["ef"]), _fmt(rec["sf"]), mode=mode)
    assert same_bits(got, rec["y"]), cname


def test_mx_scale_formula_agreement():
    """The GPU scale expression amax*(1/pmn) and the CPU amax/pmn agreed on
    every golden MX block (E8M0 / E5M2 scales)."""
    for cname, rec in cases("mx"):
        assert int(rec["cpu_formula_diff"]) == 0, cname


@pytest.mark.parametrize("cname,rec", list(cases("gemm")), ids=lambda v: v if isinstance(v, str) else "")
def test_gemm(cname, rec):
    D = O.gemm(rec["A"], rec["B"], int(rec["mbits"]), alpha=float(rec["alpha"]))
    assert same_bits(D, rec["D"]), cname


def codec_from_fields(cf):
    bw, m, bias, inf, nan, sgn, inf_or, inf_match, pos, neg, qn, sn, kind, n2n = (int(v) for v in cf)
    return O.codec_fmt(bw, m, bias, saturating=bool(inf), signed=not sgn, nan_754=bool(nan),
                       inf_or=inf_or, inf_match=inf_match, pos_inf=pos, neg_inf=neg, qnan=qn,
                       snan=sn, nan_kind=kind, neg_to_nan=bool(n2n))


@pytest.mark.parametrize("cname,rec", list(cases("codec")), ids=lambda v: v if isinstance(v, str) else "")
def test_codec(cname, rec):
    """The codec oracle against the reference's own LoF_encode / LoF_decode
    (src/lo_pack.hpp) for every deterministic mode, the three saturation modes
    and both group orders: packed bytes identical, decoded bits identical."""
    f = codec_from_fields(rec["fields"])
    x = rec["x"]
    for key, want in rec.items():
        if not key.startswith("enc_"):
            continue
        _, m, s, r = key.split("_")
        got = O.encode(x, f, mode=int(m[1:]), sat=int(s[1:]), reverse=int(r[1:]))
        assert np.array_equal(got, want), (cname, key, int(np.sum(got != want)))
    for rev in (0, 1):
        got = O.decode(rec["raw"], 2048, f, reverse=rev)
        assert same_bits(got, rec[f"dec_r{rev}"]), (cname, rev)
