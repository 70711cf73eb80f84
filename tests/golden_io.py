"""Loader for the committed golden fixtures (tests/golden/*.npz)."""
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest():
    with open(os.path.join(GOLDEN, "MANIFEST.json")) as fh:
        return json.load(fh)


def verify_sha(name):
    with open(os.path.join(GOLDEN, name), "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest() == manifest()["files"][name]["sha256"]


def load(name):
    """One fixture file, after checking it against its MANIFEST.json sha256."""
    assert verify_sha(name), f"{name} does not match MANIFEST.json"
    return np.load(os.path.join(GOLDEN, name))


def cases(group):
    """Yield (case_name, dict of arrays) for one fixture group."""
    z = np.load(os.path.join(GOLDEN, f"golden_{group}.npz"))
    recs = {}
    for k in z.files:
        cname, field = k.split("__", 1)
        recs.setdefault(cname, {})[field] = z[k]
    for cname in sorted(recs):
        yield cname, recs[cname]


def fmt_tuple(a):
    bw, m, bias, sat, signed = (int(v) for v in a)
    return bw, m, bias, bool(sat), bool(signed)


def same_bits(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    u = {2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]
    return np.array_equal(a.view(u), b.view(u))


def same_bits_nan_class(a, b):
    """Bit equality, except that any NaN matches any NaN (payloads differ
    between host and GPU arithmetic)."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    u = {2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]
    if a.dtype == np.uint16:
        an = ((a & 0x7C00) == 0x7C00) & ((a & 0x3FF) != 0)
        bn = ((b & 0x7C00) == 0x7C00) & ((b & 0x3FF) != 0)
    else:
        an, bn = np.isnan(a), np.isnan(b)
    eq = (a.view(u) == b.view(u)) | (an & bn)
    return bool(np.all(eq)), np.nonzero(~eq)[0]
