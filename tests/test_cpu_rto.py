"""The GEMM leaf's round-to-odd word, computed on the device as "ru if ru is
odd, else rd" from the two directed results, equals the reference's form
rz | (rd != ru) with rz = rd >= 0 ? rd : ru (src/cutlass_gemms.cuh:73-88) for
every pair the two directed roundings can produce: equal words (exact
results, infinities, canonical NaN), the exact-zero pair (-0, +0) and every
adjacent pair, across zero and the overflow edge."""
import numpy as np


def _f(bits):
    return np.asarray(bits, dtype=np.uint32).view(np.float32)


def _reference_word(rd_bits, ru_bits):
    rd, ru = _f(rd_bits), _f(ru_bits)
    with np.errstate(invalid="ignore"):
        rz = np.where(rd >= 0, rd_bits, ru_bits).astype(np.uint32)
        inexact = (ru != rd).astype(np.uint32)
    return rz | inexact


def _odd_select(rd_bits, ru_bits):
    return np.where(ru_bits & 1, ru_bits, rd_bits).astype(np.uint32)


def _pairs():
    rng = np.random.default_rng(7)
    pos = np.concatenate([
        np.arange(0, 1 << 12, dtype=np.uint32),                     # zero and subnormals
        rng.integers(0, 0x7F800000, 1 << 20, dtype=np.uint32),      # every binade
        np.arange(0x7F7FF000, 0x7F800000, dtype=np.uint32),         # near the largest finite
        np.array([0x7F800000], dtype=np.uint32),                    # +inf
    ])
    # inexact positive results: rd = x, ru = next word up (0x7F7FFFFF -> +inf)
    up = pos[pos < 0x7F800000]
    rd = [up, up + 1]
    # inexact negative results: ru = -x, rd = next word down in value
    neg = up | np.uint32(0x80000000)
    rd_n, ru_n = neg + 1, neg
    # exact results: rd == ru (finite, +-inf, canonical NaN)
    ex = np.concatenate([pos, pos | np.uint32(0x80000000), np.array([0x7FFFFFFF], np.uint32)])
    rds = np.concatenate([rd[0], rd_n, ex, np.array([0x80000000], np.uint32)])
    rus = np.concatenate([rd[1], ru_n, ex, np.array([0x00000000], np.uint32)])
    return rds.astype(np.uint32), rus.astype(np.uint32)


def test_odd_select_equals_reference_form():
    rd, ru = _pairs()
    assert rd.size > 2_000_000
    got, want = _odd_select(rd, ru), _reference_word(rd, ru)
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, [(hex(rd[i]), hex(ru[i]), hex(got[i]), hex(want[i])) for i in bad[:5]]


def test_exact_zero_keeps_negative_zero():
    # x + (-x) = 0: RD gives -0, RU gives +0; the reference keeps -0
    assert _odd_select(np.uint32(0x80000000), np.uint32(0))[()] == 0x80000000
    assert _reference_word(np.uint32(0x80000000), np.uint32(0))[()] == 0x80000000
