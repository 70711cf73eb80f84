"""Format factories with the reference's signatures and field values
(LoFloat/formats.py:55-165): P3109 formats, FP16, FP32 and the E8M0 MX scale.

The inf/NaN checker objects answer the same questions as the reference's
(bit predicates plus the canonical inf/NaN patterns); the GPU rounding path
never calls them.
"""
from __future__ import annotations

from .binding import FloatFormatDescriptor, InfBehavior, NaNBehavior, Signedness


class P3109_NaNChecker:
    """NaN of a k-bit P3109 format: the single pattern 1 << (k-1) when signed,
    all ones when unsigned."""

    def __init__(self, k, is_signed=True):
        self.k = k
        self.is_signed = is_signed

    def _pattern(self):
        return (1 << (self.k - 1)) if self.is_signed else ((1 << self.k) - 1)

    def __call__(self, bits):
        return bits == self._pattern()

    def qNanBitPattern(self):
        return self._pattern()

    def sNanBitPattern(self):
        return self._pattern()


class P3109_InfChecker:
    """Infinities of a k-bit P3109 format; a saturating format has none."""

    def __init__(self, k, is_signed=True, has_inf_saturating=True):
        self.k = k
        self.is_signed = is_signed
        self.has_inf_saturating = has_inf_saturating

    def __call__(self, bits):
        if self.has_inf_saturating:
            return False
        top = (1 << self.k) - 1 if self.is_signed else (1 << self.k) - 2
        return (bits | (1 << (self.k - 1))) == top

    def minNegInf(self):
        return (1 << self.k) - 1 if self.is_signed else 0

    def minPosInf(self):
        return (1 << (self.k - 1)) - 1 if self.is_signed else (1 << self.k) - 2


def create_p3109_params(k, p, is_signed=True, saturating=True, bias=None):
    """P3109 <k, p>: k bits, precision p (p-1 stored mantissa bits), default
    bias 2^(k-p-1)."""
    if bias is None:
        bias = 1 << (k - p - 1)
    return FloatFormatDescriptor(
        k, p - 1, bias,
        inf_behavior=InfBehavior.Saturating if saturating else InfBehavior.Extended,
        nan_behavior=NaNBehavior._3109,
        signedness=Signedness.Signed if is_signed else Signedness.Unsigned,
        is_inf_checker=P3109_InfChecker(k, is_signed, saturating),
        is_nan_checker=P3109_NaNChecker(k, is_signed))


def create_e8m0_params():
    """E8M0 shared MX scale: 8-bit unsigned, no mantissa bits, bias 127."""
    return FloatFormatDescriptor(
        8, 0, 127, inf_behavior=InfBehavior.Extended, nan_behavior=NaNBehavior._3109,
        signedness=Signedness.Unsigned, is_inf_checker=P3109_InfChecker(8, False, False),
        is_nan_checker=P3109_NaNChecker(8, False))


class _IEEEInfChecker:
    def __init__(self, exp_mask, mant_mask, neg_inf, pos_inf):
        self.exp_mask, self.mant_mask = exp_mask, mant_mask
        self.neg_inf, self.pos_inf = neg_inf, pos_inf

    def __call__(self, bits):
        return (bits & self.exp_mask) == self.exp_mask and (bits & self.mant_mask) == 0

    def minNegInf(self):
        return self.neg_inf

    def minPosInf(self):
        return self.pos_inf


class _IEEENaNChecker:
    def __init__(self, exp_mask, mant_mask, qnan, snan):
        self.exp_mask, self.mant_mask = exp_mask, mant_mask
        self.qnan, self.snan = qnan, snan

    def __call__(self, bits):
        return (bits & self.exp_mask) == self.exp_mask and (bits & self.mant_mask) != 0

    def qNanBitPattern(self):
        return self.qnan

    def sNanBitPattern(self):
        return self.snan


class HalfPrecisionInfChecker(_IEEEInfChecker):
    def __init__(self):
        super().__init__(0x7C00, 0x03FF, 0xFC00, 0x7C00)


class HalfPrecisionNaNChecker(_IEEENaNChecker):
    def __init__(self):
        super().__init__(0x7C00, 0x03FF, 0x7E00, 0x7D00)


class SinglePrecisionInfChecker(_IEEEInfChecker):
    def __init__(self):
        super().__init__(0x7F800000, 0x007FFFFF, 0xFF800000, 0x7F800000)


class SinglePrecisionNaNChecker(_IEEENaNChecker):
    def __init__(self):
        super().__init__(0x7F800000, 0x007FFFFF, 0x7FC00000, 0x7FA00000)


def create_half_params():
    return FloatFormatDescriptor(16, 10, 15, inf_behavior=InfBehavior.Extended,
                                 nan_behavior=NaNBehavior._3109, signedness=Signedness.Signed,
                                 is_inf_checker=HalfPrecisionInfChecker(),
                                 is_nan_checker=HalfPrecisionNaNChecker())


def create_single_params():
    return FloatFormatDescriptor(32, 23, 127, inf_behavior=InfBehavior.Extended,
                                 nan_behavior=NaNBehavior._3109, signedness=Signedness.Signed,
                                 is_inf_checker=SinglePrecisionInfChecker(),
                                 is_nan_checker=SinglePrecisionNaNChecker())


def make_format(exp_bits: int, mant_bits: int, bias: int | None = None, saturating: bool = True,
                signed: bool = True) -> FloatFormatDescriptor:
    """Convenience: a signed (or unsigned) format with `exp_bits` exponent and
    `mant_bits` mantissa bits; bias defaults to 2^(exp_bits-1) - 1."""
    if bias is None:
        bias = (1 << (exp_bits - 1)) - 1
    k = exp_bits + mant_bits + (1 if signed else 0)
    return FloatFormatDescriptor(
        k, mant_bits, bias,
        inf_behavior=InfBehavior.Saturating if saturating else InfBehavior.Extended,
        nan_behavior=NaNBehavior._754, signedness=Signedness.Signed if signed else Signedness.Unsigned,
        is_inf_checker=P3109_InfChecker(k, signed, saturating),
        is_nan_checker=P3109_NaNChecker(k, signed))
