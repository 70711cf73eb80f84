// ref_shim.cpp — TEST INFRASTRUCTURE ONLY.
//
// Exposes the reference's own scalar rounding functions
// (lo_float::virtual_round, src/lo_float.h:2715-2756 and :2843-2939, public
// wrappers :4258-4274) through a C ABI so tests/golden/make_golden.py can
// produce golden vectors. It is compiled against the reference headers where
// they lie (oracle/build_oracle.py, -DUSE_CUDA so the header needs no xsimd);
// the output goes to oracle/_ref/ and never ships.
//
// Stochastic modes: the reference's host helpers build std::mt19937(lof_seed)
// afresh on every call (src/lo_float.h:666, 705, 764, 835, 872), so setting
// lo_float::set_seed(s_i) before element i makes the draw a function of s_i.
// The shim draws the same distribution from std::mt19937(s_i) again to
// record the value the reference consumed, so the oracle can be fed the same
// random bits.
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>

#include "lo_float.h"
#include "lo_pack.hpp"

using namespace lo_float;
using Params = FloatingPointParams<DeviceInfChecker, DeviceNaNChecker>;

namespace {

Params make(int bw, int m, int bias, int inf, int nan, int sgn) {
    return Params(bw, m, bias, inf ? Inf_Behaviors::Saturating : Inf_Behaviors::Extended,
                  nan ? NaN_Behaviors::_754 : NaN_Behaviors::_3109,
                  sgn ? Signedness::Unsigned : Signedness::Signed,
                  DeviceInfChecker{0, 0, 0, 0}, DeviceNaNChecker{0, 0, 0, 0},
                  Unsigned_behavior::NegtoZero);
}

// Record the random value the reference's host helper draws for `mode`
// from std::mt19937(seed). rbits receives the integer draw laid out the way
// the oracle consumes it (SR-D: low len bits + coin at bit len); usamp the
// uniform double of True_StochasticRounding.
void record_draw(int mode, int len, unsigned seed, uint64_t* rbits, double* usamp) {
    std::mt19937 mt(seed);
    *rbits = 0;
    *usamp = 0.0;
    switch ((Rounding_Mode)mode) {
    case Rounding_Mode::StochasticRoundingA: {
        if (len <= 0) return;
        const unsigned maxv = (1u << unsigned(len)) - 1u;
        std::uniform_int_distribution<unsigned> dist(0u, maxv);
        *rbits = dist(mt);
        return;
    }
    case Rounding_Mode::StochasticRoundingB:
    case Rounding_Mode::StochasticRoundingC: {
        std::uniform_int_distribution<unsigned int> distribution(0, (1 << (len)) - 1);
        *rbits = distribution(mt);
        return;
    }
    case Rounding_Mode::StochasticRoundingD: {
        if (len <= 0) return;
        const unsigned maxv = (1u << unsigned(len)) - 1u;
        std::uniform_int_distribution<unsigned> dist(0u, maxv);
        std::uniform_int_distribution<int> coin(0, 1);
        const uint64_t s = static_cast<uint32_t>(dist(mt) + static_cast<unsigned>(coin(mt)));
        // the sum r + c is what the reference adds; encode it as (r, c)
        const uint64_t r = s > maxv ? maxv : s;
        const uint64_t c = s > maxv ? 1 : 0;
        *rbits = r | (c << len);
        return;
    }
    case Rounding_Mode::True_StochasticRounding: {
        std::uniform_real_distribution<double> distribution(0.0, 1.0);
        *usamp = distribution(mt);
        return;
    }
    case Rounding_Mode::ProbabilisticRounding: {
        std::uniform_int_distribution<int> d01(0, 1);
        *rbits = (uint64_t)d01(mt);
        return;
    }
    default:
        return;
    }
}

inline c10::Half half_from_bits(uint16_t b) { return c10::Half(b, c10::Half::from_bits()); }

// The device leaf's round-to-odd FMA (src/cutlass_gemms.cuh:73-88), rebuilt on
// the host with directed-rounding fmaf under <cfenv> (the device intrinsics
// __fmaf_rd / __fmaf_ru have no host form).
float rto_fma_fenv(float a, float b, float c) {
    volatile float va = a, vb = b, vc = c;
    std::fesetround(FE_DOWNWARD);
    volatile float rd = std::fma(va, vb, vc);
    std::fesetround(FE_UPWARD);
    volatile float ru = std::fma(va, vb, vc);
    std::fesetround(FE_TONEAREST);
    float frd = rd, fru = ru;
    uint32_t inexact = (fru != frd) ? 1u : 0u;
    float rz = (frd >= 0.0f) ? frd : fru;
    uint32_t bits;
    std::memcpy(&bits, &rz, 4);
    bits |= inexact;
    std::memcpy(&rz, &bits, 4);
    return rz;
}

}  // namespace

extern "C" {

// Format-overload rounding of n values; seeds[i] seeds the reference draw of
// element i (may be NULL for deterministic modes).
int ref_round_f32(const float* in, float* out, int64_t n, int bw, int m, int bias, int inf,
                  int nan, int sgn, int mode, int len, const uint32_t* seeds,
                  uint64_t* rbits, double* usamp) {
    Params p = make(bw, m, bias, inf, nan, sgn);
    ProjSpec ps{(Rounding_Mode)mode, Saturation_Mode::OvfInf, len};
    for (int64_t i = 0; i < n; ++i) {
        if (seeds) {
            set_seed(seeds[i]);
            record_draw(mode, len, seeds[i], &rbits[i], &usamp[i]);
        }
        out[i] = lo_float::virtual_round(in[i], p, ps);
    }
    return 0;
}

int ref_round_f64(const double* in, double* out, int64_t n, int bw, int m, int bias,
                  int inf, int nan, int sgn, int mode, int len, const uint32_t* seeds,
                  uint64_t* rbits, double* usamp) {
    Params p = make(bw, m, bias, inf, nan, sgn);
    ProjSpec ps{(Rounding_Mode)mode, Saturation_Mode::OvfInf, len};
    for (int64_t i = 0; i < n; ++i) {
        if (seeds) {
            set_seed(seeds[i]);
            record_draw(mode, len, seeds[i], &rbits[i], &usamp[i]);
        }
        out[i] = lo_float::virtual_round(in[i], p, ps);
    }
    return 0;
}

// (The reference's half-source format overload does not compile against this
// torch's c10/util/Half.h: c10 re-exports std::bit_cast, so the unqualified
// bit_cast<FromBits>(c10::Half) calls at src/lo_float.h:2855, 2864, 2905,
// 2921 are ambiguous. The half-source mantissa overload below uses
// cuda::std::bit_cast and compiles.)

// Mantissa-overload rounding.
int ref_round_mantissa_f32(const float* in, float* out, int64_t n, int mbits, int mode,
                           int len, const uint32_t* seeds, uint64_t* rbits, double* usamp) {
    ProjSpec ps{(Rounding_Mode)mode, Saturation_Mode::OvfInf, len};
    for (int64_t i = 0; i < n; ++i) {
        if (seeds) {
            set_seed(seeds[i]);
            record_draw(mode, len, seeds[i], &rbits[i], &usamp[i]);
        }
        out[i] = lo_float::virtual_round(in[i], mbits, ps);
    }
    return 0;
}

int ref_round_mantissa_f64(const double* in, double* out, int64_t n, int mbits, int mode,
                           int len, const uint32_t* seeds, uint64_t* rbits, double* usamp) {
    ProjSpec ps{(Rounding_Mode)mode, Saturation_Mode::OvfInf, len};
    for (int64_t i = 0; i < n; ++i) {
        if (seeds) {
            set_seed(seeds[i]);
            record_draw(mode, len, seeds[i], &rbits[i], &usamp[i]);
        }
        out[i] = lo_float::virtual_round(in[i], mbits, ps);
    }
    return 0;
}

int ref_round_mantissa_f16(const uint16_t* in, uint16_t* out, int64_t n, int mbits,
                           int mode, int len, const uint32_t* seeds, uint64_t* rbits,
                           double* usamp) {
    ProjSpec ps{(Rounding_Mode)mode, Saturation_Mode::OvfInf, len};
    for (int64_t i = 0; i < n; ++i) {
        if (seeds) {
            set_seed(seeds[i]);
            record_draw(mode, len, seeds[i], &rbits[i], &usamp[i]);
        }
        c10::Half h = half_from_bits(in[i]);
        out[i] = lo_float::virtual_round(h, mbits, ps).x;
    }
    return 0;
}

// MX block loop of src/LoPy_bind.cpp:199-214 around the reference's scalar
// virtual_round; formula 0 uses the GPU scale expression amax * (1/pmn)
// (src/mx_round.cuh:52-65), formula 1 the CPU one amax / pmn. Deterministic
// element and scale modes only.
int ref_mx_round_f32(const float* in, float* out, int64_t n, int block, int ebw, int em,
                     int ebias, int einf, int esgn, int sbw, int sm, int sbias, int sinf,
                     int ssgn, int mode, int scale_mode, int formula) {
    Params priv = make(ebw, em, ebias, einf, 0, esgn);
    Params pub = make(sbw, sm, sbias, sinf, 0, ssgn);
    const int me = priv.is_signed == Signedness::Signed
                       ? (1 << (priv.bitwidth - priv.mantissa_bits - 1)) - 1 - priv.bias
                       : (1 << (priv.bitwidth - priv.mantissa_bits)) - 1 - priv.bias;
    const float pmn = ldexpf(1.0f, me) * (2.0f - ldexpf(1.0f, -priv.mantissa_bits));
    for (int64_t b = 0; b < n; b += block) {
        const int len = (int)std::min<int64_t>(block, n - b);
        float amax = 0.0f;
        for (int i = 0; i < len; ++i) amax = std::max(amax, std::fabs(in[b + i]));
        float sin = formula ? amax / pmn : amax * (1.0f / pmn);
        float scale = lo_float::virtual_round(sin, pub, ProjSpec{(Rounding_Mode)scale_mode});
        for (int i = 0; i < len; ++i) {
            if (scale > 0.0f)
                out[b + i] = lo_float::virtual_round(in[b + i] / scale, priv,
                                                     ProjSpec{(Rounding_Mode)mode}) *
                             scale;
            else
                out[b + i] = 0.0f;
        }
    }
    return 0;
}

// Emulated-accumulation GEMM, A M×K row-major, B K×N row-major: the leaf of
// src/cutlass_gemms.cuh:139-166 in sequential k order with the reference's
// mantissa rounding, then D = alpha * acc.
int ref_gemm_f32(const float* A, const float* B, float* D, int M, int N, int K, int mbits,
                 float alpha) {
    for (int i = 0; i < M; ++i)
        for (int j = 0; j < N; ++j) {
            float acc = 0.0f;
            for (int k = 0; k < K; ++k)
                acc = lo_float::virtual_round(
                    rto_fma_fenv(A[(int64_t)i * K + k], B[(int64_t)k * N + j], acc), mbits);
            D[(int64_t)i * N + j] = alpha * acc;
        }
    return 0;
}

// ---- storage codec (src/lo_pack.hpp) --------------------------------------------
// Runtime checker functors with the two predicate forms the reference's
// checkers take (masked compare for infinities; single pattern, IEEE-style or
// none for NaN), so that one shim function covers every format.
struct RtInf {
    uint32_t inf_or, inf_match, pos, neg;
    bool operator()(uint64_t bits) const { return ((uint32_t)bits | inf_or) == inf_match; }
    uint64_t minNegInf() const { return neg; }
    uint64_t minPosInf() const { return pos; }
};
struct RtNaN {
    int kind;  // 0 pattern, 1 IEEE-style, 2 none
    uint32_t qnan, snan, sign_mask, exp_all;
    bool operator()(uint64_t bits) const {
        if (kind == 2) return false;
        if (kind == 0) return (uint32_t)bits == qnan;
        return ((uint32_t)bits & ~sign_mask) > exp_all;
    }
    uint64_t qNanBitPattern() const { return qnan; }
    uint64_t sNanBitPattern() const { return snan; }
};
using CodecParams = FloatingPointParams<RtInf, RtNaN>;

// cf: bw, m, bias, inf(1 = saturating), nan(1 = 754), sgn(1 = unsigned),
//     inf_or, inf_match, pos_inf, neg_inf, qnan, snan, nan_kind, neg_to_nan
static CodecParams make_codec(const int64_t* cf) {
    const int bw = (int)cf[0], m = (int)cf[1], sgn = (int)cf[5];
    RtInf inf{(uint32_t)cf[6], (uint32_t)cf[7], (uint32_t)cf[8], (uint32_t)cf[9]};
    const uint32_t sign_mask = sgn ? 0u : (1u << (bw - 1));
    const int ebits = bw - m - (sgn ? 0 : 1);
    RtNaN nan{(int)cf[12], (uint32_t)cf[10], (uint32_t)cf[11], sign_mask,
              ((1u << ebits) - 1u) << m};
    return CodecParams(bw, m, (int)cf[2], cf[3] ? Inf_Behaviors::Saturating : Inf_Behaviors::Extended,
                       cf[4] ? NaN_Behaviors::_754 : NaN_Behaviors::_3109,
                       sgn ? Signedness::Unsigned : Signedness::Signed, inf, nan,
                       cf[13] ? Unsigned_behavior::NegtoNaN : Unsigned_behavior::NegtoZero);
}

int ref_encode_f32(uint8_t* dst, const float* src, int64_t count, const int64_t* cf, int mode,
                   int sat, int len, int reverse) {
    const CodecParams P = make_codec(cf);
    const ProjSpec ps{(Rounding_Mode)mode, (Saturation_Mode)sat, len};
    return reverse ? LoF_encode<PackEndian::Reverse>(dst, src, P, (size_t)count, ps)
                   : LoF_encode<PackEndian::Forward>(dst, src, P, (size_t)count, ps);
}

int ref_decode_f32(float* dst, const uint8_t* src, int64_t count, const int64_t* cf,
                   int reverse) {
    const CodecParams P = make_codec(cf);
    return reverse ? LoF_decode<PackEndian::Reverse>(dst, src, P, (size_t)count)
                   : LoF_decode<PackEndian::Forward>(dst, src, P, (size_t)count);
}

int64_t ref_packed_size(int n, int64_t count) { return (int64_t)LoF_packed_size(n, (size_t)count); }

}  // extern "C"
