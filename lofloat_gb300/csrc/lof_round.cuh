// lof_round.cuh — device rounding core shared by every kernel in liblofgb.
//
// Bit-level semantics follow the reference's scalar functions
// (SudhanvaKulkarni123/LoFloat):
//   RoundMantissa and helpers         src/lo_float.h:570-1272
//   virtual_round(x, ToMantissaBits)  src/lo_float.h:2715-2756
//   virtual_round(x, params, ps)      src/lo_float.h:2843-2939
// The host precomputes a RoundPlan per (source type, format, mode) so the
// device path is integer-only: every float comparison of the reference
// (|x| < tiny, |x| vs tiny/2, |x| > 0 after narrowing to float) becomes a
// comparison of the magnitude's bit pattern against a precomputed threshold,
// exact because non-negative IEEE bit patterns order like their values.
//
// Defined behaviour where the reference's is undefined (shared with the
// oracle): roundoff 0 leaves every mode unchanged; the random addend of
// SR-A/B/C/D keeps the low min(len, W) bits of R (W the source word width);
// an addend wider than the dropped bits is shifted right instead of left by a
// negative count; SR-C
// on 64-bit words uses 64-bit arithmetic; a subnormal-branch shift wider than
// the word is clamped to width-1 (reachable only when the result is ±0).
#pragma once
#include <cuda_fp16.h>

#include <cstdint>
#include <type_traits>

#include "lofgb_internal.h"

namespace lofgb {

// ---- counter-based RNG: SplitMix64 (Steele, Lea, Flood 2014) ---------------
// The idx-th output of a SplitMix64 stream whose state starts at `seed`.
constexpr uint64_t SM64_GAMMA = 0x9E3779B97F4A7C15ull;

__device__ __forceinline__ uint64_t sm64_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t rng64(uint64_t seed, uint64_t idx) {
    return sm64_mix(seed + (idx + 1ull) * SM64_GAMMA);
}

// Random word of element g: lane g mod 2^lg of output g >> lg, lanes of
// 64 >> lg bits from the low end (RoundPlan::rng_lg). The bits above the
// lane belong to the next elements; every mode masks to the bits it reads.
__device__ __forceinline__ uint64_t rng_elem(uint64_t seed, uint64_t g, int lg) {
    const uint64_t w = rng64(seed, g >> lg);
    return w >> (((uint32_t)g & ((1u << lg) - 1u)) << (6 - lg));
}

// Elements g .. g+3. With lanes of 16 or 8 bits and g a multiple of 4 the
// four lanes sit in one output, with 32-bit lanes and g even in two: one
// or two SplitMix64 mixes for four elements instead of four. lg is uniform
// across the launch, and so is g's alignment when the stream offset is.
__device__ __forceinline__ void rng_elem4(uint64_t seed, uint64_t g, int lg, uint64_t (&r)[4]) {
    if (lg == 3 && (g & 3u) == 0) {
        // four 8-bit lanes: the low or the high half of the output
        const uint64_t w = rng64(seed, g >> 3);
        const uint32_t h = (g & 4u) ? (uint32_t)(w >> 32) : (uint32_t)w;
#pragma unroll
        for (int q = 0; q < 4; ++q) r[q] = h >> (8 * q);
    } else if (lg == 2 && (g & 3u) == 0) {
        const uint64_t w = rng64(seed, g >> 2);
#pragma unroll
        for (int q = 0; q < 4; ++q) r[q] = w >> (16 * q);
    } else if (lg == 1 && (g & 1u) == 0) {
        const uint64_t z = seed + ((g >> 1) + 1ull) * SM64_GAMMA;
        const uint64_t w0 = sm64_mix(z), w1 = sm64_mix(z + SM64_GAMMA);
        r[0] = w0;
        r[1] = w0 >> 32;
        r[2] = w1;
        r[3] = w1 >> 32;
    } else if (lg == 0) {
        const uint64_t z = seed + (g + 1ull) * SM64_GAMMA;
#pragma unroll
        for (int q = 0; q < 4; ++q) r[q] = sm64_mix(z + (uint64_t)q * SM64_GAMMA);
    } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) r[q] = rng_elem(seed, g + q, lg);
    }
}

// ---- per-thread cp.async staging (16-byte copies global -> shared) --------
// Each thread copies into and later reads its own shared-memory slots, so a
// wait_group is all the ordering it needs (no block barrier).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// ---- round-to-odd word and RNE to m mantissa bits (the GEMM leaf) ----------
// The round-to-odd result of one FP32 operation from its two directed
// roundings rd (toward -inf) and ru (toward +inf). The reference form
// (src/cutlass_gemms.cuh:73-88) is rz | (rd != ru) with rz = rd >= 0 ? rd : ru.
// Inexact: rd and ru are adjacent words (also across 0 and at the overflow
// edge), exactly one of them is odd, and that one is rz | 1. Exact: rd == ru,
// or the zero pair rd = -0, ru = +0 where the reference keeps rd. NaN: both
// are the canonical 0x7FFFFFFF. So "ru if ru is odd, else rd" gives the same
// word for every input with one test and one select.
__device__ __forceinline__ uint32_t rto_word(float rd, float ru) {
    const uint32_t d = __float_as_uint(rd), u = __float_as_uint(ru);
    return (u & 1u) ? u : d;
}

// RNE of the FP32 word v to 23 - ro mantissa bits, 1 <= ro <= 23, on the
// signed word (adding < 2^ro never carries into the sign bit of a finite
// value or of the canonical NaN). sh = 2^(32 - ro): the multiply-high is
// v >> ro on the multiply pipe, leaving the logic pipe three operations.
__device__ __forceinline__ uint32_t rne_word(uint32_t v, uint32_t sh, uint32_t half_m1, uint32_t mask) {
    return (v + (__umulhi(v, sh) & 1u) + half_m1) & mask;
}
// The same with bit ro of v taken by two multiplies, leaving the logic pipe
// two operations: v * 2^(31 - ro) has it at bit 31 and the multiply-high by
// two moves it to bit 0. `two` must be opaque to the compiler (a register the
// caller fills from an asm), which would otherwise turn the multiply-high
// into a shift on the logic pipe.
__device__ __forceinline__ uint32_t rne_word2(uint32_t v, uint32_t sh2, uint32_t two, uint32_t half_m1,
                                              uint32_t mask) {
    return (v + __umulhi(v * sh2, two) + half_m1) & mask;
}

__device__ __forceinline__ double usamp_of(uint64_t r) {
    return (double)(r >> 11) * 0x1.0p-53;
}

template <typename U>
__device__ __forceinline__ U shl_s(U v, int s) {
    constexpr int W = sizeof(U) * 8;
    if (s >= W || s <= -W) return U(0);
    return s >= 0 ? U(v << s) : U(v >> (-s));
}

template <typename U>
__device__ __forceinline__ U lowmask(int n) {
    constexpr int W = sizeof(U) * 8;
    return n >= W ? ~U(0) : U((U(1) << n) - U(1));
}

// RoundMantissa (src/lo_float.h:1231-1272) on a W-bit magnitude held in U
// (uint32_t for f32/f16 words, uint64_t for f64). `W` is the source word
// width; results are truncated to W bits as the reference's Bits type does.
// MODE < 0 selects the runtime mode `rmode`.
template <int MODE, int W, typename U>
__device__ __forceinline__ U round_mantissa(U bits, int ro, int rmode, int len, bool pos,
                                            uint64_t r) {
    const int mode = MODE >= 0 ? MODE : rmode;
    if (ro <= 0) return bits;
    if (ro > W - 1) ro = W - 1;
    const U one_ro = U(1) << ro;
    const U low = one_ro - U(1);
    const U trunc = bits & ~low;
    const U tail = bits & low;
    // the random addend keeps the low min(len, W) bits of r (the reference
    // casts it to its W-bit Bits type before shifting)
    const U rm = lowmask<U>(len < W ? len : W);
    U res;
    switch (mode) {
    case LOFGB_RNE: res = bits + ((bits >> ro) & U(1)) + (one_ro >> 1) - U(1); break;
    case LOFGB_RNO: res = bits + (((bits >> ro) & U(1)) ^ U(1)) + (one_ro >> 1) - U(1); break;
    case LOFGB_RTZ: res = trunc; break;
    case LOFGB_RAFZ: res = trunc + (tail ? one_ro : U(0)); break;
    case LOFGB_RU: res = trunc + ((pos && tail) ? one_ro : U(0)); break;
    case LOFGB_RD: res = trunc + ((!pos && tail) ? one_ro : U(0)); break;
    case LOFGB_RTA: res = trunc + (((bits >> (ro - 1)) & U(1)) << ro); break;
    case LOFGB_SR_A: {
        if (len <= 0) { res = bits; break; }
        res = bits + shl_s<U>(U(r) & rm, ro - len);
        break;
    }
    case LOFGB_SR_B: {
        const U add = (U(r) & rm) + U(1);
        res = bits + (tail ? shl_s<U>(add, ro - len) : U(0));
        break;
    }
    case LOFGB_SR_C: {
        if (len == 0 || tail == 0) { res = bits; break; }
        const U samp = U(r) & rm;
        U add = shl_s<U>((samp >> 1) + (samp & U(1)), ro - len + 1);
        if (W <= 32) add = U(uint32_t(add));
        res = bits + add;
        break;
    }
    case LOFGB_SR_D: {
        if (len <= 0) { res = bits; break; }
        const U add = (U(r) & rm) + (U(r >> len) & U(1));
        res = bits + shl_s<U>(add, ro - len);
        break;
    }
    case LOFGB_TRUE_SR: {
        const double prob = (double)tail / (double)one_ro;
        if (usamp_of(r) < prob) {
            U rounded = (trunc + one_ro) & lowmask<U>(W);
            res = rounded < trunc ? trunc : rounded;
        } else {
            res = trunc;
        }
        break;
    }
    case LOFGB_PROB: res = trunc + ((tail ? (U(r) & U(1)) : U(0)) << ro); break;
    case LOFGB_RTO: res = trunc | (tail ? one_ro : U(0)); break;
    case LOFGB_RTTZ: res = bits + (one_ro >> 1) - U(1); break;
    default: res = bits;
    }
    return res & lowmask<U>(W);
}

__device__ __forceinline__ bool mode_is_stochastic(int mode) {
    return mode == LOFGB_SR_A || mode == LOFGB_SR_B || mode == LOFGB_SR_C ||
           mode == LOFGB_SR_D || mode == LOFGB_TRUE_SR || mode == LOFGB_PROB;
}

// Source word traits.
template <int W> struct Src;
template <> struct Src<32> {
    using U = uint32_t;
    static constexpr int M = 23;
    static constexpr U SIGN = 0x80000000u, PINF = 0x7F800000u, QNAN = 0x7FC00000u;
};
template <> struct Src<64> {
    using U = uint64_t;
    static constexpr int M = 52;
    static constexpr U SIGN = 0x8000000000000000ull, PINF = 0x7FF0000000000000ull,
                       QNAN = 0x7FF8000000000000ull;
};
template <> struct Src<16> {
    using U = uint32_t;  // 16-bit words held in 32-bit registers
    static constexpr int M = 10;
    static constexpr U SIGN = 0x8000u, PINF = 0x7C00u, QNAN = 0x7E00u;
};

// from_double<From>((double)k * (double)tiny) for the subnormal branch
// (src/lo_float.h:2921). tiny is a power of two, 0, or (excluded by format
// validation) inf, so the product is exact in every source type.
template <int W>
__device__ __forceinline__ typename Src<W>::U subnormal_value(uint64_t k, const RoundPlan& p);
template <>
__device__ __forceinline__ uint32_t subnormal_value<32>(uint64_t k, const RoundPlan& p) {
    return __float_as_uint(__fmul_rn(__uint2float_rn((uint32_t)k), p.tiny_f));
}
template <>
__device__ __forceinline__ uint64_t subnormal_value<64>(uint64_t k, const RoundPlan& p) {
    return (uint64_t)__double_as_longlong(__dmul_rn(__ull2double_rn(k), (double)p.tiny_f));
}
template <>
__device__ __forceinline__ uint32_t subnormal_value<16>(uint64_t k, const RoundPlan& p) {
    const float v = __fmul_rn(__uint2float_rn((uint32_t)k), p.tiny_f);
    return (uint32_t)__half_as_ushort(__float2half_rn(v));
}

// The rare branches of virtual_round (src/lo_float.h:2869-2923): NaN, below
// the smallest subnormal, and the target-subnormal grid — computed without
// branches (every candidate, then a select), so that a warp running them
// for a few lanes pays no divergence bookkeeping.
template <int MODE, int W>
__device__ __forceinline__ typename Src<W>::U vr_special(typename Src<W>::U x, const RoundPlan& p,
                                                         uint64_t r) {
    using S = Src<W>;
    using U = typename S::U;
    using T = typename std::conditional<(W <= 32), uint32_t, uint64_t>::type;
    const U sign = x & S::SIGN;
    const U mag = x & (S::SIGN - U(1));
    // :2871-2909 below the smallest subnormal: 0 or +-tiny by mode and sign
    const T th = sign ? (T)p.tmin_neg : (T)p.tmin_pos;
    const U tiny_res = ((T)mag >= th ? U(p.tiny_bits) : U(0)) | sign;
    // :2910-2923 target-subnormal grid (shift clamped to a defined range for
    // lanes whose result is not selected)
    const int expf = (int)(mag >> S::M);
    int shift = p.d + (p.to_min_field - expf);
    shift = shift < 0 ? 0 : (shift > W - 1 ? W - 1 : shift);
    U sig = (mag & ((U(1) << S::M) - U(1))) | (U(1) << S::M);
    sig = round_mantissa<MODE, W, U>(sig, shift, p.mode, p.len, sign == 0, r);
    const U sub_res = subnormal_value<W>((uint64_t)(sig >> shift), p) | sign;
    U res = (T)mag < (T)p.tiny_thr ? tiny_res : sub_res;
    // :2869 NaN -> quiet NaN, sign dropped
    return mag > S::PINF ? U(S::QNAN) : res;
}

// Common case of virtual_round(x, params, ps) (src/lo_float.h:2925-2936), on
// the signed word: RoundMantissa never carries into the sign bit of a finite
// value, so rounding x and masking the dropped bits equals the reference's
// round-the-magnitude-then-OR-the-sign; then the overflow rule.
template <int MODE, int W>
__device__ __forceinline__ typename Src<W>::U vr_normal(typename Src<W>::U x, const RoundPlan& p,
                                                        uint64_t r) {
    using S = Src<W>;
    using U = typename S::U;
    using T = typename std::conditional<(W <= 32), uint32_t, uint64_t>::type;
    U t = x;
    if (MODE == LOFGB_RNE) {
        // d >= 1 whenever any bit is dropped; d == 0 leaves x unchanged
        if (p.d > 0) t = x + ((x >> p.d) & U(1)) + ((U(1) << (p.d - 1)) - U(1));
    } else if (p.d > 0) {
        t = round_mantissa<MODE, W, U>(x, p.d, p.mode, p.len, (x & S::SIGN) == 0, r);
    }
    U res = t & (U)p.keep_mask;
    if ((T)(res & (S::SIGN - U(1))) >= (T)p.ovf_thr) res = p.saturating ? x : S::PINF;
    return res;
}

// True when x needs the rare branches: NaN, or magnitude below the target's
// smallest normal (exponent field < to_min_field).
template <int W>
__device__ __forceinline__ bool vr_is_special(typename Src<W>::U x, const RoundPlan& p) {
    using S = Src<W>;
    using U = typename S::U;
    using T = typename std::conditional<(W <= 32), uint32_t, uint64_t>::type;
    const U mag = x & (S::SIGN - U(1));
    return (T)(mag - (U)p.norm_thr) > (T)(S::PINF - (U)p.norm_thr);
}

// Rare branches for f32 words. With a float grid (RoundPlan::grid) the tiny
// and target-subnormal branches are one directed fadd against C and one exact
// fsub; FP32-subnormal inputs that reach the target-subnormal branch (the
// reference treats them as exponent -127 with an implicit 1) and NaN keep the
// exact integer path.
template <int MODE>
__device__ __forceinline__ uint32_t vr_grid_f32(uint32_t x, const RoundPlan& p) {
    const uint32_t sign = x & 0x80000000u;
    const float a = fabsf(__uint_as_float(x));
    float s;
    if (p.grid == 1) {
        s = __fadd_rn(a, p.grid_c);
    } else {
        const bool up = sign ? p.grid_up_neg : p.grid_up_pos;
        s = up ? __fadd_ru(a, p.grid_c) : __fadd_rz(a, p.grid_c);
    }
    return __float_as_uint(__fsub_rn(s, p.grid_c)) | sign;
}

// True when the float grid does not reproduce the reference: FP32-subnormal
// inputs in the target-subnormal branch (the reference treats them as
// exponent -127 with an implicit 1), and NaN.
__device__ __forceinline__ bool vr_grid_exception(uint32_t x, const RoundPlan& p) {
    const uint32_t mag = x & 0x7FFFFFFFu;
    return (mag < 0x00800000u && mag >= (uint32_t)p.tiny_thr) || mag > 0x7F800000u;
}

template <int MODE>
__device__ __forceinline__ uint32_t vr_special_f32(uint32_t x, const RoundPlan& p, uint64_t r) {
    if (p.grid == 0) return vr_special<MODE, 32>(x, p, r);
    const uint32_t g = vr_grid_f32<MODE>(x, p);
    const bool ex = vr_grid_exception(x, p);
    if (__any_sync(__activemask(), ex)) {
        const uint32_t e = vr_special<MODE, 32>(x, p, r);
        return ex ? e : g;
    }
    return g;
}

// virtual_round(x, params, ps), src/lo_float.h:2843-2939, on one source word.
template <int MODE, int W>
__device__ __forceinline__ typename Src<W>::U vr_format(typename Src<W>::U x, const RoundPlan& p,
                                                        uint64_t r) {
    if (!vr_is_special<W>(x, p)) return vr_normal<MODE, W>(x, p, r);
    if constexpr (W == 32) return vr_special_f32<MODE>(x, p, r);
    else return vr_special<MODE, W>(x, p, r);
}

// One f32 word per lane, rare branches under a warp vote instead of a
// divergent branch (for values computed once per lane, like an MX scale).
template <int MODE>
__device__ __forceinline__ uint32_t vr_format_f32_voted(uint32_t x, const RoundPlan& p,
                                                        uint64_t r) {
    uint32_t res = vr_normal<MODE, 32>(x, p, r);
    const bool sp = vr_is_special<32>(x, p);
    if (__any_sync(__activemask(), sp)) {
        const uint32_t s = vr_special_f32<MODE>(x, p, r);
        res = sp ? s : res;
    }
    return res;
}

// Four f32 words at once: the common case for all four, then one warp vote
// decides whether any lane of the warp needs the rare branches; if so they
// run for all four words and are selected per word. `r` holds the four
// random words (zeros for deterministic modes).
template <int MODE, bool FULL = false>
__device__ __forceinline__ void vr_format_f32x4(uint32_t (&w)[4], const RoundPlan& p,
                                                const uint64_t (&r)[4]) {
    // FULL: the caller guarantees all 32 lanes are here (no __activemask())
    const unsigned mask = FULL ? 0xFFFFFFFFu : __activemask();
    uint32_t res[4];
    bool sp[4];
    bool any = false;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        res[q] = vr_normal<MODE, 32>(w[q], p, r[q]);
        sp[q] = vr_is_special<32>(w[q], p);
        any |= sp[q];
    }
    if (__any_sync(mask, any)) {
        if (p.grid == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t s = vr_special<MODE, 32>(w[q], p, r[q]);
                res[q] = sp[q] ? s : res[q];
            }
        } else {
            bool ex[4];
            bool any_ex = false;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t g = vr_grid_f32<MODE>(w[q], p);
                res[q] = sp[q] ? g : res[q];
                ex[q] = sp[q] && vr_grid_exception(w[q], p);
                any_ex |= ex[q];
            }
            if (__any_sync(mask, any_ex)) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint32_t e = vr_special<MODE, 32>(w[q], p, r[q]);
                    res[q] = ex[q] ? e : res[q];
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = res[q];
}

// virtual_round(x, params, ps) of an f32 word by float arithmetic over the
// whole range (RoundPlan::uni; UNI = 1 round to nearest even, 2 directed).
// C = 2^(clamp(e, to_min, hi) + d) puts the target's spacing at |x| in the
// last place of C, so one fadd in the mode's direction and one exact fsub
// give the rounded magnitude — the normal branch (src/lo_float.h:2925-2933),
// the target-subnormal grid (:2915-2923) and the tiny branch (:2872-2908)
// alike. Then the overflow rule (:2935-2936) and NaN -> quiet NaN (:2869).
template <int MODE, int UNI>
__device__ __forceinline__ uint32_t vr_uni_f32(uint32_t x, const RoundPlan& p) {
    const uint32_t cb = min(max(x & 0x7F800000u, p.uni_lo), p.uni_hi) + p.uni_d;
    const float c = __uint_as_float(cb);
    const float a = fabsf(__uint_as_float(x));
    float s;
    if (UNI == 1) {
        s = __fadd_rn(a, c);
    } else if (MODE == LOFGB_RTZ) {
        s = __fadd_rz(a, c);
    } else {
        const bool up = (x & 0x80000000u) ? p.grid_up_neg : p.grid_up_pos;
        s = up ? __fadd_ru(a, c) : __fadd_rz(a, c);
    }
    const uint32_t r = __float_as_uint(__fsub_rn(s, c));
    uint32_t res = r | (x & 0x80000000u);
    res = r >= (uint32_t)p.ovf_thr ? ((x & p.sat_and) | p.sat_or) : res;
    return (x & 0x7FFFFFFFu) > 0x7F800000u ? 0x7FC00000u : res;
}

// virtual_round(x, params, {RoundToOdd}) of an f32 word on the float grid
// (RoundPlan::uni == 6): t = fadd_rz(|x|, C) - C truncates |x| onto the
// target's grid; the reference's RoundToOdd ORs the target's last place into
// the truncated word when any dropped bit was set (src/lo_float.h:1203-1229).
// At or above the target's smallest normal that place is FP32 bit d of t; below
// it the grid is the multiples of tiny and t + Csub (Csub = 2^23 tiny, exact)
// holds t / tiny in its low bits, so the OR happens there and Csub comes off
// again exactly. The tiny branch (|x| < tiny gives tiny when |x| > 0) is the
// same formula with t = 0.
__device__ __forceinline__ uint32_t vr_uni_rto_f32(uint32_t x, const RoundPlan& p) {
    const uint32_t mag = x & 0x7FFFFFFFu;
    const uint32_t cb = min(max(x & 0x7F800000u, p.uni_lo), p.uni_hi) + p.uni_d;
    const float c = __uint_as_float(cb);
    const float a = __uint_as_float(mag);
    const float t = __fsub_rn(__fadd_rz(a, c), c);
    const uint32_t inexact = t != a ? 1u : 0u;
    const uint32_t vs = __float_as_uint(
        __fsub_rn(__uint_as_float(__float_as_uint(__fadd_rn(t, p.grid_c)) | inexact), p.grid_c));
    const uint32_t v = mag >= (uint32_t)p.norm_thr ? (__float_as_uint(t) | (inexact << p.d)) : vs;
    uint32_t res = v | (x & 0x80000000u);
    res = v >= (uint32_t)p.ovf_thr ? ((x & p.sat_and) | p.sat_or) : res;
    return mag > 0x7F800000u ? 0x7FC00000u : res;
}

// vr_uni_f32<RNE, 1> for a saturating format, whose overflow returns the
// input word: a NaN input rounds to a NaN word, above every overflow
// threshold, and so comes back as the input NaN rather than the canonical
// quiet NaN. Only for callers whose next operation on the result turns any
// NaN into the same canonical NaN (MX multiplies it by the block scale).
__device__ __forceinline__ uint32_t vr_uni_sat_rne_f32(uint32_t x, const RoundPlan& p) {
    const uint32_t cb = min(max(x & 0x7F800000u, p.uni_lo), p.uni_hi) + p.uni_d;
    const float c = __uint_as_float(cb);
    const uint32_t r = __float_as_uint(__fsub_rn(__fadd_rn(fabsf(__uint_as_float(x)), c), c));
    return r >= (uint32_t)p.ovf_thr ? x : (r | (x & 0x80000000u));
}

// virtual_round(x, params, {SR-A, len}) of an f32 word by float arithmetic
// (RoundPlan::sr_uni); r holds the element's random bits in its low len bits.
// The noise R' * spacing * 2^-len is built exactly as F - E with
// E = 2^(e_C - len) (e_C the exponent of C; E's word is the clamped exponent
// field plus sr_shift = (d - len) << 23) and F = E with R' in its low
// mantissa bits (R' < 2^len, len <= d <= 23, so F = E + R' * ulp(E)). The
// truncation of y to the target's spacing at y is y's word with the d low bits
// cleared where y is at or above the target's smallest normal (every such y
// then has spacing 2^(e_y - m), or overflows), and fadd_rz(y, Csub) - Csub with
// Csub = 2^(to_min + d) (ulp = tiny) below it.
// SAT: a saturating format, whose overflow returns the input word.
template <bool SAT = false>
__device__ __forceinline__ uint32_t vr_uni_sra_f32(uint32_t x, const RoundPlan& p, uint32_t r) {
    const uint32_t mag = x & 0x7FFFFFFFu;
    const uint32_t eb = min(max(x & 0x7F800000u, p.uni_lo), p.uni_hi) + p.sr_shift;
    const float noise = __fsub_rn(__uint_as_float((r & p.sr_mask) | eb), __uint_as_float(eb));
    const float y = __fadd_rz(__uint_as_float(mag), noise);
    const uint32_t yb = __float_as_uint(y);
    const uint32_t vs = __float_as_uint(__fsub_rn(__fadd_rz(y, p.grid_c), p.grid_c));
    const uint32_t v = yb >= (uint32_t)p.norm_thr ? (yb & (uint32_t)p.keep_mask) : vs;
    uint32_t res = v | (x & 0x80000000u);
    res = v >= (uint32_t)p.ovf_thr ? (SAT ? x : ((x & p.sat_and) | p.sat_or)) : res;
    res = mag < (uint32_t)p.tiny_thr ? (x & 0x80000000u) : res;
    return mag > 0x7F800000u ? 0x7FC00000u : res;
}

// virtual_round(x, ToMantissaBits, ps), src/lo_float.h:2715-2756.
template <int MODE, int W>
__device__ __forceinline__ typename Src<W>::U vr_mantissa(typename Src<W>::U x, int d,
                                                          int rmode, int len, uint64_t r) {
    using S = Src<W>;
    using U = typename S::U;
    const U sign = x & S::SIGN;
    U b = x & (S::SIGN - U(1));
    b = round_mantissa<MODE, W, U>(b, d, rmode, len, sign == 0, r);
    if (d > 0) b &= ~((U(1) << d) - U(1));
    return (b | sign) & lowmask<U>(W);
}

}  // namespace lofgb
