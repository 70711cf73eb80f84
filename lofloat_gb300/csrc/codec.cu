// codec.cu — low-precision storage codec: FP32 <-> packed n-bit codes.
//
// Replaces LoF_encode_cuda / LoF_decode_cuda (src/lo_pack.hpp:474-532), which
// run one thread per group, stage the group in a 64-float local array and
// set or read the code bits one at a time through byte read-modify-writes.
//
// Fast paths (RNE encode on the float grid, direct-bits decode, 16-byte
// aligned float buffers): a thread converts G = lcm(n, 32) / n consecutive
// values to lcm(n, 32) / 32 whole words and back, with no staging (n = 4, 8,
// 16: one float4 per thread; the direct encode streams its inputs through a
// per-thread cp.async ring). Everything else takes the staged kernels below.
//
// Staged kernels: a warp owns a tile of 1024 consecutive values (32 per lane). A tile is
// always a whole number of groups (32 n bits hold 4 gcd(n, 8) or 2 gcd(n, 16)
// groups), so every lane packs its 32 codes into exactly n 32-bit words on its
// own, with no cross-lane bit exchange. FP32 values and packed words move
// between HBM and registers through shared memory so that every global access
// is a coalesced 128-byte warp transaction; the stride of 33 words per lane in
// shared memory keeps the per-lane accesses free of bank conflicts. The code
// width n (1..16) and the group order are template parameters, so the bit
// positions fold to constants.
//
// Per element (codec_encode / codec_decode below) the arithmetic is
// convert_float_to_rep / convert_rep_to_float of src/lo_pack.hpp:109-320,
// restated with the shared RoundMantissa (round_mantissa in lof_round.cuh).
// HBM-bound: 4 + n/8 bytes per element either way.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "lof_round.cuh"
#include "mx_common.cuh"

namespace lofgb {

namespace {

constexpr int CT = 128;             // threads per CTA (4 warps)
constexpr int TILE = 1024;          // values per warp tile

struct CodecArg {
    int n, m, bias, is_signed, has_inf, nan3109;
    uint32_t inf_or, inf_match, pos_inf, qnan, snan;
    int nan_kind, neg_to_nan;
    int mode, sat, len;
    int rng_lg;               // random lanes per SplitMix64 output (RoundPlan::rng_lg)
    uint64_t seed, offset;
    // Fast encode (enc_fast 1, RNE): the magnitude is
    // rounded on the float grid (whole-range float rounding, uni_* as in
    // RoundPlan) and its code read off the bits of the rounded value.
    int enc_fast;
    uint32_t uni_lo, uni_hi, uni_d;
    uint32_t min_norm_bits;   // FP32 bits of the smallest target normal, 2^(1-bias)
    uint32_t code_off;        // normal code = (bits >> (23 - m)) - code_off
    float sub_c;              // 2^23 * tiny: subnormal code = bits(v + sub_c) - bits(sub_c)
    // Veltkamp form of the fast encode (velt, formats with 1..22 mantissa
    // bits): the normal range rounds |x| to m bits as t - (t - |x|),
    // t = |x| * sigma, sigma = 2^(23 - m) + 1, on the FMA pipe
    int velt;
    float sigma;
    uint32_t max_finite, ovf_code, inf_code, neg_zero_code, neg_code, sign_mask;
    uint32_t neg_keep, neg_or, neg_zero;  // a negative finite code: code ? (code & keep) | or : zero
    // Fast decode: every finite value is a normal FP32 number or an exact
    // FP32 subnormal, so the bits are built directly.
    int dec_fast;
    float tiny;               // 2^(1 - bias - m)
    float sub_c_dec;          // 2^23 * tiny
    uint32_t code_off_dec;    // normal value bits = (mag << (23 - m)) - code_off_dec
};

__device__ __forceinline__ bool c_is_nan(uint32_t rep, const CodecArg& a) {
    if (a.nan_kind == LOFGB_NAN_NONE) return false;
    if (a.nan_kind == LOFGB_NAN_PATTERN) return rep == a.qnan;
    const uint32_t mag = a.is_signed ? rep & ((1u << (a.n - 1)) - 1u) : rep;
    const int ebits = a.n - a.m - (a.is_signed ? 1 : 0);
    return mag > (((1u << ebits) - 1u) << a.m);
}

__device__ __forceinline__ int clz32(uint32_t v) { return __clz((int)v); }

// convert_float_to_rep, src/lo_pack.hpp:109-287. RoundMantissa sees the
// reference's default positive-sign flag (false).
template <int MODE>
__device__ __forceinline__ uint32_t codec_encode(float from, const CodecArg& a, uint64_t r) {
    const int n = a.n, toMant = a.m;
    const int toExpBits = a.is_signed ? n - toMant - 1 : n - toMant;
    const int kExponentOffset = a.bias - 127;
    const int kDigitShift = toMant - 23;
    const int toMinExp = 1 - a.bias;
    const int toMaxExp = (1 << toExpBits) - 1 - a.bias;
    const uint32_t signmask = a.is_signed ? (1u << (n - 1)) : 0u;
    const uint32_t maxFinite = a.has_inf ? a.pos_inf - 1u
                                         : (a.is_signed ? (((1u << n) - 1u) >> 1) : ((1u << n) - 1u));
    const uint32_t infRep = a.has_inf ? a.pos_inf : maxFinite;
    const uint32_t fb = __float_as_uint(from);
    const bool neg = (fb >> 31) != 0;
    auto with_sign = [&](uint32_t mag) -> uint32_t {
        if (!neg || !a.is_signed) return mag;
        if (mag == 0u && c_is_nan(signmask, a)) return 0u;
        return mag | signmask;
    };
    if (!a.is_signed && neg) return a.neg_to_nan ? (a.nan3109 ? a.qnan : a.snan) : 0u;
    const uint32_t from_bits = fb & 0x7FFFFFFFu;
    if (from_bits == 0x7F800000u)
        return with_sign((a.sat != LOFGB_SAT_FINITE && a.has_inf) ? infRep : maxFinite);
    if (from_bits > 0x7F800000u) return a.qnan;
    if (from_bits == 0u) return with_sign(0u);
    const int bfe = (int)(from_bits >> 23);
    if (toMinExp < -125 && bfe == 0) {  // branch 1
        uint64_t bits = from_bits;
        const int norm = clz32(from_bits) - (32 - 23) + 1;
        const int bexp = kExponentOffset - norm + 1;
        if (bexp <= 0) {
            if (kExponentOffset < 64) bits <<= kExponentOffset;
        } else {
            bits <<= norm;
            bits &= ~(1ull << 23);
            bits |= (uint64_t)bexp << 23;
        }
        bits = round_mantissa<MODE, 64, uint64_t>(bits, -kDigitShift, a.mode, a.len, false, r);
        bits >>= -kDigitShift;
        return with_sign((uint32_t)bits);
    }
    if (toMinExp > -125) {  // branch 2: target-subnormal or zero
        const int bte = (bfe - 127) + a.bias;
        if (bte <= 0) {
            const uint32_t lead = bfe > 0 ? 1u : 0u;
            const int shift = -kDigitShift - bte + (int)lead;
            uint32_t rfb = (from_bits & 0x7FFFFFu) | (lead << 23);
            uint32_t bits = 0;
            if (shift <= 24) {
                rfb = round_mantissa<MODE, 32, uint32_t>(rfb, shift, a.mode, a.len, false, r);
                bits = rfb >> shift;
            } else {
                const int mode = MODE >= 0 ? MODE : a.mode;
                switch (mode) {
                case LOFGB_RTO:
                case LOFGB_RAFZ: bits = rfb > 0 ? 1u : 0u; break;
                case LOFGB_RU: bits = (rfb && !neg) ? 1u : 0u; break;
                case LOFGB_RD: bits = (rfb && neg) ? 1u : 0u; break;
                case LOFGB_SR_A: case LOFGB_SR_B: case LOFGB_SR_C: case LOFGB_SR_D:
                case LOFGB_TRUE_SR: case LOFGB_PROB: {
                    // shifts of 64 or more are undefined in the reference: 0
                    const uint64_t w = round_mantissa<MODE, 64, uint64_t>(rfb, shift, a.mode, a.len,
                                                                          false, r);
                    bits = shift >= 64 ? 0u : (uint32_t)(w >> shift);
                    break;
                }
                default: bits = 0; break;
                }
            }
            return with_sign(bits);
        }
    }
    uint64_t rfb = from_bits;  // normal path
    rfb = round_mantissa<MODE, 64, uint64_t>(rfb, -kDigitShift, a.mode, a.len, false, r);
    rfb &= ~((1ull << (-kDigitShift)) - 1ull);
    rfb += (uint64_t)(int64_t)kExponentOffset << 23;
    const uint64_t aligned_highest = (uint64_t)maxFinite << (-kDigitShift);
    const uint32_t bits = (uint32_t)(rfb >> (-kDigitShift));
    const bool narrower = (toMaxExp < 128) || (toMaxExp == 128 && toMant + 1 < 24);
    if (narrower && rfb > aligned_highest)
        return with_sign((a.sat == LOFGB_OVF_INF && a.has_inf) ? infRep : maxFinite);
    return with_sign(bits);
}

// convert_float_to_rep under RNE for formats whose subnormals sit inside
// FP32's range (CodecArg::enc_fast): the same code as codec_encode,
// branch-free. The float grid reproduces RoundMantissa's RNE on the normal
// branch and on the target-subnormal branch alike (including the reference's
// shift > 24 table, 0 for RNE). A target-subnormal v is a multiple of tiny
// below 2^to_min, so v + 2^23 tiny is exact and its word minus that of
// 2^23 tiny is v / tiny, the code. Every code above the largest finite one
// becomes ovf_code, which is that code or the next (infinity), so the
// overflow test is a min. SPECIAL = false leaves out the infinity and NaN
// inputs (the caller has checked that its warp holds none).
template <bool SPECIAL>
__device__ __forceinline__ uint32_t codec_encode_fast(float from, const CodecArg& a) {
    const uint32_t fb = __float_as_uint(from);
    const bool neg = (fb >> 31) != 0;
    const uint32_t mb = fb & 0x7FFFFFFFu;
    const uint32_t cb = min(max(fb & 0x7F800000u, a.uni_lo), a.uni_hi) + a.uni_d;
    const float c = __uint_as_float(cb);
    const float ax = __uint_as_float(mb);
    const float v = __fsub_rn(__fadd_rn(ax, c), c);
    const uint32_t vb = __float_as_uint(v);
    uint32_t code = vb >= a.min_norm_bits ? (vb >> (23 - a.m)) - a.code_off
                                          : __float_as_uint(__fadd_rn(v, a.sub_c)) - __float_as_uint(a.sub_c);
    code = min(code, a.ovf_code);
    if (!SPECIAL) {
        // finite input: the sign rules of both signednesses in one form
        // (signed: -0 -> neg_zero_code, else code | sign; unsigned: neg_code)
        const uint32_t ns = code == 0u ? a.neg_zero : ((code & a.neg_keep) | a.neg_or);
        return neg ? ns : code;
    }
    code = mb == 0x7F800000u ? a.inf_code : code;
    code = (neg && a.is_signed) ? (code == 0u ? a.neg_zero_code : (code | a.sign_mask)) : code;
    code = mb > 0x7F800000u ? a.qnan : code;
    return (neg && !a.is_signed) ? a.neg_code : code;
}

// The fast encode with the target-normal range rounded by Veltkamp's split:
// for a normal FP32 |x| and 1 <= 23 - m <= 22, t - (t - |x|) with
// t = |x| (2^(23-m) + 1) is |x| rounded to m bits, ties to even, whenever t
// is finite (checked over every FP32 pattern), which is codec_encode_fast's
// float-grid result; a t that overflows only happens far above the largest
// finite code, and its NaN or infinity bits give a code above ovf_code, which
// the min clamps as before. Inputs below the smallest target normal take the
// tiny grid as in codec_encode_fast (a value that rounds up to 2^to_min
// there gives the first normal code, 2^m). Fewer ALU-pipe operations than
// the clamped grid constant.
template <bool SPECIAL>
__device__ __forceinline__ uint32_t codec_encode_velt(float from, const CodecArg& a) {
    const uint32_t fb = __float_as_uint(from);
    const bool neg = (fb >> 31) != 0;
    const uint32_t mb = fb & 0x7FFFFFFFu;
    const float ax = __uint_as_float(mb);
    const float t = __fmul_rn(ax, a.sigma);
    const float v = __fmaf_rn(__fmaf_rn(ax, -1.0f, t), -1.0f, t);
    const uint32_t nrm = (__float_as_uint(v) >> (23 - a.m)) - a.code_off;
    const uint32_t sub = __float_as_uint(__fadd_rn(ax, a.sub_c)) - __float_as_uint(a.sub_c);
    uint32_t code = min(mb < a.min_norm_bits ? sub : nrm, a.ovf_code);
    if (!SPECIAL) {
        const uint32_t ns = code == 0u ? a.neg_zero : ((code & a.neg_keep) | a.neg_or);
        return neg ? ns : code;
    }
    code = mb == 0x7F800000u ? a.inf_code : code;
    code = (neg && a.is_signed) ? (code == 0u ? a.neg_zero_code : (code | a.sign_mask)) : code;
    code = mb > 0x7F800000u ? a.qnan : code;
    return (neg && !a.is_signed) ? a.neg_code : code;
}

// The fast encode of one value: Veltkamp form where it applies, else the
// clamped float grid (a.velt is uniform over the launch).
template <bool SPECIAL>
__device__ __forceinline__ uint32_t encode_fast_any(float from, const CodecArg& a) {
    return a.velt ? codec_encode_velt<SPECIAL>(from, a) : codec_encode_fast<SPECIAL>(from, a);
}

// convert_rep_to_float for formats whose values FP32 holds exactly
// (CodecArg::dec_fast).
__device__ __forceinline__ float codec_decode_fast(uint32_t rep, const CodecArg& a) {
    const uint32_t sbit = a.is_signed ? (rep >> (a.n - 1)) & 1u : 0u;
    const uint32_t mag = rep & ~a.sign_mask;
    const uint32_t e = mag >> a.m;
    // mag * tiny for a subnormal code (mag < 2^m): the word of 2^23 tiny plus
    // mag is 2^23 tiny + mag * tiny exactly; subtracting 2^23 tiny is exact
    const float sub = __fsub_rn(__uint_as_float(__float_as_uint(a.sub_c_dec) + mag), a.sub_c_dec);
    const uint32_t nb = (mag << (23 - a.m)) - a.code_off_dec;
    uint32_t vb = e == 0 ? __float_as_uint(sub) : nb;
    vb = c_is_nan(rep, a) ? 0x7FC00000u : (vb | (sbit << 31));
    // infinity is tested first, as convert_rep_to_float does
    vb = (a.has_inf && (rep | a.inf_or) == a.inf_match) ? (0x7F800000u | (sbit << 31)) : vb;
    return __uint_as_float(vb);
}

// convert_rep_to_float, src/lo_pack.hpp:293-320.
__device__ __forceinline__ float codec_decode(uint32_t rep, const CodecArg& a) {
    const int n = a.n;
    rep &= (1u << n) - 1u;
    const bool sign = a.is_signed ? ((rep >> (n - 1)) & 1u) != 0 : false;
    const uint32_t mag = a.is_signed ? rep & ((1u << (n - 1)) - 1u) : rep;
    if (a.has_inf && (rep | a.inf_or) == a.inf_match) return sign ? -INFINITY : INFINITY;
    if (c_is_nan(rep, a)) return __uint_as_float(0x7FC00000u);
    // the value is an integer k < 2^16 times 2^x: k converts to float
    // exactly and ldexpf rounds k * 2^x once, as the reference's exact double
    // narrowed to float does
    const uint32_t e = mag >> a.m, mf = mag & ((1u << a.m) - 1u);
    const uint32_t k = e == 0 ? mf : (mf | (1u << a.m));
    const int x = (e == 0 ? 1 : (int)e) - a.bias - a.m;
    const float v = ldexpf(__uint2float_rn(k), x < -300 ? -300 : (x > 300 ? 300 : x));
    return sign ? -v : v;
}

// One code's value: the direct bit construction for the formats that allow
// it, else the general restatement.
template <bool FAST>
__device__ __forceinline__ float decode_one(uint32_t rep, const CodecArg& a) {
    if constexpr (FAST) return codec_decode_fast(rep, a);
    else return codec_decode(rep, a);
}

constexpr int cgcd(int x, int y) { return y == 0 ? x : cgcd(y, x % y); }

// Codes per group for width N: lcm(N, 8) bits for N <= 8, lcm(N, 16) above.
template <int N>
struct Group {
    static constexpr int AL = N <= 8 ? 8 : 16;
    static constexpr int BITS = N / cgcd(N, AL) * AL;
    static constexpr int GC = BITS / N;
};

// The chunk element whose code fills slot s of the lane's bit stream: slots
// run in stream order; within a group they hold elements in order (forward)
// or in reverse order (reverse).
template <int N, bool REV>
__device__ __forceinline__ int slot_element(int s) {
    constexpr int GC = Group<N>::GC;
    if (!REV) return s;
    const int g = s / GC, k = s - g * GC;
    return g * GC + (GC - 1 - k);
}

template <int N, bool REV, int MODE, int FAST>
__global__ void __launch_bounds__(CT)
encode_kernel(const float* __restrict__ src, uint32_t* __restrict__ dst, int64_t count,
              int64_t out_bytes, CodecArg a) {
    pdl_wait();
    __shared__ float sx[CT / 32][TILE + 32];
    __shared__ uint32_t sw[CT / 32][32 * (N + 1)];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t ntiles = (count + TILE - 1) / TILE;
    const int64_t wstride = (int64_t)gridDim.x * (CT / 32);
    for (int64_t t = (int64_t)blockIdx.x * (CT / 32) + wib; t < ntiles; t += wstride) {
        const int64_t e0 = t * TILE;
        const bool full = e0 + TILE <= count;
        // coalesced loads into the lane-major shared tile (element e at e + e/32)
#pragma unroll
        for (int j = 0; j < TILE / 32; ++j) {
            const int e = j * 32 + lane;
            float v = 0.0f;
            if (full || e0 + e < count) v = __ldcs(src + e0 + e);
            sx[wib][e + (e >> 5)] = v;
        }
        __syncwarp();
        // this lane's 32 codes, appended to a bit stream of N words
        uint32_t* out = &sw[wib][lane * (N + 1)];
        const float* xin = &sx[wib][lane * 33];
        if constexpr (FAST != 0) {
            // fully unrolled: every bit position and shared-memory offset is a constant
            uint64_t acc = 0;
            int fill = 0, widx = 0;
#pragma unroll
            for (int s = 0; s < 32; ++s) {
                const uint32_t code = codec_encode_fast<true>(xin[slot_element<N, REV>(s)], a) &
                                      ((1u << N) - 1u);
                acc |= (uint64_t)code << fill;
                fill += N;
                if (fill >= 32) {
                    out[widx++] = (uint32_t)acc;
                    acc >>= 32;
                    fill -= 32;
                }
            }
        } else {
            uint64_t acc = 0;
            int fill = 0, widx = 0;
#pragma unroll 2
            for (int s = 0; s < 32; ++s) {
                const int i = slot_element<N, REV>(s);
                const int e = lane * 32 + i;
                const float x = xin[i];
                const uint64_t r = mode_is_stochastic(MODE >= 0 ? MODE : a.mode)
                                       ? rng_elem(a.seed, a.offset + (uint64_t)(e0 + e), a.rng_lg) : 0ull;
                const uint32_t code = codec_encode<MODE>(x, a, r) & ((1u << N) - 1u);
                acc |= (uint64_t)code << fill;
                fill += N;
                if (fill >= 32) {
                    out[widx++] = (uint32_t)acc;
                    acc >>= 32;
                    fill -= 32;
                }
            }
        }
        __syncwarp();
        // coalesced stores of the tile's 32 N words (bytes past out_bytes are not written)
        const int64_t w0 = t * (32 * N);
        for (int w = lane; w < 32 * N; w += 32) {
            const uint32_t v = sw[wib][(w / N) * (N + 1) + (w % N)];
            const int64_t byte = (w0 + w) * 4;
            if (byte + 4 <= out_bytes) {
                dst[w0 + w] = v;
            } else if (byte < out_bytes) {
                uint8_t* d8 = reinterpret_cast<uint8_t*>(dst) + byte;
                for (int q = 0; q < 4 && byte + q < out_bytes; ++q) d8[q] = (uint8_t)(v >> (8 * q));
            }
        }
        __syncwarp();
    }
}

// ---- direct kernels for 4-, 8- and 16-bit codes -----------------------------
// With N in {4, 8, 16} the codes of four consecutive values fill exactly
// 4N bits of the stream (two bytes, four bytes, eight bytes), so a thread
// turns one float4 into one 16/32/64-bit store and back, with no staging:
// for N = 8 and 16 a group holds one code (the group order changes
// nothing); for N = 4 a byte holds two codes, low nibble first (forward) or
// high nibble first (reverse). The last count % 4 values (and the padding
// codes of +0.0 up to the group boundary, as the staged kernel writes them)
// go through one thread that writes only the bytes below the packed size.
template <int N>
struct Chunk;
template <> struct Chunk<4> { using T = uint16_t; };
template <> struct Chunk<8> { using T = uint32_t; };
template <> struct Chunk<16> { using T = uint2; };

template <int N, bool REV>
__device__ __forceinline__ uint64_t pack4(const uint32_t (&c)[4]) {
    constexpr uint32_t M = (1u << N) - 1u;
    if (N == 4 && REV)
        return (uint64_t)((c[1] & M) | (c[0] & M) << 4 | (c[3] & M) << 8 | (c[2] & M) << 12);
    return (uint64_t)(c[0] & M) | (uint64_t)(c[1] & M) << N | (uint64_t)(c[2] & M) << (2 * N) |
           (uint64_t)(c[3] & M) << (3 * N);
}

template <int N, bool REV>
__device__ __forceinline__ void unpack4(uint64_t w, uint32_t (&c)[4]) {
    constexpr uint32_t M = (1u << N) - 1u;
#pragma unroll
    for (int q = 0; q < 4; ++q) c[q] = (uint32_t)(w >> (q * N)) & M;
    if (N == 4 && REV) {
        const uint32_t t0 = c[0], t2 = c[2];
        c[0] = c[1]; c[1] = t0; c[2] = c[3]; c[3] = t2;
    }
}

template <int N, int MODE, int FAST>
__device__ __forceinline__ void encode4(const float (&x)[4], uint32_t (&c)[4], const CodecArg& a,
                                        uint64_t e) {
    if constexpr (FAST != 0) {
        // infinities and NaNs are rare: their checks run only in warps that hold one
        bool sp = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) sp |= (__float_as_uint(x[q]) & 0x7FFFFFFFu) >= 0x7F800000u;
        if (__any_sync(__activemask(), sp)) {
#pragma unroll
            for (int q = 0; q < 4; ++q) c[q] = encode_fast_any<true>(x[q], a);
        } else if (a.velt) {
#pragma unroll
            for (int q = 0; q < 4; ++q) c[q] = codec_encode_velt<false>(x[q], a);
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) c[q] = codec_encode_fast<false>(x[q], a);
        }
    } else {
        uint64_t r[4] = {0ull, 0ull, 0ull, 0ull};
        if (mode_is_stochastic(MODE >= 0 ? MODE : a.mode)) rng_elem4(a.seed, a.offset + e, a.rng_lg, r);
#pragma unroll
        for (int q = 0; q < 4; ++q) c[q] = codec_encode<MODE>(x[q], a, r[q]);
    }
}

template <int N, bool REV, int MODE, int FAST>
__global__ void __launch_bounds__(256)
encode_direct_kernel(const float4* __restrict__ src, uint8_t* __restrict__ dst, int64_t count,
                     int64_t out_bytes, CodecArg a) {
    pdl_wait();
    using T = typename Chunk<N>::T;
    constexpr int RING = 4;  // per-thread cp.async stages (RING - 1 vectors in flight)
    __shared__ float4 ring[RING][256];
    const int64_t nvec = count >> 2;
    const int64_t stride = (int64_t)gridDim.x * 256;
    T* out = reinterpret_cast<T*>(dst);
    const int64_t v0 = (int64_t)blockIdx.x * 256 + threadIdx.x;
#pragma unroll
    for (int k = 0; k < RING - 1; ++k) {
        if (v0 + k * stride < nvec) cp_async16(&ring[k][threadIdx.x], src + v0 + k * stride);
        cp_async_commit();
    }
    int stage = 0;
    for (int64_t v = v0; v < nvec; v += stride) {
        const int64_t vp = v + (RING - 1) * stride;
        if (vp < nvec) cp_async16(&ring[stage == 0 ? RING - 1 : stage - 1][threadIdx.x], src + vp);
        cp_async_commit();
        cp_async_wait<RING - 1>();
        const float4 f = ring[stage][threadIdx.x];
        stage = stage == RING - 1 ? 0 : stage + 1;
        const float x[4] = {f.x, f.y, f.z, f.w};
        uint32_t c[4];
        encode4<N, MODE, FAST>(x, c, a, (uint64_t)v * 4);
        const uint64_t w = pack4<N, REV>(c);
        if constexpr (N == 16) __stcs(out + v, make_uint2((uint32_t)w, (uint32_t)(w >> 32)));
        else out[v] = (T)w;
    }
    cp_async_wait<0>();
    if ((count & 3) && blockIdx.x == 0 && threadIdx.x == 0) {
        const float* s = reinterpret_cast<const float*>(src);
        float x[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) x[q] = nvec * 4 + q < count ? s[nvec * 4 + q] : 0.0f;
        uint32_t c[4];
        encode4<N, MODE, FAST>(x, c, a, (uint64_t)nvec * 4);
        const uint64_t w = pack4<N, REV>(c);
        const int64_t b0 = nvec * (N / 2);
        for (int q = 0; q < N / 2 && b0 + q < out_bytes; ++q) dst[b0 + q] = (uint8_t)(w >> (8 * q));
    }
}

template <int N, bool REV, bool FAST>
__global__ void __launch_bounds__(256)
decode_direct_kernel(const uint8_t* __restrict__ src, float4* __restrict__ dst, int64_t count,
                     int64_t in_bytes, CodecArg a) {
    pdl_wait();
    using T = typename Chunk<N>::T;
    constexpr int U = 1;  // code loads in flight per thread (four measured no faster)
    const int64_t nvec = count >> 2;
    const int64_t stride = (int64_t)gridDim.x * 256;
    const T* in = reinterpret_cast<const T*>(src);
    for (int64_t v0 = (int64_t)blockIdx.x * 256 + threadIdx.x; v0 < nvec; v0 += U * stride) {
        uint64_t w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            w[u] = 0;
            if (v0 + u * stride < nvec) {
                if constexpr (N == 16) {
                    const uint2 t = __ldcs(in + v0 + u * stride);
                    w[u] = (uint64_t)t.x | (uint64_t)t.y << 32;
                } else {
                    w[u] = __ldcs(in + v0 + u * stride);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t v = v0 + u * stride;
            if (v >= nvec) break;
            uint32_t c[4];
            unpack4<N, REV>(w[u], c);
            float y[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) y[q] = decode_one<FAST>(c[q], a);
            __stcs(dst + v, make_float4(y[0], y[1], y[2], y[3]));
        }
    }
    if ((count & 3) && blockIdx.x == 0 && threadIdx.x == 0) {
        const int64_t b0 = nvec * (N / 2);
        uint64_t w = 0;
        for (int q = 0; q < N / 2 && b0 + q < in_bytes; ++q) w |= (uint64_t)src[b0 + q] << (8 * q);
        uint32_t c[4];
        unpack4<N, REV>(w, c);
        float* d = reinterpret_cast<float*>(dst);
        for (int q = 0; nvec * 4 + q < count; ++q)
            d[nvec * 4 + q] = FAST ? codec_decode_fast(c[q], a) : codec_decode(c[q], a);
    }
}

// ---- chunk kernels for the other widths ------------------------------------
// G = lcm(N, 32) / N consecutive codes fill exactly W = lcm(N, 32) / 32 words
// and hold whole groups (a group is lcm(N, 8 or 16) bits, which divides
// lcm(N, 32)), so a thread encodes G values (G / 4 float4 loads) into W
// words and decodes them back without staging: slots in stream order hold
// the chunk's elements in order (forward) or reversed within each group.
// The last chunk (fewer than G values left) is done by one thread, with
// codes of +0.0 as padding and only the bytes below the packed size written.
template <int N>
struct ChunkGeo {
    static constexpr int L = N / cgcd(N, 32) * 32;  // lcm(N, 32)
    static constexpr int G = L / N;
    static constexpr int W = L / 32;
    static constexpr int V = G / 4;
};

template <int N, bool REV, int MODE, int FAST>
__device__ __forceinline__ void encode_chunk(const float (&x)[ChunkGeo<N>::G], uint32_t (&out)[ChunkGeo<N>::W],
                                             const CodecArg& a, uint64_t e0) {
    constexpr int G = ChunkGeo<N>::G;
    uint32_t c[G];
    if constexpr (FAST != 0) {
        bool sp = false;
#pragma unroll
        for (int i = 0; i < G; ++i) sp |= (__float_as_uint(x[i]) & 0x7FFFFFFFu) >= 0x7F800000u;
        if (__any_sync(__activemask(), sp)) {
#pragma unroll
            for (int i = 0; i < G; ++i) c[i] = encode_fast_any<true>(x[i], a);
        } else if (a.velt) {
#pragma unroll
            for (int i = 0; i < G; ++i) c[i] = codec_encode_velt<false>(x[i], a);
        } else {
#pragma unroll
            for (int i = 0; i < G; ++i) c[i] = codec_encode_fast<false>(x[i], a);
        }
    } else {
#pragma unroll
        for (int i = 0; i < G; i += 4) {
            uint64_t r[4] = {0ull, 0ull, 0ull, 0ull};
            if (mode_is_stochastic(MODE >= 0 ? MODE : a.mode)) rng_elem4(a.seed, a.offset + e0 + i, a.rng_lg, r);
#pragma unroll
            for (int q = 0; q < 4; ++q) c[i + q] = codec_encode<MODE>(x[i + q], a, r[q]);
        }
    }
    uint64_t acc = 0;
    int fill = 0, widx = 0;
#pragma unroll
    for (int sl = 0; sl < G; ++sl) {
        acc |= (uint64_t)(c[slot_element<N, REV>(sl)] & ((1u << N) - 1u)) << fill;
        fill += N;
        if (fill >= 32) {
            out[widx++] = (uint32_t)acc;
            acc >>= 32;
            fill -= 32;
        }
    }
}

template <int N, bool REV, int MODE, int FAST>
__global__ void __launch_bounds__(256)
encode_chunk_kernel(const float4* __restrict__ src, uint32_t* __restrict__ dst, int64_t count,
                    int64_t out_bytes, CodecArg a) {
    pdl_wait();
    using Geo = ChunkGeo<N>;
    const int64_t nch = count / Geo::G;
    for (int64_t ch = (int64_t)blockIdx.x * 256 + threadIdx.x; ch < nch; ch += (int64_t)gridDim.x * 256) {
        float x[Geo::G];
#pragma unroll
        for (int j = 0; j < Geo::V; ++j) {
            const float4 f = __ldcs(src + ch * Geo::V + j);
            x[4 * j] = f.x; x[4 * j + 1] = f.y; x[4 * j + 2] = f.z; x[4 * j + 3] = f.w;
        }
        uint32_t out[Geo::W];
        encode_chunk<N, REV, MODE, FAST>(x, out, a, (uint64_t)ch * Geo::G);
#pragma unroll
        for (int w = 0; w < Geo::W; ++w) __stcs(dst + ch * Geo::W + w, out[w]);
    }
    if (count % Geo::G != 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        const float* s = reinterpret_cast<const float*>(src);
        float x[Geo::G];
#pragma unroll
        for (int i = 0; i < Geo::G; ++i) x[i] = nch * Geo::G + i < count ? s[nch * Geo::G + i] : 0.0f;
        uint32_t out[Geo::W];
        encode_chunk<N, REV, MODE, FAST>(x, out, a, (uint64_t)nch * Geo::G);
        uint8_t* d8 = reinterpret_cast<uint8_t*>(dst);
        const int64_t b0 = nch * Geo::W * 4;
        for (int q = 0; q < Geo::W * 4 && b0 + q < out_bytes; ++q) d8[b0 + q] = (uint8_t)(out[q >> 2] >> (8 * (q & 3)));
    }
}

template <int N, bool REV, bool FAST>
__device__ __forceinline__ void decode_chunk(const uint32_t (&in)[ChunkGeo<N>::W], float (&y)[ChunkGeo<N>::G],
                                             const CodecArg& a) {
    constexpr int G = ChunkGeo<N>::G;
    uint64_t buf = 0;
    int avail = 0, widx = 0;
#pragma unroll
    for (int sl = 0; sl < G; ++sl) {
        if (avail < N) {
            buf |= (uint64_t)in[widx++] << avail;
            avail += 32;
        }
        const uint32_t code = (uint32_t)buf & ((1u << N) - 1u);
        buf >>= N;
        avail -= N;
        y[slot_element<N, REV>(sl)] = decode_one<FAST>(code, a);
    }
}

template <int N, bool REV, bool FAST>
__global__ void __launch_bounds__(256)
decode_chunk_kernel(const uint32_t* __restrict__ src, float4* __restrict__ dst, int64_t count,
                    int64_t in_bytes, CodecArg a) {
    pdl_wait();
    using Geo = ChunkGeo<N>;
    const int64_t nch = count / Geo::G;
    for (int64_t ch = (int64_t)blockIdx.x * 256 + threadIdx.x; ch < nch; ch += (int64_t)gridDim.x * 256) {
        uint32_t in[Geo::W];
#pragma unroll
        for (int w = 0; w < Geo::W; ++w) in[w] = __ldcs(src + ch * Geo::W + w);
        float y[Geo::G];
        decode_chunk<N, REV, FAST>(in, y, a);
#pragma unroll
        for (int j = 0; j < Geo::V; ++j)
            __stcs(dst + ch * Geo::V + j, make_float4(y[4 * j], y[4 * j + 1], y[4 * j + 2], y[4 * j + 3]));
    }
    if (count % Geo::G != 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        const uint8_t* s8 = reinterpret_cast<const uint8_t*>(src);
        const int64_t b0 = nch * Geo::W * 4;
        uint32_t in[Geo::W];
#pragma unroll
        for (int w = 0; w < Geo::W; ++w) in[w] = 0;
        for (int q = 0; q < Geo::W * 4 && b0 + q < in_bytes; ++q) in[q >> 2] |= (uint32_t)s8[b0 + q] << (8 * (q & 3));
        float y[Geo::G];
        decode_chunk<N, REV, FAST>(in, y, a);
        float* d = reinterpret_cast<float*>(dst);
        for (int i = 0; nch * Geo::G + i < count; ++i) d[nch * Geo::G + i] = y[i];
    }
}

// Direct-bits decode for widths N <= 7 that one float4 per lane can serve:
// the four codes of values 4q..4q+3 are the 4N bits at bit 4Nq of the
// stream, read from the two words that cover them (neighbouring lanes read
// neighbouring words, mostly from L1), and the lane writes one float4, so a
// warp's store is 512 contiguous bytes. REV (reversed groups) only where a
// group is exactly four codes (N = 2, 6). nq: quads whose two-word window
// lies inside the input; the rest of the values are decoded by one thread.
template <int N, bool REV, bool FAST>
__global__ void __launch_bounds__(256)
decode_quad_kernel(const uint32_t* __restrict__ src, float4* __restrict__ dst, int64_t nq,
                   int64_t count, int64_t in_bytes, CodecArg a) {
    pdl_wait();
    static_assert(N <= 7 && (!REV || Group<N>::GC == 4), "quad decode");
    constexpr uint32_t CM = (1u << N) - 1u;
    for (int64_t q = (int64_t)blockIdx.x * 256 + threadIdx.x; q < nq; q += (int64_t)gridDim.x * 256) {
        const int64_t b = 4 * N * q;
        const int64_t w0 = b >> 5;
        const uint64_t win = ((uint64_t)__ldg(src + w0 + 1) << 32) | __ldg(src + w0);
        const uint32_t bits = (uint32_t)(win >> (b & 31));
        float y[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) y[REV ? 3 - k : k] = decode_one<FAST>((bits >> (N * k)) & CM, a);
        __stcs(dst + q, make_float4(y[0], y[1], y[2], y[3]));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint8_t* s8 = reinterpret_cast<const uint8_t*>(src);
        float* d = reinterpret_cast<float*>(dst);
        for (int64_t i = nq * 4; i < count; ++i) {
            const int64_t sl = REV ? (i & ~(int64_t)3) + (3 - (i & 3)) : i;   // stream slot of value i
            const int64_t bit = sl * N;
            uint32_t v = 0;
            for (int k = 0; k < 2; ++k)
                if ((bit >> 3) + k < in_bytes) v |= (uint32_t)s8[(bit >> 3) + k] << (8 * k);
            d[i] = decode_one<FAST>((v >> (bit & 7)) & CM, a);
        }
    }
}

template <int N, bool REV, bool FAST>
__global__ void __launch_bounds__(CT)
decode_kernel(const uint32_t* __restrict__ src, float* __restrict__ dst, int64_t count,
              int64_t in_bytes, CodecArg a) {
    pdl_wait();
    __shared__ float sx[CT / 32][TILE + 32];
    __shared__ uint32_t sw[CT / 32][32 * (N + 1)];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t ntiles = (count + TILE - 1) / TILE;
    const int64_t wstride = (int64_t)gridDim.x * (CT / 32);
    for (int64_t t = (int64_t)blockIdx.x * (CT / 32) + wib; t < ntiles; t += wstride) {
        const int64_t e0 = t * TILE;
        const int64_t w0 = t * (32 * N);
        for (int w = lane; w < 32 * N; w += 32) {
            const int64_t byte = (w0 + w) * 4;
            uint32_t v = 0;
            if (byte + 4 <= in_bytes) {
                v = __ldcs(src + w0 + w);
            } else if (byte < in_bytes) {
                const uint8_t* s8 = reinterpret_cast<const uint8_t*>(src) + byte;
                for (int q = 0; q < 4 && byte + q < in_bytes; ++q) v |= (uint32_t)s8[q] << (8 * q);
            }
            sw[wib][(w / N) * (N + 1) + (w % N)] = v;
        }
        __syncwarp();
        const uint32_t* in = &sw[wib][lane * (N + 1)];
        float* xout = &sx[wib][lane * 33];
        uint64_t buf = 0;
        int avail = 0, widx = 0;
        if constexpr (FAST) {
#pragma unroll
            for (int s = 0; s < 32; ++s) {
                if (avail < N) {
                    buf |= (uint64_t)in[widx++] << avail;
                    avail += 32;
                }
                const uint32_t code = (uint32_t)buf & ((1u << N) - 1u);
                buf >>= N;
                avail -= N;
                xout[slot_element<N, REV>(s)] = codec_decode_fast(code, a);
            }
        } else {
#pragma unroll 2
            for (int s = 0; s < 32; ++s) {
                if (avail < N) {
                    buf |= (uint64_t)in[widx++] << avail;
                    avail += 32;
                }
                const uint32_t code = (uint32_t)buf & ((1u << N) - 1u);
                buf >>= N;
                avail -= N;
                xout[slot_element<N, REV>(s)] = codec_decode(code, a);
            }
        }
        __syncwarp();
        const bool full = e0 + TILE <= count;
#pragma unroll
        for (int j = 0; j < TILE / 32; ++j) {
            const int e = j * 32 + lane;
            if (full || e0 + e < count) __stcs(dst + e0 + e, sx[wib][e + (e >> 5)]);
        }
        __syncwarp();
    }
}

int64_t packed_bytes(int n, int64_t count) {
    const int al = n <= 8 ? 8 : 16;
    int x = n, y = al;
    while (y) { const int t = x % y; x = y; y = t; }
    const int gbits = n / x * al, gc = gbits / n;
    return (count + gc - 1) / gc * (gbits / 8);
}

int make_codec_arg(CodecArg* a, const lofgb_codec_format* f, int mode, int sat, int len) {
    if (!f) return set_error(LOFGB_ERR_NULL, "NULL codec format");
    const lofgb_format& F = f->fmt;
    if (F.bitwidth < 1 || F.bitwidth > 16)
        return set_error(LOFGB_ERR_FORMAT, "codec bitwidth %d outside [1, 16]", F.bitwidth);
    const int ebits = F.bitwidth - F.mantissa_bits - (F.signedness == LOFGB_SIGNED ? 1 : 0);
    if (F.mantissa_bits < 0 || ebits < 0)
        return set_error(LOFGB_ERR_FORMAT, "codec mantissa bits %d do not fit %d bits",
                         F.mantissa_bits, F.bitwidth);
    if (F.bias < -(1 << 20) || F.bias > (1 << 20))
        return set_error(LOFGB_ERR_FORMAT, "bias %d outside [-2^20, 2^20]", F.bias);
    if (f->nan_kind > LOFGB_NAN_NONE) return set_error(LOFGB_ERR_FORMAT, "unknown NaN kind");
    if (mode < 0 || mode >= LOFGB_NUM_MODES) return set_error(LOFGB_ERR_MODE, "unknown mode %d", mode);
    if (sat < 0 || sat > LOFGB_SAT_PROPAGATE) return set_error(LOFGB_ERR_MODE, "unknown saturation mode %d", sat);
    if (len < 0 || len > 62) return set_error(LOFGB_ERR_MODE, "stoch_len %d outside [0, 62]", len);
    a->rng_lg = rng_lanes_log2(mode, len);
    a->n = F.bitwidth;
    a->m = F.mantissa_bits;
    a->bias = F.bias;
    a->is_signed = F.signedness == LOFGB_SIGNED;
    a->has_inf = F.inf_behavior != LOFGB_INF_SATURATING;
    a->nan3109 = F.nan_behavior == LOFGB_NAN_3109;
    a->inf_or = f->inf_or;
    a->inf_match = f->inf_match;
    a->pos_inf = f->pos_inf;
    a->qnan = f->qnan;
    a->snan = f->snan;
    a->nan_kind = f->nan_kind;
    a->neg_to_nan = f->neg_to_nan;
    a->mode = mode;
    a->sat = sat;
    a->len = len;
    // fast paths (see CodecArg)
    const int n = a->n, m = a->m, bias = a->bias;
    const int to_min = 1 - bias;
    const int to_max = (1 << ebits) - 1 - bias;
    a->sign_mask = a->is_signed ? (1u << (n - 1)) : 0u;
    a->max_finite = a->has_inf ? a->pos_inf - 1u
                               : (a->is_signed ? (((1u << n) - 1u) >> 1) : ((1u << n) - 1u));
    const uint32_t inf_rep = a->has_inf ? a->pos_inf : a->max_finite;
    a->inf_code = (sat != LOFGB_SAT_FINITE && a->has_inf) ? inf_rep : a->max_finite;
    a->ovf_code = (sat == LOFGB_OVF_INF && a->has_inf) ? inf_rep : a->max_finite;
    a->neg_code = a->neg_to_nan ? (a->nan3109 ? a->qnan : a->snan) : 0u;
    bool sign_only_nan = false;  // IsNaN(sign-only code)
    if (a->is_signed) {
        const uint32_t sm = a->sign_mask;
        if (a->nan_kind == LOFGB_NAN_PATTERN) sign_only_nan = sm == a->qnan;
        else if (a->nan_kind == LOFGB_NAN_IEEE) sign_only_nan = false;  // magnitude 0
    }
    a->neg_zero_code = sign_only_nan ? 0u : a->sign_mask;
    a->neg_keep = a->is_signed ? 0xFFFFFFFFu : 0u;
    a->neg_or = a->is_signed ? a->sign_mask : a->neg_code;
    a->neg_zero = a->is_signed ? a->neg_zero_code : a->neg_code;
    const bool narrower = to_max < 128 || (to_max == 128 && m + 1 < 24);
    const int d = 23 - m;
    const int hi = to_max + 1 + 127;
    a->enc_fast = 0;
    if (mode == LOFGB_RNE && narrower &&
        to_min > -125 && bias >= -100 && bias + m - 1 <= 127 && hi + d <= 254 &&
        to_min + 127 + d >= 1 && hi >= to_min + 127 &&
        (a->ovf_code == a->max_finite || a->ovf_code == a->max_finite + 1u)) {
        a->enc_fast = 1;
        a->uni_lo = (uint32_t)(to_min + 127) << 23;
        a->uni_hi = (uint32_t)hi << 23;
        a->uni_d = (uint32_t)d << 23;
        a->min_norm_bits = (uint32_t)(to_min + 127) << 23;
        a->code_off = (uint32_t)(127 - bias) << m;
        a->sub_c = std::ldexp(1.0f, to_min - m + 23);
    }
    a->velt = 0;
    a->sigma = 0.0f;
    if (a->enc_fast == 1 && m >= 1 && m <= 22) {
        a->velt = 1;
        a->sigma = (float)((1u << (23 - m)) + 1u);
    }
    a->dec_fast = 0;
    if (to_min + 127 >= 1 && to_max + 127 <= 254 && to_min - m >= -149 && to_min - m + 23 <= 127) {
        a->dec_fast = 1;
        a->tiny = std::ldexp(1.0f, to_min - m);
        a->sub_c_dec = std::ldexp(1.0f, to_min - m + 23);
        a->code_off_dec = (uint32_t)(bias - 127) << 23;
    }
    return LOFGB_OK;
}

int grid_for(int64_t count) {
    const int64_t tiles = (count + TILE - 1) / TILE;
    int64_t g = (tiles + (CT / 32) - 1) / (CT / 32);
    const int64_t maxg = (int64_t)sm_count() * (2048 / CT);
    if (g < 1) g = 1;
    return (int)(g < maxg ? g : maxg);
}

// grid of the direct kernels: one float4 per thread per step, at most
// 8 CTAs of 256 threads per SM
int grid_direct(int64_t count) {
    const int64_t need = ((count >> 2) + 255) / 256;
    const int64_t maxg = (int64_t)sm_count() * 8;
    return (int)(need < 1 ? 1 : (need < maxg ? need : maxg));
}

// grid of the chunk kernels: one chunk of g values per thread per step
int grid_chunk(int64_t count, int g) {
    const int64_t need = (count / g + 255) / 256;
    const int64_t maxg = (int64_t)sm_count() * 8;
    return (int)(need < 1 ? 1 : (need < maxg ? need : maxg));
}

template <int N>
int launch_encode_n(const float* src, uint8_t* dst, int64_t count, int reverse, const CodecArg& a,
                    cudaStream_t st) {
    const int grid = grid_for(count);
    const int64_t ob = packed_bytes(N, count);
    if constexpr (N == 4 || N == 8 || N == 16) {
        if ((reinterpret_cast<uintptr_t>(src) & 15) == 0 &&
            (reinterpret_cast<uintptr_t>(dst) & (N / 2 - 1)) == 0) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            const int gd = grid_direct(count);
#define LOFGB_ENCD(R, M, F) launch_pdl(encode_direct_kernel<N, R, M, F>, gd, 256, 0, st, s4, dst, count, ob, a)
            if (a.enc_fast == 1) {
                if (reverse) LOFGB_ENCD(true, LOFGB_RNE, 1); else LOFGB_ENCD(false, LOFGB_RNE, 1);
            } else {
                if (reverse) LOFGB_ENCD(true, -1, 0); else LOFGB_ENCD(false, -1, 0);
            }
#undef LOFGB_ENCD
            return check_launch("encode_direct_kernel");
        }
    } else {
        // the float-grid RNE encode (the common case); other modes stay staged
        if (a.enc_fast == 1 && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            uint32_t* d32 = reinterpret_cast<uint32_t*>(dst);
            const int gc = grid_chunk(count, ChunkGeo<N>::G);
#define LOFGB_ENCC(R) launch_pdl(encode_chunk_kernel<N, R, LOFGB_RNE, 1>, gc, 256, 0, st, s4, d32, count, ob, a)
            if (reverse) LOFGB_ENCC(true); else LOFGB_ENCC(false);
#undef LOFGB_ENCC
            return check_launch("encode_chunk_kernel");
        }
    }
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
#define LOFGB_ENC(R, M, F) launch_pdl(encode_kernel<N, R, M, F>, grid, CT, 0, st, src, d, count, ob, a)
#define LOFGB_ENC_R(M, F) do { if (reverse) LOFGB_ENC(true, M, F); else LOFGB_ENC(false, M, F); } while (0)
    // the float-grid path for RNE (the codec's common mode); every other
    // mode and format through the general restatement
    if (a.enc_fast == 1) LOFGB_ENC_R(LOFGB_RNE, 1);
    else LOFGB_ENC_R(-1, 0);
#undef LOFGB_ENC_R
#undef LOFGB_ENC
    return check_launch("encode_kernel");
}

template <int N>
int launch_decode_n(const uint8_t* src, float* dst, int64_t count, int reverse, const CodecArg& a,
                    cudaStream_t st) {
    const int grid = grid_for(count);
    const int64_t ib = packed_bytes(N, count);
    if constexpr (N == 4 || N == 8 || N == 16) {
        if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0 &&
            (reinterpret_cast<uintptr_t>(src) & (N / 2 - 1)) == 0) {
            float4* d4 = reinterpret_cast<float4*>(dst);
            const int gd = grid_direct(count);
#define LOFGB_DECD(R, F) launch_pdl(decode_direct_kernel<N, R, F>, gd, 256, 0, st, src, d4, count, ib, a)
            if (a.dec_fast) {
                if (reverse) LOFGB_DECD(true, true); else LOFGB_DECD(false, true);
            } else {
                if (reverse) LOFGB_DECD(true, false); else LOFGB_DECD(false, false);
            }
#undef LOFGB_DECD
            return check_launch("decode_direct_kernel");
        }
    } else {
        // direct-bits decode (formats FP32 holds exactly); others stay staged
        if constexpr (N <= 7) {
            if (a.dec_fast && (reinterpret_cast<uintptr_t>(dst) & 15) == 0 &&
                (!reverse || Group<N>::GC == 4)) {
                // quads whose two-word window [w0, w0 + 1] lies inside the input
                const int64_t words = ib / 4;
                const int64_t qlim = words >= 2 ? (8 * (words - 1) + N - 1) / N : 0;
                const int64_t nq = std::min(count / 4, qlim);
                const int64_t need = (nq + 255) / 256;
                const int64_t maxg = (int64_t)sm_count() * 8;
                const int gq = (int)(need < 1 ? 1 : (need < maxg ? need : maxg));
                float4* d4 = reinterpret_cast<float4*>(dst);
                const uint32_t* s32 = reinterpret_cast<const uint32_t*>(src);
                if (reverse) {
                    if constexpr (Group<N>::GC == 4)
                        launch_pdl(decode_quad_kernel<N, true, true>, gq, 256, 0, st, s32, d4, nq, count, ib, a);
                } else {
                    launch_pdl(decode_quad_kernel<N, false, true>, gq, 256, 0, st, s32, d4, nq, count, ib, a);
                }
                return check_launch("decode_quad_kernel");
            }
        }
        if (a.dec_fast && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
            float4* d4 = reinterpret_cast<float4*>(dst);
            const uint32_t* s32 = reinterpret_cast<const uint32_t*>(src);
            const int gc = grid_chunk(count, ChunkGeo<N>::G);
#define LOFGB_DECC(R) launch_pdl(decode_chunk_kernel<N, R, true>, gc, 256, 0, st, s32, d4, count, ib, a)
            if (reverse) LOFGB_DECC(true); else LOFGB_DECC(false);
#undef LOFGB_DECC
            return check_launch("decode_chunk_kernel");
        }
    }
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    if (a.dec_fast) {
        if (reverse) launch_pdl(decode_kernel<N, true, true>, grid, CT, 0, st, s, dst, count, ib, a);
        else launch_pdl(decode_kernel<N, false, true>, grid, CT, 0, st, s, dst, count, ib, a);
    } else {
        if (reverse) launch_pdl(decode_kernel<N, true, false>, grid, CT, 0, st, s, dst, count, ib, a);
        else launch_pdl(decode_kernel<N, false, false>, grid, CT, 0, st, s, dst, count, ib, a);
    }
    return check_launch("decode_kernel");
}

#define LOFGB_BY_N(FN, ...)                                                                   \
    switch (n) {                                                                              \
    case 1: return FN<1>(__VA_ARGS__);   case 2: return FN<2>(__VA_ARGS__);                   \
    case 3: return FN<3>(__VA_ARGS__);   case 4: return FN<4>(__VA_ARGS__);                   \
    case 5: return FN<5>(__VA_ARGS__);   case 6: return FN<6>(__VA_ARGS__);                   \
    case 7: return FN<7>(__VA_ARGS__);   case 8: return FN<8>(__VA_ARGS__);                   \
    case 9: return FN<9>(__VA_ARGS__);   case 10: return FN<10>(__VA_ARGS__);                 \
    case 11: return FN<11>(__VA_ARGS__); case 12: return FN<12>(__VA_ARGS__);                 \
    case 13: return FN<13>(__VA_ARGS__); case 14: return FN<14>(__VA_ARGS__);                 \
    case 15: return FN<15>(__VA_ARGS__); default: return FN<16>(__VA_ARGS__);                 \
    }


// ---- MX storage: round to MX and encode, one pass --------------------------------
// A warp step covers 4 blocks of 32 values; lane l holds values 4l..4l+3 of
// the step, so each block lives in 8 lanes (amax by a 3-step butterfly) and
// each lane's 4 codes are one whole group of the forward packing for 4-, 6-
// and 8-bit codes (2, 3 or 4 bytes at byte offset 4l N / 8). A warp loads
// four steps before it computes; the 16 block scales of those steps are
// rounded one per lane and shuffled back. Per block: the MX scale
// (mx_common.cuh), the rounded quotients q = vr(x / scale, elem) (+0 when the
// scale is not positive), their codes under RNE and the codec's saturation
// (the infinity / NaN checks only in warps that hold one), and the scale's
// code, one byte per block. Values past the end take code bits 0, the
// codec's zero padding.
// DIRECT (RNE into a saturating element format, whose rounding returns an
// overflowing input unchanged): the code of the rounded quotient equals the
// codec's RNE code of the quotient itself for every finite quotient (the
// codec rounds onto the same grid and saturates what overflows), so warps
// without an infinity or NaN encode the quotients directly and only the
// others round first (a NaN quotient must become the canonical NaN).
template <int N, bool UNI, bool DIRECT>
__global__ void __launch_bounds__(256)
mx_encode_kernel(const float* __restrict__ in, uint8_t* __restrict__ codes,
                 uint8_t* __restrict__ scales, int64_t n, RoundPlan pe, RoundPlan ps,
                 float inv_pmn, CodecArg ea, CodecArg sa, uint64_t seed, uint64_t offset, int vec,
                 int64_t code_bytes) {
    static_assert(N == 4 || N == 6 || N == 8, "MX storage codes of 4, 6 or 8 bits");
    // scale codes of the values with a zero mantissa field (+0, the powers
    // of two, +inf: every E8M0 scale) by exponent field, encoded once per CTA
    __shared__ uint8_t scode[256];
    scode[threadIdx.x] = (uint8_t)codec_encode<LOFGB_RNE>(__uint_as_float(threadIdx.x << 23), sa, 0ull);
    __syncthreads();
    pdl_wait();
    constexpr int U = 4;  // steps of 128 values per warp iteration, loaded up front
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * 256 + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * 8;
    const int64_t steps = (n + 127) / 128;
    const bool codes_aligned = (reinterpret_cast<uintptr_t>(codes) & 3) == 0;
    for (int64_t s0 = warp * U; s0 < steps; s0 += nwarps * U) {
        float x[U][4];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t e = (s0 + u) * 128 + lane * 4;
            if (vec && e + 3 < n) {
                const float4 v = __ldcs(reinterpret_cast<const float4*>(in + e));
                x[u][0] = v.x; x[u][1] = v.y; x[u][2] = v.z; x[u][3] = v.w;
            } else {
#pragma unroll
                for (int q = 0; q < 4; ++q) x[u][q] = e + q < n ? __ldcs(in + e + q) : 0.0f;
            }
        }
        // block amax in the 8 lanes of each block, then one scale per block:
        // lane j < 16 rounds the scale of (step j / 4, block j % 4) and every
        // lane fetches its own blocks' scale bits
        float amax[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            amax[u] = fmaxf(fmaxf(fabsf(x[u][0]), fabsf(x[u][1])), fmaxf(fabsf(x[u][2]), fabsf(x[u][3])));
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) amax[u] = fmaxf(amax[u], __shfl_xor_sync(0xFFFFFFFFu, amax[u], o));
        }
        const int uj = (lane >> 2) & 3, bj = lane & 3;
        float aj = 0.0f;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const float g = __shfl_sync(0xFFFFFFFFu, amax[u], bj * 8);
            aj = u == uj ? g : aj;
        }
        const int64_t blkj = (s0 + uj) * 128 + (int64_t)bj * 32;
        const BlockScale bsj = block_scale<-1>(aj, ps, inv_pmn, seed, offset + (uint64_t)blkj);
        const uint32_t sbj = __float_as_uint(bsj.scale);
        if (lane < 16 && blkj < n)
            scales[blkj / 32] = (sbj & 0x807FFFFFu) == 0u ? scode[sbj >> 23]
                                                          : (uint8_t)codec_encode<LOFGB_RNE>(bsj.scale, sa, 0ull);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t e = (s0 + u) * 128 + lane * 4;
            if ((s0 + u) * 128 >= n) break;  // warp-uniform
            const BlockScale b = scale_from_bits(__shfl_sync(0xFFFFFFFFu, sbj, u * 4 + (lane >> 3)));
            uint32_t c[4];
            if constexpr (DIRECT) {
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    w[q] = __float_as_uint(b.pow2 ? __fmul_rn(x[u][q], b.inv) : __fdiv_rn(x[u][q], b.scale));
                float qv[4];
                bool sp = false;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    qv[q] = b.pos ? __uint_as_float(w[q]) : 0.0f;
                    sp |= (__float_as_uint(qv[q]) & 0x7FFFFFFFu) >= 0x7F800000u;
                }
                const bool any_sp = __any_sync(0xFFFFFFFFu, sp);
                if (any_sp) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        qv[q] = b.pos ? __uint_as_float(vr_uni_f32<LOFGB_RNE, 1>(w[q], pe)) : 0.0f;
                }
                if (!ea.enc_fast) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) c[q] = codec_encode<LOFGB_RNE>(qv[q], ea, 0ull);
                } else if (any_sp) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) c[q] = encode_fast_any<true>(qv[q], ea);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; ++q) c[q] = encode_fast_any<false>(qv[q], ea);
                }
            } else {
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    w[q] = __float_as_uint(b.pow2 ? __fmul_rn(x[u][q], b.inv) : __fdiv_rn(x[u][q], b.scale));
                float qv[4];
                bool sp = false;
                if constexpr (UNI) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) w[q] = vr_uni_f32<LOFGB_RNE, 1>(w[q], pe);
                } else {
                    uint64_t r[4] = {0ull, 0ull, 0ull, 0ull};
                    if (mode_is_stochastic(pe.mode)) rng_elem4(seed, offset + (uint64_t)e, pe.rng_lg, r);
                    vr_format_f32x4<-1, false>(w, pe, r);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    qv[q] = b.pos ? __uint_as_float(w[q]) : 0.0f;
                    sp |= (__float_as_uint(qv[q]) & 0x7FFFFFFFu) >= 0x7F800000u;
                }
                if (!ea.enc_fast) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) c[q] = codec_encode<LOFGB_RNE>(qv[q], ea, 0ull);
                } else if (__any_sync(0xFFFFFFFFu, sp)) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) c[q] = encode_fast_any<true>(qv[q], ea);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; ++q) c[q] = encode_fast_any<false>(qv[q], ea);
                }
            }
            // values of this step in the tensor: 128 except in the last step
            const int rem = (int)min((int64_t)128, n - (s0 + u) * 128);
            constexpr uint32_t CM = (1u << N) - 1u;
            uint32_t packed = 0;
            if (rem == 128) {
#pragma unroll
                for (int q = 0; q < 4; ++q) packed |= (c[q] & CM) << (q * N);
            } else {
#pragma unroll
                for (int q = 0; q < 4; ++q) packed |= (lane * 4 + q < rem ? (c[q] & CM) : 0u) << (q * N);
            }
            constexpr int BYTES = N / 2;  // 4 codes of N bits
            const int64_t off = e / 4 * BYTES;
            if (rem == 128 && codes_aligned) {
                // a whole step lies inside the stream: plain stores
                uint8_t* dst = codes + off;
                if constexpr (N == 8) {
                    *reinterpret_cast<uint32_t*>(dst) = packed;
                } else if constexpr (N == 4) {
                    *reinterpret_cast<uint16_t*>(dst) = (uint16_t)packed;
                } else {
#pragma unroll
                    for (int k = 0; k < BYTES; ++k) dst[k] = (uint8_t)(packed >> (8 * k));
                }
            } else if (off < code_bytes) {
                uint8_t* dst = codes + off;
                const bool whole = off + BYTES <= code_bytes;
                if (N == 8 && whole && (reinterpret_cast<uintptr_t>(dst) & 3) == 0) {
                    *reinterpret_cast<uint32_t*>(dst) = packed;
                } else if (N == 4 && whole && (reinterpret_cast<uintptr_t>(dst) & 1) == 0) {
                    *reinterpret_cast<uint16_t*>(dst) = (uint16_t)packed;
                } else {
#pragma unroll
                    for (int k = 0; k < BYTES; ++k)
                        if (off + k < code_bytes) dst[k] = (uint8_t)(packed >> (8 * k));
                }
            }
        }
    }
}

// One co-resident wave of mx_encode_kernel CTAs (fewer for small inputs):
// the grid-stride loop then has no second, partial wave.
template <int N, bool UNI, bool DIRECT>
int mx_encode_grid(int64_t n) {
    static const int per_sm = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, mx_encode_kernel<N, UNI, DIRECT>, 256, 0) !=
                cudaSuccess || b < 1)
            b = 1;
        return b;
    }();
    const int64_t steps = (n + 127) / 128;
    const int64_t need = (steps + 31) / 32;   // 8 warps x 4 steps per CTA iteration
    const int64_t maxg = (int64_t)sm_count() * per_sm;
    return (int)(need < 1 ? 1 : (need < maxg ? need : maxg));
}

template <int N>
int launch_mx_encode_n(const float* in, uint8_t* codes, uint8_t* scales, int64_t n,
                       const RoundPlan& pe, const RoundPlan& ps, float inv_pmn, const CodecArg& ea,
                       const CodecArg& sa, uint64_t seed, uint64_t offset, cudaStream_t st) {
    const int vec = (reinterpret_cast<uintptr_t>(in) & 15) == 0;
    const int64_t cb = packed_bytes(N, n);
    const bool uni = pe.mode == LOFGB_RNE && pe.uni == 1;
    if (uni && pe.sat_and == 0xFFFFFFFFu && pe.sat_or == 0u)
        launch_pdl(mx_encode_kernel<N, true, true>, mx_encode_grid<N, true, true>(n), 256, 0, st, in,
                   codes, scales, n, pe, ps, inv_pmn, ea, sa, seed, offset, vec, cb);
    else if (uni)
        launch_pdl(mx_encode_kernel<N, true, false>, mx_encode_grid<N, true, false>(n), 256, 0, st, in,
                   codes, scales, n, pe, ps, inv_pmn, ea, sa, seed, offset, vec, cb);
    else
        launch_pdl(mx_encode_kernel<N, false, false>, mx_encode_grid<N, false, false>(n), 256, 0, st,
                   in, codes, scales, n, pe, ps, inv_pmn, ea, sa, seed, offset, vec, cb);
    return check_launch("mx_encode_kernel");
}

// MX storage decode: value i = decode(element code i) * decode(scale code of
// block i / 32), one FP32 multiply (round to nearest), as the composition of
// two codec decodes and a product. Every CTA first decodes all 256 scale
// codes into a shared-memory table; then a lane decodes four values (their 4N
// bits from the two words that hold them), reads its block's scale code and
// the table, and writes one float4 (a warp's store is 512 contiguous bytes).
// nq: quads whose two-word window lies inside the element codes; one thread
// decodes the rest.
template <int N, bool FAST>
__global__ void __launch_bounds__(256)
mx_decode_kernel(const uint32_t* __restrict__ codes, const uint8_t* __restrict__ scales,
                 float4* __restrict__ dst, int64_t nq, int64_t count, int64_t code_bytes,
                 CodecArg ea, CodecArg sa) {
    static_assert(N == 4 || N == 6 || N == 8, "MX storage codes of 4, 6 or 8 bits");
    constexpr uint32_t CM = (1u << N) - 1u;
    __shared__ float slut[256];
    slut[threadIdx.x] = sa.dec_fast ? codec_decode_fast(threadIdx.x, sa) : codec_decode(threadIdx.x, sa);
    __syncthreads();
    pdl_wait();
    for (int64_t q = (int64_t)blockIdx.x * 256 + threadIdx.x; q < nq; q += (int64_t)gridDim.x * 256) {
        const int64_t b = 4 * N * q;
        const int64_t w0 = b >> 5;
        const uint32_t lo = __ldg(codes + w0), hi = __ldg(codes + w0 + 1);
        const float sc = slut[__ldg(scales + (q >> 3))];   // block 4q / 32
        const uint32_t bits = (uint32_t)((((uint64_t)hi << 32) | lo) >> (b & 31));
        float y[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) y[k] = __fmul_rn(decode_one<FAST>((bits >> (N * k)) & CM, ea), sc);
        __stcs(dst + q, make_float4(y[0], y[1], y[2], y[3]));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint8_t* s8 = reinterpret_cast<const uint8_t*>(codes);
        float* d = reinterpret_cast<float*>(dst);
        for (int64_t i = nq * 4; i < count; ++i) {
            const int64_t bit = i * N;
            uint32_t v = 0;
            for (int k = 0; k < 2; ++k)
                if ((bit >> 3) + k < code_bytes) v |= (uint32_t)s8[(bit >> 3) + k] << (8 * k);
            d[i] = __fmul_rn(decode_one<FAST>((v >> (bit & 7)) & CM, ea), slut[scales[i / 32]]);
        }
    }
}

template <int N>
int launch_mx_decode_n(const uint8_t* codes, const uint8_t* scales, float* dst, int64_t count,
                       const CodecArg& ea, const CodecArg& sa, cudaStream_t st) {
    const int64_t cb = packed_bytes(N, count);
    const int64_t words = cb / 4;
    const int64_t qlim = words >= 2 ? (8 * (words - 1) + N - 1) / N : 0;
    const int64_t nq = std::min(count / 4, qlim);
    const int64_t need = (nq + 255) / 256;
    const int64_t maxg = (int64_t)sm_count() * 8;
    const int grid = (int)(need < 1 ? 1 : (need < maxg ? need : maxg));
    const uint32_t* c32 = reinterpret_cast<const uint32_t*>(codes);
    float4* d4 = reinterpret_cast<float4*>(dst);
    if (ea.dec_fast)
        launch_pdl(mx_decode_kernel<N, true>, grid, 256, 0, st, c32, scales, d4, nq, count, cb, ea, sa);
    else
        launch_pdl(mx_decode_kernel<N, false>, grid, 256, 0, st, c32, scales, d4, nq, count, cb, ea, sa);
    return check_launch("mx_decode_kernel");
}

int codec_pointers(const void* a, const void* b, int64_t count) {
    if (count < 0) return set_error(LOFGB_ERR_SIZE, "negative count");
    if (count > 0 && (!a || !b)) return set_error(LOFGB_ERR_NULL, "NULL buffer");
    if (count > 0 && ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 3))
        return set_error(LOFGB_ERR_SIZE, "codec buffers must be 4-byte aligned");
    return LOFGB_OK;
}

}  // namespace

}  // namespace lofgb

using namespace lofgb;

extern "C" {

size_t lofgb_packed_size(int bitwidth, int64_t count) {
    if (bitwidth < 1 || bitwidth > 16 || count < 0) return 0;
    return (size_t)packed_bytes(bitwidth, count);
}

int lofgb_encode_f32(uint8_t* dst, const float* src, int64_t count, const lofgb_codec_format* fmt,
                     int mode, int sat_mode, int stoch_len, int reverse, uint64_t seed,
                     uint64_t offset, void* stream) {
    clear_error();
    CodecArg a;
    int st = make_codec_arg(&a, fmt, mode, sat_mode, stoch_len);
    if (st) return st;
    if ((st = codec_pointers(src, dst, count))) return st;
    if (count == 0) return LOFGB_OK;
    const int64_t ob = packed_bytes(a.n, count);
    const char* s = reinterpret_cast<const char*>(src);
    const char* d = reinterpret_cast<const char*>(dst);
    if (s < d + ob && d < s + count * 4)
        return set_error(LOFGB_ERR_ALIAS, "packed output overlaps the input");
    a.seed = seed;
    a.offset = offset;
    const int n = a.n;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    LOFGB_BY_N(launch_encode_n, src, dst, count, reverse, a, cs)
}


int lofgb_mx_encode_f32(const float* src, uint8_t* codes, uint8_t* scales, int64_t count,
                        int block_size, const lofgb_codec_format* elem_fmt,
                        const lofgb_codec_format* scale_fmt, int mode, int scale_mode,
                        int sat_mode, int stoch_len, uint64_t seed, uint64_t offset, void* stream) {
    clear_error();
    if (block_size != 32) return set_error(LOFGB_ERR_BLOCK, "MX storage blocks are 32 values (got %d)", block_size);
    if (!elem_fmt || !scale_fmt) return set_error(LOFGB_ERR_NULL, "NULL codec format");
    const int nb = elem_fmt->fmt.bitwidth;
    if (nb != 4 && nb != 6 && nb != 8)
        return set_error(LOFGB_ERR_UNSUPPORTED, "MX storage element codes of %d bits (4, 6 or 8 supported)", nb);
    if (scale_fmt->fmt.bitwidth != 8)
        return set_error(LOFGB_ERR_UNSUPPORTED, "MX storage scale codes must be 8 bits");
    CodecArg ea, sa;
    int st = make_codec_arg(&ea, elem_fmt, LOFGB_RNE, sat_mode, 0);
    if (!st) st = make_codec_arg(&sa, scale_fmt, LOFGB_RNE, sat_mode, 0);
    if (st) return st;
    RoundPlan pe, ps;
    if ((st = make_round_plan(&pe, &elem_fmt->fmt, 32, mode, stoch_len))) return st;
    if ((st = make_round_plan(&ps, &scale_fmt->fmt, 32, scale_mode, 0))) return st;
    if (count < 0) return set_error(LOFGB_ERR_SIZE, "negative count");
    if (count == 0) return LOFGB_OK;
    if (!src || !codes || !scales) return set_error(LOFGB_ERR_NULL, "NULL data pointer");
    const int64_t cbytes = packed_bytes(nb, count), sbytes = (count + 31) / 32;
    const char* s = reinterpret_cast<const char*>(src);
    const char* c = reinterpret_cast<const char*>(codes);
    const char* k = reinterpret_cast<const char*>(scales);
    if ((s < c + cbytes && c < s + count * 4) || (s < k + sbytes && k < s + count * 4) ||
        (c < k + sbytes && k < c + cbytes))
        return set_error(LOFGB_ERR_ALIAS, "input, codes and scales must not overlap");
    const float inv = mx_inv_pmn(&elem_fmt->fmt);
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    if (nb == 4) return launch_mx_encode_n<4>(src, codes, scales, count, pe, ps, inv, ea, sa, seed, offset, cs);
    if (nb == 6) return launch_mx_encode_n<6>(src, codes, scales, count, pe, ps, inv, ea, sa, seed, offset, cs);
    return launch_mx_encode_n<8>(src, codes, scales, count, pe, ps, inv, ea, sa, seed, offset, cs);
}

int lofgb_mx_decode_f32(const uint8_t* codes, const uint8_t* scales, float* dst, int64_t count,
                        int block_size, const lofgb_codec_format* elem_fmt,
                        const lofgb_codec_format* scale_fmt, void* stream) {
    clear_error();
    if (block_size != 32) return set_error(LOFGB_ERR_BLOCK, "MX storage blocks are 32 values (got %d)", block_size);
    if (!elem_fmt || !scale_fmt) return set_error(LOFGB_ERR_NULL, "NULL codec format");
    const int nb = elem_fmt->fmt.bitwidth;
    if (nb != 4 && nb != 6 && nb != 8)
        return set_error(LOFGB_ERR_UNSUPPORTED, "MX storage element codes of %d bits (4, 6 or 8 supported)", nb);
    if (scale_fmt->fmt.bitwidth != 8)
        return set_error(LOFGB_ERR_UNSUPPORTED, "MX storage scale codes must be 8 bits");
    CodecArg ea, sa;
    int st = make_codec_arg(&ea, elem_fmt, LOFGB_RNE, 0, 0);
    if (!st) st = make_codec_arg(&sa, scale_fmt, LOFGB_RNE, 0, 0);
    if (st) return st;
    if (count < 0) return set_error(LOFGB_ERR_SIZE, "negative count");
    if (count == 0) return LOFGB_OK;
    if (!codes || !scales || !dst) return set_error(LOFGB_ERR_NULL, "NULL data pointer");
    if ((reinterpret_cast<uintptr_t>(codes) & 3) || (reinterpret_cast<uintptr_t>(dst) & 15))
        return set_error(LOFGB_ERR_SIZE, "codes must be 4-byte and the output 16-byte aligned");
    const int64_t cbytes = packed_bytes(nb, count), sbytes = (count + 31) / 32;
    const char* c = reinterpret_cast<const char*>(codes);
    const char* k = reinterpret_cast<const char*>(scales);
    const char* d = reinterpret_cast<const char*>(dst);
    if ((d < c + cbytes && c < d + count * 4) || (d < k + sbytes && k < d + count * 4))
        return set_error(LOFGB_ERR_ALIAS, "the output must not overlap the codes or scales");
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    if (nb == 4) return launch_mx_decode_n<4>(codes, scales, dst, count, ea, sa, cs);
    if (nb == 6) return launch_mx_decode_n<6>(codes, scales, dst, count, ea, sa, cs);
    return launch_mx_decode_n<8>(codes, scales, dst, count, ea, sa, cs);
}

int lofgb_decode_f32(float* dst, const uint8_t* src, int64_t count, const lofgb_codec_format* fmt,
                     int reverse, void* stream) {
    clear_error();
    CodecArg a;
    int st = make_codec_arg(&a, fmt, LOFGB_RNE, 0, 0);
    if (st) return st;
    if ((st = codec_pointers(src, dst, count))) return st;
    if (count == 0) return LOFGB_OK;
    const int64_t ib = packed_bytes(a.n, count);
    const char* s = reinterpret_cast<const char*>(src);
    const char* d = reinterpret_cast<const char*>(dst);
    if (s < d + count * 4 && d < s + ib)
        return set_error(LOFGB_ERR_ALIAS, "decoded output overlaps the input");
    a.seed = a.offset = 0;
    const int n = a.n;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    LOFGB_BY_N(launch_decode_n, src, dst, count, reverse, a, cs)
}

}  // extern "C"
