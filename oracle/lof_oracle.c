/*
 * lof_oracle.c — TEST INFRASTRUCTURE ONLY (see lof_oracle.h).
 *
 * A plain-C restatement of the reference's scalar arithmetic. Every function
 * cites the reference file:line it follows (SudhanvaKulkarni123/LoFloat).
 * The code is deliberately straightforward (one element at a time, 64-bit
 * integer arithmetic with an explicit width mask standing in for the
 * reference's Bits types) so that it can be read against the reference line
 * by line; speed comes only from OpenMP over elements / rows / blocks.
 *
 * Where the reference has undefined behaviour the oracle and the kernels
 * share one defined choice:
 *   - roundoff == 0 (nothing dropped): every mode returns the bits unchanged
 *     (the reference's RTA, SR-A and SR-D would shift by a negative count);
 *   - the random addend of SR-A/B/C/D keeps the low min(stoch_len, W) bits
 *     of the random word, W the width of the word being rounded (the
 *     reference casts it to its W-bit Bits type; its shifts are undefined
 *     once stoch_len reaches W);
 *   - stochastic modes with stoch_len > roundoff: the len-bit random addend
 *     is shifted right by (len - roundoff) instead of left by a negative
 *     count (src/lo_float.h:664, 751, 810, 832);
 *   - SR-C on 64-bit sources computes its addend in 64 bits (the reference
 *     computes it in 32-bit `unsigned int`, src/lo_float.h:809-810, which is
 *     undefined once the shift reaches 32);
 *   - a subnormal-branch shift wider than the source word is clamped to
 *     width-1 (only reachable when the format's smallest subnormal rounds to
 *     0.0f, in which case the result is ±0 whatever the shift).
 */
#include "lof_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* bit helpers                                                               */
/* ------------------------------------------------------------------------ */
static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint64_t d2u(double f) { uint64_t u; memcpy(&u, &f, 8); return u; }
static inline double u2d(uint64_t u) { double f; memcpy(&f, &u, 8); return f; }

static inline uint64_t wmask(int W) { return W >= 64 ? ~0ull : ((1ull << W) - 1ull); }

/* v << s for s >= 0, v >> -s for s < 0 (see the header note on len > roundoff) */
static inline uint64_t shl_s(uint64_t v, int s) {
    if (s >= 64 || s <= -64) return 0;
    return s >= 0 ? (v << s) : (v >> (-s));
}

/* IEEE binary16 <-> binary32, round-to-nearest-even (the conversion c10::Half
 * performs in the reference's half path, src/lo_float.h:2684-2687). */
static float h2f(uint16_t h) {
    uint32_t s = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1F, m = h & 0x3FF;
    if (e == 0x1F) return u2f(s | 0x7F800000u | (m << 13));
    if (e == 0) {
        if (m == 0) return u2f(s);
        /* subnormal: m * 2^-24 */
        float v = (float)m * 5.9604644775390625e-08f;
        return s ? -v : v;
    }
    return u2f(s | ((e + 112u) << 23) | (m << 13));
}

static uint16_t f2h(float f) {
    uint32_t x = f2u(f);
    uint16_t s = (uint16_t)((x >> 16) & 0x8000u);
    uint32_t a = x & 0x7FFFFFFFu;
    if (a >= 0x7F800000u) return (uint16_t)(s | (a > 0x7F800000u ? 0x7E00u : 0x7C00u));
    int e = (int)(a >> 23) - 127;
    uint32_t sig = (a & 0x7FFFFFu) | 0x800000u;
    if (e > 15) return (uint16_t)(s | 0x7C00u);
    if (e >= -14) {
        uint32_t r = sig >> 13, rem = sig & 0x1FFFu;
        if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;
        /* r in [0x400, 0x800]; carry into the exponent is the right result */
        uint32_t out = ((uint32_t)(e + 14) << 10) + r;
        return (uint16_t)(s | (out > 0x7C00u ? 0x7C00u : out));
    }
    if ((a >> 23) == 0) return s; /* float subnormal: far below half range */
    int shift = -(e + 1); /* value in units of 2^-24 is sig * 2^(e+1) */
    if (shift >= 32) return s;
    uint32_t r = sig >> shift, rem = sig & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rem > half || (rem == half && (r & 1u))) r++;
    return (uint16_t)(s | r);
}

/* ------------------------------------------------------------------------ */
/* RNG                                                                       */
/* ------------------------------------------------------------------------ */
uint64_t orc_rng(uint64_t seed, uint64_t idx) {
    uint64_t z = seed + (idx + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int orc_rng_lanes_log2(int mode, int len) {
    int need = 0;
    switch (mode) {
    case LOFGB_SR_A: case LOFGB_SR_B: case LOFGB_SR_C: need = len; break;
    case LOFGB_SR_D: need = len + 1; break;
    case LOFGB_PROB: need = 1; break;
    case LOFGB_TRUE_SR: need = 64; break;
    default: need = 0;
    }
    return need <= 8 ? 3 : need <= 16 ? 2 : need <= 32 ? 1 : 0;
}

uint64_t orc_rng_elem(uint64_t seed, uint64_t g, int lg) {
    const uint64_t w = orc_rng(seed, g >> lg);
    const int lane = (int)(g & ((1ull << lg) - 1ull));
    return w >> (lane * (64 >> lg));
}

static inline double usamp_of(uint64_t r) { return (double)(r >> 11) * 0x1.0p-53; }

/* ------------------------------------------------------------------------ */
/* RoundMantissa: src/lo_float.h:1231-1272 and the helpers it dispatches to. */
/* `bits` is a W-bit magnitude, `ro` the number of dropped low bits, `pos` the */
/* sign flag the callers pass as (sign_bit == 0). Returns the W-bit result   */
/* before the caller's truncation mask.                                      */
/* ------------------------------------------------------------------------ */
static uint64_t round_mantissa(uint64_t bits, int ro, int mode, int len, int pos,
                               uint64_t r, double u, int W) {
    const uint64_t M = wmask(W);
    /* the random addend keeps the low min(len, W) bits of r: the reference
     * casts it to its W-bit Bits type before shifting (:662, :748, :811, :833) */
    const uint64_t RM = wmask(len < W ? len : W);
    if (ro <= 0) return bits;
    if (ro > W - 1) ro = W - 1;
    const uint64_t one_ro = 1ull << ro;
    const uint64_t low = one_ro - 1ull;
    const uint64_t trunc = bits & ~low;
    const uint64_t tail = bits & low;
    uint64_t res;
    switch (mode) {
    case LOFGB_RNE: /* RoundBitsToNearestEven, :570-596 */
        res = bits + ((bits >> ro) & 1ull) + (one_ro >> 1) - 1ull;
        break;
    case LOFGB_RNO: /* RoundBitsToNearestOdd, :1030-1057 */
        res = bits + (((bits >> ro) & 1ull) ^ 1ull) + (one_ro >> 1) - 1ull;
        break;
    case LOFGB_RTZ: /* RoundBitsTowardsZero, :946-970 */
        res = trunc;
        break;
    case LOFGB_RAFZ: /* RoundBitsAwayFromZero, :1000-1027 */
        res = trunc + (tail ? one_ro : 0ull);
        break;
    case LOFGB_RU: /* RoundUp, :1061-1100 */
        res = trunc + ((pos && tail) ? one_ro : 0ull);
        break;
    case LOFGB_RD: /* RoundDown, :1121-1156 */
        res = trunc + ((!pos && tail) ? one_ro : 0ull);
        break;
    case LOFGB_RTA: /* RoundTiesToAway, :1176-1200 */
        res = trunc + (((bits >> (ro - 1)) & 1ull) << ro);
        break;
    case LOFGB_SR_A: { /* Stochastic_Round_A, :653-696 */
        if (len <= 0) { res = bits; break; }
        uint64_t add = r & RM;
        res = bits + shl_s(add, ro - len);
        break;
    }
    case LOFGB_SR_B: { /* Stochastic_Round_B, :699-756 */
        uint64_t add = (r & RM) + 1ull;
        res = bits + (tail > 0 ? shl_s(add, ro - len) : 0ull);
        break;
    }
    case LOFGB_SR_C: { /* Stochastic_Round_C, :758-815 */
        if (len == 0 || tail == 0) { res = bits; break; }
        uint64_t samp = r & RM;
        uint64_t top = (samp >> 1) + (samp & 1ull);
        uint64_t add = shl_s(top, ro - len + 1);
        if (W <= 32) add &= 0xFFFFFFFFull; /* computed as unsigned int */
        res = bits + add;
        break;
    }
    case LOFGB_SR_D: { /* Stochastic_Round_D, :820-861 */
        if (len <= 0) { res = bits; break; }
        uint64_t add = (r & RM) + ((r >> len) & 1ull);
        res = bits + shl_s(add, ro - len);
        break;
    }
    case LOFGB_TRUE_SR: { /* True_Stochastic_Round, :865-944 */
        double prob = (double)tail / (double)one_ro;
        if (u < prob) {
            uint64_t rounded = (trunc + one_ro) & M;
            res = rounded < trunc ? trunc : rounded;
        } else {
            res = trunc;
        }
        break;
    }
    case LOFGB_PROB: /* Probabilistic_Round, :600-650 */
        res = trunc + ((tail ? (r & 1ull) : 0ull) << ro);
        break;
    case LOFGB_RTO: /* RoundToOdd, :1203-1229 */
        res = trunc | (tail ? one_ro : 0ull);
        break;
    case LOFGB_RTTZ: /* RoundTiedBitsTowardsZero, :974-998 */
        res = bits + (one_ro >> 1) - 1ull;
        break;
    default:
        res = bits;
    }
    return res & M;
}

/* ------------------------------------------------------------------------ */
/* Source-type descriptors                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    int W, M, bias; /* word width, mantissa bits, exponent bias */
} src_t;
static const src_t SRC_F32 = {32, 23, 127};
static const src_t SRC_F64 = {64, 52, 1023};
static const src_t SRC_F16 = {16, 10, 15};

int orc_validate_format(const lofgb_format* f, int src_mant_bits) {
    if (!f) return LOFGB_ERR_NULL;
    if (f->mantissa_bits < 0 || f->mantissa_bits > src_mant_bits) return LOFGB_ERR_FORMAT;
    if (f->signedness > 1 || f->inf_behavior > 1 || f->nan_behavior > 1) return LOFGB_ERR_FORMAT;
    int e = f->bitwidth - f->mantissa_bits - (f->signedness == LOFGB_SIGNED ? 1 : 0);
    if (e < 0 || e > 30) return LOFGB_ERR_FORMAT;
    if (f->bias < -(1 << 20) || f->bias > (1 << 20)) return LOFGB_ERR_FORMAT;
    /* the smallest subnormal 2^(1-bias-m) must be finite as a float */
    if (1 - f->bias - f->mantissa_bits > 127) return LOFGB_ERR_FORMAT;
    return 0;
}

static int validate_mode(int mode, int len) {
    if (mode < 0 || mode >= LOFGB_NUM_MODES) return LOFGB_ERR_MODE;
    if (len < 0 || len > 62) return LOFGB_ERR_MODE;
    return 0;
}

/* Format constants, as src/lo_float.h:2857-2861 derives them. */
typedef struct {
    int m, to_max_exp, to_min_exp, saturating;
    float tiny; /* To_min_val (a float in the reference) */
} fconst_t;

static fconst_t make_consts(const lofgb_format* f) {
    fconst_t c;
    c.m = f->mantissa_bits;
    c.to_max_exp = (f->signedness == LOFGB_SIGNED)
                       ? (1 << (f->bitwidth - f->mantissa_bits - 1)) - 1 - f->bias
                       : (1 << (f->bitwidth - f->mantissa_bits)) - 1 - f->bias;
    c.to_min_exp = 1 - f->bias;
    /* std::pow(2.0, ToMin_exp) * std::pow(2.0, -m), then narrowed to float */
    c.tiny = (float)(ldexp(1.0, c.to_min_exp) * ldexp(1.0, -c.m));
    c.saturating = f->inf_behavior == LOFGB_INF_SATURATING;
    return c;
}

/* from_double<From>(v) for the three source types (src/lo_float.h:2684-2687) */
static uint64_t from_double_bits(double v, const src_t* s) {
    if (s->W == 32) return f2u((float)v);
    if (s->W == 64) return d2u(v);
    return f2h((float)v);
}

/* |x| narrowed to float (get_float(lof_abs(value)), src/lo_float.h:2871) */
static float abs_as_float(uint64_t mag, const src_t* s) {
    if (s->W == 32) return u2f((uint32_t)mag);
    if (s->W == 64) return (float)u2d(mag);
    return h2f((uint16_t)mag);
}

static uint64_t qnan_bits(const src_t* s) {
    return s->W == 32 ? 0x7FC00000ull : (s->W == 64 ? 0x7FF8000000000000ull : 0x7E00ull);
}
static uint64_t pinf_bits(const src_t* s) {
    return s->W == 32 ? 0x7F800000ull : (s->W == 64 ? 0x7FF0000000000000ull : 0x7C00ull);
}

/* lo_float_internal::virtual_round(value, FloatingPointParams, ProjSpec),
 * src/lo_float.h:2843-2939, for a W-bit source word x. */
static uint64_t vr_fmt(uint64_t x, const src_t* s, const fconst_t* c, int mode, int len,
                       uint64_t r, double u) {
    const uint64_t signbit = 1ull << (s->W - 1);
    const uint64_t sign = x & signbit;
    const uint64_t mag = x & (signbit - 1ull);
    const uint64_t expmask = pinf_bits(s);
    const int pos = (sign == 0);

    /* :2869 NaN -> quiet NaN (sign dropped) */
    if ((mag & expmask) == expmask && (mag & ((1ull << s->M) - 1ull)) != 0)
        return qnan_bits(s);

    /* :2871-2909 below the smallest subnormal */
    const float abs_val = abs_as_float(mag, s);
    if (abs_val < c->tiny) {
        int to_min;
        switch (mode) {
        case LOFGB_RTZ: to_min = 0; break;
        case LOFGB_RTO:
        case LOFGB_RAFZ: to_min = abs_val > 0.0f; break;
        case LOFGB_RU: to_min = pos && abs_val > 0.0f; break;
        case LOFGB_RD: to_min = !pos && abs_val > 0.0f; break;
        case LOFGB_RNE:
        case LOFGB_RNO:
        case LOFGB_RTTZ:
        case LOFGB_RTA: {
            const float half = c->tiny * 0.5f;
            if (abs_val < half) to_min = 0;
            else if (abs_val > half) to_min = 1;
            else to_min = (mode == LOFGB_RNO || mode == LOFGB_RTA);
            break;
        }
        default: to_min = 0;
        }
        uint64_t mb = to_min ? from_double_bits((double)c->tiny, s) : 0ull;
        return mb | sign;
    }

    int from_exp = (int)(mag >> s->M) - s->bias;
    const int d = s->M - c->m; /* -kDigitShift */

    /* :2910-2923 target-subnormal grid */
    if (from_exp < c->to_min_exp) {
        int shift = d - (from_exp - c->to_min_exp);
        if (shift > s->W - 1) shift = s->W - 1;
        uint64_t sig = (mag & ((1ull << s->M) - 1ull)) | (1ull << s->M);
        sig = round_mantissa(sig, shift, mode, len, pos, r, u, s->W);
        uint64_t k = sig >> shift;
        uint64_t mb = from_double_bits((double)k * (double)c->tiny, s);
        return mb | sign;
    }

    /* :2925-2933 normal rounding */
    uint64_t b = mag;
    if (d > 0) {
        b = round_mantissa(b, d, mode, len, pos, r, u, s->W);
        b &= ~((1ull << d) - 1ull);
    }
    /* :2935-2936 overflow: Saturating returns the input, Extended returns +inf */
    from_exp = (int)(b >> s->M) - s->bias;
    if (from_exp > c->to_max_exp) return c->saturating ? x : pinf_bits(s);
    return (b | sign) & wmask(s->W);
}

/* lo_float_internal::virtual_round(value, int ToMantissaBits, ProjSpec),
 * src/lo_float.h:2715-2756. */
static uint64_t vr_mant(uint64_t x, const src_t* s, int mbits, int mode, int len,
                        uint64_t r, double u) {
    const uint64_t signbit = 1ull << (s->W - 1);
    const uint64_t sign = x & signbit;
    uint64_t b = x & (signbit - 1ull);
    const int d = s->M - mbits;
    b = round_mantissa(b, d, mode, len, sign == 0, r, u, s->W);
    if (d > 0) b &= ~((1ull << d) - 1ull);
    return (b | sign) & wmask(s->W);
}

/* ---- scalar entry points ------------------------------------------------ */
float orc_vr_f32(float x, const lofgb_format* f, int mode, int len, uint64_t rbits,
                 double usamp) {
    fconst_t c = make_consts(f);
    if (usamp < 0) usamp = usamp_of(rbits);
    return u2f((uint32_t)vr_fmt(f2u(x), &SRC_F32, &c, mode, len, rbits, usamp));
}
double orc_vr_f64(double x, const lofgb_format* f, int mode, int len, uint64_t rbits,
                  double usamp) {
    fconst_t c = make_consts(f);
    if (usamp < 0) usamp = usamp_of(rbits);
    return u2d(vr_fmt(d2u(x), &SRC_F64, &c, mode, len, rbits, usamp));
}
uint16_t orc_vr_f16(uint16_t x, const lofgb_format* f, int mode, int len,
                    uint64_t rbits, double usamp) {
    fconst_t c = make_consts(f);
    if (usamp < 0) usamp = usamp_of(rbits);
    return (uint16_t)vr_fmt(x, &SRC_F16, &c, mode, len, rbits, usamp);
}
float orc_vm_f32(float x, int mbits, int mode, int len, uint64_t rbits, double usamp) {
    if (usamp < 0) usamp = usamp_of(rbits);
    return u2f((uint32_t)vr_mant(f2u(x), &SRC_F32, mbits, mode, len, rbits, usamp));
}
double orc_vm_f64(double x, int mbits, int mode, int len, uint64_t rbits, double usamp) {
    if (usamp < 0) usamp = usamp_of(rbits);
    return u2d(vr_mant(d2u(x), &SRC_F64, mbits, mode, len, rbits, usamp));
}
uint16_t orc_vm_f16(uint16_t x, int mbits, int mode, int len, uint64_t rbits,
                    double usamp) {
    if (usamp < 0) usamp = usamp_of(rbits);
    return (uint16_t)vr_mant(x, &SRC_F16, mbits, mode, len, rbits, usamp);
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int nthr(int nthreads) {
    int mx = orc_max_threads();
    return (nthreads <= 0 || nthreads > mx) ? mx : nthreads;
}

/* ---- array entry points --------------------------------------------------
 * The scale multiply happens in the source type before rounding, as
 * round_fp_params_kernel / round_mantissa_kernel do (src/Lof_kernel.cu:40-41,
 * 52-53); for half sources the scale is first narrowed to half and the
 * product is taken in float and narrowed back (c10::Half arithmetic). */
#define ORC_ROUND_BODY(FMT_OR_MANT)                                                \
    for (int64_t i = 0; i < n; ++i) {                                              \
        uint64_t rb = rbits ? rbits[i] : 0ull;                                     \
        double us = usamp ? usamp[i] : usamp_of(rb);                               \
        FMT_OR_MANT;                                                               \
    }

static int check_arrays(const void* in, const void* out, int64_t n) {
    if (n < 0) return LOFGB_ERR_SIZE;
    if (n > 0 && (!in || !out)) return LOFGB_ERR_NULL;
    return 0;
}

int orc_round_f32_bits(const float* in, float* out, int64_t n, const lofgb_format* f,
                       int mode, int len, const uint64_t* rbits, const double* usamp) {
    int st = check_arrays(in, out, n);
    if (!st) st = orc_validate_format(f, 23);
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    fconst_t c = make_consts(f);
    ORC_ROUND_BODY(out[i] = u2f((uint32_t)vr_fmt(f2u(in[i]), &SRC_F32, &c, mode, len, rb, us)))
    return 0;
}
int orc_round_f64_bits(const double* in, double* out, int64_t n, const lofgb_format* f,
                       int mode, int len, const uint64_t* rbits, const double* usamp) {
    int st = check_arrays(in, out, n);
    if (!st) st = orc_validate_format(f, 52);
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    fconst_t c = make_consts(f);
    ORC_ROUND_BODY(out[i] = u2d(vr_fmt(d2u(in[i]), &SRC_F64, &c, mode, len, rb, us)))
    return 0;
}
int orc_round_f16_bits(const uint16_t* in, uint16_t* out, int64_t n,
                       const lofgb_format* f, int mode, int len, const uint64_t* rbits,
                       const double* usamp) {
    int st = check_arrays(in, out, n);
    if (!st) st = orc_validate_format(f, 10);
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    fconst_t c = make_consts(f);
    ORC_ROUND_BODY(out[i] = (uint16_t)vr_fmt(in[i], &SRC_F16, &c, mode, len, rb, us))
    return 0;
}
int orc_round_mantissa_f32_bits(const float* in, float* out, int64_t n, int mbits,
                                int mode, int len, const uint64_t* rbits,
                                const double* usamp) {
    int st = check_arrays(in, out, n);
    if (!st && (mbits < 0 || mbits > 23)) st = LOFGB_ERR_FORMAT;
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    ORC_ROUND_BODY(out[i] = u2f((uint32_t)vr_mant(f2u(in[i]), &SRC_F32, mbits, mode, len, rb, us)))
    return 0;
}
int orc_round_mantissa_f64_bits(const double* in, double* out, int64_t n, int mbits,
                                int mode, int len, const uint64_t* rbits,
                                const double* usamp) {
    int st = check_arrays(in, out, n);
    if (!st && (mbits < 0 || mbits > 52)) st = LOFGB_ERR_FORMAT;
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    ORC_ROUND_BODY(out[i] = u2d(vr_mant(d2u(in[i]), &SRC_F64, mbits, mode, len, rb, us)))
    return 0;
}
int orc_round_mantissa_f16_bits(const uint16_t* in, uint16_t* out, int64_t n, int mbits,
                                int mode, int len, const uint64_t* rbits,
                                const double* usamp) {
    int st = check_arrays(in, out, n);
    if (!st && (mbits < 0 || mbits > 10)) st = LOFGB_ERR_FORMAT;
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    ORC_ROUND_BODY(out[i] = (uint16_t)vr_mant(in[i], &SRC_F16, mbits, mode, len, rb, us))
    return 0;
}

/* seeded forms */
int orc_round_f32(const float* in, float* out, int64_t n, const lofgb_format* f,
                  int mode, int len, float scale, uint64_t seed, uint64_t offset,
                  int nthreads) {
    int st = check_arrays(in, out, n);
    if (!st) st = orc_validate_format(f, 23);
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    fconst_t c = make_consts(f);
    const int sc = scale != 1.0f;
    const int lg = orc_rng_lanes_log2(mode, len);
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
    for (int64_t i = 0; i < n; ++i) {
        float v = sc ? scale * in[i] : in[i];
        uint64_t rb = orc_rng_elem(seed, offset + (uint64_t)i, lg);
        out[i] = u2f((uint32_t)vr_fmt(f2u(v), &SRC_F32, &c, mode, len, rb, usamp_of(rb)));
    }
    return 0;
}
int orc_round_f64(const double* in, double* out, int64_t n, const lofgb_format* f,
                  int mode, int len, double scale, uint64_t seed, uint64_t offset,
                  int nthreads) {
    int st = check_arrays(in, out, n);
    if (!st) st = orc_validate_format(f, 52);
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    fconst_t c = make_consts(f);
    const int sc = scale != 1.0;
    const int lg = orc_rng_lanes_log2(mode, len);
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
    for (int64_t i = 0; i < n; ++i) {
        double v = sc ? scale * in[i] : in[i];
        uint64_t rb = orc_rng_elem(seed, offset + (uint64_t)i, lg);
        out[i] = u2d(vr_fmt(d2u(v), &SRC_F64, &c, mode, len, rb, usamp_of(rb)));
    }
    return 0;
}
int orc_round_f16(const uint16_t* in, uint16_t* out, int64_t n, const lofgb_format* f,
                  int mode, int len, float scale, uint64_t seed, uint64_t offset,
                  int nthreads) {
    int st = check_arrays(in, out, n);
    if (!st) st = orc_validate_format(f, 10);
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    fconst_t c = make_consts(f);
    const float sh = h2f(f2h(scale));
    const int sc = sh != 1.0f;
    const int lg = orc_rng_lanes_log2(mode, len);
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
    for (int64_t i = 0; i < n; ++i) {
        uint16_t v = sc ? f2h(sh * h2f(in[i])) : in[i];
        uint64_t rb = orc_rng_elem(seed, offset + (uint64_t)i, lg);
        out[i] = (uint16_t)vr_fmt(v, &SRC_F16, &c, mode, len, rb, usamp_of(rb));
    }
    return 0;
}
int orc_round_mantissa_f32(const float* in, float* out, int64_t n, int mbits, int mode,
                           int len, float scale, uint64_t seed, uint64_t offset,
                           int nthreads) {
    int st = check_arrays(in, out, n);
    if (!st && (mbits < 0 || mbits > 23)) st = LOFGB_ERR_FORMAT;
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    const int sc = scale != 1.0f;
    const int lg = orc_rng_lanes_log2(mode, len);
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
    for (int64_t i = 0; i < n; ++i) {
        float v = sc ? scale * in[i] : in[i];
        uint64_t rb = orc_rng_elem(seed, offset + (uint64_t)i, lg);
        out[i] = u2f((uint32_t)vr_mant(f2u(v), &SRC_F32, mbits, mode, len, rb, usamp_of(rb)));
    }
    return 0;
}
int orc_round_mantissa_f64(const double* in, double* out, int64_t n, int mbits,
                           int mode, int len, double scale, uint64_t seed,
                           uint64_t offset, int nthreads) {
    int st = check_arrays(in, out, n);
    if (!st && (mbits < 0 || mbits > 52)) st = LOFGB_ERR_FORMAT;
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    const int sc = scale != 1.0;
    const int lg = orc_rng_lanes_log2(mode, len);
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
    for (int64_t i = 0; i < n; ++i) {
        double v = sc ? scale * in[i] : in[i];
        uint64_t rb = orc_rng_elem(seed, offset + (uint64_t)i, lg);
        out[i] = u2d(vr_mant(d2u(v), &SRC_F64, mbits, mode, len, rb, usamp_of(rb)));
    }
    return 0;
}
int orc_round_mantissa_f16(const uint16_t* in, uint16_t* out, int64_t n, int mbits,
                           int mode, int len, float scale, uint64_t seed,
                           uint64_t offset, int nthreads) {
    int st = check_arrays(in, out, n);
    if (!st && (mbits < 0 || mbits > 10)) st = LOFGB_ERR_FORMAT;
    if (!st) st = validate_mode(mode, len);
    if (st) return st;
    const float sh = h2f(f2h(scale));
    const int sc = sh != 1.0f;
    const int lg = orc_rng_lanes_log2(mode, len);
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
    for (int64_t i = 0; i < n; ++i) {
        uint16_t v = sc ? f2h(sh * h2f(in[i])) : in[i];
        uint64_t rb = orc_rng_elem(seed, offset + (uint64_t)i, lg);
        out[i] = (uint16_t)vr_mant(v, &SRC_F16, mbits, mode, len, rb, usamp_of(rb));
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* MX: the per-block loop of src/LoPy_bind.cpp:199-214 with the GPU scale     */
/* expression amax * (1.0f / pmn) of src/mx_round.cuh:52-65 (formula 0) or   */
/* the CPU expression amax / pmn (formula 1); element step :70-75.          */
/* ------------------------------------------------------------------------ */
#define ORC_SCALE_SALT 0x5CA1E5CA1E5CA1E5ull

/* One MX block (cnt <= block values from element b0): its scale and the
 * rounded quotients q_i = vr(x_i / scale) (+0 when the scale is not
 * positive). out = q_i * scale is the MX round; the MX encode stores q_i and
 * the scale as codes. */
static float mx_block(const float* in, int64_t b0, int64_t cnt, const fconst_t* ce,
                      const fconst_t* cs, float pmn, float inv, int mode, int scale_mode, int len,
                      int lg, uint64_t seed, uint64_t offset, int scale_formula, float* q) {
    /* amax ignores NaNs of both kinds, as the reference's device fmaxf does
       (src/mx_round.cuh:101-106); a host fmaxf may return NaN for a
       signaling NaN operand */
    float amax = 0.0f;
    for (int64_t i = 0; i < cnt; ++i) {
        const float a = fabsf(in[b0 + i]);
        if (a > amax) amax = a;
    }
    const float sin = scale_formula ? amax / pmn : amax * inv;
    uint64_t rs = orc_rng(seed ^ ORC_SCALE_SALT, offset + (uint64_t)b0);
    const float scale =
        u2f((uint32_t)vr_fmt(f2u(sin), &SRC_F32, cs, scale_mode, 0, rs, usamp_of(rs)));
    for (int64_t i = 0; i < cnt; ++i) {
        if (!(scale > 0.0f)) {
            q[i] = 0.0f;
            continue;
        }
        const float x = in[b0 + i] / scale;
        uint64_t rb = orc_rng_elem(seed, offset + (uint64_t)(b0 + i), lg);
        q[i] = u2f((uint32_t)vr_fmt(f2u(x), &SRC_F32, ce, mode, len, rb, usamp_of(rb)));
    }
    return scale;
}

static int mx_check(const float* in, int64_t n, int block, const lofgb_format* ef,
                    const lofgb_format* sf, int mode, int scale_mode, int len) {
    if (n < 0) return LOFGB_ERR_SIZE;
    if (n > 0 && !in) return LOFGB_ERR_NULL;
    int st = orc_validate_format(ef, 23);
    if (!st) st = orc_validate_format(sf, 23);
    if (!st) st = validate_mode(mode, len);
    if (!st) st = validate_mode(scale_mode, 0);
    if (!st && block <= 0) st = LOFGB_ERR_BLOCK;
    return st;
}

static float mx_pmn(const fconst_t* ce, const lofgb_format* ef) {
    return ldexpf(1.0f, ce->to_max_exp) * (2.0f - ldexpf(1.0f, -ef->mantissa_bits));
}

int orc_mx_round_f32(const float* in, float* out, int64_t n, int block,
                     const lofgb_format* ef, const lofgb_format* sf, int mode,
                     int scale_mode, int len, uint64_t seed, uint64_t offset,
                     int scale_formula, int nthreads) {
    int st = check_arrays(in, out, n);
    if (!st) st = mx_check(in, n, block, ef, sf, mode, scale_mode, len);
    if (st) return st;
    fconst_t ce = make_consts(ef), cs = make_consts(sf);
    const float pmn = mx_pmn(&ce, ef);
    const float inv = 1.0f / pmn;
    const int64_t nb = (n + block - 1) / block;
    const int lg = orc_rng_lanes_log2(mode, len);
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t b0 = b * block;
        const int64_t cnt = (n - b0) < block ? (n - b0) : block;
        /* the rounded quotients go straight into out, then get rescaled */
        const float scale = mx_block(in, b0, cnt, &ce, &cs, pmn, inv, mode, scale_mode, len, lg,
                                     seed, offset, scale_formula, out + b0);
        for (int64_t i = 0; i < cnt; ++i) out[b0 + i] = scale > 0.0f ? out[b0 + i] * scale : 0.0f;
    }
    return 0;
}

/* MX storage: the block scales and rounded quotients of orc_mx_round_f32 (GPU
 * scale form), encoded with the storage codec under RNE and `sat`: element
 * codes packed as orc_encode_f32 packs them (forward groups), one scale code
 * per block packed likewise. codes holds orc_packed_size(ef bits, n) bytes,
 * scales orc_packed_size(sf bits, ceil(n / block)). */
int orc_mx_encode_f32(const float* in, int64_t n, int block, const lofgb_codec_format* ef,
                      const lofgb_codec_format* sf, int mode, int scale_mode, int len, int sat,
                      uint64_t seed, uint64_t offset, uint8_t* codes, uint8_t* scales) {
    if (!ef || !sf) return LOFGB_ERR_NULL;
    int st = mx_check(in, n, block, &ef->fmt, &sf->fmt, mode, scale_mode, len);
    if (st) return st;
    fconst_t ce = make_consts(&ef->fmt), cs = make_consts(&sf->fmt);
    const float pmn = mx_pmn(&ce, &ef->fmt);
    const float inv = 1.0f / pmn;
    const int64_t nb = (n + block - 1) / block;
    const int lg = orc_rng_lanes_log2(mode, len);
    float* q = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    float* sc = (float*)malloc(sizeof(float) * (size_t)(nb > 0 ? nb : 1));
    if (!q || !sc) {
        free(q);
        free(sc);
        return LOFGB_ERR_SIZE;
    }
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t b0 = b * block;
        const int64_t cnt = (n - b0) < block ? (n - b0) : block;
        sc[b] = mx_block(in, b0, cnt, &ce, &cs, pmn, inv, mode, scale_mode, len, lg, seed, offset, 0,
                         q + b0);
    }
    st = orc_encode_f32(codes, q, n, ef, LOFGB_RNE, sat, 0, 0, 0, 0);
    if (!st) st = orc_encode_f32(scales, sc, nb, sf, LOFGB_RNE, sat, 0, 0, 0, 0);
    free(q);
    free(sc);
    return st;
}

/* ------------------------------------------------------------------------ */
/* Emulated-accumulation GEMM                                                */
/* ------------------------------------------------------------------------ */

static float next_up(float f) {
    uint32_t b = f2u(f);
    if ((b & 0x7FFFFFFFu) == 0) return u2f(1u);
    return u2f((b >> 31) ? b - 1u : b + 1u);
}
static float next_down(float f) {
    uint32_t b = f2u(f);
    if ((b & 0x7FFFFFFFu) == 0) return u2f(0x80000001u);
    return u2f((b >> 31) ? b + 1u : b - 1u);
}

/* round_to_odd_fma<float> of the device leaf, src/cutlass_gemms.cuh:73-88:
 * rd = fma_rd, ru = fma_ru, rz = rd >= 0 ? rd : ru, result = rz | (rd != ru).
 * Restated on the host from an RN fmaf and the exact residual (the two-sum
 * construction of src/blis_lof_gemm.hpp:63-99), with the device's signed-zero
 * and overflow outcomes reproduced. NaN results are the GPU's canonical NaN. */
float orc_rto_fma(float a, float b, float c) {
    if (isnan(a) || isnan(b) || isnan(c)) return u2f(0x7FFFFFFFu);
    const double p = (double)a * (double)b;
    if (isnan(p)) return u2f(0x7FFFFFFFu); /* inf * 0 */
    if (isinf(p) || isinf(c)) {
        if (isinf(p) && isinf(c) && ((p > 0) != (c > 0))) return u2f(0x7FFFFFFFu);
        return (float)(isinf(p) ? p : (double)c);
    }
    const float rn = fmaf(a, b, c);
    const double cd = (double)c;
    const double s = p + cd;
    const double bb = s - p;
    const double e = (p - (s - bb)) + (cd - bb);
    double res;
    if (isinf(rn)) res = rn > 0 ? -1.0 : 1.0; /* exact is finite: below +inf / above -inf */
    else res = (s - (double)rn) + e;
    float rd, ru;
    if (res == 0.0) {
        if (rn == 0.0f) {
            /* exact zero: RD gives -0 unless both addends are +0 */
            const int p_pos_zero = (p == 0.0) && !signbit(p);
            const int c_pos_zero = (c == 0.0f) && !signbit(c);
            rd = (p_pos_zero && c_pos_zero) ? 0.0f : -0.0f;
        } else {
            rd = rn;
        }
        ru = rd;
        return rd; /* exact: rz = rd (rd >= 0 holds for ±0), no sticky bit */
    }
    if (res > 0.0) { rd = rn; ru = next_up(rn); }
    else { ru = rn; rd = next_down(rn); }
    const float rz = (rd >= 0.0f) ? rd : ru;
    return u2f(f2u(rz) | 1u);
}

static inline float ldA(const float* A, int64_t lda, int ta, int i, int k) {
    return ta ? A[(int64_t)k * lda + i] : A[(int64_t)i * lda + k];
}
static inline float ldB(const float* B, int64_t ldb, int tb, int k, int j) {
    return tb ? B[(int64_t)j * ldb + k] : B[(int64_t)k * ldb + j];
}

static int check_gemm(const float* A, int64_t lda, int ta, const float* B, int64_t ldb,
                      int tb, const void* D, int64_t ldd, int M, int N, int K, int mbits) {
    if (M < 0 || N < 0 || K < 0) return LOFGB_ERR_SIZE;
    if ((M && N) && !D) return LOFGB_ERR_NULL;
    if ((M && N && K) && (!A || !B)) return LOFGB_ERR_NULL;
    if (lda < (ta ? M : K) || ldb < (tb ? K : N) || ldd < N) return LOFGB_ERR_SIZE;
    if (mbits < 0 || mbits > 23) return LOFGB_ERR_FORMAT;
    return 0;
}

/* thread::Mma<OpLoFMultiplyAdd> (src/cutlass_gemms.cuh:118-167): for each
 * output, acc = +0 and k runs 0..K-1 in order with
 * acc = virtual_round(round_to_odd_fma(a, b, acc), mbits) under RNE (the leaf
 * ignores ProjSpec, :122); then D = alpha * acc (LinearCombination, beta 0). */
int orc_gemm_f32_rows(const float* A, int64_t lda, int ta, const float* B, int64_t ldb,
                      int tb, float* D, int64_t ldd, int M, int N, int K, int mbits,
                      float alpha, int row0, int rows, int nthreads) {
    int st = check_gemm(A, lda, ta, B, ldb, tb, D, ldd, M, N, K, mbits);
    if (st) return st;
    if (row0 < 0 || rows < 0 || row0 + rows > M) return LOFGB_ERR_SIZE;
    const int64_t total = (int64_t)rows * N;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthr(nthreads))
    for (int64_t t = 0; t < total; ++t) {
        const int i = row0 + (int)(t / N), j = (int)(t % N);
        float acc = 0.0f;
        for (int k = 0; k < K; ++k) {
            float v = orc_rto_fma(ldA(A, lda, ta, i, k), ldB(B, ldb, tb, k, j), acc);
            acc = u2f((uint32_t)vr_mant(f2u(v), &SRC_F32, mbits, LOFGB_RNE, 0, 0, 0.0));
        }
        D[(int64_t)i * ldd + j] = alpha * acc;
    }
    return 0;
}

int orc_gemm_f32(const float* A, int64_t lda, int ta, const float* B, int64_t ldb,
                 int tb, float* D, int64_t ldd, int M, int N, int K, int mbits,
                 float alpha, int nthreads) {
    return orc_gemm_f32_rows(A, lda, ta, B, ldb, tb, D, ldd, M, N, K, mbits, alpha, 0, M,
                             nthreads);
}

int orc_gemm_accfmt_f32(const float* A, int64_t lda, int ta, const float* B, int64_t ldb,
                        int tb, float* D, int64_t ldd, int M, int N, int K,
                        const lofgb_format* fmt, float alpha, int nthreads) {
    int st = check_gemm(A, lda, ta, B, ldb, tb, D, ldd, M, N, K, 10);
    if (st) return st;
    if ((st = orc_validate_format(fmt, 23))) return st;
    const int64_t total = (int64_t)M * N;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthr(nthreads))
    for (int64_t t = 0; t < total; ++t) {
        const int i = (int)(t / N), j = (int)(t % N);
        float acc = 0.0f;
        for (int k = 0; k < K; ++k)
            acc = orc_vr_f32(orc_rto_fma(ldA(A, lda, ta, i, k), ldB(B, ldb, tb, k, j), acc), fmt,
                             LOFGB_RNE, 0, 0, 0.0);
        D[(int64_t)i * ldd + j] = alpha * acc;
    }
    return 0;
}

int orc_gemm_chunked_f32(const float* A, int64_t lda, int ta, const float* B,
                         int64_t ldb, int tb, float* D, int64_t ldd, int M, int N, int K,
                         int mbits, int chunk, float alpha, int nthreads) {
    int st = check_gemm(A, lda, ta, B, ldb, tb, D, ldd, M, N, K, mbits);
    if (st) return st;
    if (chunk <= 0) return LOFGB_ERR_SIZE;
    const int64_t total = (int64_t)M * N;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthr(nthreads))
    for (int64_t t = 0; t < total; ++t) {
        const int i = (int)(t / N), j = (int)(t % N);
        float acc = 0.0f;
        for (int k0 = 0; k0 < K; k0 += chunk) {
            double s = 0.0;
            const int k1 = k0 + chunk < K ? k0 + chunk : K;
            for (int k = k0; k < k1; ++k)
                s += (double)ldA(A, lda, ta, i, k) * (double)ldB(B, ldb, tb, k, j);
            float v = orc_rto_fma(acc, 1.0f, (float)s);
            acc = u2f((uint32_t)vr_mant(f2u(v), &SRC_F32, mbits, LOFGB_RNE, 0, 0, 0.0));
        }
        D[(int64_t)i * ldd + j] = alpha * acc;
    }
    return 0;
}

/* ---- conv2d ------------------------------------------------------------------
 * The per-MAC leaf of orc_gemm_f32 over the conv reduction. CRS order: the
 * reference's default LoF_Conv2d path unfolds the input (F.unfold: rows
 * ordered c, then r, then s) and calls lof_gemm(w.view(K, -1), x_col[n])
 * (LoFloat/layers.py:690-705), i.e. rto_fma(w, x, acc) in that row order, with
 * +0 in the padded positions. TILED8 order: lof_conv2d runs CUTLASS's analytic
 * fprop implicit GEMM (src/cutlass_conv.cuh:78-98, TbK = 8), whose activation
 * and filter iterators advance s, then r, then the 8-channel tile, while the
 * SIMT leaf walks the 8 channels of a tile in order; channels >= C load 0 in
 * both operands. The product commutes exactly, so rto_fma(w, x, acc) equals
 * the leaf's rto_fma(x, w, acc). */
static int conv_shape_ok(const lofgb_conv2d_shape* s, int* P, int* Q) {
    if (!s) return LOFGB_ERR_NULL;
    if (s->n < 0 || s->c < 1 || s->h < 1 || s->w < 1 || s->k < 1 || s->r < 1 || s->s < 1 ||
        s->pad_h < 0 || s->pad_w < 0 || s->stride_h < 1 || s->stride_w < 1 || s->dil_h < 1 ||
        s->dil_w < 1)
        return LOFGB_ERR_SIZE;
    const int64_t ph = ((int64_t)s->h + 2 * (int64_t)s->pad_h - (int64_t)s->dil_h * (s->r - 1) - 1);
    const int64_t pw = ((int64_t)s->w + 2 * (int64_t)s->pad_w - (int64_t)s->dil_w * (s->s - 1) - 1);
    if (ph < 0 || pw < 0) return LOFGB_ERR_SIZE;
    *P = (int)(ph / s->stride_h + 1);
    *Q = (int)(pw / s->stride_w + 1);
    return 0;
}

int orc_conv2d_f32(const float* x, const float* w, float* y, const lofgb_conv2d_shape* s,
                   int mbits, float alpha, int order, int64_t col0, int64_t ncols,
                   int nthreads) {
    int P, Q;
    int st = conv_shape_ok(s, &P, &Q);
    if (st) return st;
    if (!x || !w || !y) return LOFGB_ERR_NULL;
    if (mbits < 0 || mbits > 23) return LOFGB_ERR_FORMAT;
    if (order != LOFGB_CONV_CRS && order != LOFGB_CONV_TILED8) return LOFGB_ERR_UNSUPPORTED;
    const int64_t L = (int64_t)P * Q, cols = (int64_t)s->n * L;
    if (ncols < 0) { col0 = 0; ncols = cols; }
    if (col0 < 0 || col0 + ncols > cols) return LOFGB_ERR_SIZE;
    const int C = s->c, H = s->h, W = s->w, K = s->k, R = s->r, S = s->s;
    const int ctiles = (C + 7) / 8;
    const int64_t total = ncols * K;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthr(nthreads))
    for (int64_t t = 0; t < total; ++t) {
        const int64_t col = col0 + t / K;
        const int k = (int)(t % K);
        const int n = (int)(col / L), l = (int)(col % L), p = l / Q, q = l % Q;
        const int h0 = p * s->stride_h - s->pad_h, w0 = q * s->stride_w - s->pad_w;
        float acc = 0.0f;
#define ORC_CONV_MAC(cc, rr, ss)                                                             \
    do {                                                                                     \
        float a = 0.0f, b = 0.0f;                                                            \
        if ((cc) < C) {                                                                      \
            const int hh = h0 + (rr) * s->dil_h, ww = w0 + (ss) * s->dil_w;                  \
            a = w[(((int64_t)k * C + (cc)) * R + (rr)) * S + (ss)];                          \
            if (hh >= 0 && hh < H && ww >= 0 && ww < W)                                      \
                b = x[(((int64_t)n * C + (cc)) * H + hh) * W + ww];                          \
        }                                                                                    \
        const float v = orc_rto_fma(a, b, acc);                                              \
        acc = u2f((uint32_t)vr_mant(f2u(v), &SRC_F32, mbits, LOFGB_RNE, 0, 0, 0.0));         \
    } while (0)
        if (order == LOFGB_CONV_CRS) {
            for (int c = 0; c < C; ++c)
                for (int r = 0; r < R; ++r)
                    for (int q2 = 0; q2 < S; ++q2) ORC_CONV_MAC(c, r, q2);
        } else {
            for (int ct = 0; ct < ctiles; ++ct)
                for (int r = 0; r < R; ++r)
                    for (int q2 = 0; q2 < S; ++q2)
                        for (int ci = 0; ci < 8; ++ci) ORC_CONV_MAC(ct * 8 + ci, r, q2);
        }
#undef ORC_CONV_MAC
        y[(((int64_t)n * K + k) * L) + l] = alpha * acc;
    }
    return 0;
}

/* ---- piecewise-linear SiLU (src/LoPy_bind.cpp:258-269, the CPU loop; the
 * CUDA kernel src/Lof_kernel.cu:240-256 is the same FP32 arithmetic) ------- */
int orc_pwl_silu_f32(const float* in, float* out, int64_t n, const float* lut, int segments,
                     float R) {
    if (n < 0) return LOFGB_ERR_SIZE;
    if (n > 0 && (!in || !out || !lut)) return LOFGB_ERR_NULL;
    const float inv_step = (float)segments / (2.0f * R);
    for (int64_t k = 0; k < n; ++k) {
        const float xv = in[k];
        const float xc = fminf(fmaxf(xv, -R), R);
        const float u = (xc + R) * inv_step;
        int i = (int)u;
        if (i > segments - 1) i = segments - 1;
        const float frac = u - (float)i;
        const float y0 = lut[i], y1 = lut[i + 1];
        float yv = fmaf(frac, y1 - y0, y0);
        if (fabsf(xv) > R) yv = xv > 0.0f ? xv : 0.0f;
        out[k] = yv;
    }
    return 0;
}

/* ---- storage codec -------------------------------------------------------------
 * convert_float_to_rep (src/lo_pack.hpp:109-287) with SOURCE = float, the
 * runtime format in `f`, restated branch by branch; RoundMantissa is the
 * shared round_mantissa above with the reference's default positive-sign flag
 * (false) and the word width of the reference's Bits type at each call. */
static int codec_is_inf(uint32_t rep, const lofgb_codec_format* f) {
    return (rep | f->inf_or) == f->inf_match;
}

static int codec_is_nan(uint32_t rep, const lofgb_codec_format* f) {
    if (f->nan_kind == LOFGB_NAN_NONE) return 0;
    if (f->nan_kind == LOFGB_NAN_PATTERN) return rep == f->qnan;
    const int n = f->fmt.bitwidth, m = f->fmt.mantissa_bits;
    const int sgn = f->fmt.signedness == LOFGB_SIGNED;
    const uint32_t mag = sgn ? rep & ((1u << (n - 1)) - 1u) : rep;
    const int ebits = n - m - (sgn ? 1 : 0);
    const uint32_t expall = ((1u << ebits) - 1u) << m;
    return mag > expall;
}

static int clz32(uint32_t v) {
    int c = 0;
    for (int b = 31; b >= 0 && !((v >> b) & 1u); --b) ++c;
    return c;
}

uint32_t orc_codec_encode_rep(float from, const lofgb_codec_format* F, int mode, int sat,
                              int len, uint64_t r, double u) {
    const int n = F->fmt.bitwidth, toMant = F->fmt.mantissa_bits;
    const int to_signed = F->fmt.signedness == LOFGB_SIGNED;
    const int toExpBits = to_signed ? n - toMant - 1 : n - toMant;
    const int toBias = F->fmt.bias;
    const int kExponentOffset = toBias - 127;
    const int kDigitShift = toMant - 23;
    const int toMinExp = 1 - toBias;
    const int toMaxExp = (1 << toExpBits) - 1 - toBias;
    const int toDigits = toMant + 1;
    const int has_inf = F->fmt.inf_behavior != LOFGB_INF_SATURATING;
    const uint32_t signmask = to_signed ? (1u << (n - 1)) : 0u;
    const uint32_t maxFiniteRep = has_inf ? F->pos_inf - 1u
                                          : (to_signed ? (((1u << n) - 1u) >> 1) : ((1u << n) - 1u));
    const uint32_t infRep = has_inf ? F->pos_inf : maxFiniteRep;
    const uint32_t fb = f2u(from);
    const int neg = (fb >> 31) != 0;
#define WITH_SIGN(mag) ((!neg || !to_signed) ? (uint32_t)(mag)                                  \
                        : (((uint32_t)(mag)) == 0u && codec_is_nan(signmask, F)) ? 0u           \
                        : ((uint32_t)(mag) | signmask))
    /* :164-168 negative value into an unsigned target */
    if (!to_signed && neg) {
        if (!F->neg_to_nan) return 0u;
        return F->fmt.nan_behavior == LOFGB_NAN_3109 ? F->qnan : F->snan;
    }
    const uint32_t from_bits = fb & 0x7FFFFFFFu;
    /* :172-177 inf, NaN, zero */
    if (from_bits == 0x7F800000u) {
        if (sat != LOFGB_SAT_FINITE && has_inf) return WITH_SIGN(infRep);
        return WITH_SIGN(maxFiniteRep);
    }
    if (from_bits > 0x7F800000u) return F->qnan;
    if (from_bits == 0u) return WITH_SIGN(0u);
    const int bfe = (int)(from_bits >> 23);
    /* :182-201 branch 1: the target reaches below FP32's normal range */
    if (toMinExp < -125 && bfe == 0) {
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
        if (kDigitShift > 0) {
            bits <<= kDigitShift;
        } else {
            bits = round_mantissa(bits, -kDigitShift, mode, len, 0, r, u, 64);
            bits >>= -kDigitShift;
        }
        return WITH_SIGN((uint32_t)bits);
    }
    /* :204-241 branch 2: target-subnormal or zero */
    if (toMinExp > -125) {
        const int bte = (bfe - 127) + toBias;
        if (bte <= 0) {
            const uint32_t lead = bfe > 0 ? 1u : 0u;
            const int shift = -kDigitShift - bte + (int)lead;
            uint32_t rfb = (from_bits & 0x7FFFFFu) | (lead << 23);
            uint32_t bits = 0;
            if (shift <= 24) {
                rfb = (uint32_t)round_mantissa(rfb, shift, mode, len, 0, r, u, 32);
                bits = rfb >> shift;
            } else {
                uint64_t w = rfb;
                switch (mode) {
                case LOFGB_RTO:
                case LOFGB_RAFZ: bits = rfb > 0 ? 1u : 0u; break;
                case LOFGB_RTZ: bits = 0; break;
                case LOFGB_RU: bits = (rfb && !neg) ? 1u : 0u; break;
                case LOFGB_RD: bits = (rfb && neg) ? 1u : 0u; break;
                case LOFGB_SR_A: case LOFGB_SR_B: case LOFGB_SR_C: case LOFGB_SR_D:
                case LOFGB_TRUE_SR: case LOFGB_PROB:
                    /* shifts of 64 or more are undefined in the reference: 0 */
                    w = round_mantissa(w, shift, mode, len, 0, r, u, 64);
                    bits = shift >= 64 ? 0u : (uint32_t)(w >> shift);
                    break;
                default: bits = 0; break;
                }
            }
            return WITH_SIGN(bits);
        }
    }
    /* :244-272 normal path, then the overflow rule */
    uint64_t rfb = from_bits;
    if (kDigitShift < 0) {
        rfb = round_mantissa(rfb, -kDigitShift, mode, len, 0, r, u, 64);
        rfb &= ~((1ull << (-kDigitShift)) - 1ull);
    }
    rfb += (uint64_t)(int64_t)kExponentOffset << 23;
    uint32_t bits;
    uint64_t aligned_highest = maxFiniteRep;
    if (kDigitShift < 0) {
        aligned_highest <<= -kDigitShift;
        bits = (uint32_t)(rfb >> (-kDigitShift));
    } else {
        rfb <<= kDigitShift;
        bits = (uint32_t)rfb;
    }
    const int narrower = (toMaxExp < 128) || (toMaxExp == 128 && toDigits < 24);
    if (narrower && rfb > aligned_highest) {
        const int emit_inf = sat == LOFGB_OVF_INF && has_inf;
        return WITH_SIGN(emit_inf ? infRep : maxFiniteRep);
    }
    return WITH_SIGN(bits);
#undef WITH_SIGN
}

/* convert_rep_to_float, src/lo_pack.hpp:293-320 */
float orc_codec_decode_rep(uint32_t rep, const lofgb_codec_format* F) {
    const int n = F->fmt.bitwidth, mant = F->fmt.mantissa_bits, bias = F->fmt.bias;
    const int is_signed = F->fmt.signedness == LOFGB_SIGNED;
    const int has_inf = F->fmt.inf_behavior != LOFGB_INF_SATURATING;
    rep &= n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
    const int sign = is_signed ? (int)((rep >> (n - 1)) & 1u) : 0;
    const uint32_t mag = is_signed ? rep & ((1u << (n - 1)) - 1u) : rep;
    if (has_inf && codec_is_inf(rep, F)) return sign ? -INFINITY : INFINITY;
    if (codec_is_nan(rep, F)) return u2f(0x7FC00000u);
    const uint32_t e = mag >> mant, m = mag & ((1u << mant) - 1u);
    double v;
    if (e == 0) v = ldexp((double)m, 1 - bias - mant);
    else v = ldexp(1.0 + (double)m / (double)(1u << mant), (int)e - bias);
    return (float)(sign ? -v : v);
}

/* group geometry, src/lo_pack.hpp:56-81 */
static int gcd_i(int a, int b) { return b == 0 ? a : gcd_i(b, a % b); }
static int group_bits(int n) { const int al = n <= 8 ? 8 : 16; return n / gcd_i(n, al) * al; }

int64_t orc_packed_size(int n, int64_t count) {
    const int gc = group_bits(n) / n;
    return (count + gc - 1) / gc * (int64_t)(group_bits(n) / 8);
}

/* element i of group g sits at bit g*group_bits + slot*n, slot = i or gc-1-i,
 * LSB-first within each byte (put_bits / get_bits, :85-104) */
static int64_t code_bit(int64_t i, int n, int reverse) {
    const int gc = group_bits(n) / n;
    const int64_t g = i / gc;
    const int k = (int)(i % gc);
    const int slot = reverse ? gc - 1 - k : k;
    return g * group_bits(n) + (int64_t)slot * n;
}

int orc_encode_f32(uint8_t* dst, const float* src, int64_t count, const lofgb_codec_format* f,
                   int mode, int sat, int len, int reverse, uint64_t seed, uint64_t offset) {
    if (!f || f->fmt.bitwidth < 1 || f->fmt.bitwidth > 16) return LOFGB_ERR_FORMAT;
    const int n = f->fmt.bitwidth;
    memset(dst, 0, (size_t)orc_packed_size(n, count));
    const int lg = orc_rng_lanes_log2(mode, len);
    for (int64_t i = 0; i < count; ++i) {
        const uint64_t rb = orc_rng_elem(seed, offset + (uint64_t)i, lg);
        const uint32_t code = orc_codec_encode_rep(src[i], f, mode, sat, len, rb, usamp_of(rb));
        const int64_t b0 = code_bit(i, n, reverse);
        for (int b = 0; b < n; ++b)
            if ((code >> b) & 1u) dst[(b0 + b) >> 3] |= (uint8_t)(1u << ((b0 + b) & 7));
    }
    return 0;
}

int orc_decode_f32(float* dst, const uint8_t* src, int64_t count, const lofgb_codec_format* f,
                   int reverse) {
    if (!f || f->fmt.bitwidth < 1 || f->fmt.bitwidth > 16) return LOFGB_ERR_FORMAT;
    const int n = f->fmt.bitwidth;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t b0 = code_bit(i, n, reverse);
        uint32_t code = 0;
        for (int b = 0; b < n; ++b) code |= (uint32_t)((src[(b0 + b) >> 3] >> ((b0 + b) & 7)) & 1u) << b;
        dst[i] = orc_codec_decode_rep(code, f);
    }
    return 0;
}
