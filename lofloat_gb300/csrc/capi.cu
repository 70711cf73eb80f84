// capi.cu — the extern "C" entry points of liblofgb.so: argument validation,
// host-side precomputation of the rounding plans, error reporting. Kernels
// live in round_kernels.cu, mx_kernels.cu, gemm_plain.cu, gemm_tc.cu.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "lofgb_internal.h"

namespace lofgb {

static thread_local char g_detail[512] = "";

int set_error(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_detail, sizeof(g_detail), fmt, ap);
    va_end(ap);
    return status;
}

void clear_error() { g_detail[0] = 0; }

int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(LOFGB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return LOFGB_OK;
}

int sm_count() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    static int cache[64] = {0};
    if (dev >= 0 && dev < 64 && cache[dev]) return cache[dev];
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
        n = 148;
    if (dev >= 0 && dev < 64) cache[dev] = n;
    return n;
}

// ---- format validation (same rules as the oracle) --------------------------
// Mantissa bits may not exceed the source's (the reference would shift by a
// negative count); exponent field width 0..30; |bias| <= 2^20; the smallest
// subnormal 2^(1-bias-m) must be finite as a float.
int validate_format(const lofgb_format* f, int src_mant_bits) {
    if (!f) return set_error(LOFGB_ERR_NULL, "format pointer is NULL");
    if (f->mantissa_bits < 0 || f->mantissa_bits > src_mant_bits)
        return set_error(LOFGB_ERR_FORMAT, "mantissa_bits %d outside [0, %d]", f->mantissa_bits,
                         src_mant_bits);
    if (f->signedness > 1 || f->inf_behavior > 1 || f->nan_behavior > 1)
        return set_error(LOFGB_ERR_FORMAT, "enum field out of range");
    const int e = f->bitwidth - f->mantissa_bits - (f->signedness == LOFGB_SIGNED ? 1 : 0);
    if (e < 0 || e > 30)
        return set_error(LOFGB_ERR_FORMAT, "exponent field width %d outside [0, 30]", e);
    if (f->bias < -(1 << 20) || f->bias > (1 << 20))
        return set_error(LOFGB_ERR_FORMAT, "bias %d outside [-2^20, 2^20]", f->bias);
    if (1 - f->bias - f->mantissa_bits > 127)
        return set_error(LOFGB_ERR_FORMAT, "smallest subnormal overflows float (bias %d)",
                         f->bias);
    return LOFGB_OK;
}

static int validate_mode(int mode, int len) {
    if (mode < 0 || mode >= LOFGB_NUM_MODES)
        return set_error(LOFGB_ERR_MODE, "unknown rounding mode %d", mode);
    if (len < 0 || len > 62) return set_error(LOFGB_ERR_MODE, "stoch_len %d outside [0, 62]", len);
    return LOFGB_OK;
}

// ---- host-side IEEE helpers -------------------------------------------------
static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint64_t d2u(double f) { uint64_t u; memcpy(&u, &f, 8); return u; }
static inline double u2d(uint64_t u) { double f; memcpy(&f, &u, 8); return f; }

static float half_bits_to_float(uint32_t h) { return __half2float(__ushort_as_half((unsigned short)h)); }
static uint32_t float_to_half_bits(float f) { return __half_as_ushort(__float2half_rn(f)); }

// (float)|x| for a non-negative source bit pattern b (src/lo_float.h:2871).
static float mag_as_float(uint64_t b, int src_bits) {
    if (src_bits == 32) return u2f((uint32_t)b);
    if (src_bits == 64) return (float)u2d(b);
    return half_bits_to_float((uint32_t)b);
}

static uint64_t pinf_bits(int src_bits) {
    return src_bits == 32 ? 0x7F800000ull : (src_bits == 64 ? 0x7FF0000000000000ull : 0x7C00ull);
}

// smallest b in [0, +inf bits] with pred(value(b)), or +inf bits + 1.
template <typename Pred>
static uint64_t lower_bound_bits(int src_bits, Pred pred) {
    uint64_t lo = 0, hi = pinf_bits(src_bits) + 1;  // answer in [lo, hi]
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        if (pred(mag_as_float(mid, src_bits))) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

int make_round_plan(RoundPlan* p, const lofgb_format* f, int src_bits, int mode, int len) {
    const int srcM = src_bits == 32 ? 23 : (src_bits == 64 ? 52 : 10);
    const int srcBias = src_bits == 32 ? 127 : (src_bits == 64 ? 1023 : 15);
    int st = validate_format(f, srcM);
    if (st) return st;
    if ((st = validate_mode(mode, len))) return st;
    memset(p, 0, sizeof(*p));
    const int m = f->mantissa_bits;
    const int to_max = (f->signedness == LOFGB_SIGNED)
                           ? (1 << (f->bitwidth - m - 1)) - 1 - f->bias
                           : (1 << (f->bitwidth - m)) - 1 - f->bias;
    const int to_min = 1 - f->bias;
    // std::pow(2.0, ToMin_exp) * std::pow(2.0, -m) narrowed to float (src/lo_float.h:2861)
    volatile float tiny = (float)(std::ldexp(1.0, to_min) * std::ldexp(1.0, -m));
    volatile float half = tiny * 0.5f;
    const float t = tiny, h = half;
    p->mode = mode;
    p->len = len;
    p->rng_lg = rng_lanes_log2(mode, len);
    p->d = srcM - m;
    p->to_min_field = to_min + srcBias;
    p->to_max_field = to_max + srcBias;
    p->saturating = f->inf_behavior == LOFGB_INF_SATURATING;
    p->tiny_f = t;
    p->tiny_thr = lower_bound_bits(src_bits, [&](float v) { return v >= t; });
    p->pos_thr = lower_bound_bits(src_bits, [&](float v) { return v > 0.0f; });
    p->half_lt = lower_bound_bits(src_bits, [&](float v) { return v >= h; });
    p->half_gt = lower_bound_bits(src_bits, [&](float v) { return v > h; });
    if (src_bits == 32) p->tiny_bits = f2u(t);
    else if (src_bits == 64) p->tiny_bits = d2u((double)t);
    else p->tiny_bits = float_to_half_bits(t);
    // exponent-field thresholds expressed on the magnitude bits
    const uint64_t wmax = src_bits == 64 ? ~0ull : ((1ull << src_bits) - 1);
    auto field_thr = [&](int64_t field) -> uint64_t {  // smallest b with (b >> srcM) >= field
        if (field <= 0) return 0;
        if (field > (int64_t)(wmax >> srcM)) return wmax;
        return (uint64_t)field << srcM;
    };
    p->keep_mask = ~((1ull << p->d) - 1ull) & wmax;
    p->norm_thr = field_thr((int64_t)p->to_min_field);
    p->ovf_thr = field_thr((int64_t)p->to_max_field + 1);
    // tiny-branch decision per sign (src/lo_float.h:2879-2903)
    const uint64_t never = ~0ull;
    switch (mode) {
    case LOFGB_RNE:
    case LOFGB_RTTZ: p->tmin_pos = p->tmin_neg = p->half_gt; break;
    case LOFGB_RNO:
    case LOFGB_RTA: p->tmin_pos = p->tmin_neg = p->half_lt; break;
    case LOFGB_RTO:
    case LOFGB_RAFZ: p->tmin_pos = p->tmin_neg = p->pos_thr; break;
    case LOFGB_RU: p->tmin_pos = p->pos_thr; p->tmin_neg = never; break;
    case LOFGB_RD: p->tmin_pos = never; p->tmin_neg = p->pos_thr; break;
    default: p->tmin_pos = p->tmin_neg = never;  // RTZ and the stochastic modes flush to 0
    }
    // float-grid rounding of below-normal f32 magnitudes (see RoundPlan::grid)
    p->grid = 0;
    const int gexp = to_min - m;  // tiny = 2^gexp
    if (src_bits == 32 && gexp >= -149 && gexp + 23 <= 127) {
        p->grid_c = std::ldexp(1.0f, gexp + 23);
        switch (mode) {
        case LOFGB_RNE: p->grid = 1; break;
        case LOFGB_RTZ: p->grid = 2; p->grid_up_pos = 0; p->grid_up_neg = 0; break;
        case LOFGB_RAFZ: p->grid = 2; p->grid_up_pos = 1; p->grid_up_neg = 1; break;
        case LOFGB_RU: p->grid = 2; p->grid_up_pos = 1; p->grid_up_neg = 0; break;
        case LOFGB_RD: p->grid = 2; p->grid_up_pos = 0; p->grid_up_neg = 1; break;
        default: break;
        }
    }
    // whole-range float rounding (see RoundPlan::uni)
    p->uni = 0;
    p->sat_and = p->saturating ? 0xFFFFFFFFu : 0u;
    p->sat_or = p->saturating ? 0u : 0x7F800000u;
    const int hi = p->to_max_field + 1;
    const bool uni_ok = src_bits == 32 && p->d >= 1 && p->tiny_thr >= 0x00800000ull &&
                        hi + p->d <= 254 && p->to_min_field >= 1 && hi >= p->to_min_field;
    if (uni_ok) {
        p->uni_lo = (uint32_t)p->to_min_field << 23;
        p->uni_hi = (uint32_t)hi << 23;
        p->uni_d = (uint32_t)p->d << 23;
    }
    if (uni_ok && p->grid != 0) p->uni = p->grid;
    // round-to-odd on the same grid (vr_uni_rto_f32): needs the subnormal grid constant
    if (uni_ok && mode == LOFGB_RTO && p->grid_c > 0.0f) p->uni = 6;
    // tiny * 2^-len normal: (to_min - m) - len >= -126
    p->sr_uni = 0;
    if (uni_ok && mode == LOFGB_SR_A && len <= p->d && len <= 23 && gexp - len >= -126 &&
        p->grid_c > 0.0f) {
        p->sr_uni = 1;
        p->sr_mask = len >= 32 ? 0xFFFFFFFFu : ((1u << len) - 1u);
        p->sr_shift = (uint32_t)(p->d - len) << 23;
    }
    return LOFGB_OK;
}

int make_mantissa_plan(RoundPlan* p, int src_bits, int mbits, int mode, int len) {
    const int srcM = src_bits == 32 ? 23 : (src_bits == 64 ? 52 : 10);
    if (mbits < 0 || mbits > srcM)
        return set_error(LOFGB_ERR_FORMAT, "mantissa_bits %d outside [0, %d]", mbits, srcM);
    int st = validate_mode(mode, len);
    if (st) return st;
    memset(p, 0, sizeof(*p));
    p->mode = mode;
    p->len = len;
    p->rng_lg = rng_lanes_log2(mode, len);
    p->d = srcM - mbits;
    p->keep_mask = ~((1ull << p->d) - 1ull);
    return LOFGB_OK;
}

// in/out must be identical or disjoint.
static int check_alias(const void* in, const void* out, int64_t bytes) {
    const char* a = (const char*)in;
    const char* b = (const char*)out;
    if (a == b) return LOFGB_OK;
    if (a < b + bytes && b < a + bytes)
        return set_error(LOFGB_ERR_ALIAS, "input and output partially overlap");
    return LOFGB_OK;
}

static int check_arrays(const void* in, const void* out, int64_t n, int elem) {
    if (n < 0) return set_error(LOFGB_ERR_SIZE, "negative element count");
    if (n > 0 && (!in || !out)) return set_error(LOFGB_ERR_NULL, "NULL data pointer");
    if (n > 0) return check_alias(in, out, n * elem);
    return LOFGB_OK;
}

// GEMM argument checks shared by every GEMM entry point (sizes, trans flags,
// NULL pointers, leading dimensions).
int check_gemm_args(const void* A, int64_t lda, int ta, const void* B, int64_t ldb, int tb,
                    const void* D, int64_t ldd, int M, int N, int K) {
    if (M < 0 || N < 0 || K < 0) return set_error(LOFGB_ERR_SIZE, "negative GEMM dimension");
    if ((ta != 0 && ta != 1) || (tb != 0 && tb != 1))
        return set_error(LOFGB_ERR_SIZE, "trans flags must be 0 or 1");
    if (M && N && !D) return set_error(LOFGB_ERR_NULL, "D is NULL");
    if (M && N && K && (!A || !B)) return set_error(LOFGB_ERR_NULL, "A or B is NULL");
    if (lda < (ta ? M : K) || lda < 1 || ldb < (tb ? K : N) || ldb < 1 || ldd < N || ldd < 1)
        return set_error(LOFGB_ERR_SIZE, "leading dimension too small");
    return LOFGB_OK;
}

// 1 / pmn of an MX element format (src/mx_round.cuh:52-56), in FP32.
float mx_inv_pmn(const lofgb_format* ef) {
    const int m = ef->mantissa_bits;
    const int me = (ef->signedness == LOFGB_SIGNED) ? (1 << (ef->bitwidth - m - 1)) - 1 - ef->bias
                                                    : (1 << (ef->bitwidth - m)) - 1 - ef->bias;
    volatile float a = std::ldexp(1.0f, me);
    volatile float b = 2.0f - std::ldexp(1.0f, -m);
    volatile float pmn = a * b;
    return 1.0f / pmn;
}

}  // namespace lofgb

using namespace lofgb;

extern "C" {

const char* lofgb_strerror(int status) {
    switch (status) {
    case LOFGB_OK: return "ok";
    case LOFGB_ERR_NULL: return "null pointer";
    case LOFGB_ERR_SIZE: return "invalid size or leading dimension";
    case LOFGB_ERR_FORMAT: return "unsupported float format";
    case LOFGB_ERR_MODE: return "invalid rounding mode or stoch_len";
    case LOFGB_ERR_BLOCK: return "unsupported MX block size (use 8/16/32/64/128/256)";
    case LOFGB_ERR_ALIAS: return "input and output partially overlap";
    case LOFGB_ERR_UNSUPPORTED: return "unsupported request";
    case LOFGB_ERR_CUDA: return "CUDA error";
    case LOFGB_ERR_WORKSPACE: return "workspace too small or misaligned";
    case LOFGB_ERR_TIMEOUT: return "device-side wait timed out";
    default: return "unknown status";
    }
}

const char* lofgb_last_error_detail(void) { return g_detail; }

int lofgb_version(void) { return 100; }

#define LOFGB_ROUND_FMT(NAME, T, BITS, SCALE_T)                                                  \
    int NAME(const T* in, T* out, int64_t n, const lofgb_format* fmt, int mode, int stoch_len,   \
             SCALE_T scale, uint64_t seed, uint64_t offset, void* stream) {                      \
        g_detail[0] = 0;                                                                        \
        int st = check_arrays(in, out, n, (int)sizeof(T));                                      \
        if (st) return st;                                                                      \
        RoundPlan p;                                                                            \
        if ((st = make_round_plan(&p, fmt, BITS, mode, stoch_len))) return st;                 \
        if (n == 0) return LOFGB_OK;                                                            \
        return launch_round(BITS, true, in, out, n, p, (double)scale, seed, offset, stream);    \
    }

LOFGB_ROUND_FMT(lofgb_round_f32, float, 32, float)
LOFGB_ROUND_FMT(lofgb_round_f64, double, 64, double)
LOFGB_ROUND_FMT(lofgb_round_f16, uint16_t, 16, float)

#define LOFGB_ROUND_MANT(NAME, T, BITS, SCALE_T)                                                 \
    int NAME(const T* in, T* out, int64_t n, int mantissa_bits, int mode, int stoch_len,         \
             SCALE_T scale, uint64_t seed, uint64_t offset, void* stream) {                      \
        g_detail[0] = 0;                                                                        \
        int st = check_arrays(in, out, n, (int)sizeof(T));                                      \
        if (st) return st;                                                                      \
        RoundPlan p;                                                                            \
        if ((st = make_mantissa_plan(&p, BITS, mantissa_bits, mode, stoch_len))) return st;    \
        if (n == 0) return LOFGB_OK;                                                            \
        return launch_round(BITS, false, in, out, n, p, (double)scale, seed, offset, stream);   \
    }

LOFGB_ROUND_MANT(lofgb_round_mantissa_f32, float, 32, float)
LOFGB_ROUND_MANT(lofgb_round_mantissa_f64, double, 64, double)
LOFGB_ROUND_MANT(lofgb_round_mantissa_f16, uint16_t, 16, float)

// Shared by the FP32 and BF16 MX entry points: validation, plans, pmn.
static int mx_prepare(int64_t n, int block_size, const lofgb_format* elem_fmt,
                      const lofgb_format* scale_fmt, int mode, int scale_mode, int stoch_len,
                      RoundPlan* pe, RoundPlan* ps, float* inv_pmn) {
    if (!(block_size == 8 || block_size == 16 || block_size == 32 || block_size == 64 ||
          block_size == 128 || block_size == 256))
        return set_error(LOFGB_ERR_BLOCK, "unsupported MX block size %d", block_size);
    int st;
    if ((st = make_round_plan(pe, elem_fmt, 32, mode, stoch_len))) return st;
    if ((st = make_round_plan(ps, scale_fmt, 32, scale_mode, 0))) return st;
    (void)n;
    const int m = elem_fmt->mantissa_bits;
    const int me = (elem_fmt->signedness == LOFGB_SIGNED)
                       ? (1 << (elem_fmt->bitwidth - m - 1)) - 1 - elem_fmt->bias
                       : (1 << (elem_fmt->bitwidth - m)) - 1 - elem_fmt->bias;
    volatile float a = std::ldexp(1.0f, me);
    volatile float b = 2.0f - std::ldexp(1.0f, -m);
    volatile float pmn = a * b;
    *inv_pmn = 1.0f / pmn;
    return LOFGB_OK;
}

int lofgb_mx_round_bf16(const uint16_t* in, float* out, int64_t n, int block_size,
                        const lofgb_format* elem_fmt, const lofgb_format* scale_fmt, int mode,
                        int scale_mode, int stoch_len, uint64_t seed, uint64_t offset,
                        void* stream) {
    g_detail[0] = 0;
    if (n < 0) return set_error(LOFGB_ERR_SIZE, "negative element count");
    if (n > 0 && (!in || !out)) return set_error(LOFGB_ERR_NULL, "NULL data pointer");
    if (n > 0) {
        // a 2n-byte input and a 4n-byte output must not overlap at all
        const char* a = reinterpret_cast<const char*>(in);
        const char* b = reinterpret_cast<const char*>(out);
        if (a < b + 4 * n && b < a + 2 * n)
            return set_error(LOFGB_ERR_ALIAS, "input and output overlap");
    }
    RoundPlan pe, ps;
    float inv;
    int st = mx_prepare(n, block_size, elem_fmt, scale_fmt, mode, scale_mode, stoch_len, &pe, &ps, &inv);
    if (st) return st;
    if (n == 0) return LOFGB_OK;
    return launch_mx_bf16(in, out, n, block_size, pe, ps, inv, seed, offset, stream);
}

int lofgb_mx_round_f32(const float* in, float* out, int64_t n, int block_size,
                       const lofgb_format* elem_fmt, const lofgb_format* scale_fmt, int mode,
                       int scale_mode, int stoch_len, uint64_t seed, uint64_t offset,
                       void* stream) {
    g_detail[0] = 0;
    int st = check_arrays(in, out, n, 4);
    if (st) return st;
    if (!(block_size == 8 || block_size == 16 || block_size == 32 || block_size == 64 ||
          block_size == 128 || block_size == 256))
        return set_error(LOFGB_ERR_BLOCK, "unsupported MX block size %d", block_size);
    RoundPlan pe, ps;
    if ((st = make_round_plan(&pe, elem_fmt, 32, mode, stoch_len))) return st;
    if ((st = make_round_plan(&ps, scale_fmt, 32, scale_mode, 0))) return st;
    if (n == 0) return LOFGB_OK;
    // pmn = ldexpf(1, me) * (2 - ldexpf(1, -m)) in float (src/mx_round.cuh:52-56)
    const int m = elem_fmt->mantissa_bits;
    const int me = (elem_fmt->signedness == LOFGB_SIGNED)
                       ? (1 << (elem_fmt->bitwidth - m - 1)) - 1 - elem_fmt->bias
                       : (1 << (elem_fmt->bitwidth - m)) - 1 - elem_fmt->bias;
    volatile float a = std::ldexp(1.0f, me);
    volatile float b = 2.0f - std::ldexp(1.0f, -m);
    volatile float pmn = a * b;
    volatile float inv = 1.0f / pmn;
    return launch_mx(in, out, n, block_size, pe, ps, pmn, inv, seed, offset, stream);
}

static int gemm_impl(const float* A, int64_t lda, int64_t sa, int trans_a, const float* B,
                     int64_t ldb, int64_t sb, int trans_b, float* D, int64_t ldd, int64_t sd,
                     int M, int N, int K, int batch, int accum_mant_bits, int mode, float alpha,
                     int variant, int chunk, void* workspace, size_t workspace_bytes,
                     void* stream, const RoundPlan* acc_fmt = nullptr) {
    g_detail[0] = 0;
    int st = check_gemm_args(A, lda, trans_a, B, ldb, trans_b, D, ldd, M, N, K);
    if (st) return st;
    if (accum_mant_bits < 0 || accum_mant_bits > 23)
        return set_error(LOFGB_ERR_FORMAT, "accum_mant_bits %d outside [0, 23]", accum_mant_bits);
    if (mode != LOFGB_RNE)
        return set_error(LOFGB_ERR_MODE,
                         "accumulator rounding is RNE only (the reference leaf ignores the mode)");
    if (batch < 0) return set_error(LOFGB_ERR_SIZE, "negative batch");
    if (sa < 0 || sb < 0 || sd < 0) return set_error(LOFGB_ERR_SIZE, "negative batch stride");
    if (batch > 1 && M > 0 && N > 0 && sd < (int64_t)(M - 1) * ldd + N)
        return set_error(LOFGB_ERR_ALIAS, "batch stride of D smaller than one D matrix");
    if (M == 0 || N == 0 || batch == 0) return LOFGB_OK;
    if (variant == LOFGB_GEMM_PLAIN)
        return launch_gemm_plain(A, lda, sa, trans_a, B, ldb, sb, trans_b, D, ldd, sd, M, N, K,
                                 batch, accum_mant_bits, acc_fmt, alpha, stream);
    if (variant == LOFGB_GEMM_TC) {
        if (chunk <= 0 || chunk % 16 != 0 || chunk > 256)
            return set_error(LOFGB_ERR_SIZE, "chunk %d must be a multiple of 16 in [16, 256]",
                             chunk);
        return launch_gemm_tc(A, lda, sa, trans_a, B, ldb, sb, trans_b, D, ldd, sd, M, N, K,
                              batch, accum_mant_bits, acc_fmt, alpha, chunk, workspace,
                              workspace_bytes, stream);
    }
    return set_error(LOFGB_ERR_UNSUPPORTED, "unknown GEMM variant %d", variant);
}

int lofgb_gemm_f32(const float* A, int64_t lda, int trans_a, const float* B, int64_t ldb,
                   int trans_b, float* D, int64_t ldd, int M, int N, int K, int accum_mant_bits,
                   int mode, float alpha, int variant, int chunk, void* workspace,
                   size_t workspace_bytes, void* stream) {
    return gemm_impl(A, lda, 0, trans_a, B, ldb, 0, trans_b, D, ldd, 0, M, N, K, 1,
                     accum_mant_bits, mode, alpha, variant, chunk, workspace, workspace_bytes,
                     stream);
}

size_t lofgb_gemm_tc_workspace_size(int M, int N, int K) {
    if (M <= 0 || N <= 0 || K <= 0) return 0;
    return gemm_tc_workspace(M, N, K, 1);
}

int lofgb_gemm_batched_f32(const float* A, int64_t lda, int64_t stride_a, int trans_a,
                           const float* B, int64_t ldb, int64_t stride_b, int trans_b, float* D,
                           int64_t ldd, int64_t stride_d, int M, int N, int K, int batch,
                           int accum_mant_bits, int mode, float alpha, int variant, int chunk,
                           void* workspace, size_t workspace_bytes, void* stream) {
    return gemm_impl(A, lda, stride_a, trans_a, B, ldb, stride_b, trans_b, D, ldd, stride_d, M,
                     N, K, batch, accum_mant_bits, mode, alpha, variant, chunk, workspace,
                     workspace_bytes, stream);
}

int lofgb_gemm_accfmt_f32(const float* A, int64_t lda, int trans_a, const float* B, int64_t ldb,
                          int trans_b, float* D, int64_t ldd, int M, int N, int K,
                          const lofgb_format* accum_fmt, float alpha, int variant, int chunk,
                          void* workspace, size_t workspace_bytes, void* stream) {
    g_detail[0] = 0;
    RoundPlan plan;
    int st = make_round_plan(&plan, accum_fmt, 32, LOFGB_RNE, 0);
    if (st) return st;
    return gemm_impl(A, lda, 0, trans_a, B, ldb, 0, trans_b, D, ldd, 0, M, N, K, 1,
                     23 - plan.d, LOFGB_RNE, alpha, variant, chunk, workspace, workspace_bytes,
                     stream, &plan);
}

size_t lofgb_gemm_batched_tc_workspace_size(int M, int N, int K, int batch) {
    if (M <= 0 || N <= 0 || K <= 0 || batch <= 0) return 0;
    return gemm_tc_workspace(M, N, K, batch);
}

int lofgb_gemm_f64_ref(const float* A, int64_t lda, int trans_a, const float* B, int64_t ldb,
                       int trans_b, double* D, int64_t ldd, int M, int N, int K, void* stream) {
    g_detail[0] = 0;
    int st = check_gemm_args(A, lda, trans_a, B, ldb, trans_b, D, ldd, M, N, K);
    if (st) return st;
    if (M == 0 || N == 0) return LOFGB_OK;
    return launch_gemm_f64(A, lda, trans_a, B, ldb, trans_b, D, ldd, M, N, K, stream);
}

}  // extern "C"
