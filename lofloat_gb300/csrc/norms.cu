// norms.cu — the BatchNorm approximations (L1, L-infinity, FISR, PWL) as
// two kernels: per-channel statistics, then one fused normalise-and-affine
// pass.
//
// Replaces the torch compositions of L1BatchNorm, LinfBatchNorm,
// FISRBatchNorm and PWLBatchNorm (LoFloat/layers.py:805-1047), which run a
// mean, a centring pass, a deviation reduction and four to six elementwise
// passes over the activation. Layout: x is [n, c, inner] contiguous (NCHW
// with inner = H*W; a 2-D (N, C) input has inner = 1); channel ch owns the n
// rows of `inner` consecutive values at (nn * c + ch) * inner.
//
// Statistics (HBM-bound, 4 B read per element and pass):
//   stats_pass_kernel      a grid of (row splits) x (channels), sized to one
//                          co-resident wave; every CTA reduces its slice of
//                          one channel to a pair of doubles: sum x, or the
//                          shifted sums sum (x - K), sum (x - K)^2 (K = the
//                          channel's first value), or sum |x - mean| with the
//                          FP32 mean of the previous pass (the centring the
//                          reference performs in FP32), or sum x with the
//                          FP32 max and min of x packed in the second double;
//                          the channel's last CTA (a ticket per channel)
//                          combines the splits in double, writes the FP32
//                          statistic and the running-average update
//                          r = r (1 - m) + m s.
// L1 takes two statistics passes (mean, then the deviation about it);
// L-infinity and the variance variants one. L-infinity's max |x - mean| is
// max(max x - mean, mean - min x) with both differences rounded in FP32:
// rounding is monotone, so the largest rounded |x - mean| comes from the
// largest or the smallest x, and the bits equal those of the maximum taken
// over every centred value. A NaN input makes the sum, the mean and so the
// deviation NaN; an infinite x makes one difference inf - inf = NaN, as the
// centred value of that x is.
//
// Normalisation (HBM-bound, 4 B read + 4 B written per element): per element
// in FP32, in the reference's operation order,
//   L1 / L-inf  y = ((x - mean) / (dev + eps)) * scale,   FISR / PWL  y = (x - mean) * r
//   then y = y * w + b with the affine parameters,
// where r is the channel's approximate 1/sqrt(var + eps): the bit-trick seed
// 0x5F3759DF - (bits >> 1) and two Newton steps y (1.5 - (v/2) y y) (FISR),
// or the PWL table interpolated on the mantissa in [1, 2) times
// 2^-floor(e/2) and 1/sqrt(2) for odd e (PWL). Every operation is a single
// IEEE FP32 operation with no contraction, as torch evaluates the chain, so
// given the same statistics the output has the reference's bits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "lofgb_internal.h"

namespace lofgb {

namespace {

constexpr int NT = 256;            // threads per CTA
constexpr int TARGET_CTAS = 1216;  // statistics grid: about 8 CTAs per SM
constexpr int MAX_SPLITS = 1024;
constexpr int UNR = 4;             // 16-byte vectors in flight per thread

enum { P_SUM = 0, P_SHIFTED = 1, P_ABSDEV = 2, P_SUMRANGE = 3 };

struct BnGeo {
    int64_t n, c, inner;
    int splits;        // row splits (row path) or element splits (flat path)
    int rows_per;      // rows per split (row path)
    int64_t elems_per; // elements per split (flat path)
    int vec;           // row path with 16-byte vectors
    int flat;          // small rows: walk the channel's flattened values
};

int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

BnGeo bn_geo(int64_t n, int64_t c, int64_t inner, const void* x) {
    BnGeo g;
    g.n = n;
    g.c = c;
    g.inner = inner;
    g.flat = inner < 64;
    g.vec = !g.flat && inner % 4 == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0;
    // as many splits per channel as keep the whole grid one co-resident wave
    // (no tail of a few CTAs), at least one
    int64_t want = std::max<int64_t>(1, TARGET_CTAS / std::max<int64_t>(c, 1));
    if (g.flat) {
        const int64_t per_ch = n * inner;
        int64_t s = std::min<int64_t>(want, cdiv(per_ch, 4096));
        s = std::max<int64_t>(1, std::min<int64_t>(s, MAX_SPLITS));
        g.splits = (int)s;
        g.elems_per = cdiv(per_ch, s);
        g.rows_per = 0;
    } else {
        int64_t s = std::max<int64_t>(1, std::min<int64_t>({want, n, (int64_t)MAX_SPLITS}));
        g.rows_per = (int)cdiv(n, s);
        g.splits = (int)cdiv(n, g.rows_per);
        g.elems_per = 0;
    }
    return g;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}
// The FP32 max and min of a P_SUMRANGE pass travel as the two halves of one
// double's bits (moved and stored, never used in arithmetic).
__device__ __forceinline__ double pack_range(float hi, float lo) {
    return __hiloint2double(__float_as_int(hi), __float_as_int(lo));
}
__device__ __forceinline__ float range_hi(double v) { return __int_as_float(__double2hiint(v)); }
__device__ __forceinline__ float range_lo(double v) { return __int_as_float(__double2loint(v)); }
__device__ __forceinline__ double range_join(double u, double v) {
    return pack_range(fmaxf(range_hi(u), range_hi(v)), fminf(range_lo(u), range_lo(v)));
}
__device__ __forceinline__ double warp_range(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = range_join(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

// Per-thread accumulation of one value in FP32 (a few hundred values per
// thread at most), combined across the CTA and the splits in double.
template <int P>
struct Acc {
    float a = 0.0f, b = 0.0f;
    float k = 0.0f;  // shift (P_SHIFTED) or FP32 mean (P_ABSDEV)
    float hi = -INFINITY, lo = INFINITY;  // P_SUMRANGE
    __device__ __forceinline__ void add(float x) {
        if constexpr (P == P_SUM) {
            a = __fadd_rn(a, x);
        } else if constexpr (P == P_SUMRANGE) {
            a = __fadd_rn(a, x);
            hi = fmaxf(hi, x);  // NaNs are skipped here and carried by the sum
            lo = fminf(lo, x);
        } else if constexpr (P == P_SHIFTED) {
            const float d = __fsub_rn(x, k);
            a = __fadd_rn(a, d);
            b = __fmaf_rn(d, d, b);
        } else {
            a = __fadd_rn(a, fabsf(__fsub_rn(x, k)));
        }
    }
};

// Combines a channel's split results in double (one warp) and writes the
// FP32 statistic. P_SUM writes mean; P_SHIFTED mean and the biased variance
// (to dev); P_ABSDEV dev; P_SUMRANGE mean and max |x - mean| (to
// dev). running_mean / running_dev (NULL: not updated) take r (1 - m) + m s
// for what was written.
template <int P>
__device__ __forceinline__ void finalize_channel(const double2* part, const BnGeo& g, int64_t ch,
                                                 const float* x, float* mean, float* dev,
                                                 float* running_mean, float* running_dev,
                                                 float momentum) {
    const int lane = threadIdx.x & 31;
    double a = 0.0, b = P == P_SUMRANGE ? pack_range(-INFINITY, INFINITY) : 0.0;
    for (int s = lane; s < g.splits; s += 32) {
        const double2 p = __ldcg(part + ch * g.splits + s);
        a += p.x;
        b = (P == P_SUMRANGE) ? range_join(b, p.y) : b + p.y;
    }
    a = warp_sum(a);
    b = (P == P_SUMRANGE) ? warp_range(b) : warp_sum(b);
    if (lane != 0) return;
    const double cnt = (double)g.n * (double)g.inner;
    const float keep = __fsub_rn(1.0f, momentum);
    auto track = [&](float* r, float v) {
        if (r) r[ch] = __fadd_rn(__fmul_rn(r[ch], keep), __fmul_rn(momentum, v));
    };
    if constexpr (P == P_SUM) {
        const float m = (float)(a / cnt);
        mean[ch] = m;
        track(running_mean, m);
    } else if constexpr (P == P_SUMRANGE) {
        const float m = (float)(a / cnt);
        const float d1 = __fsub_rn(range_hi(b), m), d2 = __fsub_rn(m, range_lo(b));
        // the larger difference is never below zero; clearing the sign makes
        // a zero deviation +0 as |x - mean| is (all x -0: -0 - (+0) = -0)
        const float d = (d1 != d1 || d2 != d2) ? __int_as_float(0x7FC00000)
                                               : __int_as_float(__float_as_int(fmaxf(d1, d2)) & 0x7FFFFFFF);
        mean[ch] = m;
        dev[ch] = d;
        track(running_mean, m);
        track(running_dev, d);
    } else if constexpr (P == P_SHIFTED) {
        const double k = (double)x[ch * g.inner];
        const double d = a / cnt;
        const float m = (float)(k + d);
        double var = b / cnt - d * d;
        if (var < 0.0) var = 0.0;
        mean[ch] = m;
        dev[ch] = (float)var;
        track(running_mean, m);
        track(running_dev, (float)var);
    } else {
        dev[ch] = (float)(a / cnt);
        track(running_dev, dev[ch]);
    }
}

// One statistics pass. Every CTA reduces its slice of one channel to a pair
// of doubles; the last CTA of the channel to finish (a ticket per channel)
// combines them (finalize_channel) and resets the ticket for the next pass.
template <int P>
__global__ void __launch_bounds__(NT)
stats_pass_kernel(const float* __restrict__ x, BnGeo g, const float* __restrict__ center,
                  double2* __restrict__ part, unsigned* __restrict__ tickets, float* mean,
                  float* dev, float* running_mean, float* running_dev, float momentum) {
    pdl_wait();
    const int s = blockIdx.x;
    const int64_t ch = blockIdx.y;
    Acc<P> acc;
    if constexpr (P == P_SHIFTED) acc.k = x[ch * g.inner];
    if constexpr (P == P_ABSDEV) acc.k = center[ch];
    if (g.flat) {
        const int64_t per_ch = g.n * g.inner;
        const int64_t j0 = (int64_t)s * g.elems_per;
        const int64_t j1 = min(per_ch, j0 + g.elems_per);
        for (int64_t j = j0 + threadIdx.x; j < j1; j += NT) {
            const int64_t nn = j / g.inner, ii = j - nn * g.inner;
            acc.add(x[(nn * g.c + ch) * g.inner + ii]);
        }
    } else {
        const int64_t r0 = (int64_t)s * g.rows_per;
        const int64_t r1 = min(g.n, r0 + g.rows_per);
        for (int64_t nn = r0; nn < r1; ++nn) {
            const float* row = x + (nn * g.c + ch) * g.inner;
            if (g.vec) {
                // UNR vectors per thread in flight before they are consumed
                const float4* v = reinterpret_cast<const float4*>(row);
                const int64_t nv = g.inner / 4;
                for (int64_t i0 = threadIdx.x; i0 < nv; i0 += (int64_t)NT * UNR) {
                    float4 q[UNR];
#pragma unroll
                    for (int u = 0; u < UNR; ++u) {
                        const int64_t i = i0 + (int64_t)u * NT;
                        q[u] = i < nv ? __ldg(v + i) : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
#pragma unroll
                    for (int u = 0; u < UNR; ++u) {
                        if (i0 + (int64_t)u * NT < nv) {
                            acc.add(q[u].x);
                            acc.add(q[u].y);
                            acc.add(q[u].z);
                            acc.add(q[u].w);
                        }
                    }
                }
            } else {
                for (int64_t i = threadIdx.x; i < g.inner; i += NT) acc.add(__ldg(row + i));
            }
        }
    }
    __shared__ double red[2][NT / 32];
    __shared__ int last;
    double a = acc.a, b = P == P_SUMRANGE ? pack_range(acc.hi, acc.lo) : (double)acc.b;
    a = warp_sum(a);
    b = (P == P_SUMRANGE) ? warp_range(b) : warp_sum(b);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = a;
        red[1][w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = red[0][0], tb = red[1][0];
        for (int i = 1; i < NT / 32; ++i) {
            ta += red[0][i];
            tb = (P == P_SUMRANGE) ? range_join(tb, red[1][i]) : tb + red[1][i];
        }
        part[ch * g.splits + s] = make_double2(ta, tb);
        __threadfence();
        last = atomicAdd(tickets + ch, 1u) == (unsigned)g.splits - 1;
    }
    __syncthreads();
    if (last && w == 0) {
        __threadfence();
        finalize_channel<P>(part, g, ch, x, mean, dev, running_mean, running_dev, momentum);
        if (threadIdx.x == 0) tickets[ch] = 0;
    }
}

// ---- normalisation ---------------------------------------------------------------
struct ApplyArgs {
    const float* x;
    float* y;
    int64_t n, c, inner;
    const float* mean;
    const float* dev;
    const float* scale;   // per channel, or NULL
    const float* weight;  // per channel, or NULL (no affine step)
    const float* bias;
    const float* lut;     // PWL table (norm == LOFGB_BN_PWL)
    int segments;
    float eps;
    int norm;
    int vec;
};

// Approximate 1/sqrt(v) of FISRBatchNorm (bit-trick seed, two Newton steps).
__device__ __forceinline__ float fisr(float v) {
    const float half = __fmul_rn(v, 0.5f);
    float y = __int_as_float(0x5F3759DF - (__float_as_int(v) >> 1));
#pragma unroll
    for (int i = 0; i < 2; ++i)
        y = __fmul_rn(y, __fsub_rn(1.5f, __fmul_rn(__fmul_rn(half, y), y)));
    return y;
}

// Approximate 1/sqrt(v) of PWLBatchNorm: v = m 2^e with m in [1, 2); the
// table over [1, 2] interpolated at m, times 2^-floor(e/2), times 1/sqrt(2)
// (in FP32) for odd e.
__device__ __forceinline__ float pwl_rsqrt(float v, const float* __restrict__ lut, int nseg) {
    int e;
    const float m = __fmul_rn(frexpf(v, &e), 2.0f);
    e -= 1;
    const float u = __fmul_rn(__fsub_rn(m, 1.0f), (float)nseg);
    int i = (int)floorf(u);
    i = i < 0 ? 0 : (i > nseg - 1 ? nseg - 1 : i);
    const float frac = __fsub_rn(u, (float)i);
    const float f = __ldg(lut + i), gv = __ldg(lut + i + 1);
    const float r = __fadd_rn(f, __fmul_rn(frac, __fsub_rn(gv, f)));
    const int eh = e >> 1;  // floor(e / 2)
    float sc = ldexpf(1.0f, -eh);
    if (e & 1) sc = __fmul_rn(sc, 0.70710677f);
    return __fmul_rn(r, sc);
}

struct ChanFactors {
    float mean, dpe, r, sc, w, b;
};

__device__ __forceinline__ ChanFactors chan_factors(const ApplyArgs& a, int64_t ch) {
    ChanFactors f;
    f.mean = __ldg(a.mean + ch);
    const float d = __fadd_rn(__ldg(a.dev + ch), a.eps);
    f.dpe = d;
    f.r = a.norm == LOFGB_BN_FISR ? fisr(d) : a.norm == LOFGB_BN_PWL ? pwl_rsqrt(d, a.lut, a.segments) : 0.0f;
    f.sc = a.scale ? __ldg(a.scale + ch) : 1.0f;
    f.w = a.weight ? __ldg(a.weight + ch) : 1.0f;
    f.b = a.weight ? __ldg(a.bias + ch) : 0.0f;
    return f;
}

__device__ __forceinline__ float normalise(float x, const ChanFactors& f, const ApplyArgs& a) {
    const float xc = __fsub_rn(x, f.mean);
    float y;
    if (a.norm == LOFGB_BN_DIVIDE) {
        y = __fdiv_rn(xc, f.dpe);
        if (a.scale) y = __fmul_rn(y, f.sc);
    } else {
        y = __fmul_rn(xc, f.r);
    }
    if (a.weight) y = __fadd_rn(__fmul_rn(y, f.w), f.b);
    return y;
}

// Row path: CTAs stride over the n * c rows; per row the channel factors
// once, then the row's values as 16-byte vectors (or scalars).
__global__ void __launch_bounds__(NT, 6)
bn_apply_rows_kernel(ApplyArgs a) {
    pdl_wait();
    const int64_t rows = a.n * a.c;
    for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
        const float* xr = a.x + row * a.inner;
        float* yr = a.y + row * a.inner;
        if (a.vec) {
            const int64_t nv = a.inner / 4;
            const float4* xv = reinterpret_cast<const float4*>(xr);
            float4* yv = reinterpret_cast<float4*>(yr);
            // the row's first vectors are requested before the channel
            // factors, so the two reads overlap
            float4 q[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
                const int64_t i = threadIdx.x + (int64_t)u * NT;
                if (i < nv) q[u] = __ldcs(xv + i);
            }
            const ChanFactors f = chan_factors(a, row % a.c);
            for (int64_t i0 = threadIdx.x; i0 < nv; i0 += (int64_t)NT * UNR) {
                if (i0 != threadIdx.x) {
#pragma unroll
                    for (int u = 0; u < UNR; ++u) {
                        const int64_t i = i0 + (int64_t)u * NT;
                        if (i < nv) q[u] = __ldcs(xv + i);
                    }
                }
#pragma unroll
                for (int u = 0; u < UNR; ++u) {
                    const int64_t i = i0 + (int64_t)u * NT;
                    if (i < nv) {
                        q[u].x = normalise(q[u].x, f, a);
                        q[u].y = normalise(q[u].y, f, a);
                        q[u].z = normalise(q[u].z, f, a);
                        q[u].w = normalise(q[u].w, f, a);
                        __stcs(yv + i, q[u]);
                    }
                }
            }
        } else {
            const ChanFactors f = chan_factors(a, row % a.c);
            for (int64_t i = threadIdx.x; i < a.inner; i += NT) yr[i] = normalise(xr[i], f, a);
        }
    }
}

// Flat path (short rows): one value per thread, grid-stride.
__global__ void __launch_bounds__(NT)
bn_apply_flat_kernel(ApplyArgs a) {
    pdl_wait();
    const int64_t total = a.n * a.c * a.inner;
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < total; i += (int64_t)gridDim.x * NT) {
        const int64_t ch = (i / a.inner) % a.c;
        a.y[i] = normalise(a.x[i], chan_factors(a, ch), a);
    }
}

int check_geo(const float* x, int64_t n, int64_t c, int64_t inner) {
    if (n < 0 || c < 0 || inner < 0) return set_error(LOFGB_ERR_SIZE, "negative BatchNorm size");
    if (c > 65535) return set_error(LOFGB_ERR_SIZE, "more than 65535 channels");
    if (n > 0 && c > 0 && inner > 0 && !x) return set_error(LOFGB_ERR_NULL, "NULL input");
    return LOFGB_OK;
}

template <int P>
int run_pass(const float* x, const BnGeo& g, const float* center, double2* part, unsigned* tickets,
             float* mean, float* dev, float* rmean, float* rdev, float momentum, cudaStream_t st) {
    cudaError_t e = launch_pdl(stats_pass_kernel<P>, dim3(g.splits, (unsigned)g.c), dim3(NT), 0, st,
                               x, g, center, part, tickets, mean, dev, rmean, rdev, momentum);
    if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "stats_pass_kernel: %s", cudaGetErrorString(e));
    return LOFGB_OK;
}

size_t part_bytes(const BnGeo& g) { return ((size_t)g.splits * (size_t)g.c * sizeof(double2) + 255) & ~(size_t)255; }

}  // namespace

}  // namespace lofgb

using namespace lofgb;

extern "C" {

size_t lofgb_bn_workspace_size(int64_t n, int64_t c, int64_t inner) {
    if (n <= 0 || c <= 0 || inner <= 0) return 0;
    const BnGeo g = bn_geo(n, c, inner, nullptr);
    return part_bytes(g) + (size_t)c * sizeof(unsigned);
}

int lofgb_bn_stats_f32(const float* x, int64_t n, int64_t c, int64_t inner, int stat, float* mean,
                       float* dev, float* running_mean, float* running_dev, float momentum,
                       void* workspace, size_t workspace_bytes, void* stream) {
    clear_error();
    int rc = check_geo(x, n, c, inner);
    if (rc) return rc;
    if (stat < LOFGB_BN_MEAN_ABS_DEV || stat > LOFGB_BN_VARIANCE)
        return set_error(LOFGB_ERR_UNSUPPORTED, "unknown BatchNorm statistic %d", stat);
    if (c == 0) return LOFGB_OK;
    if (n == 0 || inner == 0) return set_error(LOFGB_ERR_SIZE, "BatchNorm statistics of no values");
    if (!mean || !dev) return set_error(LOFGB_ERR_NULL, "NULL mean or deviation output");
    const BnGeo g = bn_geo(n, c, inner, x);
    const size_t need = part_bytes(g) + (size_t)c * sizeof(unsigned);
    if (!workspace || workspace_bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 15))
        return set_error(LOFGB_ERR_WORKSPACE, "need %zu bytes of 16-byte aligned workspace", need);
    auto* part = static_cast<double2*>(workspace);
    auto* tickets = reinterpret_cast<unsigned*>(static_cast<uint8_t*>(workspace) + part_bytes(g));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the tickets start every call at zero (each pass's last CTA resets them)
    cudaError_t e = cudaMemsetAsync(tickets, 0, (size_t)c * sizeof(unsigned), st);
    if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
    if (stat == LOFGB_BN_VARIANCE) {
        if ((rc = run_pass<P_SHIFTED>(x, g, nullptr, part, tickets, mean, dev, running_mean, running_dev,
                                      momentum, st)))
            return rc;
    } else if (stat == LOFGB_BN_MAX_ABS_DEV) {
        if ((rc = run_pass<P_SUMRANGE>(x, g, nullptr, part, tickets, mean, dev, running_mean, running_dev,
                                       momentum, st)))
            return rc;
    } else {
        if ((rc = run_pass<P_SUM>(x, g, nullptr, part, tickets, mean, dev, running_mean, nullptr, momentum, st)))
            return rc;
        if ((rc = run_pass<P_ABSDEV>(x, g, mean, part, tickets, mean, dev, nullptr, running_dev, momentum,
                                     st)))
            return rc;
    }
    return check_launch("BatchNorm statistics");
}

int lofgb_bn_apply_f32(const float* x, float* y, int64_t n, int64_t c, int64_t inner,
                       const float* mean, const float* dev, float eps, int norm, const float* scale,
                       const float* weight, const float* bias, const float* lut, int segments,
                       void* stream) {
    clear_error();
    int rc = check_geo(x, n, c, inner);
    if (rc) return rc;
    if (norm < LOFGB_BN_DIVIDE || norm > LOFGB_BN_PWL)
        return set_error(LOFGB_ERR_UNSUPPORTED, "unknown BatchNorm normaliser %d", norm);
    if (norm == LOFGB_BN_PWL && (segments < 1 || segments > 65536 || !lut))
        return set_error(LOFGB_ERR_SIZE, "PWL normaliser needs a table of 1..65536 segments");
    const int64_t total = n * c * inner;
    if (total == 0) return LOFGB_OK;
    if (!y || !mean || !dev) return set_error(LOFGB_ERR_NULL, "NULL output or statistics");
    if (weight && !bias) return set_error(LOFGB_ERR_NULL, "affine weight without bias");
    const int64_t bytes = total * 4;
    const char* a = reinterpret_cast<const char*>(x);
    const char* b = reinterpret_cast<const char*>(y);
    if (a != b && a < b + bytes && b < a + bytes)
        return set_error(LOFGB_ERR_ALIAS, "input and output partially overlap");
    ApplyArgs args{x, y, n, c, inner, mean, dev, scale, weight, bias, lut, segments, eps, norm, 0};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t maxg = (int64_t)sm_count() * (2048 / NT);
    cudaError_t e;
    if (inner >= 64) {
        args.vec = inner % 4 == 0 &&
                   ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0;
        // equal row counts per CTA: ceil(rows / maxg) rows each
        const int64_t rows = n * c, per = cdiv(rows, maxg);
        const int64_t g = cdiv(rows, per);
        e = launch_pdl(bn_apply_rows_kernel, dim3((unsigned)g), dim3(NT), 0, st, args);
    } else {
        const int64_t g = std::max<int64_t>(1, std::min<int64_t>(cdiv(total, NT), maxg));
        e = launch_pdl(bn_apply_flat_kernel, dim3((unsigned)g), dim3(NT), 0, st, args);
    }
    if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "bn apply: %s", cudaGetErrorString(e));
    return check_launch("BatchNorm normalisation");
}

}  // extern "C"
