// pwl_silu.cu — piecewise-linear SiLU from a knot table.
//
// Replaces pwl_silu_kernel / pwl_silu (src/Lof_kernel.cu:240-264, dispatched
// from src/LoPy_bind.cpp:228-272): one element per thread with a grid of
// ceil(n/256) CTAs on the legacy stream, one template instantiation per table
// length. Here the table length is a run-time argument, each thread moves
// 16-byte vectors in a grid-stride loop sized to the SM count, and the table
// (at most 4097 floats) is read through the read-only path, where it stays
// cache resident. The arithmetic is the reference's, in FP32, operation for
// operation:
//   xc = fminf(fmaxf(x, -R), R); u = (xc + R) * inv_step; i = min((int)u, N-1)
//   y = fmaf(u - i, lut[i+1] - lut[i], lut[i]);  |x| > R: y = x > 0 ? x : 0
// with inv_step = N / (2R) computed in FP32 on the host. HBM-bound:
// 2 * sizeof(T) algorithmic bytes per element.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lofgb_internal.h"

namespace lofgb {

namespace {

constexpr int PT = 256;

__device__ __forceinline__ float pwl(float x, const float* __restrict__ lut, int nseg, float R,
                                     float inv_step) {
    const float xc = fminf(fmaxf(x, -R), R);
    const float u = __fmul_rn(__fadd_rn(xc, R), inv_step);
    int i = __float2int_rz(u);
    if (i > nseg - 1) i = nseg - 1;
    const float frac = __fsub_rn(u, __int2float_rn(i));
    const float y0 = __ldg(lut + i), y1 = __ldg(lut + i + 1);
    float y = __fmaf_rn(frac, __fsub_rn(y1, y0), y0);
    if (fabsf(x) > R) y = x > 0.0f ? x : 0.0f;
    return y;
}

template <typename T> struct Io;
template <> struct Io<float> {
    static __device__ __forceinline__ float in(float v) { return v; }
    static __device__ __forceinline__ float out(float v) { return v; }
};
template <> struct Io<double> {
    static __device__ __forceinline__ float in(double v) { return __double2float_rn(v); }
    static __device__ __forceinline__ double out(float v) { return (double)v; }
};
template <> struct Io<__half> {
    static __device__ __forceinline__ float in(__half v) { return __half2float(v); }
    static __device__ __forceinline__ __half out(float v) { return __float2half_rn(v); }
};

// 16-byte vectors of 16 / sizeof(T) elements, then a scalar tail.
template <typename T>
__global__ void __launch_bounds__(PT)
pwl_silu_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t n,
                const float* __restrict__ lut, int nseg, float R, float inv_step, int vec) {
    pdl_wait();
    constexpr int EPV = 16 / sizeof(T);
    const int64_t stride = (int64_t)gridDim.x * PT;
    int64_t done = 0;
    if (vec) {
        const int64_t nvec = n / EPV;
        const uint4* vin = reinterpret_cast<const uint4*>(in);
        uint4* vout = reinterpret_cast<uint4*>(out);
        for (int64_t v = (int64_t)blockIdx.x * PT + threadIdx.x; v < nvec; v += stride) {
            union { uint4 u; T e[EPV]; } a, b;
            a.u = __ldcs(vin + v);
#pragma unroll
            for (int q = 0; q < EPV; ++q) b.e[q] = Io<T>::out(pwl(Io<T>::in(a.e[q]), lut, nseg, R, inv_step));
            __stcs(vout + v, b.u);
        }
        done = nvec * EPV;
    }
    for (int64_t i = done + (int64_t)blockIdx.x * PT + threadIdx.x; i < n; i += stride)
        out[i] = Io<T>::out(pwl(Io<T>::in(in[i]), lut, nseg, R, inv_step));
}

template <typename T>
int launch_pwl(const T* in, T* out, int64_t n, const float* lut, int nseg, float R, void* stream) {
    clear_error();
    if (n < 0) return set_error(LOFGB_ERR_SIZE, "negative size");
    if (nseg < 2 || nseg > 4096 || (nseg & (nseg - 1)))
        return set_error(LOFGB_ERR_SIZE, "pwl_silu: lut length %d is not a power of 2 in [2, 4096]",
                         nseg);
    if (!(R > 0.0f)) return set_error(LOFGB_ERR_SIZE, "pwl_silu: R must be positive");
    if (n == 0) return LOFGB_OK;
    if (!in || !out || !lut) return set_error(LOFGB_ERR_NULL, "NULL pointer");
    const char* a = reinterpret_cast<const char*>(in);
    const char* b = reinterpret_cast<const char*>(out);
    const int64_t bytes = n * (int64_t)sizeof(T);
    if (a != b && a < b + bytes && b < a + bytes)
        return set_error(LOFGB_ERR_ALIAS, "input and output partially overlap");
    const float inv_step = (float)nseg / (2.0f * R);
    const int vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
    const int64_t per = vec ? (int64_t)(16 / sizeof(T)) : 1;
    int64_t g = (n / per + PT - 1) / PT;
    const int64_t maxg = (int64_t)sm_count() * (2048 / PT);
    if (g < 1) g = 1;
    if (g > maxg) g = maxg;
    launch_pdl(pwl_silu_kernel<T>, (int)g, PT, 0, static_cast<cudaStream_t>(stream), in, out, n, lut,
               nseg, R, inv_step, vec);
    return check_launch("pwl_silu_kernel");
}

}  // namespace

}  // namespace lofgb

using namespace lofgb;

extern "C" {

int lofgb_pwl_silu_f32(const float* in, float* out, int64_t n, const float* lut, int segments,
                       float R, void* stream) {
    return launch_pwl<float>(in, out, n, lut, segments, R, stream);
}

int lofgb_pwl_silu_f64(const double* in, double* out, int64_t n, const float* lut, int segments,
                       float R, void* stream) {
    return launch_pwl<double>(in, out, n, lut, segments, R, stream);
}

int lofgb_pwl_silu_f16(const uint16_t* in, uint16_t* out, int64_t n, const float* lut,
                       int segments, float R, void* stream) {
    return launch_pwl<__half>(reinterpret_cast<const __half*>(in), reinterpret_cast<__half*>(out), n,
                              lut, segments, R, stream);
}

}  // extern "C"
