// tc_split.cuh — FP32 -> BF16 hi/lo operand split for the tensor-core GEMM,
// shared by the GEMM (gemm_tc.cu) and conv2d (conv.cu) split kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

namespace lofgb {
namespace {

// Exponent range of an operand, for the tensor-core epilogue's choice of
// fold: every thread keeps the largest FP32 exponent field it has seen (255
// for inf / NaN) and 255 minus the smallest field of a non-zero value (255
// for an FP32 subnormal); range_flush publishes them with atomicMax into the
// first two of the operand's three words, which the host cleared before the
// split. The third word records whether any lo part is non-zero: when none
// is (every value exact in 8 significant bits), the GEMM neither loads the
// lo tiles nor issues their MMAs, whose products would all be zero.
struct ExpRange {
    uint32_t emax = 0, emin_c = 0, lo = 0;
    __device__ __forceinline__ void add(float x) {
        const uint32_t b = __float_as_uint(x) & 0x7FFFFFFFu;
        const uint32_t f = b >> 23;
        emax = max(emax, f);
        if (b) emin_c = max(emin_c, 255u - f);
    }
};

// CTA-wide maximum of the range words and OR of the lo flag, then one
// atomic per word from thread 0, skipped when the published value already
// covers it (most CTAs). Called by all threads of the CTA (blockDim.x a
// multiple of 32, <= 1024); range == nullptr publishes nothing.
__device__ __forceinline__ void range_flush(uint32_t* range, const ExpRange& er) {
    __shared__ uint32_t red[3][32];
    const uint32_t a = __reduce_max_sync(0xFFFFFFFFu, er.emax);
    const uint32_t b = __reduce_max_sync(0xFFFFFFFFu, er.emin_c);
    const uint32_t l = __reduce_or_sync(0xFFFFFFFFu, er.lo);
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = a;
        red[1][w] = b;
        red[2][w] = l;
    }
    __syncthreads();
    if (threadIdx.x == 0 && range) {
        uint32_t ma = 0, mb = 0, ml = 0;
        for (int i = 0; i < nw; ++i) {
            ma = max(ma, red[0][i]);
            mb = max(mb, red[1][i]);
            ml |= red[2][i];
        }
        if (ma > *reinterpret_cast<volatile uint32_t*>(range)) atomicMax(range, ma);
        if (mb > *reinterpret_cast<volatile uint32_t*>(range + 1)) atomicMax(range + 1, mb);
        if (ml && !*reinterpret_cast<volatile uint32_t*>(range + 2)) atomicOr(range + 2, 1u);
    }
    __syncthreads();
}

// Writes a staged 32-row x 64-k FP32 tile (tile[row][k]) to the K-major BF16
// operands hi / lo (R rows x Kp columns) at rows r0.., columns k0..:
// hi = RZ_bf16(x), lo = RN_bf16(x - hi) (the difference is exact in FP32),
// lo = 0 for non-finite x; er collects the exponent range of the values and
// whether a lo part is non-zero.
// Called by all 256 threads of the CTA.
__device__ __forceinline__ void split_store_tile(const float (*tile)[65], int r0, int k0, int R,
                                                 int Kp, __nv_bfloat16* hi, __nv_bfloat16* lo,
                                                 ExpRange& er) {
    for (int i = threadIdx.x; i < 32 * 32; i += 256) {
        const int rr = i / 32, kp = (i % 32) * 2;
        const int r = r0 + rr, k = k0 + kp;
        if (r >= R || k >= Kp) continue;
        __nv_bfloat162 h2, l2;
        const float x0 = tile[rr][kp], x1 = tile[rr][kp + 1];
        er.add(x0);
        er.add(x1);
        const __nv_bfloat16 h0 = __float2bfloat16_rz(x0), h1 = __float2bfloat16_rz(x1);
        float d0 = x0 - __bfloat162float(h0), d1 = x1 - __bfloat162float(h1);
        if (!isfinite(x0)) d0 = 0.0f;
        if (!isfinite(x1)) d1 = 0.0f;
        h2.x = h0;
        h2.y = h1;
        l2.x = __float2bfloat16_rn(d0);
        l2.y = __float2bfloat16_rn(d1);
        uint32_t lbits;
        memcpy(&lbits, &l2, 4);
        er.lo |= (lbits & 0x7FFF7FFFu) != 0u;
        *reinterpret_cast<__nv_bfloat162*>(hi + (int64_t)r * Kp + k) = h2;
        *reinterpret_cast<__nv_bfloat162*>(lo + (int64_t)r * Kp + k) = l2;
    }
}

}  // namespace
}  // namespace lofgb
