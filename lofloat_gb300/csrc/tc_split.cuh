// tc_split.cuh — FP32 -> BF16 hi/lo operand split for the tensor-core GEMM,
// shared by the GEMM (gemm_tc.cu) and conv2d (conv.cu) split kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace lofgb {
namespace {

// Writes a staged 32-row x 64-k FP32 tile (tile[row][k]) to the K-major BF16
// operands hi / lo (R rows x Kp columns) at rows r0.., columns k0..:
// hi = RZ_bf16(x), lo = RN_bf16(x - hi) (the difference is exact in FP32),
// lo = 0 for non-finite x. Called by all 256 threads of the CTA.
__device__ __forceinline__ void split_store_tile(const float (*tile)[65], int r0, int k0, int R,
                                                 int Kp, __nv_bfloat16* hi, __nv_bfloat16* lo) {
    for (int i = threadIdx.x; i < 32 * 32; i += 256) {
        const int rr = i / 32, kp = (i % 32) * 2;
        const int r = r0 + rr, k = k0 + kp;
        if (r >= R || k >= Kp) continue;
        __nv_bfloat162 h2, l2;
        const float x0 = tile[rr][kp], x1 = tile[rr][kp + 1];
        const __nv_bfloat16 h0 = __float2bfloat16_rz(x0), h1 = __float2bfloat16_rz(x1);
        float d0 = x0 - __bfloat162float(h0), d1 = x1 - __bfloat162float(h1);
        if (!isfinite(x0)) d0 = 0.0f;
        if (!isfinite(x1)) d1 = 0.0f;
        h2.x = h0;
        h2.y = h1;
        l2.x = __float2bfloat16_rn(d0);
        l2.y = __float2bfloat16_rn(d1);
        *reinterpret_cast<__nv_bfloat162*>(hi + (int64_t)r * Kp + k) = h2;
        *reinterpret_cast<__nv_bfloat162*>(lo + (int64_t)r * Kp + k) = l2;
    }
}

}  // namespace
}  // namespace lofgb
