// gemm_plain_core.cuh — the per-MAC emulated-accumulation core shared by the
// plain GEMM (gemm_plain.cu) and the plain implicit-GEMM conv2d (conv.cu):
// the leaf, the 128 x 128 x 16 shared-memory tile shape and the MAC loop over
// one k-tile.
#pragma once
#include <cuda_runtime.h>

#include "lof_round.cuh"

namespace lofgb {
namespace {

constexpr int BM = 128, BN = 128, BK = 16, NT = 256;
constexpr int PAD = 4;

// How the accumulator is re-rounded after every MAC: ACC_NONE (23 mantissa
// bits: the round-to-odd word itself), ACC_MANT (RNE to m mantissa bits, the
// reference leaf), ACC_UNI / ACC_FMT (RNE into a whole format — exponent
// range, subnormals, overflow — by the whole-range float rounding or by the
// integer rounding core; an extension without a reference counterpart).
enum { ACC_NONE = 0, ACC_MANT = 1, ACC_UNI = 2, ACC_FMT = 3 };

struct AccRound {
    int ro;                       // 23 - mantissa bits
    uint32_t sh, half_m1, mask;   // RNE constants for ACC_MANT (rne_word)
    RoundPlan plan;               // the accumulator format for ACC_UNI / ACC_FMT
};

// One emulated MAC: the round-to-odd word of the two directed FMAs
// (rto_word), then the accumulator rounding. Round-to-odd keeps a sticky bit
// below FP32's last place, so rounding v to the (narrower) accumulator equals
// rounding the exact a*b + acc.
template <int ACC>
__device__ __forceinline__ float emac(float a, float b, float acc, const AccRound& r) {
    const uint32_t v = rto_word(__fmaf_rd(a, b, acc), __fmaf_ru(a, b, acc));
    if (ACC == ACC_NONE) return __uint_as_float(v);
    if (ACC == ACC_UNI) return __uint_as_float(vr_uni_f32<LOFGB_RNE, 1>(v, r.plan));
    if (ACC == ACC_FMT) return __uint_as_float(vr_format<LOFGB_RNE, 32>(v, r.plan, 0ull));
    return __uint_as_float(rne_word(v, r.sh, r.half_m1, r.mask));
}

AccRound acc_mant(int mbits) {
    AccRound r = {};
    r.ro = 23 - mbits;
    r.sh = r.ro > 0 ? 1u << (32 - r.ro) : 0u;
    r.half_m1 = r.ro > 0 ? (1u << (r.ro - 1)) - 1u : 0u;
    r.mask = r.ro > 0 ? ~((1u << r.ro) - 1u) : ~0u;
    return r;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async4(uint32_t dst, const float* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src),
                 "r"(valid ? 4 : 0)
                 : "memory");
}

// One staged k-tile: k-major shared tiles As[k][m], Bs[k][n]; thread (tx, ty)
// owns rows {ty*4 .. ty*4+3, 64+ty*4 .. 64+ty*4+3} and the same columns of tx.
// One 8x8 MAC block per k (640 instructions) stays resident in the
// instruction cache; unrolling k as well overflows it.
// RI = 4: only the first four rows (the 64-row half tile of the plain GEMM).
template <int ACC, int RI = 8>
__device__ __forceinline__ void mac_ktile(const float (*As)[BM + PAD], const float (*Bs)[BN + PAD],
                                          float (&acc)[8][8], int kmax, int tx, int ty,
                                          const AccRound& r) {
#pragma unroll 1
    for (int kk = 0; kk < kmax; ++kk) {
        const float4 a0 = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
        const float4 a1 = *reinterpret_cast<const float4*>(&As[kk][64 + ty * 4]);
        const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
        const float4 b1 = *reinterpret_cast<const float4*>(&Bs[kk][64 + tx * 4]);
        const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < RI; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = emac<ACC>(av[i], bv[j], acc[i][j], r);
    }
}

}  // namespace
}  // namespace lofgb
