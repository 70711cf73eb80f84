// mx_common.cuh — the MX block scale, shared by the MX rounding kernels
// (mx_kernels.cu) and the MX storage encode (codec.cu).
//
// Per block (src/mx_round.cuh:52-65): scale = virtual_round(amax * (1/pmn),
// scale_fmt, {scale_mode, 0}); elements are then divided by the scale, taken
// as a multiply by 1/scale when the scale is a power of two in
// [2^-126, 2^127] (one rounding of the same exact value either way).
#pragma once
#include <cuda_runtime.h>

#include "lof_round.cuh"

namespace lofgb {
namespace {

constexpr uint64_t SCALE_SALT = 0x5CA1E5CA1E5CA1E5ull;

template <int MODE>
__device__ __forceinline__ bool stoch(int rmode) {
    const int m = MODE >= 0 ? MODE : rmode;
    return mode_is_stochastic(m);
}

struct BlockScale {
    float scale, inv;
    bool pos, pow2;
};

__device__ __forceinline__ BlockScale scale_from_bits(uint32_t sb) {
    BlockScale b;
    b.scale = __uint_as_float(sb);
    b.pos = b.scale > 0.0f;
    // scale = 2^(E-127) with exponent field E in [1, 253]: 1/scale = 2^(127-E)
    // is a normal float with field 254-E, built directly from the bits
    b.pow2 = (sb & 0x807FFFFFu) == 0 && (sb - 0x00800000u) <= 0x7E000000u;
    // a non-positive scale zeroes the block; keep the divide off that path
    b.pow2 = b.pow2 || !b.pos;
    b.inv = __uint_as_float(0x7F000000u - (sb & 0x7F800000u));
    return b;
}

template <int SMODE>
__device__ __forceinline__ BlockScale block_scale(float amax, const RoundPlan& ps, float inv_pmn,
                                                  uint64_t seed, uint64_t blk_elem) {
    const float sin = __fmul_rn(amax, inv_pmn);
    const uint64_t r = stoch<SMODE>(ps.mode) ? rng64(seed ^ SCALE_SALT, blk_elem) : 0ull;
    return scale_from_bits(vr_format_f32_voted<SMODE>(__float_as_uint(sin), ps, r));
}


}  // namespace
}  // namespace lofgb
