// lofgb_internal.h — types shared by the host launchers and the kernels of
// liblofgb.so. Not part of the public C ABI (include/lofgb.h).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <utility>

#include "../../include/lofgb.h"

namespace lofgb {

// Per-(source type, format, mode) constants, computed on the host by
// make_round_plan() and passed to kernels by value. Thresholds are bit
// patterns of the source type's magnitude, so that
//   (float)|x| <  tiny   <=>  mag <  tiny_thr
//   (float)|x| >  0      <=>  mag >= pos_thr
//   (float)|x| <  tiny/2 <=>  mag <  half_lt
//   (float)|x| >  tiny/2 <=>  mag >= half_gt
// reproduce the reference's float comparisons (src/lo_float.h:2871-2896).
struct RoundPlan {
    int32_t mode;          // lofgb_rounding_mode
    int32_t len;           // stoch_len
    int32_t d;             // source mantissa bits - target mantissa bits (>= 0)
    int32_t to_min_field;  // (1 - bias) + source exponent bias
    int32_t to_max_field;  // ToMax_exp + source exponent bias
    int32_t saturating;    // Inf_Behaviors::Saturating
    uint64_t tiny_thr, pos_thr, half_lt, half_gt;
    uint64_t tiny_bits;    // from_double<From>(tiny) bit pattern
    // Derived thresholds for the branch-light device path:
    //   mag <  norm_thr  <=>  exponent field < to_min_field (target-subnormal range)
    //   b   >= ovf_thr   <=>  exponent field of the rounded b > to_max_field
    //   in the tiny branch the result is +-tiny iff mag >= (sign ? tmin_neg : tmin_pos)
    uint64_t norm_thr, ovf_thr, tmin_pos, tmin_neg;
    // Fast path on the signed word: res = round(x) & keep_mask (keep_mask
    // clears the d dropped bits, keeps the sign); overflow iff the magnitude
    // of res >= ovf_thr; everything with magnitude < norm_thr or NaN takes the
    // special path.
    uint64_t keep_mask;
    float tiny_f;          // To_min_val (a float in the reference)
    // Below-normal magnitudes of f32 words by float arithmetic: with
    // C = 2^(23 + ToMin - m) (so ulp(C) = tiny), fadd(|x|, C) - C rounds |x| to
    // a multiple of tiny in the fadd's rounding direction — the reference's
    // tiny and target-subnormal branches for RNE (grid = 1, round to nearest
    // even) and RTZ/RAFZ/RU/RD (grid = 2, magnitude up iff grid_up_{pos,neg}).
    // grid = 0: integer path only.
    int32_t grid;
    float grid_c;
    int32_t grid_up_pos, grid_up_neg;
    // Whole-range float rounding of f32 words (uni = grid's 1 or 2, else 0):
    // the per-element constant C = 2^(clamp(e, to_min, hi) + d), e the
    // word's unbiased exponent, has ulp(C) equal to the target's spacing at
    // |x| in the normal range as well as below it, so fadd(|x|, C) - C is the
    // whole of virtual_round's rounding for RNE / RTZ / RAFZ / RU / RD. Valid
    // when d >= 1, tiny >= 2^-126 (no FP32-subnormal input reaches the
    // target-subnormal branch) and hi + d <= 254 with hi the FP32 exponent
    // field just above the target's largest finite value (every |x| at or
    // above 2^hi then still rounds to an overflow).
    // uni == 6: round-to-odd on the same grid (vr_uni_rto_f32).
    int32_t uni;
    uint32_t uni_lo, uni_hi, uni_d;  // FP32 exponent fields, shifted to bit 23
    uint32_t sat_and, sat_or;        // overflow result: (x & sat_and) | sat_or
    // Stochastic rounding A by float arithmetic (sr_uni): with the same C,
    // the noise R' * spacing * 2^-len (R' = R & sr_mask, spacing = ulp(C)) is
    // a multiple of ulp(|x|) when len <= d; y = fadd_rz(|x|, noise) then
    // truncated to the target's spacing at y is the reference's integer
    // SR-A — within a binade the bit-pattern sum is the value sum, and a carry
    // into the next binade truncates to 2^(e+1) either way; rounding y toward
    // zero never crosses a multiple of the spacing. Magnitudes below tiny
    // flush to +-0 (the stochastic modes' tiny branch). Valid when the uni
    // conditions hold, the float grid constant grid_c exists, and
    // len <= min(d, 24) with tiny * 2^-len a normal float.
    int32_t sr_uni;
    uint32_t sr_mask, sr_shift;      // R' mask; (d - len) << 23
    // Random words: element g of a stream reads lane g mod 2^rng_lg (from the
    // low end) of the SplitMix64 output number g >> rng_lg; lanes are
    // 64 >> rng_lg bits wide, the narrowest of 8/16/32/64 that holds every
    // bit the mode reads (rng_lanes_log2).
    int32_t rng_lg;
};

// log2 of the random lanes per 64-bit word for (mode, stoch_len): SR-A, SR-B
// and SR-C read the low len bits, SR-D len + 1 bits, Prob one bit, True SR
// 53 bits; the deterministic modes read none.
inline int rng_lanes_log2(int mode, int len) {
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

// Host side.
int validate_format(const lofgb_format* f, int src_mant_bits);
int make_round_plan(RoundPlan* p, const lofgb_format* f, int src_bits, int mode, int len);
int make_mantissa_plan(RoundPlan* p, int src_bits, int mbits, int mode, int len);
int sm_count();
int set_error(int status, const char* fmt, ...);
void clear_error();
int check_launch(const char* what);
int check_gemm_args(const void* A, int64_t lda, int ta, const void* B, int64_t ldb, int tb,
                    const void* D, int64_t ldd, int M, int N, int K);

// Tensor-core GEMM workspace (gemm_tc.cu): a status word, then the BF16 hi /
// lo splits of A (Mp x Kp) and B (Np x Kp), K-major and zero padded
// (Mp, Np multiples of 128, Kp of 64), each 1024-byte aligned.
// A strided batch of GEMMs stacks `batch` such splits (A rows b*Mp.., B rows
// b*Np..) in each operand region.
// Six words after the status word hold the exponent ranges and lo flags of
// A (words 0-2) and B (words 3-5) (tc_split.cuh ExpRange: largest field,
// 255 - smallest non-zero field, any non-zero lo part), which the split
// kernels publish and the GEMM reads to pick its fold and its MMAs per k
// step; the host clears WS_HEADER_CLEAR bytes from the status word before a
// launch.
struct WsLayout {
    size_t status, range, ahi, alo, bhi, blo, total;
    int Mp, Np, Kp, batch;
};
constexpr size_t WS_HEADER_CLEAR = 32;
WsLayout ws_layout(int M, int N, int K, int batch = 1);
// Runs the chunked tensor-core GEMM on operands already split into `ws`
// (laid out by ws_layout) whose status word the caller has cleared.
// img_L > 0 stores conv2d output: column j = img * img_L + l of row i goes to
// D[img * img_stride + i * ldd + l].
// D of batch entry b starts at D + b * sd.
// acc_fmt (optional) rounds the accumulator into a whole format instead of
// to mbits mantissa bits.
int launch_tc_presplit(uint8_t* ws, const WsLayout& w, float* D, int64_t ldd, int64_t sd, int M,
                       int N, int mbits, float alpha, int chunk, int64_t img_L,
                       int64_t img_stride, void* stream, const RoundPlan* acc_fmt = nullptr);

// Kernel launchers (one translation unit each).
int launch_round(int src_bits, bool fmt, const void* in, void* out, int64_t n,
                 const RoundPlan& p, double scale, uint64_t seed, uint64_t offset,
                 void* stream);
int launch_mx(const float* in, float* out, int64_t n, int block, const RoundPlan& pe,
              const RoundPlan& ps, float pmn, float inv_pmn, uint64_t seed, uint64_t offset,
              void* stream);
// 1 / pmn of an MX element format, pmn = 2^emax (2 - 2^-m) in FP32
// (src/mx_round.cuh:52-56): the scale is virtual_round(amax * (1 / pmn)).
float mx_inv_pmn(const lofgb_format* ef);
// MX rounding of BF16 bit patterns (widened to FP32 on load) to FP32 output.
int launch_mx_bf16(const uint16_t* in, float* out, int64_t n, int block, const RoundPlan& pe,
                   const RoundPlan& ps, float inv_pmn, uint64_t seed, uint64_t offset,
                   void* stream);
// Strided batches: GEMM z reads A + z*sa, B + z*sb and writes D + z*sd.
// acc_fmt (optional, RNE plan of an f32 source) rounds the accumulator into a
// whole format after every MAC / chunk instead of to mbits mantissa bits.
int launch_gemm_plain(const float* A, int64_t lda, int64_t sa, int ta, const float* B,
                      int64_t ldb, int64_t sb, int tb, float* D, int64_t ldd, int64_t sd, int M,
                      int N, int K, int batch, int mbits, const RoundPlan* acc_fmt, float alpha,
                      void* stream);
int launch_gemm_f64(const float* A, int64_t lda, int ta, const float* B, int64_t ldb, int tb,
                    double* D, int64_t ldd, int M, int N, int K, void* stream);
int launch_gemm_tc(const float* A, int64_t lda, int64_t sa, int ta, const float* B, int64_t ldb,
                   int64_t sb, int tb, float* D, int64_t ldd, int64_t sd, int M, int N, int K,
                   int batch, int mbits, const RoundPlan* acc_fmt, float alpha, int chunk,
                   void* workspace, size_t workspace_bytes, void* stream);
size_t gemm_tc_workspace(int M, int N, int K, int batch);

}  // namespace lofgb

namespace lofgb {

// Programmatic dependent launch for the streaming kernels: the launch may
// begin while the previous kernel in the stream is still running (its CTAs
// then wait at griddepcontrol.wait, before touching memory, until that kernel
// has completed and its writes are visible), which hides the gap between
// back-to-back launches. Kernels launched this way call pdl_wait() before
// their first global memory access; without the attribute it is a no-op.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace lofgb

#ifdef __CUDACC__
namespace lofgb {
// Wait for the preceding kernel (programmatic dependent launch), then let
// the next one begin its launch.
__device__ __forceinline__ void pdl_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
}  // namespace lofgb
#endif

namespace lofgb {

// Device-side row of the grouped rounding table (one per tensor).
struct GroupedTask {
    const float* in;
    float* out;
    int64_t n;
    int64_t item_begin;  // first work item of this task (exclusive prefix sum)
    RoundPlan plan;
    float scale;
    int32_t apply_scale;
    int32_t item_shift;  // work items of 2^item_shift elements
    uint64_t seed, offset;
};
constexpr int GROUPED_ITEM_SHIFT = 16;  // default work item: 2^16 elements

int launch_round_grouped(const void* table, int ntasks, int64_t num_items, void* stream);

}  // namespace lofgb
