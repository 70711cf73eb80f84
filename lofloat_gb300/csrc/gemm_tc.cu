// gemm_tc.cu — tensor-core (tcgen05 / TMEM / TMA) chunked emulated-accumulation
// GEMM for sm_103a.
//
// The reference re-rounds its FP32 accumulator after every multiply-add on
// the CUDA cores (src/cutlass_gemms.cuh:139-166). This form keeps the same
// emulated accumulator but feeds it per k-chunk: the tensor cores sum each
// chunk of `chunk` products in FP32 in TMEM, and the epilogue folds the chunk
// sum into the accumulator with one round-to-odd add and an RNE rounding to
// `accum_mant_bits`:
//     acc = RNE_m(rto(acc + chunk_sum)),   D = alpha * acc.
// It is not bit-exact to the per-MAC form; its error is stated against the
// FP64 oracle GEMM.
//
// Operands: FP32 values are split into BF16 pairs hi = RZ_bf16(x),
// lo = RN_bf16(x - hi) (x - hi is exact in FP32), stored K-major and zero
// padded by a split kernel. Each k-step of 16 issues three MMAs
// (hi·hi, hi·lo, lo·hi); the dropped lo·lo term is below 2^-16 relative.
// Values that are exact in 8 significant bits (E4M3/E5M2/E2M1 times a
// power-of-two scale) have lo = 0 and enter exactly; the split kernels flag
// an operand whose lo parts are all zero, and its lo tiles are then neither
// loaded nor multiplied (MX operands: one MMA per k-step, half the bytes).
//
// Kernel layout (one CTA per SM, persistent over 128 x BN output tiles,
// BN = 128 here; the 64- and 256-column shapes are described at TileShape):
//   warp 0      TMA producer: up to 4 tiles (A hi/lo, B hi/lo) of 64 k per
//               stage, 3 to 6 stages in 192 KiB (more when lo tiles are
//               left out), 128-byte swizzle, one mbarrier per stage;
//   warp 1      TMEM owner and MMA issuer (one lane):
//               tcgen05.mma.cta_group::1.kind::f16, M=128 N=128 K=16,
//               chunk sums in four 128-column TMEM buffers (all 512
//               columns), so the MMAs run up to three chunks ahead;
//   warps 2..17 epilogue (four per TMEM lane quarter): tcgen05.ld the chunk
//               sum of its lane quarter and one 32-column slice, in two
//               16-column loads pipelined with the folds (one piece loads
//               while the previous one is folded), fold it into 32 register
//               accumulators, release the TMEM buffer; store D at tile end.
// The fold runs on the FMA pipe in packed pairs (fold2_fast) whenever the
// operands' exponent ranges, published by the split kernels, rule out
// subnormal and overflowing partial sums; otherwise with integer rounding.
// Every wait is bounded (~2 s of %globaltimer): on expiry the CTA records
// LOFGB_ERR_TIMEOUT in the workspace status word, drains its own in-flight
// copies and MMAs (again bounded), frees its TMEM and exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "lof_round.cuh"
#include "lofgb_internal.h"
#include "tc_split.cuh"

namespace lofgb {

namespace {

constexpr int TBM = 128;          // output tile rows (UMMA M)
constexpr int TBN = 128;          // widest output tile (UMMA N); operands are padded to it
constexpr int SK = 64;            // k per pipeline stage (one 128-byte swizzle row of bf16)
constexpr int TILE_A = TBM * SK * 2;           // 16 KiB per A operand tile
constexpr int PIPE_BYTES = 192 * 1024;         // shared memory of the stage ring

// Tile shapes of the persistent kernel: 128 x BN outputs per tile.
//   BN = 128: stages of 64 KiB (A hi, A lo, B hi, B lo), 3 stages (6 of
//             32 KiB without lo tiles); four 128-column TMEM chunk buffers;
//             16 epilogue warps of 32 columns;
//   BN = 64:  stages of 48 KiB, 4 stages (8 without lo tiles); eight
//             64-column chunk buffers; 8 epilogue warps of 32 columns (the
//             grouped kernel's narrow tile, more tiles for load balance
//             across uneven GEMMs);
//   BN = 256: stages of 96 KiB, 2 stages (4 without lo tiles); two
//             256-column chunk buffers; 16 epilogue warps of 64 columns in
//             8-column pieces (one MMA covers 256 columns).
template <int BN>
struct TileShape {
    static constexpr int TILE_B = BN * SK * 2;
    static constexpr int STAGE_BYTES = 2 * TILE_A + 2 * TILE_B;
    static constexpr int STAGES = PIPE_BYTES / STAGE_BYTES;
    static constexpr int MAXST = PIPE_BYTES / (TILE_A + TILE_B);   // stages of hi tiles only
    static constexpr int EPI_WARPS = BN == 64 ? 8 : 16;    // EPI_WARPS / 4 per TMEM lane quarter
    static constexpr int EPI_COLS = BN * 4 / EPI_WARPS;    // accumulator columns per epilogue thread
    static constexpr int NBUF = 512 / BN;                  // TMEM chunk buffers (all 512 columns)
    // Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
    // (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
    static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) |
                                      ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);
    static_assert(EPI_COLS == 64 || EPI_COLS == 32, "the epilogue folds 16-column pieces, 4 or 2 per chunk");
    static_assert((NBUF & (NBUF - 1)) == 0 && NBUF * BN == 512, "TMEM chunk buffers");
    static_assert(STAGES * STAGE_BYTES <= PIPE_BYTES && STAGES >= 2, "stage ring");
    static_assert(2 * MAXST + 2 * NBUF + 1 <= 56, "barrier area");
};
constexpr int NUM_THREADS = 32 * (2 + 16);     // launch size of every shape (idle warps exit)
constexpr size_t SMEM_BYTES = 1024 /*align slack*/ + PIPE_BYTES + 512 /*barriers, flags*/;
constexpr unsigned long long WAIT_LIMIT_NS = 2000000000ull;

// Limit of every bounded wait, and for the wait self-test the pipeline stage
// whose copies the producer withholds (-1: none), so that the MMA warp's
// wait for it runs out and the CTA takes its abort path.
struct WaitCfg {
    unsigned long long limit_ns = WAIT_LIMIT_NS;
    int withhold = -1;
};

struct TcParams {
    float* D;
    int64_t ldd;
    int M, N, Kp;          // Kp: padded K (multiple of SK)
    int tiles_m, tiles_n;
    int tile_n;            // output columns per tile (128 or 256)
    int chunk16;           // chunk length in 16-k steps
    int ro;                // 23 - accum_mant_bits
    float alpha;
    int* status;           // workspace status word
    int64_t img_L;         // conv output: columns per image (0: plain row-major D)
    int64_t img_stride;    // conv output: elements per image
    int batch;             // strided batch: GEMM b reads split rows b*Mp.. / b*Np..
    int Mp, Np;            // padded rows of one GEMM's A / B split
    int64_t stride_d;      // elements between consecutive D matrices
    int acc_kind;          // 0: RNE to ro mantissa bits; 2 / 3: the format acc_plan
                           // (whole-range float rounding / integer rounding core)
    RoundPlan acc_plan;
    uint32_t* range;       // exponent ranges of A and B (workspace words)
    int fast_lim;          // fast fold iff emax_a + emax_b <= fast_lim (FAST_OFF: never)
    WaitCfg wait;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(100000u)
        : "memory");
    return ok != 0;
}

// Bounded wait: false if the CTA is aborting or the wait ran out of time
// (then the abort flag is raised and the status word set).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          int* status, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (globaltimer() - t0 > limit_ns) {
            *abort_flag = 1;
            atomicExch(status, (int)LOFGB_ERR_TIMEOUT);
            return false;
        }
    }
}

// Wait used while draining after an abort: bounded, result ignored.
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
    const unsigned long long t0 = globaltimer();
    while (!mbar_try_wait(bar, parity))
        if (globaltimer() - t0 > limit_ns) return;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

// tcgen05 shared-memory matrix descriptor: K-major operand, 128-byte swizzle,
// 8-row x 128-byte atoms stacked every 1024 bytes (SBO), LBO unused (1),
// descriptor version 1 (bits 46-47), layout type 2 = SWIZZLE_128B (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

template <uint32_t IDESC>
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(IDESC), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 consecutive TMEM columns of this warp's lane quarter, one per register.
// The registers are valid only after tmem_ld_wait16 on them.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

// Wait for the outstanding TMEM loads; the registers of r are operands, so
// no read of r is scheduled before the wait.
__device__ __forceinline__ void tmem_ld_wait16(uint32_t (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                   "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                   "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
}

// 8-column forms of the two above, for the 64-column epilogue slices of the
// 128 x 256 tile (64 accumulators plus two 8-register pieces per thread).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait8(uint32_t (&r)[8]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                   "+r"(r[6]), "+r"(r[7])
                 :
                 : "memory");
}
template <int OFF, int N>
__device__ __forceinline__ void pin8(float (&a)[N]) {
    static_assert(OFF + 8 <= N, "pin8 range");
    asm volatile(""
                 : "+f"(a[OFF + 0]), "+f"(a[OFF + 1]), "+f"(a[OFF + 2]), "+f"(a[OFF + 3]),
                   "+f"(a[OFF + 4]), "+f"(a[OFF + 5]), "+f"(a[OFF + 6]), "+f"(a[OFF + 7]));
}

// Scheduling pin for the pipelined epilogue: an empty asm that takes 16
// accumulators as in/out operands. Placed after a TMEM load it keeps the fold
// of those accumulators after the load is issued; placed before a TMEM wait it
// keeps their fold ahead of the wait. Emits no instruction.
template <int OFF, int N>
__device__ __forceinline__ void pin16(float (&a)[N]) {
    static_assert(OFF + 16 <= N, "pin16 range");
    asm volatile(""
                 : "+f"(a[OFF + 0]), "+f"(a[OFF + 1]), "+f"(a[OFF + 2]), "+f"(a[OFF + 3]),
                   "+f"(a[OFF + 4]), "+f"(a[OFF + 5]), "+f"(a[OFF + 6]), "+f"(a[OFF + 7]),
                   "+f"(a[OFF + 8]), "+f"(a[OFF + 9]), "+f"(a[OFF + 10]), "+f"(a[OFF + 11]),
                   "+f"(a[OFF + 12]), "+f"(a[OFF + 13]), "+f"(a[OFF + 14]), "+f"(a[OFF + 15]));
}

// acc = RNE_m(rto(acc + s)) with directed adds, as the per-MAC leaf does with
// directed FMAs (src/cutlass_gemms.cuh:73-88, 162-163); rto_word / rne_word
// are that leaf's round-to-odd and RNE steps.
__device__ __forceinline__ float fold(float acc, float s, int ro, uint32_t sh, uint32_t two,
                                      uint32_t half_m1, uint32_t mask) {
    const uint32_t v = rto_word(__fadd_rd(acc, s), __fadd_ru(acc, s));
    if (ro <= 0) return __uint_as_float(v);
    return __uint_as_float(rne_word2(v, sh, two, half_m1, mask));
}

// acc = RNE_format(rto(acc + s)) for a whole-format accumulator: the
// round-to-odd word keeps a sticky bit, so the format rounding of it equals
// the format rounding of the exact sum.
template <int KIND>
__device__ __forceinline__ float fold_fmt(float acc, float s, const RoundPlan& p) {
    const uint32_t v = rto_word(__fadd_rd(acc, s), __fadd_ru(acc, s));
    if (KIND == 2) return __uint_as_float(vr_uni_f32<LOFGB_RNE, 1>(v, p));
    return __uint_as_float(vr_format<LOFGB_RNE, 32>(v, p, 0ull));
}

// The fold acc = RNE_m(rto(acc + s)) for two accumulators at a time, with
// the arithmetic in packed FP32 pairs on the FMA pipe: rto is rto_word's
// select, and RNE to m = 23 - ro mantissa bits is Veltkamp's split
// hi = t - (t - v), t = v * (2^ro + 1), which for 1 <= ro <= 22 equals the
// integer RNE of rne_word2 for every zero or normal v with |v| * (2^ro + 1)
// finite (checked exhaustively over all FP32 patterns for every ro). The two
// subtractions are fused multiply-adds by -1 (exact products), which keeps
// signed zeros. The epilogue takes this fold only when the operands'
// exponent ranges guarantee those conditions for every partial sum
// (fast_fold_ok).
__device__ __forceinline__ void fold2_fast(float& a0, float& a1, float s0, float s1, float sigma) {
    const float2 a = make_float2(a0, a1), s = make_float2(s0, s1);
    const float2 rd = __fadd2_rd(a, s), ru = __fadd2_ru(a, s);
    const float2 v = make_float2(__uint_as_float(rto_word(rd.x, ru.x)),
                                 __uint_as_float(rto_word(rd.y, ru.y)));
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 t = __fmul2_rn(v, make_float2(sigma, sigma));
    const float2 h = __ffma2_rn(__ffma2_rn(v, m1, t), m1, t);   // t - (t - v)
    a0 = h.x;
    a1 = h.y;
}

constexpr int FAST_OFF = -100000;

// Largest exponent-field sum (emax_a + emax_b) for which every partial sum v
// of a K-long product keeps |v| * (2^ro + 1) finite: with |a| < 2^(emax_a -
// 126) and |b| alike, |v| <= Kp * 2^(ea + eb) * G, G the growth of nchunks
// roundings by at most (1 + 2^-(m+1)) (1 + 2^-23) each; two more bits of
// margin cover the tensor cores' chunk sums and the dropped lo * lo term.
int fast_fold_limit(int Kp, int chunk, int mbits) {
    const int ro = 23 - mbits;
    if (ro < 1 || ro > 22) return FAST_OFF;
    const int nchunks = (Kp + chunk - 1) / chunk;
    const double g = nchunks * std::log2((1.0 + std::ldexp(1.0, -(mbits + 1))) * (1.0 + 0x1p-23));
    const int L = (int)std::ceil(std::log2((double)Kp)) + (int)std::ceil(g) + 2;
    return 378 - ro - L;
}

// The fast fold is exact for the whole tile iff no partial sum can overflow
// it (the limit above) and none can be an FP32 subnormal: every operand part
// is a multiple of 2^(emin - 150), so every partial sum is a multiple of
// 2^(emin_a + emin_b - 300), which must be at least 2^-126.
__device__ __forceinline__ bool fast_fold_ok(const uint32_t (&r)[4], int lim) {
    const int emax = (int)r[0] + (int)r[2];
    const int emin = (255 - (int)r[1]) + (255 - (int)r[3]);
    return lim != FAST_OFF && emax <= lim && emin >= 174;
}

// ---- tile sources ------------------------------------------------------------
// Everything the three roles need to know about one 128 x 128 output tile.
struct TileInfo {
    const CUtensorMap* map[4];  // A hi, A lo, B hi, B lo
    float* D;
    int64_t ldd;
    int M, N, m0, n0, Kp, chunk16, ro;
    int a_r0, b_r0;             // first split rows of the A / B tiles (TMA coordinates)
    float alpha;
    // conv2d output (img_L > 0): column j = img * img_L + l of row i is
    // stored at D[img * img_stride + i * ldd + l]
    int64_t img_L, img_stride;
    int fast_lim;               // fast_fold_limit of this GEMM
};

// One GEMM; its tensor maps are kernel parameters.
struct SingleSrc {
    const CUtensorMap* m[4];
    TcParams prm;
    __device__ __forceinline__ int count() const { return prm.batch * prm.tiles_m * prm.tiles_n; }
    __device__ __forceinline__ TileInfo get(int t) const {
        TileInfo ti;
#pragma unroll
        for (int i = 0; i < 4; ++i) ti.map[i] = m[i];
        const int per = prm.tiles_m * prm.tiles_n;
        const int b = t / per, r = t - b * per;
        ti.D = prm.D + (int64_t)b * prm.stride_d;
        ti.ldd = prm.ldd;
        ti.M = prm.M;
        ti.N = prm.N;
        ti.m0 = (r / prm.tiles_n) * TBM;
        ti.n0 = (r % prm.tiles_n) * prm.tile_n;
        ti.a_r0 = b * prm.Mp + ti.m0;
        ti.b_r0 = b * prm.Np + ti.n0;
        ti.Kp = prm.Kp;
        ti.chunk16 = prm.chunk16;
        ti.ro = prm.ro;
        ti.alpha = prm.alpha;
        ti.img_L = prm.img_L;
        ti.img_stride = prm.img_stride;
        ti.fast_lim = prm.fast_lim;
        return ti;
    }
};

// Many GEMMs: a device table of per-task rows (tensor maps in global memory,
// 64-byte aligned) and a tile list whose order is the schedule.
struct GroupRow {
    CUtensorMap map[4];
    float* D;
    int64_t ldd;
    int32_t M, N, Kp, chunk16, ro;
    float alpha;
    int32_t fast_lim;
    int32_t pad[7];
};
struct TileRef {
    int32_t task, m0, n0, pad;
};
struct SplitRow {
    const float* src;
    int64_t ld;
    __nv_bfloat16* hi;
    __nv_bfloat16* lo;
    int64_t item_begin;  // first 32 x 64 split item of this operand
    int32_t kmajor, rows, K, R, Kp, operand;  // operand: 0 = A, 1 = B
};
struct GroupHeader {   // at the start of the device table; offsets from its base
    int32_t ntasks, ntiles, nsplit, tile_n;   // tile_n: 64, 128 or 256 output columns per tile
    int64_t split_items;
    int64_t rows_off, tiles_off, splits_off;
    int* status;
    // exponent ranges and lo flags of all A and all B operands (zero in the
    // prepared table; the split kernel raises them, the GEMM kernel reads
    // them and its last CTA clears them, and the reader count, for the next
    // launch)
    uint32_t range[6];
    uint32_t range_readers;
    uint32_t pad2[1];
};

struct GroupedSrc {
    const GroupHeader* h;
    __device__ __forceinline__ int count() const { return h->ntiles; }
    __device__ __forceinline__ TileInfo get(int t) const {
        const uint8_t* base = reinterpret_cast<const uint8_t*>(h);
        const TileRef r = reinterpret_cast<const TileRef*>(base + h->tiles_off)[t];
        const GroupRow* g = reinterpret_cast<const GroupRow*>(base + h->rows_off) + r.task;
        TileInfo ti;
#pragma unroll
        for (int i = 0; i < 4; ++i) ti.map[i] = &g->map[i];
        ti.D = g->D;
        ti.ldd = g->ldd;
        ti.M = g->M;
        ti.N = g->N;
        ti.m0 = r.m0;
        ti.n0 = r.n0;
        ti.a_r0 = r.m0;
        ti.b_r0 = r.n0;
        ti.Kp = g->Kp;
        ti.chunk16 = g->chunk16;
        ti.ro = g->ro;
        ti.alpha = g->alpha;
        ti.img_L = 0;
        ti.img_stride = 0;
        ti.fast_lim = g->fast_lim;
        return ti;
    }
};

// ---- the persistent tensor-core body (shared by both launches) ---------------
// ACCK: 0 RNE to ro mantissa bits; 2 / 3 a whole-format accumulator (acc_plan)
// by the whole-range float rounding / by the integer rounding core.
// range: the six words the split kernels published (A's largest field,
// 255 - its smallest non-zero field, whether a lo part is non-zero; the
// same for B); reset_range: the last CTA to read them clears them (and
// range[6], the reader count) for the next launch of the same device table.
// An operand whose lo parts are all zero has its lo tiles neither loaded nor
// multiplied: one, two or three MMAs per k step of 16.
template <int ACCK, int BN, class Src>
__device__ __forceinline__ void tc_body(const Src& src, int* status, uint8_t* smem_raw,
                                       uint32_t* range, bool reset_range, const WaitCfg wcfg,
                                       const RoundPlan* acc_plan = nullptr) {
    using Shape = TileShape<BN>;
    constexpr int TBN = BN, MAXST = Shape::MAXST;
    constexpr int TILE_B = Shape::TILE_B, EPI_WARPS = Shape::EPI_WARPS, EPI_COLS = Shape::EPI_COLS;
    constexpr int NBUF = Shape::NBUF, TMEM_COLS = NBUF * TBN;
    constexpr uint32_t IDESC = Shape::IDESC;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    uint8_t* tiles = smem;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + PIPE_BYTES);
    // bars: full[MAXST], empty[MAXST], tfull[NBUF], tempty[NBUF], drain
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * MAXST + 2 * NBUF + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    uint32_t* range_s = tmem_slot + 2;  // six words

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t bar_full = smem_u32(bars);
    const uint32_t bar_empty = smem_u32(bars + MAXST);
    const uint32_t bar_tfull = smem_u32(bars + 2 * MAXST);
    const uint32_t bar_tempty = smem_u32(bars + 2 * MAXST + NBUF);
    const uint32_t bar_drain = smem_u32(bars + 2 * MAXST + 2 * NBUF);

    if (threadIdx.x == 0) {
        for (int s = 0; s < MAXST; ++s) {
            mbar_init(bar_full + 8 * s, 1);
            mbar_init(bar_empty + 8 * s, 1);
        }
        for (int b = 0; b < NBUF; ++b) {
            mbar_init(bar_tfull + 8 * b, 1);
            mbar_init(bar_tempty + 8 * b, EPI_WARPS * 32);
        }
        mbar_init(bar_drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int i = 0; i < 6; ++i)
            range_s[i] = range ? *reinterpret_cast<volatile uint32_t*>(range + i) : 255u;
        if (range && reset_range) {
            __threadfence();
            if (atomicAdd(range + 6, 1u) == gridDim.x - 1) {
                for (int i = 0; i < 7; ++i) range[i] = 0;
            }
        }
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"((uint32_t)TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    const int num_tiles = src.count();
    // Stage layout [A hi][A lo][B hi][B lo], the lo tiles only for operands
    // that have non-zero lo parts; as many stages as the ring holds.
    const bool use_alo = range_s[2] != 0u, use_blo = range_s[5] != 0u;
    const uint32_t o_bhi = TILE_A * (use_alo ? 2 : 1), o_blo = o_bhi + TILE_B;
    const uint32_t stage_bytes = o_bhi + TILE_B * (use_blo ? 2 : 1);
    const uint32_t nst = min((uint32_t)MAXST, (uint32_t)PIPE_BYTES / stage_bytes);

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t it = 0, s = 0, ph = 0;   // stages issued; stage and its phase
            bool ok = true;
            for (int tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x) {
                const TileInfo ti = src.get(tile);
                const int ksteps = ti.Kp / SK;
                for (int ks = 0; ks < ksteps; ++ks, ++it) {
                    if (!mbar_wait(bar_empty + 8 * s, ph ^ 1u, abort_flag, status, wcfg.limit_ns)) { ok = false; break; }
                    if ((int)it != wcfg.withhold) {   // wait self-test: the withheld stage never fills
                        const uint32_t base = smem_u32(tiles + s * stage_bytes);
                        const uint32_t fb = bar_full + 8 * s;
                        mbar_arrive_expect_tx(fb, stage_bytes);
                        tma_load_2d(base, ti.map[0], ks * SK, ti.a_r0, fb);
                        if (use_alo) tma_load_2d(base + TILE_A, ti.map[1], ks * SK, ti.a_r0, fb);
                        tma_load_2d(base + o_bhi, ti.map[2], ks * SK, ti.b_r0, fb);
                        if (use_blo) tma_load_2d(base + o_blo, ti.map[3], ks * SK, ti.b_r0, fb);
                    }
                    if (++s == nst) { s = 0; ph ^= 1u; }
                }
            }
            if (!ok) {
                // drain: every issued stage completes (or the drain wait expires)
                for (uint32_t j = (it >= nst ? it - nst : 0); j < it; ++j)
                    mbar_drain(bar_full + 8 * (j % nst), (j / nst) & 1u, wcfg.limit_ns);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        // Lean issue loop (one thread): stage, phase, chunk position and
        // TMEM buffer kept as counters (no divisions), descriptors as a
        // per-stage base plus constant offsets (the start-address field,
        // bits 0-13, is the byte address >> 4 and never carries: shared
        // memory is below 256 KiB).
        if (lane == 0) {
            const uint64_t dbase = smem_desc_sw128(smem_u32(tiles));
            constexpr uint64_t ALO = TILE_A >> 4;
            const uint64_t BHI = o_bhi >> 4, BLO = o_blo >> 4, SSTEP = stage_bytes >> 4;
            uint32_t s = 0, sph = 0;         // stage and its phase
            uint32_t buf = 0, bph = 0;       // TMEM chunk buffer and its phase
            bool ok = true;
            for (int tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x) {
                const TileInfo ti = src.get(tile);
                const int ksteps = ti.Kp / SK;
                const int chunk16 = ti.chunk16;
                int pos = 0;                 // k16 step within the chunk
                for (int ks = 0; ks < ksteps && ok; ++ks) {
                    if (!mbar_wait(bar_full + 8 * s, sph, abort_flag, status, wcfg.limit_ns)) { ok = false; break; }
                    tc_fence_after();
                    const uint64_t sd = dbase + s * SSTEP;
                    const bool last_stage = ks == ksteps - 1;
#pragma unroll
                    for (int j = 0; j < SK / 16; ++j) {
                        if (pos == 0) {
                            if (!mbar_wait(bar_tempty + 8 * buf, bph ^ 1u, abort_flag, status, wcfg.limit_ns)) { ok = false; break; }
                            tc_fence_after();
                        }
                        const uint32_t d = tmem_base + buf * TBN;
                        const uint64_t ahi = sd + 2 * j, alo = sd + ALO + 2 * j;
                        const uint64_t bhi = sd + BHI + 2 * j, blo = sd + BLO + 2 * j;
                        umma_f16<IDESC>(d, ahi, bhi, pos > 0 ? 1u : 0u);
                        if (use_blo) umma_f16<IDESC>(d, ahi, blo, 1u);
                        if (use_alo) umma_f16<IDESC>(d, alo, bhi, 1u);
                        if (++pos == chunk16 || (last_stage && j == SK / 16 - 1)) {
                            umma_commit(bar_tfull + 8 * buf);
                            pos = 0;
                            if (++buf == NBUF) { buf = 0; bph ^= 1u; }
                        }
                    }
                    if (!ok) break;
                    umma_commit(bar_empty + 8 * s);  // stage's smem free once its MMAs finish
                    if (++s == nst) { s = 0; sph ^= 1u; }
                }
            }
            // all issued MMAs complete before the TMEM is released
            umma_commit(bar_drain);
            mbar_drain(bar_drain, 0, wcfg.limit_ns);
        }
    } else if (warp < 2 + EPI_WARPS) {
        // ---------------- epilogue ----------------
        const int ew = warp - 2;              // 0 .. EPI_WARPS-1
        const int quarter = warp & 3;         // TMEM lane quarter this warp may access
        const int slice = ew >> 2;            // column slice of EPI_COLS columns
        const uint32_t lane_base = tmem_base + ((uint32_t)(quarter * 32) << 16) + slice * EPI_COLS;
        uint32_t cg = 0;
        bool ok = true;
        const uint32_t rng[4] = {range_s[0], range_s[1], range_s[3], range_s[4]};
        // every lane waits; the warp goes on only when all lanes saw the phase
        // complete, reconverged for the .sync.aligned TMEM loads
        auto wait_full = [&](uint32_t g) -> bool {
            const bool got = mbar_wait(bar_tfull + 8 * (g % NBUF), (g / NBUF) & 1u, abort_flag, status,
                                       wcfg.limit_ns);
            if (!__all_sync(0xFFFFFFFFu, got)) return false;
            __syncwarp();
            tc_fence_after();
            return true;
        };
        for (int tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x) {
            const TileInfo ti = src.get(tile);
            const int nchunks = (ti.Kp / 16 + ti.chunk16 - 1) / ti.chunk16;
            const int ro = ti.ro;
            const uint32_t sh = ro > 0 ? 1u << (31 - ro) : 0u;   // rne_word2 constants
            uint32_t two;
            asm volatile("mov.u32 %0, 2;" : "=r"(two));
            const uint32_t half_m1 = ro > 0 ? (1u << (ro - 1)) - 1u : 0u;
            const uint32_t mask = ro > 0 ? ~((1u << ro) - 1u) : ~0u;
            const bool fast = ACCK == 0 && fast_fold_ok(rng, ti.fast_lim);
            const float sigma = (float)((1u << (ro & 31)) + 1u);
            float acc[EPI_COLS];
#pragma unroll
            for (int i = 0; i < EPI_COLS; ++i) acc[i] = 0.0f;
            auto fold16 = [&](int off, const uint32_t (&r)[16]) {
                if constexpr (ACCK == 0) {
                    if (fast) {
#pragma unroll
                        for (int i = 0; i < 16; i += 2)
                            fold2_fast(acc[off + i], acc[off + i + 1], __uint_as_float(r[i]),
                                       __uint_as_float(r[i + 1]), sigma);
                    } else {
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            acc[off + i] = fold(acc[off + i], __uint_as_float(r[i]), ro, sh, two, half_m1, mask);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        acc[off + i] = fold_fmt<ACCK>(acc[off + i], __uint_as_float(r[i]), *acc_plan);
                }
            };
            auto fold8 = [&](int off, const uint32_t (&r)[8]) {
                if constexpr (ACCK == 0) {
                    if (fast) {
#pragma unroll
                        for (int i = 0; i < 8; i += 2)
                            fold2_fast(acc[off + i], acc[off + i + 1], __uint_as_float(r[i]),
                                       __uint_as_float(r[i + 1]), sigma);
                    } else {
#pragma unroll
                        for (int i = 0; i < 8; ++i)
                            acc[off + i] = fold(acc[off + i], __uint_as_float(r[i]), ro, sh, two, half_m1, mask);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                        acc[off + i] = fold_fmt<ACCK>(acc[off + i], __uint_as_float(r[i]), *acc_plan);
                }
            };
            if constexpr (EPI_COLS == 64) {
                // 64-column slices: eight pieces of 8 columns per chunk over
                // two 8-register sets, each piece loading while the previous
                // one is folded, piece 0 of chunk c+1 during piece 7 of chunk c
                uint32_t qa[8], qb[8];
                if (!wait_full(cg)) { ok = false; break; }
                tmem_ld8(lane_base + (cg % NBUF) * TBN, qa);
                tmem_ld_wait8(qa);
                for (int c = 0; c < nchunks; ++c) {
                    const uint32_t col = lane_base + (cg % NBUF) * TBN;
#define LOFGB_EPI8(LD, DST, OFF, SRC)  \
    tmem_ld8(col + (LD), DST);         \
    pin8<OFF>(acc);                    \
    fold8(OFF, SRC);                   \
    pin8<OFF>(acc);                    \
    tmem_ld_wait8(DST);
                    LOFGB_EPI8(8, qb, 0, qa)
                    LOFGB_EPI8(16, qa, 8, qb)
                    LOFGB_EPI8(24, qb, 16, qa)
                    LOFGB_EPI8(32, qa, 24, qb)
                    LOFGB_EPI8(40, qb, 32, qa)
                    LOFGB_EPI8(48, qa, 40, qb)
                    LOFGB_EPI8(56, qb, 48, qa)
#undef LOFGB_EPI8
                    tc_fence_before();
                    mbar_arrive(bar_tempty + 8 * (cg % NBUF));   // all of chunk c is in registers
                    ++cg;
                    const bool more = c + 1 < nchunks;
                    if (more) {
                        if (!wait_full(cg)) { ok = false; break; }
                        tmem_ld8(lane_base + (cg % NBUF) * TBN, qa);
                    }
                    pin8<56>(acc);
                    fold8(56, qb);
                    pin8<56>(acc);
                    if (more) tmem_ld_wait8(qa);
                }
            } else {
            // EPI_COLS / 16 = 2 pieces of 16 columns per chunk, software-
            // pipelined over two register sets: each piece loads while the
            // previous one is folded, and piece 0 of chunk c+1 loads during
            // the last piece of chunk c.
            static_assert(EPI_COLS == 32, "32- or 64-column epilogue slices");
            uint32_t ra[16], rb[16];
            if (!wait_full(cg)) { ok = false; break; }
            tmem_ld16(lane_base + (cg % NBUF) * TBN, ra);
            tmem_ld_wait16(ra);
            for (int c = 0; c < nchunks; ++c) {
                const uint32_t col = lane_base + (cg % NBUF) * TBN;
                tmem_ld16(col + 16, rb);
                pin16<0>(acc);
                fold16(0, ra);
                pin16<0>(acc);
                tmem_ld_wait16(rb);
                tc_fence_before();
                mbar_arrive(bar_tempty + 8 * (cg % NBUF));   // all of chunk c is in registers
                ++cg;
                const bool more = c + 1 < nchunks;
                if (more) {
                    if (!wait_full(cg)) { ok = false; break; }
                    tmem_ld16(lane_base + (cg % NBUF) * TBN, ra);
                }
                pin16<16>(acc);
                fold16(16, rb);
                pin16<16>(acc);
                if (more) tmem_ld_wait16(ra);
            }
            }
            if (!ok) break;
            const int row = ti.m0 + quarter * 32 + lane;
            const int64_t col0 = ti.n0 + slice * EPI_COLS;
            const int ncol = min(EPI_COLS, ti.N - (int)col0);
            if (row < ti.M && ti.img_L > 0) {
                // conv2d output: walk (image, column-in-image) along the columns
                int64_t img = col0 / ti.img_L;
                int64_t l = col0 - img * ti.img_L;
#pragma unroll
                for (int i = 0; i < EPI_COLS; ++i) {
                    if (i < ncol) ti.D[img * ti.img_stride + (int64_t)row * ti.ldd + l] = __fmul_rn(ti.alpha, acc[i]);
                    if (++l == ti.img_L) { l = 0; ++img; }
                }
            } else if (row < ti.M) {
                float* drow = ti.D + (int64_t)row * ti.ldd + col0;
                if (ncol == EPI_COLS && ((reinterpret_cast<uintptr_t>(drow) & 15) == 0)) {
#pragma unroll
                    for (int i = 0; i < EPI_COLS; i += 4) {
                        float4 v = make_float4(__fmul_rn(ti.alpha, acc[i]), __fmul_rn(ti.alpha, acc[i + 1]),
                                               __fmul_rn(ti.alpha, acc[i + 2]), __fmul_rn(ti.alpha, acc[i + 3]));
                        *reinterpret_cast<float4*>(drow + i) = v;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < EPI_COLS; ++i)
                        if (i < ncol) drow[i] = __fmul_rn(ti.alpha, acc[i]);
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                     "r"((uint32_t)TMEM_COLS)
                     : "memory");
    }
}

template <int ACCK, int BN>
__global__ void __launch_bounds__(NUM_THREADS, 1)
gemm_tc_kernel(const __grid_constant__ CUtensorMap tm_ahi, const __grid_constant__ CUtensorMap tm_alo,
               const __grid_constant__ CUtensorMap tm_bhi, const __grid_constant__ CUtensorMap tm_blo,
               const __grid_constant__ TcParams prm) {
    extern __shared__ uint8_t smem_raw[];
    SingleSrc src;
    src.m[0] = &tm_ahi;
    src.m[1] = &tm_alo;
    src.m[2] = &tm_bhi;
    src.m[3] = &tm_blo;
    src.prm = prm;
    tc_body<ACCK, BN>(src, prm.status, smem_raw, prm.range, false, prm.wait, &prm.acc_plan);
}

// One body per tile width, each compiled as its own function so that its
// registers are allocated for it alone (inlined together, the widest
// shape's register pressure spilled the others).
template <int BN>
__device__ __noinline__ void grouped_body(const GroupHeader* h, uint8_t* smem_raw) {
    GroupedSrc src{h};
    tc_body<0, BN>(src, h->status, smem_raw, const_cast<uint32_t*>(h->range), true, WaitCfg{});
}

__global__ void __launch_bounds__(NUM_THREADS, 1)
gemm_tc_grouped_kernel(const GroupHeader* __restrict__ h) {
    extern __shared__ uint8_t smem_raw[];
    // the tile width the table was prepared for (uniform over the launch)
    if (h->tile_n == 64) grouped_body<64>(h, smem_raw);
    else if (h->tile_n == 256) grouped_body<256>(h, smem_raw);
    else grouped_body<128>(h, smem_raw);
}

// The same for a tile width the host names at launch; a table prepared for
// another width is refused on the device (status LOFGB_ERR_UNSUPPORTED,
// nothing computed). The 64- and 128-column bodies are inlined here (on the
// mix of 64 GEMMs of 256..4096 14.69 / 11.56 ms against 16.27 / 12.17
// through the call);
// the 256-column body measured faster through its own function (11.51
// against 11.67 ms inlined) and is called.
template <int BN>
__global__ void __launch_bounds__(NUM_THREADS, 1)
gemm_tc_grouped_w_kernel(const GroupHeader* __restrict__ h) {
    extern __shared__ uint8_t smem_raw[];
    if (h->tile_n != BN) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(h->status, (int)LOFGB_ERR_UNSUPPORTED);
        return;
    }
    if constexpr (BN == 256) {
        grouped_body<256>(h, smem_raw);
    } else {
        GroupedSrc src{h};
        tc_body<0, BN>(src, h->status, smem_raw, const_cast<uint32_t*>(h->range), true, WaitCfg{});
    }
}

// ---- operand split: FP32 -> K-major BF16 hi/lo, zero padded -----------------
// One 32-row x 64-k tile of an operand. Output rows [0, R) x cols [0, Kp)
// (bf16). Source element (r, k) is src[r*ld + k] when kmajor, else
// src[k*ld + r]. Rows >= rows or k >= K are 0. hi = RZ_bf16(x),
// lo = RN_bf16(x - hi) (exact difference), lo = 0 for non-finite x.
__device__ __forceinline__ void split_tile(const float* __restrict__ src, int64_t ld, int kmajor,
                                           int rows, int K, int R, int Kp, __nv_bfloat16* hi,
                                           __nv_bfloat16* lo, int tr, int tk, float (*tile)[65],
                                           ExpRange& er) {
    const int r0 = tr * 32, k0 = tk * 64;
    const int t = threadIdx.x;
    if (kmajor) {
        for (int i = t; i < 32 * 64; i += 256) {
            const int rr = i / 64, kk = i % 64;
            const int r = r0 + rr, k = k0 + kk;
            tile[rr][kk] = (r < rows && k < K) ? src[(int64_t)r * ld + k] : 0.0f;
        }
    } else {
        for (int i = t; i < 32 * 64; i += 256) {
            const int kk = i / 32, rr = i % 32;
            const int r = r0 + rr, k = k0 + kk;
            tile[rr][kk] = (r < rows && k < K) ? src[(int64_t)k * ld + r] : 0.0f;
        }
    }
    __syncthreads();
    split_store_tile(tile, r0, k0, R, Kp, hi, lo, er);
    __syncthreads();
}

// blockIdx.z walks a strided batch: operand z at src + z * src_stride, its
// split at hi / lo + z * R * Kp. range: the operand's two exponent-range words.
__global__ void __launch_bounds__(256)
split_bf16_kernel(const float* __restrict__ src, int64_t ld, int64_t src_stride, int kmajor,
                  int rows, int K, int R, int Kp, int batch, __nv_bfloat16* __restrict__ hi,
                  __nv_bfloat16* __restrict__ lo, uint32_t* __restrict__ range) {
    __shared__ float tile[32][65];
    ExpRange er;
    for (int z = blockIdx.z; z < batch; z += gridDim.z) {
        const int64_t off = (int64_t)z * R * Kp;
        split_tile(src + (int64_t)z * src_stride, ld, kmajor, rows, K, R, Kp, hi + off, lo + off,
                   blockIdx.y, blockIdx.x, tile, er);
    }
    range_flush(range, er);
}

// All operands of a grouped launch: items are 32 x 64 tiles, walked
// grid-stride; each finds its operand by binary search over item_begin.
__global__ void __launch_bounds__(256)
split_grouped_kernel(const GroupHeader* __restrict__ h) {
    __shared__ float tile[32][65];
    __shared__ SplitRow row;
    const SplitRow* rows = reinterpret_cast<const SplitRow*>(
        reinterpret_cast<const uint8_t*>(h) + h->splits_off);
    const int nrows = h->nsplit;
    ExpRange era, erb;  // all A operands, all B operands
    // the device status word starts every launch cleared (this kernel runs
    // first on the stream; the GEMM kernel only ever sets it)
    if (blockIdx.x == 0 && threadIdx.x == 0) *h->status = 0;
    for (int64_t item = blockIdx.x; item < h->split_items; item += gridDim.x) {
        if (threadIdx.x == 0) {
            int lo = 0, hi = nrows - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (rows[mid].item_begin <= item) lo = mid;
                else hi = mid - 1;
            }
            row = rows[lo];
        }
        __syncthreads();
        const SplitRow r = row;
        __syncthreads();
        const int64_t local = item - r.item_begin;
        const int tiles_k = r.Kp / 64;
        ExpRange cur;
        split_tile(r.src, r.ld, r.kmajor, r.rows, r.K, r.R, r.Kp, r.hi, r.lo,
                   (int)(local / tiles_k), (int)(local % tiles_k), tile, cur);
        ExpRange& dst = r.operand ? erb : era;
        dst.emax = max(dst.emax, cur.emax);
        dst.emin_c = max(dst.emin_c, cur.emin_c);
        dst.lo |= cur.lo;
    }
    uint32_t* range = const_cast<uint32_t*>(h->range);
    range_flush(range, era);
    range_flush(range + 3, erb);
}

// ---- host side ---------------------------------------------------------------
size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

WsLayout ws_layout(int M, int N, int K, int batch) {
    WsLayout w;
    w.Mp = (int)align_up((size_t)M, TBM);
    w.Np = (int)align_up((size_t)N, TBN);
    w.Kp = (int)align_up((size_t)K, SK);
    w.batch = batch;
    const size_t a = (size_t)batch * w.Mp * w.Kp * 2, b = (size_t)batch * w.Np * w.Kp * 2;
    w.status = 0;
    w.range = 4;
    w.ahi = 1024;
    w.alo = align_up(w.ahi + a, 1024);
    w.bhi = align_up(w.alo + a, 1024);
    w.blo = align_up(w.bhi + b, 1024);
    w.total = align_up(w.blo + b, 1024);
    return w;
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

int make_map(CUtensorMap* map, void* base, int rows, int Kp, int box_rows = TBM) {
    auto fn = encode_fn();
    if (!fn) return set_error(LOFGB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)SK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(LOFGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return LOFGB_OK;
}

}  // namespace

size_t gemm_tc_workspace(int M, int N, int K, int batch) { return ws_layout(M, N, K, batch).total; }

namespace {
int launch_tc_presplit_cfg(uint8_t* ws, const WsLayout& w, float* D, int64_t ldd, int64_t sd, int M,
                           int N, int mbits, float alpha, int chunk, int64_t img_L,
                           int64_t img_stride, void* stream, const RoundPlan* acc_fmt,
                           const WaitCfg& wait);

int launch_gemm_tc_cfg(const float* A, int64_t lda, int64_t sa, int ta, const float* B, int64_t ldb,
                       int64_t sb, int tb, float* D, int64_t ldd, int64_t sd, int M, int N, int K,
                       int batch, int mbits, const RoundPlan* acc_fmt, float alpha, int chunk,
                       void* workspace, size_t workspace_bytes, void* stream, const WaitCfg& wait) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (K == 0) {
        // no products: D = alpha * (+0), one pitched clear per batch entry
        for (int z = 0; z < batch; ++z) {
            cudaError_t e = cudaMemset2DAsync(D + (int64_t)z * sd, sizeof(float) * (size_t)ldd, 0,
                                              sizeof(float) * (size_t)N, (size_t)M, st);
            if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
        }
        return LOFGB_OK;
    }
    const WsLayout w = ws_layout(M, N, K, batch);
    if (!workspace || workspace_bytes < w.total || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return set_error(LOFGB_ERR_WORKSPACE, "need %zu bytes of 256-byte aligned workspace", w.total);
    uint8_t* ws = static_cast<uint8_t*>(workspace);
    auto* ahi = reinterpret_cast<__nv_bfloat16*>(ws + w.ahi);
    auto* alo = reinterpret_cast<__nv_bfloat16*>(ws + w.alo);
    auto* bhi = reinterpret_cast<__nv_bfloat16*>(ws + w.bhi);
    auto* blo = reinterpret_cast<__nv_bfloat16*>(ws + w.blo);
    int* status = reinterpret_cast<int*>(ws + w.status);
    auto* range = reinterpret_cast<uint32_t*>(ws + w.range);
    cudaError_t e = cudaMemsetAsync(status, 0, WS_HEADER_CLEAR, st);
    if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));

    dim3 sb256(256);
    const unsigned gz = batch < 65535 ? batch : 65535;
    split_bf16_kernel<<<dim3(w.Kp / 64, w.Mp / 32, gz), sb256, 0, st>>>(A, lda, sa, ta ? 0 : 1, M, K,
                                                                        w.Mp, w.Kp, batch, ahi, alo,
                                                                        range);
    int rc = check_launch("split_bf16_kernel(A)");
    if (rc) return rc;
    split_bf16_kernel<<<dim3(w.Kp / 64, w.Np / 32, gz), sb256, 0, st>>>(B, ldb, sb, tb ? 1 : 0, N, K,
                                                                        w.Np, w.Kp, batch, bhi, blo,
                                                                        range + 3);
    if ((rc = check_launch("split_bf16_kernel(B)"))) return rc;
    return launch_tc_presplit_cfg(ws, w, D, ldd, sd, M, N, mbits, alpha, chunk, 0, 0, stream, acc_fmt,
                                  wait);
}
}  // namespace

int launch_gemm_tc(const float* A, int64_t lda, int64_t sa, int ta, const float* B, int64_t ldb,
                   int64_t sb, int tb, float* D, int64_t ldd, int64_t sd, int M, int N, int K,
                   int batch, int mbits, const RoundPlan* acc_fmt, float alpha, int chunk,
                   void* workspace, size_t workspace_bytes, void* stream) {
    return launch_gemm_tc_cfg(A, lda, sa, ta, B, ldb, sb, tb, D, ldd, sd, M, N, K, batch, mbits,
                              acc_fmt, alpha, chunk, workspace, workspace_bytes, stream, WaitCfg{});
}

int launch_tc_presplit(uint8_t* ws, const WsLayout& w, float* D, int64_t ldd, int64_t sd, int M,
                       int N, int mbits, float alpha, int chunk, int64_t img_L,
                       int64_t img_stride, void* stream, const RoundPlan* acc_fmt) {
    return launch_tc_presplit_cfg(ws, w, D, ldd, sd, M, N, mbits, alpha, chunk, img_L, img_stride,
                                  stream, acc_fmt, WaitCfg{});
}

namespace {
int launch_tc_presplit_cfg(uint8_t* ws, const WsLayout& w, float* D, int64_t ldd, int64_t sd, int M,
                           int N, int mbits, float alpha, int chunk, int64_t img_L,
                           int64_t img_stride, void* stream, const RoundPlan* acc_fmt,
                           const WaitCfg& wait) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto* ahi = reinterpret_cast<__nv_bfloat16*>(ws + w.ahi);
    auto* alo = reinterpret_cast<__nv_bfloat16*>(ws + w.alo);
    auto* bhi = reinterpret_cast<__nv_bfloat16*>(ws + w.bhi);
    auto* blo = reinterpret_cast<__nv_bfloat16*>(ws + w.blo);
    // Output tile 128 x 256 (one MMA covers twice the columns, halving the
    // MMA instructions per output) or 128 x 128, for the mantissa
    // accumulator: the persistent grid takes ceil(tiles / SMs) tile times,
    // and a wide tile measured about 1.1x the outputs per second of two
    // narrow ones (4096^3: 183 vs 167 TFLOP/s per full wave), so the wide
    // tile is taken only where its fewer, coarser waves still come out
    // ahead (not at 4096^2: 4 wide waves against 7 narrow ones).
    // LOFGB_TC_TILE_N=128|256 overrides the choice (tests, tuning).
    const int64_t tiles_m = w.Mp / TBM;
    const int64_t sms = sm_count();
    const int64_t t128 = (int64_t)w.batch * tiles_m * (w.Np / 128);
    const int64_t t256 = (int64_t)w.batch * tiles_m * ((w.Np + 255) / 256);
    const int64_t waves128 = (t128 + sms - 1) / sms, waves256 = (t256 + sms - 1) / sms;
    int tile_n = (!acc_fmt && waves256 * 20 < waves128 * 11) ? 256 : 128;
    if (const char* ov = std::getenv("LOFGB_TC_TILE_N")) {
        if (std::strcmp(ov, "128") == 0) tile_n = 128;
        else if (std::strcmp(ov, "256") == 0 && !acc_fmt) tile_n = 256;
    }
    int rc;
    CUtensorMap m_ahi, m_alo, m_bhi, m_blo;
    if ((rc = make_map(&m_ahi, ahi, w.batch * w.Mp, w.Kp))) return rc;
    if ((rc = make_map(&m_alo, alo, w.batch * w.Mp, w.Kp))) return rc;
    if ((rc = make_map(&m_bhi, bhi, w.batch * w.Np, w.Kp, tile_n))) return rc;
    if ((rc = make_map(&m_blo, blo, w.batch * w.Np, w.Kp, tile_n))) return rc;

    TcParams p;
    p.D = D;
    p.ldd = ldd;
    p.M = M;
    p.N = N;
    p.Kp = w.Kp;
    p.tiles_m = (int)tiles_m;
    p.tile_n = tile_n;
    p.tiles_n = (w.Np + tile_n - 1) / tile_n;
    p.chunk16 = chunk / 16;
    p.ro = 23 - mbits;
    p.alpha = alpha;
    p.status = reinterpret_cast<int*>(ws + w.status);
    p.img_L = img_L;
    p.img_stride = img_stride;
    p.batch = w.batch;
    p.Mp = w.Mp;
    p.Np = w.Np;
    p.stride_d = sd;
    p.acc_kind = 0;
    memset(&p.acc_plan, 0, sizeof(p.acc_plan));
    if (acc_fmt) {
        p.acc_kind = acc_fmt->uni == 1 ? 2 : 3;
        p.acc_plan = *acc_fmt;
    }
    p.range = reinterpret_cast<uint32_t*>(ws + w.range);
    p.fast_lim = acc_fmt ? FAST_OFF : fast_fold_limit(w.Kp, chunk, mbits);
    p.wait = wait;

    int dev = 0;
    cudaGetDevice(&dev);
    static bool attr_set[4][64] = {};
    const int ki = p.acc_kind == 0 ? (tile_n == 256 ? 3 : 0) : p.acc_kind - 1;
    const void* fn = ki == 3 ? (const void*)gemm_tc_kernel<0, 256>
                     : ki == 0 ? (const void*)gemm_tc_kernel<0, 128>
                     : ki == 1 ? (const void*)gemm_tc_kernel<2, 128> : (const void*)gemm_tc_kernel<3, 128>;
    if (dev < 0 || dev >= 64 || !attr_set[ki][dev]) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
        if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "smem attribute: %s", cudaGetErrorString(e));
        if (dev >= 0 && dev < 64) attr_set[ki][dev] = true;
    }
    const int64_t tiles = (int64_t)p.batch * p.tiles_m * p.tiles_n;
    if (tiles >= ((int64_t)1 << 31)) return set_error(LOFGB_ERR_SIZE, "too many output tiles");
    const int grid = tiles < sm_count() ? (int)tiles : sm_count();
    if (ki == 3)
        gemm_tc_kernel<0, 256><<<grid, NUM_THREADS, SMEM_BYTES, st>>>(m_ahi, m_alo, m_bhi, m_blo, p);
    else if (ki == 0)
        gemm_tc_kernel<0, 128><<<grid, NUM_THREADS, SMEM_BYTES, st>>>(m_ahi, m_alo, m_bhi, m_blo, p);
    else if (ki == 1)
        gemm_tc_kernel<2, 128><<<grid, NUM_THREADS, SMEM_BYTES, st>>>(m_ahi, m_alo, m_bhi, m_blo, p);
    else
        gemm_tc_kernel<3, 128><<<grid, NUM_THREADS, SMEM_BYTES, st>>>(m_ahi, m_alo, m_bhi, m_blo, p);
    return check_launch("gemm_tc_kernel");
}
}  // namespace

}  // namespace lofgb

// ---- the no-allocation entry point -------------------------------------------
// Scratch for lofgb_gemm_tc_noalloc_f32: a fixed device array in this module.
// Host code must not use the symbol as a pointer; its device address comes
// from cudaGetSymbolAddress, once per device.
namespace lofgb {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 64ull << 20;
__device__ __align__(256) uint8_t g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device (first call per
// device resolves it), or nullptr with the error recorded.
void* noalloc_scratch(int* status) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        *status = set_error(LOFGB_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
        return nullptr;
    }
    if (dev < 0 || dev >= 64) {
        *status = set_error(LOFGB_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            *status = set_error(LOFGB_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return nullptr;
        }
        g_noalloc_ptr[dev] = p;
    }
    *status = LOFGB_OK;
    return g_noalloc_ptr[dev];
}

}  // namespace
}  // namespace lofgb

extern "C" int lofgb_gemm_tc_noalloc_f32(const float* A, int64_t lda, int trans_a, const float* B,
                                         int64_t ldb, int trans_b, float* D, int64_t ldd, int M,
                                         int N, int K, int accum_mant_bits, float alpha, int chunk,
                                         void* stream) {
    using namespace lofgb;
    // the arguments first, with the codes lofgb_gemm_f32 returns for them;
    // only a valid request is measured against the scratch array
    int st = check_gemm_args(A, lda, trans_a, B, ldb, trans_b, D, ldd, M, N, K);
    if (st) return st;
    if (accum_mant_bits < 0 || accum_mant_bits > 23)
        return set_error(LOFGB_ERR_FORMAT, "accum_mant_bits %d outside [0, 23]", accum_mant_bits);
    if (chunk <= 0 || chunk % 16 != 0 || chunk > 256)
        return set_error(LOFGB_ERR_SIZE, "chunk %d must be a multiple of 16 in [16, 256]", chunk);
    const bool work = M > 0 && N > 0 && K > 0;
    if (work) {
        const size_t need = gemm_tc_workspace(M, N, K, 1);
        if (need > NOALLOC_SCRATCH_BYTES)
            return set_error(LOFGB_ERR_WORKSPACE,
                             "no-alloc GEMM needs %zu bytes of scratch; the built-in array holds %zu",
                             need, NOALLOC_SCRATCH_BYTES);
    }
    void* scratch = nullptr;
    if (work) {
        scratch = noalloc_scratch(&st);
        if (!scratch) return st;
    }
    return lofgb_gemm_f32(A, lda, trans_a, B, ldb, trans_b, D, ldd, M, N, K, accum_mant_bits,
                          LOFGB_RNE, alpha, LOFGB_GEMM_TC, chunk, scratch,
                          scratch ? NOALLOC_SCRATCH_BYTES : 0, stream);
}

// ---- bounded-wait self-test ----------------------------------------------------
extern "C" int lofgb_gemm_tc_wait_selftest(const float* A, const float* B, float* D, int M, int N,
                                           int K, void* workspace, size_t workspace_bytes,
                                           uint32_t wait_limit_us, void* stream) {
    using namespace lofgb;
    clear_error();
    if (M <= 0 || N <= 0 || K <= 0) return set_error(LOFGB_ERR_SIZE, "self-test needs M, N, K > 0");
    if (!A || !B || !D) return set_error(LOFGB_ERR_NULL, "NULL operand");
    if (wait_limit_us < 100 || wait_limit_us > 100000)
        return set_error(LOFGB_ERR_SIZE, "wait limit %u us outside [100, 100000]", wait_limit_us);
    WaitCfg wait;
    wait.limit_ns = (unsigned long long)wait_limit_us * 1000ull;
    wait.withhold = 0;  // the first stage of every CTA never fills
    return launch_gemm_tc_cfg(A, K, 0, 0, B, N, 0, 0, D, N, 0, M, N, K, 1, 10, nullptr, 1.0f, 32,
                              workspace, workspace_bytes, stream, wait);
}

// ---- grouped launch: host side -----------------------------------------------
#include <algorithm>
#include <vector>

namespace lofgb {
namespace {

struct GroupLayout {
    size_t ws_total;
    std::vector<size_t> ahi, alo, bhi, blo;
    std::vector<int> Mp, Np, Kp;
    int64_t tiles = 0, split_items = 0;
    size_t rows_off, tiles_off, splits_off, table_total;
};

int check_task(const lofgb_gemm_task& t, int i) {
    if (t.M < 0 || t.N < 0 || t.K < 0)
        return set_error(LOFGB_ERR_SIZE, "task %d: negative dimension", i);
    if ((t.trans_a != 0 && t.trans_a != 1) || (t.trans_b != 0 && t.trans_b != 1))
        return set_error(LOFGB_ERR_SIZE, "task %d: trans flags must be 0 or 1", i);
    if (t.M && t.N && !t.D) return set_error(LOFGB_ERR_NULL, "task %d: D is NULL", i);
    if (t.M && t.N && t.K && (!t.A || !t.B)) return set_error(LOFGB_ERR_NULL, "task %d: A or B is NULL", i);
    if (t.lda < (t.trans_a ? t.M : t.K) || t.lda < 1 || t.ldb < (t.trans_b ? t.K : t.N) || t.ldb < 1 ||
        t.ldd < t.N || t.ldd < 1)
        return set_error(LOFGB_ERR_SIZE, "task %d: leading dimension too small", i);
    if (t.accum_mant_bits < 0 || t.accum_mant_bits > 23)
        return set_error(LOFGB_ERR_FORMAT, "task %d: accum_mant_bits %d outside [0, 23]", i, t.accum_mant_bits);
    if (t.chunk <= 0 || t.chunk % 16 != 0 || t.chunk > 256)
        return set_error(LOFGB_ERR_SIZE, "task %d: chunk %d must be a multiple of 16 in [16, 256]", i, t.chunk);
    if (t.M > 0 && t.N > 0 && t.K == 0)
        return set_error(LOFGB_ERR_UNSUPPORTED, "task %d: K == 0 in a grouped launch", i);
    return LOFGB_OK;
}

GroupLayout group_layout(const lofgb_gemm_task* tasks, int n) {
    GroupLayout g;
    size_t off = 1024;  // status word
    for (int i = 0; i < n; ++i) {
        const lofgb_gemm_task& t = tasks[i];
        const bool empty = t.M <= 0 || t.N <= 0 || t.K <= 0;
        const int Mp = empty ? 0 : (int)align_up((size_t)t.M, TBM);
        const int Np = empty ? 0 : (int)align_up((size_t)t.N, TBN);
        const int Kp = empty ? 0 : (int)align_up((size_t)t.K, SK);
        g.Mp.push_back(Mp);
        g.Np.push_back(Np);
        g.Kp.push_back(Kp);
        const size_t a = (size_t)Mp * Kp * 2, b = (size_t)Np * Kp * 2;
        g.ahi.push_back(off); off = align_up(off + a, 1024);
        g.alo.push_back(off); off = align_up(off + a, 1024);
        g.bhi.push_back(off); off = align_up(off + b, 1024);
        g.blo.push_back(off); off = align_up(off + b, 1024);
        g.tiles += (int64_t)(Mp / TBM) * (Np / 64);  // room for the narrow tile's count
        g.split_items += (int64_t)(Mp / 32) * (Kp / 64) + (int64_t)(Np / 32) * (Kp / 64);
    }
    g.ws_total = off;
    g.rows_off = align_up(sizeof(GroupHeader), 256);
    g.tiles_off = align_up(g.rows_off + sizeof(GroupRow) * (size_t)n, 256);
    g.splits_off = align_up(g.tiles_off + sizeof(TileRef) * (size_t)g.tiles, 256);
    g.table_total = align_up(g.splits_off + sizeof(SplitRow) * (size_t)(2 * n), 256);
    return g;
}

}  // namespace
}  // namespace lofgb

using namespace lofgb;

extern "C" {

size_t lofgb_gemm_grouped_workspace_size(const lofgb_gemm_task* tasks, int ntasks) {
    if (!tasks || ntasks <= 0) return 0;
    return group_layout(tasks, ntasks).ws_total;
}

size_t lofgb_gemm_grouped_table_size(const lofgb_gemm_task* tasks, int ntasks) {
    if (!tasks || ntasks <= 0) return 0;
    return group_layout(tasks, ntasks).table_total;
}

int lofgb_gemm_grouped_prepare(const lofgb_gemm_task* tasks, int ntasks, void* workspace,
                               size_t workspace_bytes, int schedule, int grid, void* table,
                               size_t table_bytes, int64_t* num_tiles, int64_t* split_items) {
    if (ntasks <= 0) return set_error(LOFGB_ERR_SIZE, "need at least one task");
    if (!tasks || !table || !workspace || !num_tiles || !split_items)
        return set_error(LOFGB_ERR_NULL, "NULL tasks, workspace, table or output count");
    if ((schedule & LOFGB_GROUPED_TILE_N64) && (schedule & LOFGB_GROUPED_TILE_N256))
        return set_error(LOFGB_ERR_UNSUPPORTED, "one tile width per table");
    const int tile_n = (schedule & LOFGB_GROUPED_TILE_N64) ? 64 : (schedule & LOFGB_GROUPED_TILE_N256) ? 256 : 128;
    schedule &= ~(LOFGB_GROUPED_TILE_N64 | LOFGB_GROUPED_TILE_N256);
    if (schedule < 0 || schedule > 2) return set_error(LOFGB_ERR_UNSUPPORTED, "schedule %d", schedule);
    for (int i = 0; i < ntasks; ++i) {
        const int st = check_task(tasks[i], i);
        if (st) return st;
    }
    const GroupLayout g = group_layout(tasks, ntasks);
    if (workspace_bytes < g.ws_total || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return set_error(LOFGB_ERR_WORKSPACE, "need %zu bytes of 256-byte aligned workspace", g.ws_total);
    if (table_bytes < g.table_total)
        return set_error(LOFGB_ERR_WORKSPACE, "table needs %zu bytes", g.table_total);
    if (grid <= 0) grid = sm_count();
    uint8_t* tb = static_cast<uint8_t*>(table);
    memset(tb, 0, g.table_total);
    uint8_t* ws = static_cast<uint8_t*>(workspace);
    GroupHeader* h = reinterpret_cast<GroupHeader*>(tb);
    h->ntasks = ntasks;
    h->tile_n = tile_n;
    h->nsplit = 2 * ntasks;
    h->split_items = g.split_items;
    h->rows_off = (int64_t)g.rows_off;
    h->tiles_off = (int64_t)g.tiles_off;
    h->splits_off = (int64_t)g.splits_off;
    h->status = reinterpret_cast<int*>(ws);
    GroupRow* rows = reinterpret_cast<GroupRow*>(tb + g.rows_off);
    SplitRow* splits = reinterpret_cast<SplitRow*>(tb + g.splits_off);
    struct Cand { int32_t task, m0, n0; int64_t cost; };
    std::vector<Cand> cands;
    cands.reserve((size_t)g.tiles);
    int64_t item = 0;
    for (int i = 0; i < ntasks; ++i) {
        const lofgb_gemm_task& t = tasks[i];
        GroupRow& r = rows[i];
        auto* ahi = reinterpret_cast<__nv_bfloat16*>(ws + g.ahi[i]);
        auto* alo = reinterpret_cast<__nv_bfloat16*>(ws + g.alo[i]);
        auto* bhi = reinterpret_cast<__nv_bfloat16*>(ws + g.bhi[i]);
        auto* blo = reinterpret_cast<__nv_bfloat16*>(ws + g.blo[i]);
        r.D = t.D;
        r.ldd = t.ldd;
        r.M = t.M;
        r.N = t.N;
        r.Kp = g.Kp[i];
        r.chunk16 = t.chunk / 16;
        r.ro = 23 - t.accum_mant_bits;
        r.alpha = t.alpha;
        r.fast_lim = g.Kp[i] > 0 ? fast_fold_limit(g.Kp[i], t.chunk, t.accum_mant_bits) : FAST_OFF;
        SplitRow& sa = splits[2 * i];
        SplitRow& sbr = splits[2 * i + 1];
        sa.src = t.A; sa.ld = t.lda; sa.kmajor = t.trans_a ? 0 : 1; sa.rows = t.M; sa.K = t.K;
        sa.R = g.Mp[i]; sa.Kp = g.Kp[i]; sa.hi = ahi; sa.lo = alo; sa.item_begin = item;
        sa.operand = 0;
        item += (int64_t)(g.Mp[i] / 32) * (g.Kp[i] / 64);
        sbr.src = t.B; sbr.ld = t.ldb; sbr.kmajor = t.trans_b ? 1 : 0; sbr.rows = t.N; sbr.K = t.K;
        sbr.R = g.Np[i]; sbr.Kp = g.Kp[i]; sbr.hi = bhi; sbr.lo = blo; sbr.item_begin = item;
        sbr.operand = 1;
        item += (int64_t)(g.Np[i] / 32) * (g.Kp[i] / 64);
        if (g.Mp[i] == 0 || g.Np[i] == 0 || g.Kp[i] == 0) continue;
        int rc;
        if ((rc = make_map(&r.map[0], ahi, g.Mp[i], g.Kp[i]))) return rc;
        if ((rc = make_map(&r.map[1], alo, g.Mp[i], g.Kp[i]))) return rc;
        if ((rc = make_map(&r.map[2], bhi, g.Np[i], g.Kp[i], tile_n))) return rc;
        if ((rc = make_map(&r.map[3], blo, g.Np[i], g.Kp[i], tile_n))) return rc;
        const int nchunks = (g.Kp[i] / 16 + r.chunk16 - 1) / r.chunk16;
        const int64_t cost = 4 * (int64_t)nchunks + g.Kp[i] / SK;
        for (int mt = 0; mt < g.Mp[i] / TBM; ++mt)
            for (int nt = 0; nt < (g.Np[i] + tile_n - 1) / tile_n; ++nt)
                cands.push_back({i, mt * TBM, nt * tile_n, cost});
    }
    if (schedule >= 1)
        std::stable_sort(cands.begin(), cands.end(),
                         [](const Cand& a, const Cand& b) { return a.cost > b.cost; });
    TileRef* tl = reinterpret_cast<TileRef*>(tb + g.tiles_off);
    const int64_t nt = (int64_t)cands.size();
    for (int64_t pidx = 0; pidx < nt; ++pidx) {
        int64_t src_idx = pidx;
        if (schedule == 2) {  // boustrophedon deal: odd rounds run the CTAs backwards
            const int64_t round = pidx / grid, c = pidx % grid;
            const int64_t base = round * grid;
            const int64_t width = std::min<int64_t>(grid, nt - base);
            src_idx = (round & 1) ? base + (width - 1 - c) : pidx;
            if (src_idx >= nt) src_idx = pidx;
        }
        tl[pidx] = TileRef{cands[src_idx].task, cands[src_idx].m0, cands[src_idx].n0, 0};
    }
    h->ntiles = (int32_t)nt;
    *num_tiles = nt;
    *split_items = g.split_items;
    return LOFGB_OK;
}

}  // extern "C"

namespace lofgb {
namespace {
int grouped_launch(const void* kernel, int ki, const void* device_table, int64_t num_tiles,
                   int64_t split_items, int grid, void* stream) {
    if (!device_table) return set_error(LOFGB_ERR_NULL, "NULL device table");
    if ((reinterpret_cast<uintptr_t>(device_table) & 255) != 0)
        return set_error(LOFGB_ERR_WORKSPACE, "device table must be 256-byte aligned");
    if (num_tiles < 0 || split_items < 0) return set_error(LOFGB_ERR_SIZE, "negative count");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const auto* h = static_cast<const GroupHeader*>(device_table);
    if (split_items > 0) {
        const int64_t maxg = (int64_t)sm_count() * 8;
        const int sg = (int)std::min<int64_t>(split_items, maxg);
        split_grouped_kernel<<<sg, 256, 0, st>>>(h);
        const int rc = check_launch("split_grouped_kernel");
        if (rc) return rc;
    }
    if (num_tiles == 0) return LOFGB_OK;
    int dev = 0;
    cudaGetDevice(&dev);
    static bool attr_set[4][64] = {};
    if (dev < 0 || dev >= 64 || !attr_set[ki][dev]) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
        if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "smem attribute: %s", cudaGetErrorString(e));
        if (dev >= 0 && dev < 64) attr_set[ki][dev] = true;
    }
    if (grid <= 0) grid = sm_count();
    if (grid > num_tiles) grid = (int)num_tiles;
    void* args[] = {const_cast<void*>(static_cast<const void*>(&h))};
    cudaError_t e = cudaLaunchKernel(kernel, dim3(grid), dim3(NUM_THREADS), args, SMEM_BYTES, st);
    if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "gemm_tc_grouped_kernel: %s", cudaGetErrorString(e));
    return LOFGB_OK;
}
}  // namespace
}  // namespace lofgb

extern "C" {

int lofgb_gemm_grouped_launch(const void* device_table, int64_t num_tiles, int64_t split_items,
                              int grid, void* stream) {
    return grouped_launch((const void*)gemm_tc_grouped_kernel, 0, device_table, num_tiles, split_items,
                          grid, stream);
}

int lofgb_gemm_grouped_launch_w(const void* device_table, int64_t num_tiles, int64_t split_items,
                                int grid, int tile_n, void* stream) {
    if (tile_n == 64)
        return grouped_launch((const void*)gemm_tc_grouped_w_kernel<64>, 1, device_table, num_tiles,
                              split_items, grid, stream);
    if (tile_n == 128)
        return grouped_launch((const void*)gemm_tc_grouped_w_kernel<128>, 2, device_table, num_tiles,
                              split_items, grid, stream);
    if (tile_n == 256)
        return grouped_launch((const void*)gemm_tc_grouped_w_kernel<256>, 3, device_table, num_tiles,
                              split_items, grid, stream);
    return set_error(LOFGB_ERR_UNSUPPORTED, "tile width %d (64, 128 or 256)", tile_n);
}

}  // extern "C"
