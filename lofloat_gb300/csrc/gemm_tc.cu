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
// power-of-two scale) have lo = 0 and enter exactly.
//
// Kernel layout (one CTA per SM, persistent over 128 x 128 output tiles):
//   warp 0      TMA producer: 4 tiles (A hi/lo, B hi/lo) of 64 k per stage,
//               3 stages, 128-byte swizzle, one mbarrier per stage;
//   warp 1      TMEM owner and MMA issuer (one elected lane):
//               tcgen05.mma.cta_group::1.kind::f16, M=128 N=128 K=16,
//               chunk sums double-buffered in 2 x 128 TMEM columns;
//   warps 2..9  epilogue: tcgen05.ld the chunk sum of one TMEM lane quarter
//               and one 64-column half, fold it into 64 register
//               accumulators, release the TMEM buffer; store D at tile end.
// Every wait is bounded (~2 s of %globaltimer): on expiry the CTA records
// LOFGB_ERR_TIMEOUT in the workspace status word, drains its own in-flight
// copies and MMAs (again bounded), frees its TMEM and exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "lofgb_internal.h"

namespace lofgb {

namespace {

constexpr int TBM = 128;          // output tile rows (UMMA M)
constexpr int TBN = 128;          // output tile cols (UMMA N)
constexpr int SK = 64;            // k per pipeline stage (one 128-byte swizzle row of bf16)
constexpr int STAGES = 3;
constexpr int TILE_BYTES = TBM * SK * 2;       // 16 KiB per operand tile
constexpr int STAGE_BYTES = 4 * TILE_BYTES;    // A hi, A lo, B hi, B lo
constexpr int EPI_WARPS = 8;
constexpr int NUM_THREADS = 32 * (2 + EPI_WARPS);
constexpr int TMEM_COLS = 2 * TBN;             // two chunk buffers
constexpr size_t SMEM_BYTES = 1024 /*align slack*/ + STAGES * STAGE_BYTES + 256 /*barriers*/;
constexpr unsigned long long WAIT_LIMIT_NS = 2000000000ull;

struct TcParams {
    float* D;
    int64_t ldd;
    int M, N, Kp;          // Kp: padded K (multiple of SK)
    int tiles_m, tiles_n;
    int chunk16;           // chunk length in 16-k steps
    int ro;                // 23 - accum_mant_bits
    float alpha;
    int* status;           // workspace status word
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
                                          int* status) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (globaltimer() - t0 > WAIT_LIMIT_NS) {
            *abort_flag = 1;
            atomicExch(status, (int)LOFGB_ERR_TIMEOUT);
            return false;
        }
    }
}

// Wait used while draining after an abort: bounded, result ignored.
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = globaltimer();
    while (!mbar_try_wait(bar, parity))
        if (globaltimer() - t0 > WAIT_LIMIT_NS) return;
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

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TBN >> 3) << 17) |
                           ((uint32_t)(TBM >> 4) << 24);

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

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// acc = RNE_m(rto(acc + s)) with directed adds, as the per-MAC leaf does with
// directed FMAs (src/cutlass_gemms.cuh:73-88, 162-163).
__device__ __forceinline__ float fold(float acc, float s, int ro, uint32_t half_m1, uint32_t mask) {
    const float rd = __fadd_rd(acc, s);
    const float ru = __fadd_ru(acc, s);
    const uint32_t rz = __float_as_uint(rd >= 0.0f ? rd : ru);
    const uint32_t v = rz | ((__float_as_uint(rd) | __float_as_uint(ru)) & 1u);
    if (ro <= 0) return __uint_as_float(v);
    const uint32_t t = v + ((v >> ro) & 1u) + half_m1;
    return __uint_as_float(t & mask);
}

__global__ void __launch_bounds__(NUM_THREADS, 1)
gemm_tc_kernel(const __grid_constant__ CUtensorMap tm_ahi, const __grid_constant__ CUtensorMap tm_alo,
               const __grid_constant__ CUtensorMap tm_bhi, const __grid_constant__ CUtensorMap tm_blo,
               TcParams prm) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    uint8_t* tiles = smem;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    // bars: full[STAGES], empty[STAGES], tfull[2], tempty[2], drain
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t bar_full = smem_u32(bars);
    const uint32_t bar_empty = smem_u32(bars + STAGES);
    const uint32_t bar_tfull = smem_u32(bars + 2 * STAGES);
    const uint32_t bar_tempty = smem_u32(bars + 2 * STAGES + 2);
    const uint32_t bar_drain = smem_u32(bars + 2 * STAGES + 4);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(bar_full + 8 * s, 1);
            mbar_init(bar_empty + 8 * s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(bar_tfull + 8 * b, 1);
            mbar_init(bar_tempty + 8 * b, EPI_WARPS * 32);
        }
        mbar_init(bar_drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
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

    const int num_tiles = prm.tiles_m * prm.tiles_n;
    const int ksteps = prm.Kp / SK;        // pipeline stages per tile
    const int k16 = prm.Kp / 16;           // MMA k-steps per tile
    const int nchunks = (k16 + prm.chunk16 - 1) / prm.chunk16;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x) {
                const int m0 = (tile / prm.tiles_n) * TBM;
                const int n0 = (tile % prm.tiles_n) * TBN;
                for (int ks = 0; ks < ksteps; ++ks, ++it) {
                    const uint32_t s = it % STAGES;
                    const uint32_t ph = (it / STAGES) & 1u;
                    if (!mbar_wait(bar_empty + 8 * s, ph ^ 1u, abort_flag, prm.status)) { ok = false; break; }
                    const uint32_t base = smem_u32(tiles + s * STAGE_BYTES);
                    mbar_arrive_expect_tx(bar_full + 8 * s, STAGE_BYTES);
                    tma_load_2d(base + 0 * TILE_BYTES, &tm_ahi, ks * SK, m0, bar_full + 8 * s);
                    tma_load_2d(base + 1 * TILE_BYTES, &tm_alo, ks * SK, m0, bar_full + 8 * s);
                    tma_load_2d(base + 2 * TILE_BYTES, &tm_bhi, ks * SK, n0, bar_full + 8 * s);
                    tma_load_2d(base + 3 * TILE_BYTES, &tm_blo, ks * SK, n0, bar_full + 8 * s);
                }
            }
            if (!ok) {
                // drain: every issued stage completes (or the drain wait expires)
                for (uint32_t j = (it >= STAGES ? it - STAGES : 0); j < it; ++j)
                    mbar_drain(bar_full + 8 * (j % STAGES), (j / STAGES) & 1u);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint32_t it = 0;      // stage counter
            uint32_t cg = 0;      // global chunk counter
            bool ok = true;
            for (int tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x) {
                int kk16 = 0;
                for (int ks = 0; ks < ksteps && ok; ++ks, ++it) {
                    const uint32_t s = it % STAGES;
                    if (!mbar_wait(bar_full + 8 * s, (it / STAGES) & 1u, abort_flag, prm.status)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t base = smem_u32(tiles + s * STAGE_BYTES);
                    for (int j = 0; j < SK / 16; ++j, ++kk16) {
                        const int pos = kk16 % prm.chunk16;
                        const uint32_t buf = cg & 1u;
                        if (pos == 0) {
                            if (!mbar_wait(bar_tempty + 8 * buf, ((cg >> 1) & 1u) ^ 1u, abort_flag, prm.status)) { ok = false; break; }
                            tc_fence_after();
                        }
                        const uint32_t d = tmem_base + buf * TBN;
                        const uint64_t ahi = smem_desc_sw128(base + 0 * TILE_BYTES + j * 32);
                        const uint64_t alo = smem_desc_sw128(base + 1 * TILE_BYTES + j * 32);
                        const uint64_t bhi = smem_desc_sw128(base + 2 * TILE_BYTES + j * 32);
                        const uint64_t blo = smem_desc_sw128(base + 3 * TILE_BYTES + j * 32);
                        umma_f16(d, ahi, bhi, pos > 0 ? 1u : 0u);
                        umma_f16(d, ahi, blo, 1u);
                        umma_f16(d, alo, bhi, 1u);
                        if (pos == prm.chunk16 - 1 || kk16 == k16 - 1) {
                            umma_commit(bar_tfull + 8 * buf);
                            ++cg;
                        }
                    }
                    if (!ok) break;
                    umma_commit(bar_empty + 8 * s);  // stage's smem free once its MMAs finish
                }
            }
            // all issued MMAs complete before the TMEM is released
            umma_commit(bar_drain);
            mbar_drain(bar_drain, 0);
        }
    } else {
        // ---------------- epilogue ----------------
        const int ew = warp - 2;              // 0..7
        const int quarter = warp & 3;         // TMEM lane quarter this warp may access
        const int half = ew >> 2;             // column half
        const int ro = prm.ro;
        const uint32_t half_m1 = ro > 0 ? (1u << (ro - 1)) - 1u : 0u;
        const uint32_t mask = ro > 0 ? ~((1u << ro) - 1u) : ~0u;
        uint32_t cg = 0;
        bool ok = true;
        for (int tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x) {
            const int m0 = (tile / prm.tiles_n) * TBM;
            const int n0 = (tile % prm.tiles_n) * TBN;
            float acc[64];
#pragma unroll
            for (int i = 0; i < 64; ++i) acc[i] = 0.0f;
            for (int c = 0; c < nchunks; ++c, ++cg) {
                const uint32_t buf = cg & 1u;
                // every lane waits; the warp proceeds only when all lanes saw the
                // phase complete, reconverged for the .sync.aligned TMEM loads
                const bool got = mbar_wait(bar_tfull + 8 * buf, (cg >> 1) & 1u, abort_flag, prm.status);
                if (!__all_sync(0xFFFFFFFFu, got)) { ok = false; break; }
                __syncwarp();
                tc_fence_after();
                const uint32_t taddr = tmem_base + ((uint32_t)(quarter * 32) << 16) + buf * TBN + half * 64;
                uint32_t r0[32], r1[32];
                tmem_ld32(taddr, r0);
                tmem_ld32(taddr + 32, r1);
                tmem_ld_wait();
                tc_fence_before();
                mbar_arrive(bar_tempty + 8 * buf);
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[i] = fold(acc[i], __uint_as_float(r0[i]), ro, half_m1, mask);
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[32 + i] = fold(acc[32 + i], __uint_as_float(r1[i]), ro, half_m1, mask);
            }
            if (!ok) break;
            const int row = m0 + quarter * 32 + lane;
            if (row < prm.M) {
                float* drow = prm.D + (int64_t)row * prm.ldd + n0 + half * 64;
                const int ncol = min(64, prm.N - (n0 + half * 64));
                if (ncol == 64 && ((reinterpret_cast<uintptr_t>(drow) & 15) == 0)) {
#pragma unroll
                    for (int i = 0; i < 64; i += 4) {
                        float4 v = make_float4(__fmul_rn(prm.alpha, acc[i]), __fmul_rn(prm.alpha, acc[i + 1]),
                                               __fmul_rn(prm.alpha, acc[i + 2]), __fmul_rn(prm.alpha, acc[i + 3]));
                        *reinterpret_cast<float4*>(drow + i) = v;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 64; ++i)
                        if (i < ncol) drow[i] = __fmul_rn(prm.alpha, acc[i]);
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

// ---- operand split: FP32 -> K-major BF16 hi/lo, zero padded -----------------
// Output rows [0, R) x cols [0, Kp) (bf16). Source element (r, k) is
// src[r*ld + k] when kmajor, else src[k*ld + r]. Rows >= rows or k >= K are 0.
__global__ void __launch_bounds__(256)
split_bf16_kernel(const float* __restrict__ src, int64_t ld, int kmajor, int rows, int K, int R,
                  int Kp, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
    __shared__ float tile[32][65];
    const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 64;
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
    for (int i = t; i < 32 * 32; i += 256) {
        const int rr = i / 32, kp = (i % 32) * 2;
        const int r = r0 + rr, k = k0 + kp;
        if (r >= R || k >= Kp) continue;
        __nv_bfloat162 h2, l2;
        float x0 = tile[rr][kp], x1 = tile[rr][kp + 1];
        __nv_bfloat16 h0 = __float2bfloat16_rz(x0), h1 = __float2bfloat16_rz(x1);
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

// ---- host side ---------------------------------------------------------------
struct WsLayout {
    size_t status, ahi, alo, bhi, blo, total;
    int Mp, Np, Kp;
};

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

WsLayout ws_layout(int M, int N, int K) {
    WsLayout w;
    w.Mp = (int)align_up((size_t)M, TBM);
    w.Np = (int)align_up((size_t)N, TBN);
    w.Kp = (int)align_up((size_t)K, SK);
    const size_t a = (size_t)w.Mp * w.Kp * 2, b = (size_t)w.Np * w.Kp * 2;
    w.status = 0;
    w.ahi = 1024;
    w.alo = align_up(w.ahi + a, 1024);
    w.bhi = align_up(w.alo + a, 1024);
    w.blo = align_up(w.bhi + b, 1024);
    w.total = align_up(w.blo + b, 1024);
    return w;
}

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

int make_map(CUtensorMap* map, void* base, int rows, int Kp) {
    auto fn = encode_fn();
    if (!fn) return set_error(LOFGB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)SK, (cuuint32_t)TBM};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(LOFGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return LOFGB_OK;
}

}  // namespace

size_t gemm_tc_workspace(int M, int N, int K) { return ws_layout(M, N, K).total; }

int launch_gemm_tc(const float* A, int64_t lda, int ta, const float* B, int64_t ldb, int tb,
                   float* D, int64_t ldd, int M, int N, int K, int mbits, float alpha, int chunk,
                   void* workspace, size_t workspace_bytes, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (K == 0) {
        // no products: D = alpha * (+0)
        for (int i = 0; i < M; ++i) {
            cudaError_t e = cudaMemsetAsync(D + (int64_t)i * ldd, 0, sizeof(float) * N, st);
            if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
        }
        return LOFGB_OK;
    }
    const WsLayout w = ws_layout(M, N, K);
    if (!workspace || workspace_bytes < w.total || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return set_error(LOFGB_ERR_WORKSPACE, "need %zu bytes of 256-byte aligned workspace", w.total);
    uint8_t* ws = static_cast<uint8_t*>(workspace);
    auto* ahi = reinterpret_cast<__nv_bfloat16*>(ws + w.ahi);
    auto* alo = reinterpret_cast<__nv_bfloat16*>(ws + w.alo);
    auto* bhi = reinterpret_cast<__nv_bfloat16*>(ws + w.bhi);
    auto* blo = reinterpret_cast<__nv_bfloat16*>(ws + w.blo);
    int* status = reinterpret_cast<int*>(ws + w.status);
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), st);
    if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));

    dim3 sb(256);
    split_bf16_kernel<<<dim3(w.Kp / 64, w.Mp / 32), sb, 0, st>>>(A, lda, ta ? 0 : 1, M, K, w.Mp, w.Kp, ahi, alo);
    int rc = check_launch("split_bf16_kernel(A)");
    if (rc) return rc;
    split_bf16_kernel<<<dim3(w.Kp / 64, w.Np / 32), sb, 0, st>>>(B, ldb, tb ? 1 : 0, N, K, w.Np, w.Kp, bhi, blo);
    if ((rc = check_launch("split_bf16_kernel(B)"))) return rc;

    CUtensorMap m_ahi, m_alo, m_bhi, m_blo;
    if ((rc = make_map(&m_ahi, ahi, w.Mp, w.Kp))) return rc;
    if ((rc = make_map(&m_alo, alo, w.Mp, w.Kp))) return rc;
    if ((rc = make_map(&m_bhi, bhi, w.Np, w.Kp))) return rc;
    if ((rc = make_map(&m_blo, blo, w.Np, w.Kp))) return rc;

    TcParams p;
    p.D = D;
    p.ldd = ldd;
    p.M = M;
    p.N = N;
    p.Kp = w.Kp;
    p.tiles_m = w.Mp / TBM;
    p.tiles_n = w.Np / TBN;
    p.chunk16 = chunk / 16;
    p.ro = 23 - mbits;
    p.alpha = alpha;
    p.status = status;

    int dev = 0;
    cudaGetDevice(&dev);
    static bool attr_set[64] = {false};
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
        e = cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
        if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "smem attribute: %s", cudaGetErrorString(e));
        if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
    const int tiles = p.tiles_m * p.tiles_n;
    const int grid = tiles < sm_count() ? tiles : sm_count();
    gemm_tc_kernel<<<grid, NUM_THREADS, SMEM_BYTES, st>>>(m_ahi, m_alo, m_bhi, m_blo, p);
    return check_launch("gemm_tc_kernel");
}

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
    if (M > 0 && N > 0 && K > 0) {
        const size_t need = gemm_tc_workspace(M, N, K);
        if (need > NOALLOC_SCRATCH_BYTES)
            return set_error(LOFGB_ERR_WORKSPACE,
                             "no-alloc GEMM needs %zu bytes of scratch; the built-in array holds %zu",
                             need, NOALLOC_SCRATCH_BYTES);
    }
    int st = LOFGB_OK;
    void* scratch = nullptr;
    if (M > 0 && N > 0 && K > 0) {
        scratch = noalloc_scratch(&st);
        if (!scratch) return st;
    }
    return lofgb_gemm_f32(A, lda, trans_a, B, ldb, trans_b, D, ldd, M, N, K, accum_mant_bits,
                          LOFGB_RNE, alpha, LOFGB_GEMM_TC, chunk, scratch,
                          scratch ? NOALLOC_SCRATCH_BYTES : 0, stream);
}
