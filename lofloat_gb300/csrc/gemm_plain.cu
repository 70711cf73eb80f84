// gemm_plain.cu — bit-exact emulated-accumulation GEMM on the CUDA cores, and
// the FP64 oracle GEMM used to state the tensor-core form's error.
//
// Replaces the forked-CUTLASS SIMT GEMM (src/cutlass_gemms.cuh:1629-1896,
// launched from src/Lof_kernel.cu:96-154). Semantics of the leaf
// thread::Mma<OpLoFMultiplyAdd> (src/cutlass_gemms.cuh:118-167):
//   acc_0 = +0;  acc_{k+1} = RNE_m(rto_fma(A[i,k], B[k,j], acc_k)), k = 0..K-1
//   D[i,j] = alpha * acc_K
// with rto_fma the round-to-odd FMA of src/cutlass_gemms.cuh:73-88
// (rd = fma.rm, ru = fma.rp, rz = rd >= 0 ? rd : ru, sticky = rd != ru;
// computed here as the same word by rto_word).
// Every output keeps that exact k order, so any M/N tiling is bit-exact;
// K is never split.
//
// Tiling: 128x128 CTA tile, 256 threads, 8x8 outputs per thread, k-tiles of
// 16 staged through double-buffered shared memory (k-major for both
// operands) by 4-byte cp.async copies, zero-filled out of range, so every
// layout / leading dimension / tail works. Two CTAs per SM (<= 128 registers);
// the kernel is bound by ~10 integer+FP instructions per emulated MAC, not by
// memory.
#include <cuda_runtime.h>

#include "gemm_plain_core.cuh"

namespace lofgb {

namespace {

// One 128 x 128 output tile of one GEMM of the batch (HALF: a 64-row tile,
// blockIdx.y counting 64-row steps).
template <int ACC, bool HALF>
__device__ __forceinline__ void plain_tile(float (*As)[BK][BM + PAD], float (*Bs)[BK][BN + PAD],
                                           const float* __restrict__ A, int64_t lda, int ta,
                                           const float* __restrict__ B, int64_t ldb, int tb,
                                           float* __restrict__ D, int64_t ldd, int M, int N,
                                           int K, const AccRound& r, float alpha) {
    constexpr int ROWS = HALF ? BM / 2 : BM;   // A rows staged per k-tile
    constexpr int RI = HALF ? 4 : 8;           // accumulator rows per thread
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int m0 = blockIdx.y * ROWS, n0 = blockIdx.x * BN;

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

    // Next k-tile: 4-byte cp.async copies straight from global memory into
    // the k-major shared tiles (no register staging); out-of-range elements
    // are zero-filled (src-size 0, the source pointer stays in bounds).
    auto issue = [&](int buf, int k0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int idx = tid + q * NT;
            if (q < ROWS * BK / NT) {
                int m, k;
                if (ta) { k = idx / ROWS; m = idx % ROWS; } else { m = idx / BK; k = idx % BK; }
                const int gm = m0 + m, gk = k0 + k;
                const bool va = gm < M && gk < K;
                const float* src = va ? (ta ? A + (int64_t)gk * lda + gm : A + (int64_t)gm * lda + gk) : A;
                cp_async4(smem_addr(&As[buf][k][m]), src, va);
            }
            int n, kb;
            if (tb) { n = idx / BK; kb = idx % BK; } else { kb = idx / BN; n = idx % BN; }
            const int gn = n0 + n, gkb = k0 + kb;
            const bool vb = gn < N && gkb < K;
            const float* srcb = vb ? (tb ? B + (int64_t)gn * ldb + gkb : B + (int64_t)gkb * ldb + gn) : B;
            cp_async4(smem_addr(&Bs[buf][kb][n]), srcb, vb);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    const int ktiles = (K + BK - 1) / BK;
    issue(0, 0);
    for (int kt = 0; kt < ktiles; ++kt) {
        const int buf = kt & 1;
        if (kt + 1 < ktiles) {
            issue(buf ^ 1, (kt + 1) * BK);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        mac_ktile<ACC, RI>(As[buf], Bs[buf], acc, min(BK, K - kt * BK), tx, ty, r);
        __syncthreads();  // buffer `buf` is refilled by the next iteration's issue()
    }

#pragma unroll
    for (int i = 0; i < RI; ++i) {
        const int gm = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int gn = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
            if (gn < N) D[(int64_t)gm * ldd + gn] = __fmul_rn(alpha, acc[i][j]);
        }
    }
}

// blockIdx.z walks the batch (strided-batched GEMM; batch 1 for a single one).
template <int ACC, bool HALF>
__global__ void __launch_bounds__(NT, 2)
gemm_plain_kernel(const float* __restrict__ A, int64_t lda, int64_t sa, int ta,
                  const float* __restrict__ B, int64_t ldb, int64_t sb, int tb,
                  float* __restrict__ D, int64_t ldd, int64_t sd, int M, int N, int K, int batch,
                  const __grid_constant__ AccRound r, float alpha) {
    __shared__ __align__(16) float As[2][BK][BM + PAD];
    __shared__ __align__(16) float Bs[2][BK][BN + PAD];
    for (int z = blockIdx.z; z < batch; z += gridDim.z) {
        plain_tile<ACC, HALF>(As, Bs, A + (int64_t)z * sa, lda, ta, B + (int64_t)z * sb, ldb, tb,
                              D + (int64_t)z * sd, ldd, M, N, K, r, alpha);
        __syncthreads();  // the next batch entry refills the shared tiles
    }
}

// FP64 oracle: D = sum_k (double)A[i,k] * (double)B[k,j], 64x64 tiles,
// 256 threads, 4x4 outputs per thread.
__global__ void __launch_bounds__(256)
gemm_f64_kernel(const float* __restrict__ A, int64_t lda, int ta, const float* __restrict__ B,
                int64_t ldb, int tb, double* __restrict__ D, int64_t ldd, int M, int N, int K) {
    __shared__ double As[16][64 + 1];
    __shared__ double Bs[16][64 + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int idx = tid; idx < 64 * 16; idx += 256) {
            const int m = idx % 64, k = idx / 64;
            const int gm = m0 + m, gk = k0 + k;
            As[k][m] = (gm < M && gk < K) ? (double)(ta ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk]) : 0.0;
            const int n = idx % 64;
            const int gn = n0 + n;
            Bs[k][n] = (gn < N && gk < K) ? (double)(tb ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn]) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; ++k)
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(As[k][ty * 4 + i], Bs[k][tx * 4 + j], acc[i][j]);
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
            if (gm < M && gn < N) D[(int64_t)gm * ldd + gn] = acc[i][j];
        }
}

}  // namespace

int launch_gemm_plain(const float* A, int64_t lda, int64_t sa, int ta, const float* B,
                      int64_t ldb, int64_t sb, int tb, float* D, int64_t ldd, int64_t sd, int M,
                      int N, int K, int batch, int mbits, const RoundPlan* acc_fmt, float alpha,
                      void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // Two CTAs per SM run at once. A single GEMM of fewer 128 x 128 tiles than
    // that runs as 64-row tiles, twice the CTAs for half the work each
    // (1024^2: 128 CTAs instead of 64); every output keeps its whole k order,
    // so the bits do not change.
    const int64_t tiles = (int64_t)((N + BN - 1) / BN) * ((M + BM - 1) / BM);
    const bool half = batch == 1 && tiles < 2 * (int64_t)sm_count();
    dim3 grid((N + BN - 1) / BN, half ? (M + BM / 2 - 1) / (BM / 2) : (M + BM - 1) / BM,
              batch < 65535 ? batch : 65535);
    if (grid.y > 65535) return set_error(LOFGB_ERR_SIZE, "M too large for the plain GEMM grid");
    AccRound r = acc_mant(mbits);
#define LOFGB_PLAIN(ACC)                                                                        \
    do {                                                                                        \
        if (half)                                                                               \
            gemm_plain_kernel<ACC, true><<<grid, NT, 0, st>>>(A, lda, sa, ta, B, ldb, sb, tb, D, \
                                                              ldd, sd, M, N, K, batch, r, alpha); \
        else                                                                                    \
            gemm_plain_kernel<ACC, false><<<grid, NT, 0, st>>>(A, lda, sa, ta, B, ldb, sb, tb, D, \
                                                               ldd, sd, M, N, K, batch, r, alpha); \
    } while (0)
    if (acc_fmt) {
        r.plan = *acc_fmt;
        if (acc_fmt->uni == 1) LOFGB_PLAIN(ACC_UNI);
        else LOFGB_PLAIN(ACC_FMT);
    } else if (r.ro > 0) {
        LOFGB_PLAIN(ACC_MANT);
    } else {
        LOFGB_PLAIN(ACC_NONE);
    }
#undef LOFGB_PLAIN
    return check_launch("gemm_plain_kernel");
}

int launch_gemm_f64(const float* A, int64_t lda, int ta, const float* B, int64_t ldb, int tb,
                    double* D, int64_t ldd, int M, int N, int K, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    if (grid.y > 65535) return set_error(LOFGB_ERR_SIZE, "M too large for the FP64 GEMM grid");
    gemm_f64_kernel<<<grid, 256, 0, st>>>(A, lda, ta, B, ldb, tb, D, ldd, M, N, K);
    return check_launch("gemm_f64_kernel");
}

}  // namespace lofgb
