// conv.cu — emulated-accumulation conv2d as an implicit GEMM.
//
// Replaces LoF_conv2d (src/Lof_kernel.cu:156-227), which permutes NCHW / OIHW
// to NHWC / KRSC copies, runs the forked-CUTLASS analytic fprop
// (src/cutlass_conv.cuh:57-184) with the OpLoFMultiplyAdd leaf, syncs the
// device and permutes the result back; and the default im2col path of
// LoF_Conv2d (LoFloat/layers.py:684-713), which materialises F.unfold and
// loops lof_gemm over the batch in Python.
//
// Here the GEMM view is M = output channels (rows of the OIHW weight, read in
// place), N = N·P·Q output pixels, and the reduction index t walks (c, r, s)
// in one of two orders (lofgb_conv_order). No operand is rearranged in
// memory: the loaders decode t into (c, r, s) and the column into
// (image, p, q) with multiply-high divisions and gather straight from the
// NCHW input with zero fill for padding, into the same shared-memory tiles
// and per-MAC core as the plain GEMM (gemm_plain_core.cuh). The output is
// written in NCHW directly.
//
// The tensor-core form splits the weight (in t order) and the implicit im2col
// matrix into BF16 hi / lo operands in the workspace and runs the chunked
// tensor-core GEMM on them (launch_tc_presplit), storing NCHW.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "gemm_plain_core.cuh"
#include "tc_split.cuh"

namespace lofgb {

namespace {

// Division by a run-time invariant d >= 1 for 0 <= n < 2^31 with one
// multiply-high, one add and one shift (Granlund and Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994): l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (mulhi(n, m) + n) >> l.
struct FastDiv {
    uint32_t m, l;
};

FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    f.l = l;
    f.m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    return f;
}

__device__ __forceinline__ int fdiv(int n, FastDiv f) {
    return (int)((__umulhi((uint32_t)n, f.m) + (uint32_t)n) >> f.l);
}

struct ConvGeo {
    const float* x;
    const float* w;
    float* y;
    int C, H, W, K, R, S, P, Q;
    int pad_h, pad_w, str_h, str_w, dil_h, dil_w;
    int RS, CRS;       // R*S and the weight row length C*R*S
    int kseq;          // reduction length in t order
    int L, ncols;      // P*Q output pixels per image, N*P*Q in all
    int64_t HW, CHW;
    FastDiv fd_rs, fd_s, fd_tile, fd_l, fd_q;
};

// t -> (c, r, s) and the weight column c*R*S + r*S + s.
template <int ORDER>
__device__ __forceinline__ void decode_t(const ConvGeo& g, int t, int& c, int& r, int& s,
                                         int& kflat) {
    int rs;
    if (ORDER == LOFGB_CONV_CRS) {
        c = fdiv(t, g.fd_rs);
        rs = t - c * g.RS;
    } else {  // 8-channel tiles outer, then r, s, then the channel within the tile
        const int ct = fdiv(t, g.fd_tile);
        const int rem = t - ct * 8 * g.RS;
        rs = rem >> 3;
        c = ct * 8 + (rem & 7);
    }
    r = fdiv(rs, g.fd_s);
    s = rs - r * g.S;
    kflat = c * g.RS + rs;
}

// Output pixel column -> first input row / column of its window and the
// image's base offset.
__device__ __forceinline__ void decode_col(const ConvGeo& g, int col, int& h0, int& w0,
                                           int64_t& xbase) {
    const int img = fdiv(col, g.fd_l);
    const int l = col - img * g.L;
    const int p = fdiv(l, g.fd_q);
    const int q = l - p * g.Q;
    h0 = p * g.str_h - g.pad_h;
    w0 = q * g.str_w - g.pad_w;
    xbase = (int64_t)img * g.CHW;
}

template <int ACC, int ORDER>
__global__ void __launch_bounds__(NT, 2)
conv_plain_kernel(ConvGeo g, AccRound r, float alpha) {
    __shared__ __align__(16) float As[2][BK][BM + PAD];
    __shared__ __align__(16) float Bs[2][BK][BN + PAD];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

    // The loader mapping of the plain GEMM with row-major A and B: this
    // thread fills A column ka of every k-tile (rows ty + 16q) and B column
    // bn (rows kb0 + 2q), so its B pixel is decoded once.
    const int ka = tid & 15;
    const int bn = tid & (BN - 1);
    const int kb0 = tid >> 7;
    const int col = n0 + bn;
    const bool colv = col < g.ncols;
    int h0 = 0, w0 = 0;
    int64_t xbase = 0;
    if (colv) decode_col(g, col, h0, w0, xbase);

    auto issue = [&](int buf, int k0) {
        {
            const int t = k0 + ka;
            int c, r, s, kf;
            decode_t<ORDER>(g, t, c, r, s, kf);
            const bool tv = t < g.kseq && c < g.C;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int m = ty + 16 * q;
                const int gm = m0 + m;
                const bool va = tv && gm < g.K;
                const float* src = va ? g.w + (int64_t)gm * g.CRS + kf : g.w;
                cp_async4(smem_addr(&As[buf][ka][m]), src, va);
            }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int kb = kb0 + 2 * q;
            const int t = k0 + kb;
            int c, r, s, kf;
            decode_t<ORDER>(g, t, c, r, s, kf);
            const int hh = h0 + r * g.dil_h, ww = w0 + s * g.dil_w;
            const bool vb = colv && t < g.kseq && c < g.C && (unsigned)hh < (unsigned)g.H &&
                            (unsigned)ww < (unsigned)g.W;
            const float* src = vb ? g.x + xbase + (int64_t)c * g.HW + (int64_t)hh * g.W + ww : g.x;
            cp_async4(smem_addr(&Bs[buf][kb][bn]), src, vb);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    const int ktiles = (g.kseq + BK - 1) / BK;
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
        mac_ktile<ACC>(As[buf], Bs[buf], acc, min(BK, g.kseq - kt * BK), tx, ty, r);
        __syncthreads();
    }

    // NCHW store: y[img][k][l]
    int64_t ycol[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int gn = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
        ycol[j] = -1;
        if (gn < g.ncols) {
            const int img = fdiv(gn, g.fd_l);
            ycol[j] = (int64_t)img * g.K * g.L + (gn - img * g.L);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int gm = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        if (gm >= g.K) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (ycol[j] >= 0) g.y[ycol[j] + (int64_t)gm * g.L] = __fmul_rn(alpha, acc[i][j]);
    }
}

// ---- tensor-core operands ------------------------------------------------------
// Weight in t order: row o, column t -> W[o][c][r][s] (0 for channels past C).
// Items are 32-row x 64-t tiles; loads walk t fastest.
template <int ORDER>
__global__ void __launch_bounds__(256)
split_conv_weight_kernel(ConvGeo g, int Mp, int Kp, __nv_bfloat16* __restrict__ hi,
                         __nv_bfloat16* __restrict__ lo, uint32_t* __restrict__ range) {
    __shared__ float tile[32][65];
    ExpRange er;
    const int tiles_k = Kp / 64;
    const int64_t items = (int64_t)(Mp / 32) * tiles_k;
    for (int64_t item = blockIdx.x; item < items; item += gridDim.x) {
        const int r0 = (int)(item / tiles_k) * 32, k0 = (int)(item % tiles_k) * 64;
        for (int i = threadIdx.x; i < 32 * 64; i += 256) {
            const int rr = i / 64, kk = i % 64;
            const int o = r0 + rr, t = k0 + kk;
            float v = 0.0f;
            if (o < g.K && t < g.kseq) {
                int c, r, s, kf;
                decode_t<ORDER>(g, t, c, r, s, kf);
                if (c < g.C) v = g.w[(int64_t)o * g.CRS + kf];
            }
            tile[rr][kk] = v;
        }
        __syncthreads();
        split_store_tile(tile, r0, k0, Mp, Kp, hi, lo, er);
        __syncthreads();
    }
    range_flush(range, er);
}

// Implicit im2col: row j (output pixel), column t -> x[img][c][h][w] or 0.
// Loads walk the pixel fastest (adjacent output columns read adjacent input
// columns at unit stride).
template <int ORDER>
__global__ void __launch_bounds__(256)
split_im2col_kernel(ConvGeo g, int Np, int Kp, __nv_bfloat16* __restrict__ hi,
                    __nv_bfloat16* __restrict__ lo, uint32_t* __restrict__ range) {
    __shared__ float tile[32][65];
    ExpRange er;
    const int tiles_k = Kp / 64;
    const int64_t items = (int64_t)(Np / 32) * tiles_k;
    for (int64_t item = blockIdx.x; item < items; item += gridDim.x) {
        const int r0 = (int)(item / tiles_k) * 32, k0 = (int)(item % tiles_k) * 64;
        const int rr = threadIdx.x & 31;
        const int j = r0 + rr;
        const bool jv = j < g.ncols;
        int h0 = 0, w0 = 0;
        int64_t xbase = 0;
        if (jv) decode_col(g, j, h0, w0, xbase);
        for (int kk = threadIdx.x >> 5; kk < 64; kk += 8) {
            const int t = k0 + kk;
            float v = 0.0f;
            if (jv && t < g.kseq) {
                int c, r, s, kf;
                decode_t<ORDER>(g, t, c, r, s, kf);
                const int hh = h0 + r * g.dil_h, ww = w0 + s * g.dil_w;
                if (c < g.C && (unsigned)hh < (unsigned)g.H && (unsigned)ww < (unsigned)g.W)
                    v = g.x[xbase + (int64_t)c * g.HW + (int64_t)hh * g.W + ww];
            }
            tile[rr][kk] = v;
        }
        __syncthreads();
        split_store_tile(tile, r0, k0, Np, Kp, hi, lo, er);
        __syncthreads();
    }
    range_flush(range, er);
}

int conv_geometry(const lofgb_conv2d_shape* s, int* P, int* Q) {
    if (!s) return set_error(LOFGB_ERR_NULL, "NULL conv2d shape");
    if (s->n < 0 || s->c < 1 || s->h < 1 || s->w < 1 || s->k < 1 || s->r < 1 || s->s < 1)
        return set_error(LOFGB_ERR_SIZE, "conv2d sizes must be positive (n >= 0)");
    if (s->pad_h < 0 || s->pad_w < 0 || s->stride_h < 1 || s->stride_w < 1 || s->dil_h < 1 ||
        s->dil_w < 1)
        return set_error(LOFGB_ERR_SIZE, "conv2d padding >= 0, stride and dilation >= 1");
    const int64_t ph = (int64_t)s->h + 2 * (int64_t)s->pad_h - (int64_t)s->dil_h * (s->r - 1) - 1;
    const int64_t pw = (int64_t)s->w + 2 * (int64_t)s->pad_w - (int64_t)s->dil_w * (s->s - 1) - 1;
    if (ph < 0 || pw < 0)
        return set_error(LOFGB_ERR_SIZE, "non-positive output spatial size");
    *P = (int)(ph / s->stride_h + 1);
    *Q = (int)(pw / s->stride_w + 1);
    return LOFGB_OK;
}

int64_t conv_kseq(const lofgb_conv2d_shape* s, int order) {
    const int64_t rs = (int64_t)s->r * s->s;
    return order == LOFGB_CONV_CRS ? (int64_t)s->c * rs : (int64_t)((s->c + 7) / 8) * 8 * rs;
}

int make_geo(ConvGeo* g, const float* x, const float* w, float* y, const lofgb_conv2d_shape* s,
             int P, int Q, int order) {
    const int64_t L = (int64_t)P * Q, ncols = (int64_t)s->n * L, kseq = conv_kseq(s, order);
    const int64_t limit = (int64_t)1 << 31;
    if (ncols >= limit || kseq >= limit || (int64_t)s->c * s->r * s->s >= limit ||
        (int64_t)s->k * L >= limit)
        return set_error(LOFGB_ERR_SIZE, "conv2d too large (output pixels and reduction < 2^31)");
    g->x = x;
    g->w = w;
    g->y = y;
    g->C = s->c;
    g->H = s->h;
    g->W = s->w;
    g->K = s->k;
    g->R = s->r;
    g->S = s->s;
    g->P = P;
    g->Q = Q;
    g->pad_h = s->pad_h;
    g->pad_w = s->pad_w;
    g->str_h = s->stride_h;
    g->str_w = s->stride_w;
    g->dil_h = s->dil_h;
    g->dil_w = s->dil_w;
    g->RS = s->r * s->s;
    g->CRS = s->c * g->RS;
    g->kseq = (int)kseq;
    g->L = (int)L;
    g->ncols = (int)ncols;
    g->HW = (int64_t)s->h * s->w;
    g->CHW = (int64_t)s->c * g->HW;
    g->fd_rs = make_fastdiv((uint32_t)g->RS);
    g->fd_s = make_fastdiv((uint32_t)s->s);
    g->fd_tile = make_fastdiv((uint32_t)(8 * g->RS));
    g->fd_l = make_fastdiv((uint32_t)L);
    g->fd_q = make_fastdiv((uint32_t)Q);
    return LOFGB_OK;
}

bool overlaps(const void* a, int64_t abytes, const void* b, int64_t bbytes) {
    const char* p = static_cast<const char*>(a);
    const char* q = static_cast<const char*>(b);
    return p < q + bbytes && q < p + abytes;
}

template <int ORDER>
int launch_conv_plain(const ConvGeo& g, int mbits, float alpha, cudaStream_t st) {
    dim3 grid((g.ncols + BN - 1) / BN, (g.K + BM - 1) / BM);
    if (grid.y > 65535) return set_error(LOFGB_ERR_SIZE, "too many output channels for the grid");
    const AccRound r = acc_mant(mbits);
    if (r.ro > 0) conv_plain_kernel<ACC_MANT, ORDER><<<grid, NT, 0, st>>>(g, r, alpha);
    else conv_plain_kernel<ACC_NONE, ORDER><<<grid, NT, 0, st>>>(g, r, alpha);
    return check_launch("conv_plain_kernel");
}

template <int ORDER>
int launch_conv_tc(const ConvGeo& g, int mbits, float alpha, int chunk, void* workspace,
                   size_t workspace_bytes, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const WsLayout w = ws_layout(g.K, g.ncols, g.kseq);
    if (!workspace || workspace_bytes < w.total || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return set_error(LOFGB_ERR_WORKSPACE, "need %zu bytes of 256-byte aligned workspace", w.total);
    uint8_t* ws = static_cast<uint8_t*>(workspace);
    cudaError_t e = cudaMemsetAsync(ws + w.status, 0, WS_HEADER_CLEAR, st);
    if (e != cudaSuccess) return set_error(LOFGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
    auto* range = reinterpret_cast<uint32_t*>(ws + w.range);
    auto* ahi = reinterpret_cast<__nv_bfloat16*>(ws + w.ahi);
    auto* alo = reinterpret_cast<__nv_bfloat16*>(ws + w.alo);
    auto* bhi = reinterpret_cast<__nv_bfloat16*>(ws + w.bhi);
    auto* blo = reinterpret_cast<__nv_bfloat16*>(ws + w.blo);
    const int64_t maxg = (int64_t)sm_count() * 8;
    const int64_t ia = (int64_t)(w.Mp / 32) * (w.Kp / 64), ib = (int64_t)(w.Np / 32) * (w.Kp / 64);
    split_conv_weight_kernel<ORDER><<<(int)(ia < maxg ? ia : maxg), 256, 0, st>>>(g, w.Mp, w.Kp, ahi, alo,
                                                                               range);
    int rc = check_launch("split_conv_weight_kernel");
    if (rc) return rc;
    split_im2col_kernel<ORDER><<<(int)(ib < maxg ? ib : maxg), 256, 0, st>>>(g, w.Np, w.Kp, bhi, blo,
                                                                          range + 3);
    if ((rc = check_launch("split_im2col_kernel"))) return rc;
    return launch_tc_presplit(ws, w, g.y, g.L, 0, g.K, g.ncols, mbits, alpha, chunk, g.L,
                              (int64_t)g.K * g.L, stream);
}

}  // namespace

}  // namespace lofgb

using namespace lofgb;

extern "C" {

int lofgb_conv2d_out_size(const lofgb_conv2d_shape* shape, int32_t* p, int32_t* q) {
    clear_error();
    int P, Q;
    int st = conv_geometry(shape, &P, &Q);
    if (st) return st;
    if (p) *p = P;
    if (q) *q = Q;
    return LOFGB_OK;
}

size_t lofgb_conv2d_workspace_size(const lofgb_conv2d_shape* shape, int order, int variant) {
    int P, Q;
    if (variant != LOFGB_GEMM_TC || conv_geometry(shape, &P, &Q)) return 0;
    if (order != LOFGB_CONV_CRS && order != LOFGB_CONV_TILED8) return 0;
    const int64_t ncols = (int64_t)shape->n * P * Q, kseq = conv_kseq(shape, order);
    if (ncols == 0 || ncols >= ((int64_t)1 << 31) || kseq >= ((int64_t)1 << 31)) return 0;
    return ws_layout(shape->k, (int)ncols, (int)kseq).total;
}

int lofgb_conv2d_f32(const float* input, const float* weight, float* output,
                     const lofgb_conv2d_shape* shape, int accum_mant_bits, int mode,
                     float alpha, int order, int variant, int chunk, void* workspace,
                     size_t workspace_bytes, void* stream) {
    clear_error();
    int P, Q;
    int st = conv_geometry(shape, &P, &Q);
    if (st) return st;
    if (accum_mant_bits < 0 || accum_mant_bits > 23)
        return set_error(LOFGB_ERR_FORMAT, "accum_mant_bits %d outside [0, 23]", accum_mant_bits);
    if (mode != LOFGB_RNE)
        return set_error(LOFGB_ERR_MODE,
                         "accumulator rounding is RNE only (the reference leaf ignores the mode)");
    if (order != LOFGB_CONV_CRS && order != LOFGB_CONV_TILED8)
        return set_error(LOFGB_ERR_UNSUPPORTED, "unknown conv2d order %d", order);
    if (variant != LOFGB_GEMM_PLAIN && variant != LOFGB_GEMM_TC)
        return set_error(LOFGB_ERR_UNSUPPORTED, "unknown conv2d variant %d", variant);
    if (variant == LOFGB_GEMM_TC && (chunk <= 0 || chunk % 16 != 0 || chunk > 256))
        return set_error(LOFGB_ERR_SIZE, "chunk %d must be a multiple of 16 in [16, 256]", chunk);
    if (shape->n == 0) return LOFGB_OK;
    if (!input || !weight || !output) return set_error(LOFGB_ERR_NULL, "NULL conv2d operand");
    const int64_t xb = (int64_t)shape->n * shape->c * shape->h * shape->w * 4;
    const int64_t wb = (int64_t)shape->k * shape->c * shape->r * shape->s * 4;
    const int64_t yb = (int64_t)shape->n * shape->k * P * Q * 4;
    if (overlaps(output, yb, input, xb) || overlaps(output, yb, weight, wb))
        return set_error(LOFGB_ERR_ALIAS, "conv2d output overlaps an operand");
    ConvGeo g;
    if ((st = make_geo(&g, input, weight, output, shape, P, Q, order))) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    if (variant == LOFGB_GEMM_PLAIN)
        return order == LOFGB_CONV_CRS ? launch_conv_plain<LOFGB_CONV_CRS>(g, accum_mant_bits, alpha, cs)
                                       : launch_conv_plain<LOFGB_CONV_TILED8>(g, accum_mant_bits, alpha, cs);
    return order == LOFGB_CONV_CRS
               ? launch_conv_tc<LOFGB_CONV_CRS>(g, accum_mant_bits, alpha, chunk, workspace, workspace_bytes, stream)
               : launch_conv_tc<LOFGB_CONV_TILED8>(g, accum_mant_bits, alpha, chunk, workspace, workspace_bytes, stream);
}

}  // extern "C"
