// mx_kernels.cu — MX block rounding with a shared per-block scale.
//
// Replaces run_virtual_mx_round / virtual_mx_round<float,256,MX,NX>
// (src/Lof_kernel.cu:70-94, src/mx_round.cuh:27-214), which uses one element
// per thread, 65535-CTA grid caps and, above 32-element blocks, shared-memory
// or CUB reductions. Here a block of BS contiguous elements lives in the
// registers of BS/4 adjacent lanes (two float4s per lane for BS = 256), so the
// amax is a log2(lanes)-step __shfl_xor butterfly and the whole operation is
// one HBM read and one HBM write per element (8 algorithmic bytes).
//
// Per block (src/mx_round.cuh:52-75):
//   amax  = max |x_i|                 (fmaxf; NaN lanes are ignored)
//   scale = virtual_round(amax * (1/pmn), scale_fmt, {scale_mode, 0})
//   x_i   = scale > 0 ? virtual_round(x_i / scale, elem_fmt, ps) * scale : +0
// When the scale is a power of two in [2^-126, 2^127] the quotient is taken
// as x * (1/scale), which is bit-identical to the IEEE division (both are one
// rounding of the same exact value); other scales use __fdiv_rn.
// Inputs stream through a per-thread cp.async ring; scales are rounded once
// per (slot, block) pair and shuffled back; RNE elements round on the float
// grid (a saturating element format with block 32 folds the NaN case into the
// overflow select). Launched with programmatic dependent launch.
#include <cuda_runtime.h>

#include "lof_round.cuh"
#include "mx_common.cuh"

namespace lofgb {

namespace {

constexpr int MT = 256;
constexpr int RING = 3;  // cp.async stages per thread (RING - 1 runs prefetched)


// Element sources: FP32, or BF16 bit patterns widened to FP32 on load (exact),
// so that rounding a BF16 tensor equals rounding its FP32 copy without
// making one. Raw is what one lane's four elements occupy in memory.
template <typename T> struct Src;
template <> struct Src<float> {
    using Raw = float4;
    static __device__ __forceinline__ float4 cvt(Raw r) { return r; }
    static __device__ __forceinline__ float one(float v) { return v; }
};
template <> struct Src<uint16_t> {
    using Raw = uint2;
    static __device__ __forceinline__ float4 cvt(Raw r) {
        return make_float4(__uint_as_float(r.x << 16), __uint_as_float(r.x & 0xFFFF0000u),
                           __uint_as_float(r.y << 16), __uint_as_float(r.y & 0xFFFF0000u));
    }
    static __device__ __forceinline__ float one(uint16_t v) { return __uint_as_float((uint32_t)v << 16); }
};

template <typename T>
__device__ __forceinline__ void cp_async_raw(void* smem, const T* gmem) {
    if constexpr (sizeof(typename Src<T>::Raw) == 16) {
        cp_async16(smem, gmem);
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(smem)),
                     "l"(gmem)
                     : "memory");
    }
}

template <typename T, bool ALIGNED>
__device__ __forceinline__ float4 load4(const T* in, int64_t e, int64_t n) {
    if (ALIGNED && e + 3 < n)
        return Src<T>::cvt(__ldcs(reinterpret_cast<const typename Src<T>::Raw*>(in + e)));
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (e + 0 < n) v.x = Src<T>::one(__ldcs(in + e + 0));
    if (e + 1 < n) v.y = Src<T>::one(__ldcs(in + e + 1));
    if (e + 2 < n) v.z = Src<T>::one(__ldcs(in + e + 2));
    if (e + 3 < n) v.w = Src<T>::one(__ldcs(in + e + 3));
    return v;
}

template <bool ALIGNED>
__device__ __forceinline__ void store4(float* out, int64_t e, int64_t n, float4 v) {
    if (ALIGNED && e + 3 < n) { __stcs(reinterpret_cast<float4*>(out + e), v); return; }
    if (e + 0 < n) __stcs(out + e + 0, v.x);
    if (e + 1 < n) __stcs(out + e + 1, v.y);
    if (e + 2 < n) __stcs(out + e + 2, v.z);
    if (e + 3 < n) __stcs(out + e + 3, v.w);
}

// Four elements of one block: q = x / scale (x * (1/scale) for power-of-two
// scales, chosen once per warp), round, rescale; a block whose scale is not
// positive gives +0 (src/mx_round.cuh:70-75). UNI != 0: the element format
// takes the whole-range float rounding (RoundPlan::uni).
template <int EMODE, bool FULL, int UNI>
__device__ __forceinline__ float4 quant4(float4 x, const BlockScale& b, const RoundPlan& pe,
                                        uint64_t seed, uint64_t e) {
    const unsigned mask = FULL ? 0xFFFFFFFFu : __activemask();
    float q[4] = {x.x, x.y, x.z, x.w};
    if (__all_sync(mask, b.pow2)) {
#pragma unroll
        for (int i = 0; i < 4; ++i) q[i] = __fmul_rn(q[i], b.inv);
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) q[i] = b.pow2 ? __fmul_rn(q[i], b.inv) : __fdiv_rn(q[i], b.scale);
    }
    uint32_t w[4];
    if constexpr (UNI == 4) {
        // saturating element format: a NaN q comes back as itself and the
        // rescale below turns it into the canonical NaN, as for qNaN
#pragma unroll
        for (int i = 0; i < 4; ++i) w[i] = vr_uni_sat_rne_f32(__float_as_uint(q[i]), pe);
    } else if constexpr (UNI != 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) w[i] = vr_uni_f32<EMODE, UNI>(__float_as_uint(q[i]), pe);
    } else {
        uint64_t r[4] = {0ull, 0ull, 0ull, 0ull};
        if (stoch<EMODE>(pe.mode)) rng_elem4(seed, e, pe.rng_lg, r);
#pragma unroll
        for (int i = 0; i < 4; ++i) w[i] = __float_as_uint(q[i]);
        vr_format_f32x4<EMODE, FULL>(w, pe, r);
    }
    float4 o;
    o.x = b.pos ? __fmul_rn(__uint_as_float(w[0]), b.scale) : 0.0f;
    o.y = b.pos ? __fmul_rn(__uint_as_float(w[1]), b.scale) : 0.0f;
    o.z = b.pos ? __fmul_rn(__uint_as_float(w[2]), b.scale) : 0.0f;
    o.w = b.pos ? __fmul_rn(__uint_as_float(w[3]), b.scale) : 0.0f;
    return o;
}

// BS: block size; VPT float4s per lane per block; L lanes per block.
// Geometry of one block size: BS elements per block, VPT float4s per lane per
// block, L lanes per block, SLOT elements per warp per slot, U slots per warp
// iteration; NB blocks per slot and P = U * NB (slot, block) pairs per
// iteration. With P <= 32 the scales are computed transposed (one pair per
// lane).
template <int BS>
struct MxGeo {
    static constexpr int VPT = BS >= 256 ? BS / 128 : 1;
    static constexpr int L = BS / (4 * VPT);
    static constexpr int SLOT = 128 * VPT;
    static constexpr int U = VPT == 1 ? 4 : 2;
    static constexpr int NB = 32 / L;
    static constexpr int P = U * NB;
    static constexpr bool TRANSPOSED = VPT == 1 && P <= 32;
    static_assert(L >= 1 && L <= 32 && (L & (L - 1)) == 0, "lanes per block");
};

// U full slots starting at slot s0, already in registers.
template <int BS, int EMODE, int SMODE, int UNI>
__device__ __forceinline__ void mx_full_slots(const float4 (&v)[MxGeo<BS>::U][MxGeo<BS>::VPT],
                                              float* out, int64_t s0, int lane, const RoundPlan& pe,
                                              const RoundPlan& ps, float inv_pmn, uint64_t seed,
                                              uint64_t offset) {
    using G = MxGeo<BS>;
    constexpr int U = G::U, VPT = G::VPT, L = G::L, NB = G::NB, P = G::P, SLOT = G::SLOT;
    float amax[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        amax[u] = 0.0f;
#pragma unroll
        for (int j = 0; j < VPT; ++j)
            amax[u] = fmaxf(amax[u], fmaxf(fmaxf(fabsf(v[u][j].x), fabsf(v[u][j].y)),
                                           fmaxf(fabsf(v[u][j].z), fabsf(v[u][j].w))));
#pragma unroll
        for (int off = L / 2; off > 0; off >>= 1)
            amax[u] = fmaxf(amax[u], __shfl_xor_sync(0xFFFFFFFFu, amax[u], off));
    }
    if constexpr (G::TRANSPOSED) {
        // one scale per lane for the P (slot, block) pairs of this iteration
        // instead of one per lane and slot: lane j takes pair j mod P, gathers
        // its amax, rounds the scale, and every lane then fetches the scale
        // bits of its own blocks
        const int pj = lane % P;
        const int uj = pj / NB, bj = pj % NB;
        float aj = 0.0f;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const float g = __shfl_sync(0xFFFFFFFFu, amax[u], bj * L);
            aj = u == uj ? g : aj;
        }
        const int64_t blkj = (s0 + uj) * SLOT + (int64_t)bj * BS;
        const uint32_t sbj = __float_as_uint(block_scale<SMODE>(aj, ps, inv_pmn, seed, offset + blkj).scale);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t sb = __shfl_sync(0xFFFFFFFFu, sbj, u * NB + lane / L);
            const BlockScale b = scale_from_bits(sb);
            const int64_t e = (s0 + u) * SLOT + lane * 4;
            __stcs(reinterpret_cast<float4*>(out + e), quant4<EMODE, true, UNI>(v[u][0], b, pe, seed, offset + (uint64_t)e));
        }
    } else {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t blk0 = (s0 + u) * SLOT + (int64_t)(lane / L) * BS;
            const BlockScale b = block_scale<SMODE>(amax[u], ps, inv_pmn, seed, offset + blk0);
#pragma unroll
            for (int j = 0; j < VPT; ++j) {
                const int64_t e = (s0 + u) * SLOT + j * 128 + lane * 4;
                __stcs(reinterpret_cast<float4*>(out + e), quant4<EMODE, true, UNI>(v[u][j], b, pe, seed, offset + (uint64_t)e));
            }
        }
    }
}

// The float-grid instantiations fit 5 CTAs of 256 threads per SM (<= 48
// registers, the occupancy the HBM stream needs); the general ones would
// spill under that bound.
template <typename T, int BS, int EMODE, int SMODE, bool ALIGNED, int UNI = 0>
__global__ void __launch_bounds__(MT, UNI != 0 ? 5 : 1)
mx_kernel(const T* in, float* out, int64_t n, RoundPlan pe, RoundPlan ps, float inv_pmn,
          uint64_t seed, uint64_t offset) {
    pdl_wait();
    using G = MxGeo<BS>;
    constexpr int U = G::U, VPT = G::VPT, L = G::L, SLOT = G::SLOT;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * MT + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * MT) >> 5;
    const int64_t nslots = (n + SLOT - 1) / SLOT;
    const int64_t full_slots = n / SLOT;  // slots entirely inside the tensor
    const int64_t step = nwarps * U;
    int64_t s0 = warp * U;
    if (ALIGNED) {
        // common case: runs of U full slots, no bounds checks. Each thread
        // streams its own 16-byte pieces of the next RING - 1 runs into
        // shared memory with cp.async while it rounds the current run, so the
        // HBM reads in flight do not occupy registers; a thread only reads
        // back what it copied itself, so no CTA barrier is needed.
        __shared__ typename Src<T>::Raw ring[RING][U * VPT][MT];
        auto issue = [&](int stage, int64_t s) {
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int j = 0; j < VPT; ++j)
                    cp_async_raw(&ring[stage][u * VPT + j][threadIdx.x],
                                 in + (s + u) * SLOT + j * 128 + lane * 4);
        };
        int64_t sp = s0;  // next run to prefetch
#pragma unroll
        for (int k = 0; k < RING - 1; ++k, sp += step) {
            if (sp + U <= full_slots) issue(k, sp);
            cp_async_commit();
        }
        int stage = 0;
        for (; s0 + U <= full_slots; s0 += step, sp += step) {
            if (sp + U <= full_slots) issue(stage == 0 ? RING - 1 : stage - 1, sp);
            cp_async_commit();
            cp_async_wait<RING - 1>();  // this run's group has landed
            float4 v[U][VPT];
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int j = 0; j < VPT; ++j) v[u][j] = Src<T>::cvt(ring[stage][u * VPT + j][threadIdx.x]);
            mx_full_slots<BS, EMODE, SMODE, UNI>(v, out, s0, lane, pe, ps, inv_pmn, seed, offset);
            stage = stage == RING - 1 ? 0 : stage + 1;
        }
        cp_async_wait<0>();
    }
    // partial runs (and every run of a misaligned tensor)
    for (; s0 < nslots; s0 += step) {
        float4 v[U][VPT];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int j = 0; j < VPT; ++j) {
                const int64_t e = (s0 + u) * SLOT + j * 128 + lane * 4;
                v[u][j] = (s0 + u < nslots) ? load4<T, ALIGNED>(in, e, n) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (s0 + u >= nslots) break;  // warp-uniform
            float amax = 0.0f;
#pragma unroll
            for (int j = 0; j < VPT; ++j)
                amax = fmaxf(amax, fmaxf(fmaxf(fabsf(v[u][j].x), fabsf(v[u][j].y)),
                                         fmaxf(fabsf(v[u][j].z), fabsf(v[u][j].w))));
#pragma unroll
            for (int off = L / 2; off > 0; off >>= 1)
                amax = fmaxf(amax, __shfl_xor_sync(0xFFFFFFFFu, amax, off));
            const int64_t blk0 = (s0 + u) * SLOT + (int64_t)(lane / L) * BS;
            const BlockScale b = block_scale<SMODE>(amax, ps, inv_pmn, seed, offset + blk0);
#pragma unroll
            for (int j = 0; j < VPT; ++j) {
                const int64_t e = (s0 + u) * SLOT + j * 128 + lane * 4;
                const uint64_t g = offset + (uint64_t)e;
                store4<ALIGNED>(out, e, n, quant4<EMODE, false, UNI>(v[u][j], b, pe, seed, g));
            }
        }
    }
}

template <int BS>
int launch_bs(const float* in, float* out, int64_t n, const RoundPlan& pe, const RoundPlan& ps,
              float inv_pmn, uint64_t seed, uint64_t offset, cudaStream_t st);

// BF16 sources: the float-grid RNE instantiations when the buffers allow
// vectors (input 8-byte, output 16-byte aligned), the general one otherwise.
template <int BS>
int launch_bs_bf16(const uint16_t* in, float* out, int64_t n, const RoundPlan& pe,
                   const RoundPlan& ps, float inv_pmn, uint64_t seed, uint64_t offset,
                   cudaStream_t st) {
    constexpr int VPT = BS >= 256 ? BS / 128 : 1;
    constexpr int SLOT = 128 * VPT;
    constexpr int U = VPT == 1 ? 4 : 2;
    const int64_t warps_needed = ((n + SLOT - 1) / SLOT + U - 1) / U;
    int64_t g = (warps_needed + (MT / 32) - 1) / (MT / 32);
    const int maxg = sm_count() * (2048 / MT);
    const int grid = (int)(g < 1 ? 1 : (g < maxg ? g : maxg));
    const bool aligned = ((reinterpret_cast<uintptr_t>(in) & 7) | (reinterpret_cast<uintptr_t>(out) & 15)) == 0;
    const bool rne = pe.mode == LOFGB_RNE && ps.mode == LOFGB_RNE && pe.uni == 1;
    if (aligned && rne && BS == 32 && pe.saturating)
        launch_pdl(mx_kernel<uint16_t, 32, LOFGB_RNE, LOFGB_RNE, true, 4>, grid, MT, 0, st, in, out, n,
                   pe, ps, inv_pmn, seed, offset);
    else if (aligned && rne)
        launch_pdl(mx_kernel<uint16_t, BS, LOFGB_RNE, LOFGB_RNE, true, 1>, grid, MT, 0, st, in, out, n,
                   pe, ps, inv_pmn, seed, offset);
    else
        launch_pdl(mx_kernel<uint16_t, BS, -1, -1, false>, grid, MT, 0, st, in, out, n, pe, ps,
                   inv_pmn, seed, offset);
    return check_launch("mx_kernel(bf16)");
}

template <int BS>
int launch_bs(const float* in, float* out, int64_t n, const RoundPlan& pe, const RoundPlan& ps,
              float inv_pmn, uint64_t seed, uint64_t offset, cudaStream_t st) {
    constexpr int VPT = BS >= 256 ? BS / 128 : 1;
    constexpr int SLOT = 128 * VPT;
    constexpr int U = VPT == 1 ? 4 : 2;
    const int64_t nslots = (n + SLOT - 1) / SLOT;
    const int64_t warps_needed = (nslots + U - 1) / U;
    int64_t g = (warps_needed + (MT / 32) - 1) / (MT / 32);
    const int maxg = sm_count() * (2048 / MT);
    const int grid = (int)(g < 1 ? 1 : (g < maxg ? g : maxg));
    const bool aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
    if (!aligned)
        launch_pdl(mx_kernel<float, BS, -1, -1, false>, grid, MT, 0, st, in, out, n, pe, ps, inv_pmn, seed, offset);
    else if (BS == 32 && pe.mode == LOFGB_RNE && ps.mode == LOFGB_RNE && pe.uni == 1 && pe.saturating)
        launch_pdl(mx_kernel<float, 32, LOFGB_RNE, LOFGB_RNE, true, 4>, grid, MT, 0, st, in, out, n, pe, ps, inv_pmn, seed, offset);
    else if (pe.mode == LOFGB_RNE && ps.mode == LOFGB_RNE && pe.uni == 1)
        launch_pdl(mx_kernel<float, BS, LOFGB_RNE, LOFGB_RNE, true, 1>, grid, MT, 0, st, in, out, n, pe, ps, inv_pmn, seed, offset);
    else if (pe.mode == LOFGB_RNE && ps.mode == LOFGB_RNE)
        launch_pdl(mx_kernel<float, BS, LOFGB_RNE, LOFGB_RNE, true>, grid, MT, 0, st, in, out, n, pe, ps, inv_pmn, seed, offset);
    else if (ps.mode == LOFGB_RNE)
        launch_pdl(mx_kernel<float, BS, -1, LOFGB_RNE, true>, grid, MT, 0, st, in, out, n, pe, ps, inv_pmn, seed, offset);
    else
        launch_pdl(mx_kernel<float, BS, -1, -1, true>, grid, MT, 0, st, in, out, n, pe, ps, inv_pmn, seed, offset);
    return check_launch("mx_kernel");
}

}  // namespace

int launch_mx(const float* in, float* out, int64_t n, int block, const RoundPlan& pe,
              const RoundPlan& ps, float pmn, float inv_pmn, uint64_t seed, uint64_t offset,
              void* stream) {
    (void)pmn;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (block) {
    case 8: return launch_bs<8>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 16: return launch_bs<16>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 32: return launch_bs<32>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 64: return launch_bs<64>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 128: return launch_bs<128>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 256: return launch_bs<256>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    default: return set_error(LOFGB_ERR_BLOCK, "unsupported MX block size %d", block);
    }
}

int launch_mx_bf16(const uint16_t* in, float* out, int64_t n, int block, const RoundPlan& pe,
                   const RoundPlan& ps, float inv_pmn, uint64_t seed, uint64_t offset,
                   void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (block) {
    case 8: return launch_bs_bf16<8>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 16: return launch_bs_bf16<16>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 32: return launch_bs_bf16<32>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 64: return launch_bs_bf16<64>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 128: return launch_bs_bf16<128>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    case 256: return launch_bs_bf16<256>(in, out, n, pe, ps, inv_pmn, seed, offset, st);
    default: return set_error(LOFGB_ERR_BLOCK, "unsupported MX block size %d", block);
    }
}

}  // namespace lofgb
