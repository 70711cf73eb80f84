// round_kernels.cu — elementwise virtual rounding (format and mantissa-only
// overloads) for f32 / f64 / f16 sources.
//
// Replaces round_fp_params_kernel / round_mantissa_kernel
// (src/Lof_kernel.cu:37-60): those launch one element per thread with scalar
// loads and, for the format overload, round in place on a clone of the input.
// Here each thread moves 16-byte vectors (4 f32, 2 f64 or 8 f16 values), RU of
// them per iteration, over a grid-stride loop sized to the SM count; the next
// iterations' vectors stream into a per-thread cp.async ring in shared memory
// while the current one is rounded. f32 sources in RNE, the directed modes,
// round-to-odd and SR-A round on the float grid (lof_round.cuh vr_uni_*); the
// other modes and sources take the integer rounding core. Launched with
// programmatic dependent launch. The output is written out of place (in ==
// out also works). HBM-bound: 2 * sizeof(T) algorithmic bytes per element.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lof_round.cuh"

namespace lofgb {

namespace {

constexpr int RT = 256;  // threads per CTA
constexpr int RU = 4;    // 16-byte vectors per thread per iteration
constexpr int RING = 3;  // cp.async stages per thread (RING - 1 iterations prefetched)
static_assert(RU % 2 == 0, "SR-A draws are shared over pairs of steps");


struct ScaleArg {
    float f;      // f32 scale, or the f16 scale widened to float
    double d;     // f64 scale
    int apply;    // scale != 1 in the source type
};

template <int MODE>
__device__ __forceinline__ bool needs_rng(const RoundPlan& p) {
    if (MODE >= 0) return MODE == LOFGB_SR_A || MODE == LOFGB_SR_B || MODE == LOFGB_SR_C ||
                          MODE == LOFGB_SR_D || MODE == LOFGB_TRUE_SR || MODE == LOFGB_PROB;
    return mode_is_stochastic(p.mode);
}

// One source word: optional fused scale (in the source type, as
// src/Lof_kernel.cu:40-41 and :52-53 do), then the rounding.
template <int MODE, int W, bool FMT, bool SCALED = true>
__device__ __forceinline__ typename Src<W>::U process(typename Src<W>::U w, const RoundPlan& p,
                                                      const ScaleArg& s, uint64_t seed,
                                                      uint64_t idx) {
    using U = typename Src<W>::U;
    if (SCALED && s.apply) {
        if constexpr (W == 32) {
            w = __float_as_uint(__fmul_rn(s.f, __uint_as_float(w)));
        } else if constexpr (W == 64) {
            w = (U)__double_as_longlong(__dmul_rn(s.d, __longlong_as_double((long long)w)));
        } else {
            const float prod = __fmul_rn(s.f, __half2float(__ushort_as_half((unsigned short)w)));
            w = (U)__half_as_ushort(__float2half_rn(prod));
        }
    }
    const uint64_t r = needs_rng<MODE>(p) ? rng_elem(seed, idx, p.rng_lg) : 0ull;
    if constexpr (FMT) return vr_format<MODE, W>(w, p, r);
    else return vr_mantissa<MODE, W>(w, p.d, p.mode, p.len, r);
}

template <int MODE, int W, bool FMT, bool SCALED, int UNI = 0>
__global__ void __launch_bounds__(RT)
round_vec_kernel(const uint4* vin, uint4* vout, int64_t n,
                 RoundPlan p, ScaleArg s, uint64_t seed, uint64_t offset) {
    pdl_wait();
    using U = typename Src<W>::U;
    constexpr int EPV = 128 / W;  // elements per 16-byte vector
    const int64_t nvec = n / EPV;
    const int64_t stride = (int64_t)gridDim.x * RT * RU;
    // one 16-byte vector: element index vi * EPV .. vi * EPV + EPV - 1; `full`:
    // every lane of the warp is here (the voted rare-branch path may use the
    // full mask)
    auto round_vec = [&](const uint4& vv, int64_t vi, bool full) -> uint4 {
        const uint64_t e0 = offset + (uint64_t)vi * EPV;
        uint4 o;
        if constexpr (W == 32 && FMT && (UNI == 3 || UNI == 5)) {
            // SR-A by float arithmetic (RoundPlan::sr_uni); UNI 5: saturating format
            uint32_t w[4] = {vv.x, vv.y, vv.z, vv.w};
            uint64_t r[4];
            rng_elem4(seed, e0, p.rng_lg, r);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (SCALED) w[q] = __float_as_uint(__fmul_rn(s.f, __uint_as_float(w[q])));
                w[q] = vr_uni_sra_f32<UNI == 5>(w[q], p, r[q]);
            }
            o = make_uint4(w[0], w[1], w[2], w[3]);
        } else if constexpr (W == 32 && FMT && UNI == 6) {
            uint32_t w[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (SCALED) w[q] = __float_as_uint(__fmul_rn(s.f, __uint_as_float(w[q])));
                w[q] = vr_uni_rto_f32(w[q], p);
            }
            o = make_uint4(w[0], w[1], w[2], w[3]);
        } else if constexpr (W == 32 && FMT && UNI != 0) {
            uint32_t w[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (SCALED) w[q] = __float_as_uint(__fmul_rn(s.f, __uint_as_float(w[q])));
                w[q] = vr_uni_f32<MODE, UNI>(w[q], p);
            }
            o = make_uint4(w[0], w[1], w[2], w[3]);
        } else if constexpr (W == 32 && FMT) {
            uint32_t w[4] = {vv.x, vv.y, vv.z, vv.w};
            uint64_t r[4] = {0ull, 0ull, 0ull, 0ull};
            if (needs_rng<MODE>(p)) rng_elem4(seed, e0, p.rng_lg, r);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (SCALED) w[q] = __float_as_uint(__fmul_rn(s.f, __uint_as_float(w[q])));
            if (full) vr_format_f32x4<MODE, true>(w, p, r);
            else vr_format_f32x4<MODE, false>(w, p, r);
            o = make_uint4(w[0], w[1], w[2], w[3]);
        } else if constexpr (W == 32) {
            o.x = process<MODE, 32, FMT, SCALED>(vv.x, p, s, seed, e0 + 0);
            o.y = process<MODE, 32, FMT, SCALED>(vv.y, p, s, seed, e0 + 1);
            o.z = process<MODE, 32, FMT, SCALED>(vv.z, p, s, seed, e0 + 2);
            o.w = process<MODE, 32, FMT, SCALED>(vv.w, p, s, seed, e0 + 3);
        } else if constexpr (W == 64) {
            const uint64_t a = ((uint64_t)vv.y << 32) | vv.x;
            const uint64_t b = ((uint64_t)vv.w << 32) | vv.z;
            const uint64_t ra = process<MODE, 64, FMT, SCALED>(a, p, s, seed, e0 + 0);
            const uint64_t rb = process<MODE, 64, FMT, SCALED>(b, p, s, seed, e0 + 1);
            o.x = (uint32_t)ra;
            o.y = (uint32_t)(ra >> 32);
            o.z = (uint32_t)rb;
            o.w = (uint32_t)(rb >> 32);
        } else {
            const uint32_t in4[4] = {vv.x, vv.y, vv.z, vv.w};
            uint32_t out4[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const U lo = process<MODE, 16, FMT, SCALED>(in4[q] & 0xFFFFu, p, s, seed, e0 + 2 * q);
                const U hi = process<MODE, 16, FMT, SCALED>(in4[q] >> 16, p, s, seed, e0 + 2 * q + 1);
                out4[q] = (lo & 0xFFFFu) | (hi << 16);
            }
            o = make_uint4(out4[0], out4[1], out4[2], out4[3]);
        }
        return o;
    };
    int64_t base = (int64_t)blockIdx.x * RT * RU;
    {
        // full iterations: each thread streams its own vectors of the next
        // RING - 1 iterations into shared memory with cp.async while it
        // rounds the current one (reads in flight without registers; a thread
        // reads back only what it copied, so no CTA barrier)
        __shared__ uint4 ring[RING][RU][RT];
        auto issue = [&](int stage, int64_t b) {
#pragma unroll
            for (int u = 0; u < RU; ++u) cp_async16(&ring[stage][u][threadIdx.x], vin + b + u * RT + threadIdx.x);
        };
        int64_t bp = base;
#pragma unroll
        for (int k = 0; k < RING - 1; ++k, bp += stride) {
            if (bp + RT * RU <= nvec) issue(k, bp);
            cp_async_commit();
        }
        // SR-A with 8-bit random lanes: one 64-bit draw serves 8 elements,
        // two neighbouring lanes' vectors. With the element offset a multiple
        // of 8, each lane computes one draw (its pair's, of step u or u + 1)
        // and the pair shares it by shuffles, half the draws of rng_elem4.
        constexpr bool SRA = W == 32 && FMT && (UNI == 3 || UNI == 5);
        const bool pair_draws = SRA && p.rng_lg == 3 && (offset & 7u) == 0;
        const int lane = threadIdx.x & 31;
        int stage = 0;
        for (; base + RT * RU <= nvec; base += stride, bp += stride) {
            if (bp + RT * RU <= nvec) issue(stage == 0 ? RING - 1 : stage - 1, bp);
            cp_async_commit();
            cp_async_wait<RING - 1>();
            if (SRA && pair_draws) {
#pragma unroll
                for (int u = 0; u < RU; u += 2) {
                    const int64_t vj = base + (u + (lane & 1)) * RT + (threadIdx.x & ~1);
                    const uint64_t w = rng64(seed, (offset + (uint64_t)vj * 4) >> 3);
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const uint64_t wu = __shfl_sync(0xFFFFFFFFu, w, h ? (lane | 1) : (lane & ~1));
                        const uint32_t half = (lane & 1) ? (uint32_t)(wu >> 32) : (uint32_t)wu;
                        const int64_t vi = base + (u + h) * RT + threadIdx.x;
                        const uint4 vv = ring[stage][u + h][threadIdx.x];
                        uint32_t x[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            if (SCALED) x[q] = __float_as_uint(__fmul_rn(s.f, __uint_as_float(x[q])));
                            x[q] = vr_uni_sra_f32<UNI == 5>(x[q], p, (uint64_t)(half >> (8 * q)));
                        }
                        __stcs(vout + vi, make_uint4(x[0], x[1], x[2], x[3]));
                    }
                }
            } else {
#pragma unroll
                for (int u = 0; u < RU; ++u) {
                    const int64_t vi = base + u * RT + threadIdx.x;
                    __stcs(vout + vi, round_vec(ring[stage][u][threadIdx.x], vi, true));
                }
            }
            stage = stage == RING - 1 ? 0 : stage + 1;
        }
        cp_async_wait<0>();
    }
    // the last, partial iteration of this CTA
    for (; base < nvec; base += stride) {
#pragma unroll
        for (int u = 0; u < RU; ++u) {
            const int64_t vi = base + u * RT + threadIdx.x;
            if (vi < nvec) __stcs(vout + vi, round_vec(__ldcs(vin + vi), vi, false));
        }
    }
    // tail of fewer than EPV elements
    if (blockIdx.x == 0) {
        for (int64_t i = nvec * EPV + threadIdx.x; i < n; i += RT) {
            if constexpr (W == 32) {
                const uint32_t w = reinterpret_cast<const uint32_t*>(vin)[i];
                reinterpret_cast<uint32_t*>(vout)[i] =
                    process<MODE, 32, FMT, SCALED>(w, p, s, seed, offset + i);
            } else if constexpr (W == 64) {
                const uint64_t w = reinterpret_cast<const uint64_t*>(vin)[i];
                reinterpret_cast<uint64_t*>(vout)[i] =
                    process<MODE, 64, FMT, SCALED>(w, p, s, seed, offset + i);
            } else {
                const uint32_t w = reinterpret_cast<const uint16_t*>(vin)[i];
                reinterpret_cast<uint16_t*>(vout)[i] =
                    (uint16_t)process<MODE, 16, FMT, SCALED>(w, p, s, seed, offset + i);
            }
        }
    }
}

// Fallback for pointers that are not 16-byte aligned: one element per thread.
template <int W, bool FMT>
__global__ void __launch_bounds__(RT)
round_scalar_kernel(const void* in, void* out, int64_t n, RoundPlan p,
                    ScaleArg s, uint64_t seed, uint64_t offset) {
    pdl_wait();
    for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n; i += (int64_t)gridDim.x * RT) {
        if constexpr (W == 32) {
            const uint32_t w = static_cast<const uint32_t*>(in)[i];
            static_cast<uint32_t*>(out)[i] = process<-1, 32, FMT>(w, p, s, seed, offset + i);
        } else if constexpr (W == 64) {
            const uint64_t w = static_cast<const uint64_t*>(in)[i];
            static_cast<uint64_t*>(out)[i] = process<-1, 64, FMT>(w, p, s, seed, offset + i);
        } else {
            const uint32_t w = static_cast<const uint16_t*>(in)[i];
            static_cast<uint16_t*>(out)[i] =
                (uint16_t)process<-1, 16, FMT>(w, p, s, seed, offset + i);
        }
    }
}

template <int W, bool FMT>
int launch_w(const void* in, void* out, int64_t n, const RoundPlan& p, const ScaleArg& s,
             uint64_t seed, uint64_t offset, cudaStream_t st) {
    const bool aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
    const int maxg = sm_count() * (2048 / RT);
    if (!aligned) {
        int64_t g = (n + RT - 1) / RT;
        const int grid = (int)(g < maxg ? g : maxg);
        launch_pdl(round_scalar_kernel<W, FMT>, grid, RT, 0, st, in, out, n, p, s, seed, offset);
        return check_launch("round_scalar_kernel");
    }
    constexpr int EPV = 128 / W;
    const int64_t nvec = n / EPV;
    int64_t g = (nvec + RT * RU - 1) / (RT * RU);
    if (g < 1) g = 1;
    const int grid = (int)(g < maxg ? g : maxg);
    auto vi = static_cast<const uint4*>(in);
    auto vo = static_cast<uint4*>(out);
#define LOFGB_RVU(M, UNI)                                                                    \
    (s.apply ? launch_pdl(round_vec_kernel<M, W, FMT, true, UNI>, grid, RT, 0, st, vi, vo, n, p, s, seed, offset) \
             : launch_pdl(round_vec_kernel<M, W, FMT, false, UNI>, grid, RT, 0, st, vi, vo, n, p, s, seed, offset))
#define LOFGB_RV(M) LOFGB_RVU(M, 0)
    if constexpr (W == 32 && FMT) {
        // whole-range float rounding: RNE (uni 1) or the directed modes (uni 2)
        if (p.uni == 1) {
            LOFGB_RVU(LOFGB_RNE, 1);
            return check_launch("round_vec_kernel");
        }
        if (p.uni == 2) {
            if (p.mode == LOFGB_RTZ) LOFGB_RVU(LOFGB_RTZ, 2);
            else LOFGB_RVU(-1, 2);
            return check_launch("round_vec_kernel");
        }
        if (p.uni == 6) {
            LOFGB_RVU(LOFGB_RTO, 6);
            return check_launch("round_vec_kernel");
        }
        if (p.sr_uni) {
            if (p.saturating) LOFGB_RVU(LOFGB_SR_A, 5);
            else LOFGB_RVU(LOFGB_SR_A, 3);
            return check_launch("round_vec_kernel");
        }
    }
    // mode-specialised element loops for f32 sources; f64 and f16 sources
    // share the runtime-mode loop
    if constexpr (W == 32) {
        switch (p.mode) {
        case LOFGB_RNE: LOFGB_RV(LOFGB_RNE); break;
        case LOFGB_RTZ: LOFGB_RV(LOFGB_RTZ); break;
        case LOFGB_RTO: LOFGB_RV(LOFGB_RTO); break;
        case LOFGB_SR_A: LOFGB_RV(LOFGB_SR_A); break;
        default: LOFGB_RV(-1); break;
        }
    } else {
        LOFGB_RV(-1);
    }
#undef LOFGB_RV
#undef LOFGB_RVU
    return check_launch("round_vec_kernel");
}

}  // namespace

int launch_round(int src_bits, bool fmt, const void* in, void* out, int64_t n,
                 const RoundPlan& p, double scale, uint64_t seed, uint64_t offset,
                 void* stream) {
    ScaleArg s;
    s.d = scale;
    s.f = (float)scale;
    if (src_bits == 16) {  // the scale is narrowed to half first (c10::Half)
        s.f = __half2float(__float2half_rn((float)scale));
        s.apply = s.f != 1.0f;
    } else if (src_bits == 32) {
        s.apply = s.f != 1.0f;
    } else {
        s.apply = s.d != 1.0;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (src_bits == 32) return fmt ? launch_w<32, true>(in, out, n, p, s, seed, offset, st)
                                   : launch_w<32, false>(in, out, n, p, s, seed, offset, st);
    if (src_bits == 64) return fmt ? launch_w<64, true>(in, out, n, p, s, seed, offset, st)
                                   : launch_w<64, false>(in, out, n, p, s, seed, offset, st);
    return fmt ? launch_w<16, true>(in, out, n, p, s, seed, offset, st)
               : launch_w<16, false>(in, out, n, p, s, seed, offset, st);
}

}  // namespace lofgb
