// grouped_round.cu — one persistent launch that rounds many FP32 tensors, each
// with its own format, mode, scale and RNG stream.
//
// The host splits every tensor into work items of 2^item_shift elements (2^16
// unless the caller picks another size) and
// writes one GroupedTask row per tensor (with the prefix sum of item counts)
// into a table the caller uploads once. CTAs walk the item space with a
// grid-stride loop; each item finds its task by binary search over the
// prefix sums, then rounds its slice with 16-byte vectors. The mode is
// uniform per item, so the specialised element loops for RNE, RTZ,
// round-to-odd and SR-A are chosen once per item; other modes use the
// runtime-dispatched loop. Results are bit-identical to lofgb_round_f32 on
// each task.
#include <cuda_runtime.h>

#include <cstring>

#include "lof_round.cuh"

namespace lofgb {

namespace {

constexpr int GT = 256;
constexpr int GRING = 3;  // cp.async stages per thread (GRING - 1 vectors prefetched)

template <int MODE>
__device__ __forceinline__ uint32_t elem(uint32_t w, const GroupedTask& t, uint64_t idx) {
    if (t.apply_scale) w = __float_as_uint(__fmul_rn(t.scale, __uint_as_float(w)));
    const int mode = MODE >= 0 ? MODE : t.plan.mode;
    const uint64_t r = mode_is_stochastic(mode) ? rng_elem(t.seed, t.offset + idx, t.plan.rng_lg) : 0ull;
    return vr_format<MODE, 32>(w, t.plan, r);
}

template <int MODE, int UNI>
__device__ void run_item(const GroupedTask& t, int64_t e0, int64_t e1, uint4 (*ring)[GT]) {
    const bool aligned =
        ((reinterpret_cast<uintptr_t>(t.in) | reinterpret_cast<uintptr_t>(t.out)) & 15) == 0 &&
        (e0 & 3) == 0;
    if (aligned) {
        const int64_t v0 = e0 >> 2, v1 = e1 >> 2;  // full float4s
        const uint4* vin = reinterpret_cast<const uint4*>(t.in);
        uint4* vout = reinterpret_cast<uint4*>(t.out);
        // per-thread cp.async ring: the loads of the next RING - 1 vectors are
        // in flight (in shared memory, not registers) while one is rounded
        auto vec = [&](int k) { return v0 + threadIdx.x + (int64_t)k * GT; };
#pragma unroll
        for (int k = 0; k < GRING - 1; ++k) {
            if (vec(k) < v1) cp_async16(&ring[k][threadIdx.x], vin + vec(k));
            cp_async_commit();
        }
        int stage = 0;
        for (int k = 0; vec(k) < v1; ++k) {
            const int64_t v = vec(k);
            const int64_t vp = vec(k + GRING - 1);
            if (vp < v1) cp_async16(&ring[stage == 0 ? GRING - 1 : stage - 1][threadIdx.x], vin + vp);
            cp_async_commit();
            cp_async_wait<GRING - 1>();
            const uint4 cur = ring[stage][threadIdx.x];
            stage = stage == GRING - 1 ? 0 : stage + 1;
            const uint64_t i = (uint64_t)v * 4;
            uint32_t w[4] = {cur.x, cur.y, cur.z, cur.w};
            uint64_t r[4] = {0ull, 0ull, 0ull, 0ull};
            const int mode = MODE >= 0 ? MODE : t.plan.mode;
            if (mode_is_stochastic(mode)) rng_elem4(t.seed, t.offset + i, t.plan.rng_lg, r);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (t.apply_scale) w[q] = __float_as_uint(__fmul_rn(t.scale, __uint_as_float(w[q])));
            if constexpr (UNI == 3) {
#pragma unroll
                for (int q = 0; q < 4; ++q) w[q] = vr_uni_sra_f32(w[q], t.plan, r[q]);
            } else if constexpr (UNI == 6) {
#pragma unroll
                for (int q = 0; q < 4; ++q) w[q] = vr_uni_rto_f32(w[q], t.plan);
            } else if constexpr (UNI != 0) {
#pragma unroll
                for (int q = 0; q < 4; ++q) w[q] = vr_uni_f32<MODE, UNI>(w[q], t.plan);
            } else {
                vr_format_f32x4<MODE>(w, t.plan, r);
            }
            __stcs(vout + v, make_uint4(w[0], w[1], w[2], w[3]));
        }
        cp_async_wait<0>();
        for (int64_t i = (v1 << 2) + threadIdx.x; i < e1; i += GT) {
            const uint32_t w = reinterpret_cast<const uint32_t*>(t.in)[i];
            reinterpret_cast<uint32_t*>(t.out)[i] = elem<MODE>(w, t, (uint64_t)i);
        }
    } else {
        for (int64_t i = e0 + threadIdx.x; i < e1; i += GT) {
            const uint32_t w = reinterpret_cast<const uint32_t*>(t.in)[i];
            reinterpret_cast<uint32_t*>(t.out)[i] = elem<MODE>(w, t, (uint64_t)i);
        }
    }
}

__global__ void __launch_bounds__(GT)
grouped_round_kernel(const GroupedTask* __restrict__ tasks, int ntasks, int64_t num_items) {
    __shared__ GroupedTask st;
    __shared__ uint4 ring[GRING][GT];
    for (int64_t item = blockIdx.x; item < num_items; item += gridDim.x) {
        if (threadIdx.x == 0) {
            int lo = 0, hi = ntasks - 1;  // last task with item_begin <= item
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (tasks[mid].item_begin <= item) lo = mid;
                else hi = mid - 1;
            }
            st = tasks[lo];
        }
        __syncthreads();
        const GroupedTask t = st;
        __syncthreads();
        const int64_t e0 = (item - t.item_begin) << t.item_shift;
        const int64_t e1 = min(e0 + ((int64_t)1 << t.item_shift), t.n);
        // uni is 1 only for RNE, 2 only for RTZ / RAFZ / RU / RD, 6 only for
        // round-to-odd; sr_uni only for SR-A
        switch (t.plan.mode) {
        case LOFGB_RNE:
            if (t.plan.uni) run_item<LOFGB_RNE, 1>(t, e0, e1, ring);
            else run_item<LOFGB_RNE, 0>(t, e0, e1, ring);
            break;
        case LOFGB_RTZ:
            if (t.plan.uni) run_item<LOFGB_RTZ, 2>(t, e0, e1, ring);
            else run_item<LOFGB_RTZ, 0>(t, e0, e1, ring);
            break;
        case LOFGB_RTO:
            if (t.plan.uni == 6) run_item<LOFGB_RTO, 6>(t, e0, e1, ring);
            else run_item<LOFGB_RTO, 0>(t, e0, e1, ring);
            break;
        case LOFGB_SR_A:
            if (t.plan.sr_uni) run_item<LOFGB_SR_A, 3>(t, e0, e1, ring);
            else run_item<LOFGB_SR_A, 0>(t, e0, e1, ring);
            break;
        default:
            if (t.plan.uni) run_item<-1, 2>(t, e0, e1, ring);
            else run_item<-1, 0>(t, e0, e1, ring);
            break;
        }
    }
}

}  // namespace

int launch_round_grouped(const void* table, int ntasks, int64_t num_items, void* stream) {
    if (num_items == 0) return LOFGB_OK;
    const int64_t maxg = (int64_t)sm_count() * (2048 / GT);
    const int grid = (int)(num_items < maxg ? num_items : maxg);
    grouped_round_kernel<<<grid, GT, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const GroupedTask*>(table), ntasks, num_items);
    return check_launch("grouped_round_kernel");
}

}  // namespace lofgb

using namespace lofgb;

extern "C" {

size_t lofgb_round_grouped_table_size(int ntasks) {
    return ntasks <= 0 ? 0 : (size_t)ntasks * sizeof(GroupedTask);
}

int lofgb_round_grouped_prepare(const lofgb_round_task* tasks, int ntasks, void* table,
                                size_t table_bytes, int64_t* num_items) {
    return lofgb_round_grouped_prepare_items(tasks, ntasks, table, table_bytes,
                                             (int64_t)1 << GROUPED_ITEM_SHIFT, num_items);
}

int lofgb_round_grouped_prepare_items(const lofgb_round_task* tasks, int ntasks, void* table,
                                      size_t table_bytes, int64_t item_elems, int64_t* num_items) {
    int shift = 0;
    while (shift < 31 && ((int64_t)1 << shift) < item_elems) ++shift;
    if (item_elems < 1024 || item_elems > (1 << 24) || ((int64_t)1 << shift) != item_elems)
        return set_error(LOFGB_ERR_SIZE, "item size %lld: a power of two in [2^10, 2^24]",
                         (long long)item_elems);
    if (ntasks < 0) return set_error(LOFGB_ERR_SIZE, "negative task count");
    if (ntasks > 0 && (!tasks || !table || !num_items))
        return set_error(LOFGB_ERR_NULL, "NULL tasks, table or num_items");
    if (table_bytes < lofgb_round_grouped_table_size(ntasks))
        return set_error(LOFGB_ERR_WORKSPACE, "table needs %zu bytes",
                         lofgb_round_grouped_table_size(ntasks));
    GroupedTask* rows = static_cast<GroupedTask*>(table);
    int64_t items = 0;
    for (int i = 0; i < ntasks; ++i) {
        const lofgb_round_task& t = tasks[i];
        if (t.n < 0) return set_error(LOFGB_ERR_SIZE, "task %d: negative size", i);
        if (t.n > 0 && (!t.in || !t.out)) return set_error(LOFGB_ERR_NULL, "task %d: NULL data", i);
        if (t.n > 0) {
            const char* a = (const char*)t.in;
            const char* b = (const char*)t.out;
            if (a != b && a < b + t.n * 4 && b < a + t.n * 4)
                return set_error(LOFGB_ERR_ALIAS, "task %d: input and output partially overlap", i);
        }
        GroupedTask g;
        memset(&g, 0, sizeof(g));
        int st = make_round_plan(&g.plan, &t.fmt, 32, t.mode, t.stoch_len);
        if (st) {
            char why[256];
            strncpy(why, lofgb_last_error_detail(), sizeof(why) - 1);
            why[sizeof(why) - 1] = 0;
            return set_error(st, "task %d: %s", i, why);
        }
        g.in = t.in;
        g.out = t.out;
        g.n = t.n;
        g.item_begin = items;
        g.scale = t.scale;
        g.apply_scale = t.scale != 1.0f;
        g.item_shift = shift;
        g.seed = t.seed;
        g.offset = t.offset;
        rows[i] = g;
        items += (t.n + ((int64_t)1 << shift) - 1) >> shift;
    }
    if (num_items) *num_items = items;
    return LOFGB_OK;
}

int lofgb_round_grouped_f32(const void* device_table, int ntasks, int64_t num_items,
                            void* stream) {
    if (ntasks < 0 || num_items < 0) return set_error(LOFGB_ERR_SIZE, "negative count");
    if (num_items > 0 && (!device_table || ntasks == 0))
        return set_error(LOFGB_ERR_NULL, "NULL device table");
    if ((reinterpret_cast<uintptr_t>(device_table) & 255) != 0)
        return set_error(LOFGB_ERR_WORKSPACE, "device table must be 256-byte aligned");
    return launch_round_grouped(device_table, ntasks, num_items, stream);
}

}  // extern "C"
