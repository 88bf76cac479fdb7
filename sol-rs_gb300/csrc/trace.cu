// trace.cu — the `extend` stage: closest hits for a queue of rays. This is
// the work traceRayEXT hands to RT cores in the reference
// (assets/glsl/pathtrace.rgen:65-76); here it is a persistent kernel whose
// warps take 32 rays at a time from an atomic work counter (Aila & Laine
// 2009 persistent threads), so that short and long traversals balance
// across the 152 SMs without a host round trip for the queue length.
#include "bvh8_traverse.cuh"
#include "internal.h"

namespace solrt {

namespace {

constexpr int kExtendBlock = 128;

template <int KIND, bool kCount>
SOLRT_D void trace_one(const DevScene& sc, float4 o, float4 d, HitRec& h, TraceCounters& cnt, uint32_t& ef) {
    if (KIND == SOLRT_BVH8_Q8)
        trace_bvh8<kCount>(sc, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
    else
        trace_bvh2<kCount>(sc, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
}

SOLRT_D void flush_counters(DevStats* stats, const TraceCounters& cnt, uint32_t ef, bool count_nodes) {
    const uint32_t fb = __reduce_add_sync(0xffffffffu, cnt.fallbacks);
    const uint32_t e = __reduce_or_sync(0xffffffffu, ef);
    uint32_t nn = 0, nt = 0;
    if (count_nodes) {
        nn = __reduce_add_sync(0xffffffffu, cnt.nodes);
        nt = __reduce_add_sync(0xffffffffu, cnt.tris);
    }
    if ((threadIdx.x & 31) == 0) {
        if (fb) atomicAdd(&stats->fp64_fallbacks, (unsigned long long)fb);
        if (e) atomicOr(&stats->eflags, e);
        if (nn) atomicAdd(&stats->node_visits, (unsigned long long)nn);
        if (nt) atomicAdd(&stats->tri_tests, (unsigned long long)nt);
    }
}

// Wavefront queue: o_tmin / d_tmax SoA, hit = (t, prim bits, u, v).
template <int KIND, bool kCount>
__global__ void __launch_bounds__(kExtendBlock) k_extend(DevScene sc, const float4* __restrict__ o_tmin,
                                                         const float4* __restrict__ d_tmax, float4* __restrict__ hits,
                                                         const unsigned int* __restrict__ count,
                                                         unsigned int* __restrict__ work, DevStats* stats) {
    const unsigned int n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0 && n) atomicAdd(&stats->segments, (unsigned long long)n);
    TraceCounters cnt{0, 0, 0};
    uint32_t ef = 0;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned int base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const unsigned int i = base + lane;
        if (i < n) {
            HitRec h;
            trace_one<KIND, kCount>(sc, o_tmin[i], d_tmax[i], h, cnt, ef);
            hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
        }
    }
    flush_counters(stats, cnt, ef, kCount);
}

// Ray-file API: AoS solrt_ray (2 float4) -> solrt_hit (float4).
template <int KIND>
__global__ void __launch_bounds__(kExtendBlock) k_trace_rays(DevScene sc, const float4* __restrict__ rays,
                                                             float4* __restrict__ hits, uint32_t n,
                                                             DevStats* stats) {
    TraceCounters cnt{0, 0, 0};
    uint32_t ef = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
    // uniform trip count per warp so the counter flush can use full-warp reductions
    const uint32_t warp_first = first - (threadIdx.x & 31);
    for (uint32_t wb = warp_first; wb < n; wb += stride) {
        const uint32_t i = wb + (threadIdx.x & 31);
        if (i < n) {
            HitRec h;
            trace_one<KIND, false>(sc, rays[2 * (size_t)i], rays[2 * (size_t)i + 1], h, cnt, ef);
            hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
        }
    }
    flush_counters(stats, cnt, ef, false);
}

}  // namespace

int extend_blocks_per_sm(uint32_t kind, bool counters) {
    int b = 0;
    if (kind == SOLRT_BVH8_Q8)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, counters ? k_extend<SOLRT_BVH8_Q8, true> : k_extend<SOLRT_BVH8_Q8, false>, kExtendBlock, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, counters ? k_extend<SOLRT_BVH2, true> : k_extend<SOLRT_BVH2, false>, kExtendBlock, 0);
    return b > 0 ? b : 1;
}

solrt_status launch_extend(Context& ctx, const Scene& sc, const PathQueue& q, float4* hits, const unsigned int* count,
                           unsigned int* work, uint32_t /*capacity*/) {
    const DevScene d = sc.view();
    const int bps = extend_blocks_per_sm(d.bvh_kind, ctx.counters);
    const uint32_t grid = (uint32_t)(ctx.sm_count * bps);
    DevStats* st = ctx.stats.as<DevStats>();
    if (d.bvh_kind == SOLRT_BVH8_Q8) {
        if (ctx.counters)
            k_extend<SOLRT_BVH8_Q8, true><<<grid, kExtendBlock, 0, ctx.stream>>>(d, q.o_tmin, q.d_tmax, hits, count, work, st);
        else
            k_extend<SOLRT_BVH8_Q8, false><<<grid, kExtendBlock, 0, ctx.stream>>>(d, q.o_tmin, q.d_tmax, hits, count, work, st);
    } else {
        if (ctx.counters)
            k_extend<SOLRT_BVH2, true><<<grid, kExtendBlock, 0, ctx.stream>>>(d, q.o_tmin, q.d_tmax, hits, count, work, st);
        else
            k_extend<SOLRT_BVH2, false><<<grid, kExtendBlock, 0, ctx.stream>>>(d, q.o_tmin, q.d_tmax, hits, count, work, st);
    }
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}

solrt_status launch_trace_rays(Context& ctx, const Scene& sc, const solrt_ray* rays, uint32_t n, solrt_hit* hits) {
    if (n == 0) return SOLRT_OK;
    const DevScene d = sc.view();
    const uint32_t want = (n + kExtendBlock - 1) / kExtendBlock;
    const uint32_t cap = (uint32_t)ctx.sm_count * 16u;
    const uint32_t grid = want < cap ? want : cap;
    const float4* r = reinterpret_cast<const float4*>(rays);
    float4* h = reinterpret_cast<float4*>(hits);
    DevStats* st = ctx.stats.as<DevStats>();
    if (d.bvh_kind == SOLRT_BVH8_Q8)
        k_trace_rays<SOLRT_BVH8_Q8><<<grid, kExtendBlock, 0, ctx.stream>>>(d, r, h, n, st);
    else
        k_trace_rays<SOLRT_BVH2><<<grid, kExtendBlock, 0, ctx.stream>>>(d, r, h, n, st);
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}

}  // namespace solrt
