// trace.cu — the `extend` stage: closest hits for a queue of rays. This is
// the work traceRayEXT hands to RT cores in the reference
// (assets/glsl/pathtrace.rgen:65-76). Persistent kernels: one grid of
// (SMs x resident blocks) whose warps take rays from an atomic work counter,
// so the queue length can stay on the device (no host round trip).
//   BVH2: while-while traversal with per-lane refill (bvh2_ww.cuh).
//   BVH8: one ray per lane, 32 rays per fetch (bvh8_traverse.cuh).
#include "bvh2_ww.cuh"
#include "bvh8_traverse.cuh"
#include "internal.h"

namespace solrt {

namespace {

#ifndef SOLRT_EXTEND_BLOCK
#define SOLRT_EXTEND_BLOCK 128
#endif
// Minimum resident blocks per SM requested from the register allocator
// (0 = no constraint).
#ifndef SOLRT_EXTEND_MINB
#define SOLRT_EXTEND_MINB 0
#endif
constexpr int kExtendBlock = SOLRT_EXTEND_BLOCK;

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

// Wavefront queue: o_tmin / d_tmax SoA, hit = (t, prim bits, u, v); the
// scene of ray i is that of its job (meta[i].y >> kDepthBits).
struct QueueIO {
    const float4* __restrict__ o_tmin;
    const float4* __restrict__ d_tmax;
    const uint2* __restrict__ meta;
    const DevJob* __restrict__ jobs;
    float4* __restrict__ hits;
    SOLRT_D void load(uint32_t i, float4& o, float4& d, TravScene& ts) const {
        o = o_tmin[i];
        d = d_tmax[i];
        const DevScene* s = &jobs[meta[i].y >> kDepthBits].sc;
        ts.nodes = s->nodes;
        ts.tris = s->tri_wt;
        ts.node_count = s->node_count;
        ts.tri_count = s->tri_count;
    }
    SOLRT_D void store(uint32_t i, const HitRec& h) const {
        hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
    }
};

// Ray-file API: AoS solrt_ray (2 float4) -> solrt_hit (float4), one scene.
struct RayFileIO {
    const float4* __restrict__ rays;
    float4* __restrict__ hits;
    TravScene scene;
    SOLRT_D void load(uint32_t i, float4& o, float4& d, TravScene& ts) const {
        o = rays[2 * (size_t)i];
        d = rays[2 * (size_t)i + 1];
        ts = scene;
    }
    SOLRT_D void store(uint32_t i, const HitRec& h) const {
        hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
    }
};

// n = *count when count != nullptr (queue length on the device), else n_static.
template <int KIND, class IO, bool kCount>
__global__ void __launch_bounds__(kExtendBlock, SOLRT_EXTEND_MINB) k_extend(IO io, const unsigned int* __restrict__ count,
                                                         uint32_t n_static, unsigned int* __restrict__ work,
                                                         DevStats* stats) {
    const uint32_t n = count ? *count : n_static;
    if (count && blockIdx.x == 0 && threadIdx.x == 0 && n) atomicAdd(&stats->segments, (unsigned long long)n);
    TraceCounters cnt{0, 0, 0};
    uint32_t ef = 0;
    if constexpr (KIND == SOLRT_BVH2) {
        extend_bvh2_ww<IO, kCount, kExtendBlock>(io, n, work, cnt, ef);
    } else {
        const int lane = threadIdx.x & 31;
        for (;;) {
            unsigned int base = 0;
            if (lane == 0) base = atomicAdd(work, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= n) break;
            const unsigned int i = base + lane;
            if (i < n) {
                float4 o, d;
                TravScene ts;
                io.load(i, o, d, ts);
                HitRec h;
                trace_bvh8<kCount>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
                io.store(i, h);
            }
        }
    }
    flush_counters(stats, cnt, ef, kCount);
}

template <int KIND, class IO>
void launch_kind(const Context& ctx, uint32_t grid, const IO& io, const unsigned int* count, uint32_t n_static,
                 unsigned int* work, DevStats* st) {
    if (ctx.counters)
        k_extend<KIND, IO, true><<<grid, kExtendBlock, 0, ctx.stream>>>(io, count, n_static, work, st);
    else
        k_extend<KIND, IO, false><<<grid, kExtendBlock, 0, ctx.stream>>>(io, count, n_static, work, st);
}

template <class IO>
int blocks_per_sm(uint32_t kind, bool counters) {
    int b = 0;
    if (kind == SOLRT_BVH8_Q8)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, counters ? k_extend<SOLRT_BVH8_Q8, IO, true> : k_extend<SOLRT_BVH8_Q8, IO, false>, kExtendBlock, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, counters ? k_extend<SOLRT_BVH2, IO, true> : k_extend<SOLRT_BVH2, IO, false>, kExtendBlock, 0);
    return b > 0 ? b : 1;
}

}  // namespace

int extend_blocks_per_sm(uint32_t kind, bool counters) { return blocks_per_sm<QueueIO>(kind, counters); }

solrt_status launch_extend(Context& ctx, uint32_t kind, const DevJob* jobs, const PathQueue& q, float4* hits,
                           const unsigned int* count, unsigned int* work) {
    const uint32_t grid = (uint32_t)(ctx.sm_count * blocks_per_sm<QueueIO>(kind, ctx.counters));
    const QueueIO io{q.o_tmin, q.d_tmax, q.meta, jobs, hits};
    DevStats* st = ctx.stats.as<DevStats>();
    if (kind == SOLRT_BVH8_Q8) launch_kind<SOLRT_BVH8_Q8>(ctx, grid, io, count, 0, work, st);
    else launch_kind<SOLRT_BVH2>(ctx, grid, io, count, 0, work, st);
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}

solrt_status launch_trace_rays(Context& ctx, const Scene& sc, const solrt_ray* rays, uint32_t n, solrt_hit* hits) {
    if (n == 0) return SOLRT_OK;
    const DevScene d = sc.view();
    const uint32_t per_sm = (uint32_t)blocks_per_sm<RayFileIO>(d.bvh_kind, ctx.counters);
    const uint32_t want = (n + kExtendBlock - 1) / kExtendBlock;
    const uint32_t cap = (uint32_t)ctx.sm_count * per_sm;
    const uint32_t grid = want < cap ? want : cap;
    const RayFileIO io{reinterpret_cast<const float4*>(rays), reinterpret_cast<float4*>(hits), trav_scene(d)};
    unsigned int* work = ctx.trace_work.as<unsigned int>();
    SOLRT_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned int), ctx.stream));
    DevStats* st = ctx.stats.as<DevStats>();
    if (d.bvh_kind == SOLRT_BVH8_Q8) launch_kind<SOLRT_BVH8_Q8>(ctx, grid, io, nullptr, n, work, st);
    else launch_kind<SOLRT_BVH2>(ctx, grid, io, nullptr, n, work, st);
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}

}  // namespace solrt
