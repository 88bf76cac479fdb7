// trace.cu — the `extend` stage: closest hits for a queue of rays. This is
// the work traceRayEXT hands to RT cores in the reference
// (assets/glsl/pathtrace.rgen:65-76). Persistent kernels: one grid of
// (SMs x resident blocks) whose warps take rays from an atomic work counter,
// so the queue length can stay on the device (no host round trip).
//   BVH2: while-while traversal with per-lane refill (bvh2_ww.cuh); two-level
//   scenes: the same loop over a TLAS and object-space BLASes (bvh2_2l.cuh).
//   BVH8 / BVH4: the same warp-uniform organisation over quantised wide
//   nodes (bvh8_ww.cuh, bvh4_ww.cuh).
#include <algorithm>

#include "bvh2_2l.cuh"
#include "bvh2_ww.cuh"
#include "bvh4_ww.cuh"
#include "bvh8_ww.cuh"
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
// The same for the 8-wide kinds (their node test holds a whole 80-byte node
// in registers).
#ifndef SOLRT_BVH8_MINB
#define SOLRT_BVH8_MINB 0
#endif
// Group-stack entries of the 8-wide traversal kept in shared memory (the
// rest in local memory), 0..SOLRT_BVH8_STACK.
#ifndef SOLRT_BVH8_SMEM
#define SOLRT_BVH8_SMEM 0
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
    bool any_hit;  // occlusion queries (shadow rays): any hit in (tmin, tmax), not the closest
    SOLRT_D void load(uint32_t i, float4& o, float4& d, TravScene& ts) const {
        o = o_tmin[i];
        d = d_tmax[i];
        const DevScene* s = &jobs[meta[i].y >> kDepthBits].sc;
        ts.nodes = s->nodes;
        ts.tris = s->tri_wt;
        ts.node_count = s->node_count;
        ts.tri_count = s->tri_count;
        ts.tlas = s->tlas;
        ts.inst = s->inst;
        ts.tlas_count = s->tlas_count;
        ts.inst_count = s->inst_count;
    }
    SOLRT_D void load_ray(uint32_t i, float4& o, float4& d) const {
        o = o_tmin[i];
        d = d_tmax[i];
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
    static constexpr bool any_hit = false;
    SOLRT_D void load(uint32_t i, float4& o, float4& d, TravScene& ts) const {
        o = rays[2 * (size_t)i];
        d = rays[2 * (size_t)i + 1];
        ts = scene;
    }
    SOLRT_D void load_ray(uint32_t i, float4& o, float4& d) const {
        o = rays[2 * (size_t)i];
        d = rays[2 * (size_t)i + 1];
    }
    SOLRT_D void store(uint32_t i, const HitRec& h) const {
        hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
    }
};

// n = *count when count != nullptr (queue length on the device), else n_static.
// kBlock threads per block; kSmem traversal-stack slots per thread in
// shared memory (BVH2).
// Two-level scenes: registers capped at 64 so that 1024 threads fit an SM
// (as the single-level BVH2 kernel does by itself).
template <int KIND, int kBlock>
constexpr int extend_min_blocks() {
    return KIND == SOLRT_BVH2_TWO_LEVEL ? 1024 / kBlock
           : (KIND == SOLRT_BVH8_Q8 || KIND == SOLRT_BVH8_F32) ? SOLRT_BVH8_MINB * 128 / kBlock
                                                                : SOLRT_EXTEND_MINB;
}

template <int KIND, class IO, bool kCount, int kBlock, int kSmem>
__global__ void __launch_bounds__(kBlock, (extend_min_blocks<KIND, kBlock>())) k_extend(IO io, const unsigned int* __restrict__ count,
                                                                      uint32_t n_static, unsigned int* __restrict__ work,
                                                                      DevStats* stats) {
    const uint32_t n = count ? *count : n_static;
    if (count && blockIdx.x == 0 && threadIdx.x == 0 && n) atomicAdd(&stats->segments, (unsigned long long)n);
    TraceCounters cnt{0, 0, 0};
    uint32_t ef = 0;
    if constexpr (KIND == SOLRT_BVH2) {
        extend_bvh2_ww<IO, kCount, kBlock, kSmem, false>(io, n, work, cnt, ef);
    } else if constexpr (KIND == SOLRT_BVH2_Q16) {
        extend_bvh2_ww<IO, kCount, kBlock, kSmem, true>(io, n, work, cnt, ef);
    } else if constexpr (KIND == SOLRT_BVH2_TWO_LEVEL) {
        extend_bvh2_2l_ww<IO, kCount, kBlock, kSmem>(io, n, work, cnt, ef);
    } else if constexpr (KIND == SOLRT_BVH4_Q8) {
        extend_bvh4_ww<IO, kCount, kBlock, kSmem>(io, n, work, cnt, ef);
    } else if constexpr (KIND == SOLRT_BVH8_F32) {
        extend_bvh8_ww<IO, kCount, true, kBlock, kSmem>(io, n, work, cnt, ef);
    } else {
        extend_bvh8_ww<IO, kCount, false, kBlock, kSmem>(io, n, work, cnt, ef);
    }
    flush_counters(stats, cnt, ef, kCount);
}

// One extend launch of a kernel variant: a persistent grid of (SMs x
// resident blocks), or fewer blocks when `n_cap` (> 0) rays need fewer.
template <int KIND, class IO, bool kCount, int kBlock, int kSmem>
void launch_variant(const Context& ctx, const IO& io, const unsigned int* count, uint32_t n_static, uint32_t n_cap,
                    unsigned int* work, DevStats* st) {
    auto kern = k_extend<KIND, IO, kCount, kBlock, kSmem>;
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kBlock, 0);
    uint32_t grid = (uint32_t)ctx.sm_count * (uint32_t)(b > 0 ? b : 1);
    if (n_cap) grid = std::min(grid, (n_cap + kBlock - 1) / kBlock);
    kern<<<grid, kBlock, 0, ctx.stream>>>(io, count, n_static, work, st);
}

// The variant of the context's tuning (solrt_context_set_tune /
// solrt_batch_autotune); counting launches use the default shape.
template <int KIND, class IO>
solrt_status launch_tuned(const Context& ctx, const IO& io, const unsigned int* count, uint32_t n_static,
                          uint32_t n_cap, unsigned int* work, DevStats* st) {
    if constexpr (KIND == SOLRT_BVH8_Q8 || KIND == SOLRT_BVH8_F32) {
        // 8-wide kinds: SOLRT_BVH8_SMEM group-stack entries (8 B each) in
        // shared memory whatever the tuned depth; the block size is tuned
        constexpr int M8 = SOLRT_BVH8_SMEM;
        if (ctx.counters) launch_variant<KIND, IO, true, kExtendBlock, M8>(ctx, io, count, n_static, n_cap, work, st);
        else if (ctx.tune.block == 64) launch_variant<KIND, IO, false, 64, M8>(ctx, io, count, n_static, n_cap, work, st);
        else if (ctx.tune.block == 256) launch_variant<KIND, IO, false, 256, M8>(ctx, io, count, n_static, n_cap, work, st);
        else launch_variant<KIND, IO, false, 128, M8>(ctx, io, count, n_static, n_cap, work, st);
        return SOLRT_OK;
    } else {
        if (ctx.counters) {
            launch_variant<KIND, IO, true, kExtendBlock, SOLRT_SMEM_STACK>(ctx, io, count, n_static, n_cap, work, st);
            return SOLRT_OK;
        }
        const uint32_t blk = ctx.tune.block, sm = ctx.tune.smem;
#define SOLRT_VARIANT(B, M)                                                                              \
        if (blk == B && sm == M) {                                                                       \
            launch_variant<KIND, IO, false, B, M>(ctx, io, count, n_static, n_cap, work, st);            \
            return SOLRT_OK;                                                                             \
        }
        SOLRT_VARIANT(64, 16)
        SOLRT_VARIANT(64, 32)
        SOLRT_VARIANT(128, 16)
        SOLRT_VARIANT(128, 32)
        SOLRT_VARIANT(256, 16)
        SOLRT_VARIANT(256, 32)
#undef SOLRT_VARIANT
        set_error("no extend kernel for block %u, stack %u", blk, sm);
        return SOLRT_ERR_INVALID;
    }
}

}  // namespace

bool extend_variant_ok(uint32_t block, uint32_t smem) {
    return (block == 64 || block == 128 || block == 256) && (smem == 16 || smem == 32);
}

solrt_status launch_extend(Context& ctx, uint32_t kind, const DevJob* jobs, const PathQueue& q, float4* hits,
                           const unsigned int* count, unsigned int* work, DevStats* st, bool any_hit) {
    const QueueIO io{q.o_tmin, q.d_tmax, q.meta, jobs, hits, any_hit};
    if (!st) st = ctx.stats.as<DevStats>();
    if (kind == SOLRT_BVH8_Q8) SOLRT_TRY((launch_tuned<SOLRT_BVH8_Q8>(ctx, io, count, 0, 0, work, st)));
    else if (kind == SOLRT_BVH4_Q8) SOLRT_TRY((launch_tuned<SOLRT_BVH4_Q8>(ctx, io, count, 0, 0, work, st)));
    else if (kind == SOLRT_BVH8_F32) SOLRT_TRY((launch_tuned<SOLRT_BVH8_F32>(ctx, io, count, 0, 0, work, st)));
    else if (kind == SOLRT_BVH2_Q16) SOLRT_TRY((launch_tuned<SOLRT_BVH2_Q16>(ctx, io, count, 0, 0, work, st)));
    else if (kind == SOLRT_BVH2_TWO_LEVEL)
        SOLRT_TRY((launch_tuned<SOLRT_BVH2_TWO_LEVEL>(ctx, io, count, 0, 0, work, st)));
    else SOLRT_TRY((launch_tuned<SOLRT_BVH2>(ctx, io, count, 0, 0, work, st)));
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}

solrt_status launch_trace_rays(Context& ctx, const Scene& sc, const solrt_ray* rays, uint32_t n, solrt_hit* hits) {
    if (n == 0) return SOLRT_OK;
    const DevScene d = sc.view();
    const RayFileIO io{reinterpret_cast<const float4*>(rays), reinterpret_cast<float4*>(hits), trav_scene(d)};
    unsigned int* work = ctx.trace_work.as<unsigned int>();
    SOLRT_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned int), ctx.stream));
    DevStats* st = ctx.stats.as<DevStats>();
    if (d.bvh_kind == SOLRT_BVH8_Q8) SOLRT_TRY((launch_tuned<SOLRT_BVH8_Q8>(ctx, io, nullptr, n, n, work, st)));
    else if (d.bvh_kind == SOLRT_BVH4_Q8) SOLRT_TRY((launch_tuned<SOLRT_BVH4_Q8>(ctx, io, nullptr, n, n, work, st)));
    else if (d.bvh_kind == SOLRT_BVH8_F32) SOLRT_TRY((launch_tuned<SOLRT_BVH8_F32>(ctx, io, nullptr, n, n, work, st)));
    else if (d.bvh_kind == SOLRT_BVH2_Q16) SOLRT_TRY((launch_tuned<SOLRT_BVH2_Q16>(ctx, io, nullptr, n, n, work, st)));
    else if (d.bvh_kind == SOLRT_BVH2_TWO_LEVEL)
        SOLRT_TRY((launch_tuned<SOLRT_BVH2_TWO_LEVEL>(ctx, io, nullptr, n, n, work, st)));
    else SOLRT_TRY((launch_tuned<SOLRT_BVH2>(ctx, io, nullptr, n, n, work, st)));
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}

}  // namespace solrt
