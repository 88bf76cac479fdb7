// bvh2_ww.cuh — BVH2 traversal organised for SIMT efficiency.
//
// A warp keeps 32 rays in flight. Every step of its loop is warp-uniform
// (full-warp votes decide the phases), so lanes re-converge at each step:
//   refill  lanes whose ray has finished take new rays from the global queue
//           (one atomic per warp), once at least SOLRT_BVH2_REFILL lanes are
//           free;
//   nodes   lanes visit inner nodes until every lane has parked a leaf or has
//           no inner node left, or until fewer than SOLRT_WW_NODE_MIN lanes
//           still have inner nodes while others hold leaves; a lane that
//           already parked a leaf keeps descending until it reaches a second
//           one ("while-while" with speculative traversal, after Aila &
//           Laine, HPG 2009);
//   leaves  lanes test their parked leaves together.
// Each lane carries its own scene (IO::load), so one launch can serve rays of
// many scenes. The closest hit does not depend on visiting order, so results
// equal those of a plain per-ray loop.
#pragma once

#include "traverse.cuh"

namespace solrt {

constexpr int kBvh2Sentinel = 0x7fffffff;
#ifndef SOLRT_BVH2_REFILL
#define SOLRT_BVH2_REFILL 16
#endif
// The node phase ends early when fewer than this many lanes have inner
// nodes to visit and some lane holds a leaf (0 = only when no lane without
// a parked leaf has inner nodes left).
#ifndef SOLRT_WW_NODE_MIN
#define SOLRT_WW_NODE_MIN 12
#endif
// 1: a lane that has parked a leaf keeps visiting inner nodes until it
// reaches a second leaf; 0: it waits for the leaf phase.
#ifndef SOLRT_WW_SPECULATE
#define SOLRT_WW_SPECULATE 1
#endif
// Default traversal stack entries kept in shared memory (slot-major, one
// column per thread, so lanes at different depths hit different banks);
// deeper entries go to a local-memory array. The launch may pick 16 or 32
// (solrt_context_set_tune / solrt_batch_autotune).
#ifndef SOLRT_SMEM_STACK
#define SOLRT_SMEM_STACK 32
#endif

// The 4 float4 of BVH2 node `node` (64-byte aligned) in two 256-bit loads.
SOLRT_D void load_bvh2_node(const float4* nodes, int node, float4& n0, float4& n1, float4& n2, int4& n3) {
    const float4* np = nodes + 4 * (size_t)node;
    float4 r;
    ldg_2x4(np, n0, n1);
    ldg_2x4(np + 2, n2, r);
    n3 = make_int4(__float_as_int(r.x), __float_as_int(r.y), __float_as_int(r.z), __float_as_int(r.w));
}

// Per-thread traversal stack: slots [0, kSmem) in shared memory, the rest
// in local memory; SOLRT_BVH2_STACK + 1 slots in all.
template <int kBlock, int kSmem>
struct Bvh2Stack {
    int* sh;  // slot k at sh[k * kBlock]
    int lo[SOLRT_BVH2_STACK + 1 - kSmem];
    SOLRT_D void put(int k, int v) {
        if (k < kSmem) sh[k * kBlock] = v;
        else lo[k - kSmem] = v;
    }
    SOLRT_D int get(int k) const { return k < kSmem ? sh[k * kBlock] : lo[k - kSmem]; }
};
template <int kBlock>
struct Bvh2Stack<kBlock, 0> {
    int* sh;
    int lo[SOLRT_BVH2_STACK + 1];
    SOLRT_D void put(int k, int v) { lo[k] = v; }
    SOLRT_D int get(int k) const { return lo[k]; }
};

// One node test in either node format (kQ16: 32-byte
// BVH2-q16 nodes, one 256-bit load; else 64-byte FP32 nodes, two).
template <bool kQ16>
SOLRT_D void bvh2_node_step(const float4* nodes, int node, float ix, float iy, float iz, float nox, float noy,
                            float noz, float tmin, float tmax, bool& h0, float& t0, bool& h1, float& t1, int& ref0,
                            int& ref1) {
    if constexpr (kQ16) {
        float4 a, b;
        ldg_2x4(nodes + 2 + 2 * (size_t)node, a, b);
        slab2_q16(a, b, ix, iy, iz, nox, noy, noz, tmin, tmax, h0, t0, h1, t1);
        ref0 = __float_as_int(a.x);
        ref1 = __float_as_int(a.y);
    } else {
        float4 n0, n1, n2;
        int4 n3;
        load_bvh2_node(nodes, node, n0, n1, n2, n3);
        slab2_fma(n0, n1, n2, ix, iy, iz, nox, noy, noz, tmin, tmax, h0, t0, h1, t1);
        ref0 = n3.x;
        ref1 = n3.y;
    }
}

// Per-ray constants of the slab test: (1/d, -o/d) per axis for FP32 nodes,
// (c/d, (G - o)/d - 2^23 c/d) for BVH2-q16 nodes (q16_ray).
template <bool kQ16>
SOLRT_D void bvh2_ray_consts(const float4* nodes, float ox, float oy, float oz, float dx, float dy, float dz,
                             float& ix, float& iy, float& iz, float& nox, float& noy, float& noz) {
    if constexpr (kQ16) {
        q16_ray(nodes, ox, oy, oz, dx, dy, dz, ix, iy, iz, nox, noy, noz);
    } else {
        ix = 1.0f / box_dir(dx);
        iy = 1.0f / box_dir(dy);
        iz = 1.0f / box_dir(dz);
        nox = -(ox * ix);
        noy = -(oy * iy);
        noz = -(oz * iz);
    }
}

template <class IO, bool kCount, int kBlock, int kSmem, bool kQ16 = false>
SOLRT_D void extend_bvh2_ww(const IO& io, uint32_t n, unsigned int* work, TraceCounters& cnt, uint32_t& ef) {
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    Bvh2Stack<kBlock, kSmem> stack;
    __shared__ int s_stack[(kSmem > 0 ? kSmem : 1) * kBlock];
    stack.sh = s_stack + threadIdx.x;
    int sp = 0;
    int node = kBvh2Sentinel;  // >= 0 inner node, < 0 leaf ~k, sentinel = nothing left
    int leaf = 0;              // parked leaf (< 0) or none (>= 0)
    bool has = false;
    bool drained = false;      // the queue has no more rays for this warp
    uint32_t idx = 0, budget = 0;
    RayWT r;
    TravScene ts{nullptr, nullptr, 0u, 0u};
    float ix = 0.0f, iy = 0.0f, iz = 0.0f;     // 1 / box_dir(d)
    float nox = 0.0f, noy = 0.0f, noz = 0.0f;  // -o / box_dir(d)
    HitRec best{0.0f, SOLRT_NO_HIT, 0.0f, 0.0f};
    for (;;) {
        const bool idle = node == kBvh2Sentinel && leaf >= 0;
        if (idle && has) {
            io.store(idx, best);
            has = false;
        }
        const uint32_t need = __ballot_sync(0xffffffffu, idle);
        if (!drained && __popc(need) >= SOLRT_BVH2_REFILL) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(work, (unsigned int)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base + (uint32_t)__popc(need) >= n) drained = true;
            if (idle) {
                const uint32_t i = base + (uint32_t)__popc(need & lane_lt);
                if (i < n) {
                    float4 o, d;
                    io.load(i, o, d, ts);
                    idx = i;
                    has = true;
                    r = setup_ray(o.x, o.y, o.z, d.x, d.y, d.z, o.w);
                    if (ts.tri_count)
                        bvh2_ray_consts<kQ16>(ts.nodes, o.x, o.y, o.z, d.x, d.y, d.z, ix, iy, iz, nox, noy, noz);
                    best = HitRec{d.w, SOLRT_NO_HIT, 0.0f, 0.0f};
                    budget = 2u * (ts.node_count + ts.tri_count) + 64u;
                    stack.put(0, kBvh2Sentinel);
                    sp = 1;
                    node = ts.tri_count ? 0 : kBvh2Sentinel;
                    leaf = 0;
                }
            }
        }
        if (!__any_sync(0xffffffffu, has)) {
            if (drained) break;
            continue;
        }
        // node phase
        for (;;) {
            const bool inner = (unsigned)node < (unsigned)kBvh2Sentinel;
            // two ballots decide the phase: stop when no lane without a
            // parked leaf has inner nodes, or when few lanes still have inner
            // nodes while others hold leaves (test the leaves first; the leaf
            // phase then has work, so this ends)
            const uint32_t b_inner = __ballot_sync(0xffffffffu, inner);
            const uint32_t b_leaf = __ballot_sync(0xffffffffu, leaf < 0);
            const uint32_t b_free = b_inner & ~b_leaf;  // inner nodes, no parked leaf
            if (b_free == 0u) break;
#if SOLRT_WW_NODE_MIN > 0
            if (__popc(SOLRT_WW_SPECULATE ? b_inner : b_free) < SOLRT_WW_NODE_MIN && b_leaf) break;
#endif
            if (inner && (SOLRT_WW_SPECULATE || leaf >= 0)) {
                if (--budget == 0u || (uint32_t)node >= ts.node_count) {
                    ef |= SOLRT_EFLAG_INDEX;
                    node = kBvh2Sentinel;
                    leaf = 0;
                } else {
                    if (kCount) ++cnt.nodes;
                    float t0, t1;
                    bool h0, h1;
                    int c0, c1;
                    bvh2_node_step<kQ16>(ts.nodes, node, ix, iy, iz, nox, noy, noz, r.tmin, best.t, h0, t0, h1, t1,
                                         c0, c1);
                    if (h0 && h1) {
                        const bool swap = t1 < t0;
                        if (sp <= SOLRT_BVH2_STACK) stack.put(sp++, swap ? c0 : c1);
                        else ef |= SOLRT_EFLAG_STACK;
                        node = swap ? c1 : c0;
                    } else if (h0) {
                        node = c0;
                    } else if (h1) {
                        node = c1;
                    } else {
                        node = stack.get(--sp);
                    }
                    if (node < 0 && leaf >= 0) {  // park the leaf, keep descending
                        leaf = node;
                        node = stack.get(--sp);
                    }
                }
            }
        }
        // leaf phase
        while (__any_sync(0xffffffffu, leaf < 0)) {
            if (leaf < 0) {
                const uint32_t k = (uint32_t)(~leaf);
                if (--budget == 0u || k >= ts.tri_count) {
                    ef |= SOLRT_EFLAG_INDEX;
                    node = kBvh2Sentinel;
                    leaf = 0;
                } else {
                    const float4* tp = ts.tris + 3 * (size_t)k;
                    if (kCount) ++cnt.tris;
                    cnt.fallbacks += intersect_tri(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), best);
                    if (io.any_hit && best.prim != SOLRT_NO_HIT) {  // occlusion query: done at the first hit
                        node = kBvh2Sentinel;
                        leaf = 0;
                    } else {
                        leaf = node;
                        if (node < 0) node = stack.get(--sp);
                    }
                }
            }
        }
    }
}

// One ray, plain depth-first loop (nearer child first): the traversal of the
// per-pixel megakernel.
template <bool kQ16 = false>
SOLRT_D void trace_bvh2_ray(const TravScene& ts, float ox, float oy, float oz, float dx, float dy, float dz,
                            float tmin, float tmax, HitRec& best, TraceCounters& cnt, uint32_t& ef) {
    best = HitRec{tmax, SOLRT_NO_HIT, 0.0f, 0.0f};
    if (ts.tri_count == 0) return;
    const RayWT r = setup_ray(ox, oy, oz, dx, dy, dz, tmin);
    float ix, iy, iz, nox, noy, noz;
    bvh2_ray_consts<kQ16>(ts.nodes, ox, oy, oz, dx, dy, dz, ix, iy, iz, nox, noy, noz);
    int stack[SOLRT_BVH2_STACK + 1];
    stack[0] = kBvh2Sentinel;
    int sp = 1;
    int node = 0;
    uint32_t budget = 2u * (ts.node_count + ts.tri_count) + 64u;
    while (node != kBvh2Sentinel) {
        if (--budget == 0u) {
            ef |= SOLRT_EFLAG_INDEX;
            return;
        }
        if (node >= 0) {
            if ((uint32_t)node >= ts.node_count) {
                ef |= SOLRT_EFLAG_INDEX;
                return;
            }
            float t0, t1;
            bool h0, h1;
            int c0, c1;
            bvh2_node_step<kQ16>(ts.nodes, node, ix, iy, iz, nox, noy, noz, tmin, best.t, h0, t0, h1, t1, c0, c1);
            if (h0 && h1) {
                const bool swap = t1 < t0;
                if (sp <= SOLRT_BVH2_STACK) stack[sp++] = swap ? c0 : c1;
                else ef |= SOLRT_EFLAG_STACK;
                node = swap ? c1 : c0;
                continue;
            }
            if (h0) { node = c0; continue; }
            if (h1) { node = c1; continue; }
        } else {
            const uint32_t k = (uint32_t)(~node);
            if (k >= ts.tri_count) {
                ef |= SOLRT_EFLAG_INDEX;
                return;
            }
            const float4* tp = ts.tris + 3 * (size_t)k;
            cnt.fallbacks += intersect_tri(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), best);
        }
        node = stack[--sp];
    }
}

}  // namespace solrt
