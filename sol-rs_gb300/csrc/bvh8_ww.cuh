// bvh8_ww.cuh — traversal of the 8-wide quantised BVH (bvh8.cuh) organised
// like bvh2_ww.cuh: a warp keeps 32 rays in flight and every step of its loop
// is warp-uniform.
//   refill  lanes whose ray has finished take new rays from the global queue
//           once at least SOLRT_BVH8_REFILL lanes are free;
//   nodes   lanes with no parked triangles visit one 8-wide node per step:
//           the nearest remaining internal child of their current node group
//           (octant order), pushing the rest of the group; the node's hit
//           internal children become the new group and its hit triangles are
//           parked. The phase ends when no lane can step, or when fewer than
//           SOLRT_BVH8_NODE_MIN lanes can while others hold triangles;
//   leaves  lanes test their parked triangles, one per step.
// The child-box tests are those of trace_bvh8 (bvh8_traverse.cuh: quantised
// or, for SOLRT_BVH8_F32, full-precision nodes), so the closest hit equals
// that of the per-ray loop.
#pragma once

#include "bvh8_traverse.cuh"

namespace solrt {

#ifndef SOLRT_BVH8_REFILL
#define SOLRT_BVH8_REFILL 16
#endif
#ifndef SOLRT_BVH8_NODE_MIN
#define SOLRT_BVH8_NODE_MIN 12
#endif

// Per-thread stack of node groups: entries [0, kSmem) in shared memory
// (slot-major, one column per thread), the rest in local memory.
template <int kBlock, int kSmem>
struct Bvh8Stack {
    uint2* sh;  // entry k at sh[k * kBlock]
    uint2 lo[SOLRT_BVH8_STACK - kSmem];
    SOLRT_D void put(int k, uint2 v) {
        if (k < kSmem) sh[k * kBlock] = v;
        else lo[k - kSmem] = v;
    }
    SOLRT_D uint2 get(int k) const { return k < kSmem ? sh[k * kBlock] : lo[k - kSmem]; }
};
template <int kBlock>
struct Bvh8Stack<kBlock, 0> {
    uint2* sh;
    uint2 lo[SOLRT_BVH8_STACK];
    SOLRT_D void put(int k, uint2 v) { lo[k] = v; }
    SOLRT_D uint2 get(int k) const { return lo[k]; }
};

template <class IO, bool kCount, bool kF32 = false, int kBlock = 128, int kSmem = 0>
SOLRT_D void extend_bvh8_ww(const IO& io, uint32_t n, unsigned int* work, TraceCounters& cnt, uint32_t& ef) {
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    Bvh8Stack<kBlock, kSmem> stack;
    __shared__ uint2 s_stack8[(kSmem > 0 ? kSmem : 1) * kBlock];
    stack.sh = s_stack8 + threadIdx.x;
    int sp = 0;
    uint2 grp = make_uint2(0u, 0u);   // (child base, hit bits << 24 | internal mask)
    uint2 tgrp = make_uint2(0u, 0u);  // parked triangles: (triangle base, hit bits)
    bool has = false;
    bool drained = false;
    uint32_t idx = 0, budget = 0, oct = 0;
    bool negx = false, negy = false, negz = false;
    RayWT r;
    TravScene ts{nullptr, nullptr, 0u, 0u};
    float ix = 0.0f, iy = 0.0f, iz = 0.0f;
    float nox = 0.0f, noy = 0.0f, noz = 0.0f;  // -o / box_dir(d) (FP32 nodes)
    HitRec best{0.0f, SOLRT_NO_HIT, 0.0f, 0.0f};
    const uint4* nodes = nullptr;
    for (;;) {
        const bool idle = (grp.y >> 24) == 0u && sp == 0 && tgrp.y == 0u;
        if (idle && has) {
            io.store(idx, best);
            has = false;
        }
        const uint32_t need = __ballot_sync(0xffffffffu, idle);
        if (!drained && __popc(need) >= SOLRT_BVH8_REFILL) {
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
                    const float bx = box_dir(d.x), by = box_dir(d.y), bz = box_dir(d.z);
                    ix = 1.0f / bx;
                    iy = 1.0f / by;
                    iz = 1.0f / bz;
                    negx = signbit(bx);
                    negy = signbit(by);
                    negz = signbit(bz);
                    nox = -(o.x * ix);
                    noy = -(o.y * iy);
                    noz = -(o.z * iz);
                    oct = (negx ? 1u : 0u) | (negy ? 2u : 0u) | (negz ? 4u : 0u);
                    best = HitRec{d.w, SOLRT_NO_HIT, 0.0f, 0.0f};
                    budget = 2u * (ts.node_count + ts.tri_count) + 64u;
                    nodes = reinterpret_cast<const uint4*>(ts.nodes);
                    sp = 0;
                    tgrp = make_uint2(0u, 0u);
                    // the root as a group of one internal child in slot 0
                    grp = ts.tri_count ? make_uint2(0u, (1u << (24u + oct)) | 1u) : make_uint2(0u, 0u);
                }
            }
        }
        if (!__any_sync(0xffffffffu, has)) {
            if (drained) break;
            continue;
        }
        // node phase
        for (;;) {
            const bool want = tgrp.y == 0u && ((grp.y >> 24) != 0u || sp > 0);
            const uint32_t wb = __ballot_sync(0xffffffffu, want);
            if (wb == 0u) break;
            if (__popc(wb) < SOLRT_BVH8_NODE_MIN && __any_sync(0xffffffffu, tgrp.y != 0u)) break;
            if (want) {
                if ((grp.y >> 24) == 0u) grp = stack.get(--sp);
                const uint32_t j = (uint32_t)(__ffs(grp.y >> 24) - 1);
                grp.y &= ~(1u << (24u + j));
                const uint32_t s = j ^ oct;
                const uint32_t node = grp.x + (uint32_t)__popc(grp.y & ((1u << s) - 1u) & 0xffu);
                if (grp.y >> 24) {
                    if (sp < SOLRT_BVH8_STACK) stack.put(sp++, grp);
                    else ef |= SOLRT_EFLAG_STACK;
                }
                grp = make_uint2(0u, 0u);
                if (--budget == 0u || node >= ts.node_count) {
                    ef |= SOLRT_EFLAG_INDEX;
                    sp = 0;
                } else {
                    if (kCount) ++cnt.nodes;
                    uint32_t hi = 0, ht = 0;
                    if constexpr (kF32) {
                        uint32_t cbase = 0, tbase = 0, imask = 0;
                        bvh8f_node_test(ts.nodes + 14 * (size_t)node, ix, iy, iz, nox, noy, noz, oct, r.tmin, best.t,
                                        hi, ht, cbase, tbase, imask);
                        if (hi) grp = make_uint2(cbase, (hi << 24) | imask);
                        tgrp = make_uint2(tbase, ht);
                    } else {
                        const uint4* np = nodes + 5 * (size_t)node;
                        const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3),
                                    w4 = __ldg(np + 4);
                        bvh8_node_test(w0, w1, w2, w3, w4, r.ox, r.oy, r.oz, ix, iy, iz, negx, negy, negz, oct,
                                       r.tmin, best.t, hi, ht);
                        if (hi) grp = make_uint2(w1.x, (hi << 24) | (w0.w >> 24));
                        tgrp = make_uint2(w1.y, ht);
                    }
                }
            }
        }
        // leaf phase
        while (__any_sync(0xffffffffu, tgrp.y != 0u)) {
            if (tgrp.y) {
                const uint32_t k = (uint32_t)(__ffs(tgrp.y) - 1);
                tgrp.y &= tgrp.y - 1u;
                const uint32_t ti = tgrp.x + k;
                if (--budget == 0u || ti >= ts.tri_count) {
                    ef |= SOLRT_EFLAG_INDEX;
                    tgrp.y = 0u;
                    grp = make_uint2(0u, 0u);
                    sp = 0;
                } else {
                    const float4* tp = ts.tris + 3 * (size_t)ti;
                    if (kCount) ++cnt.tris;
                    cnt.fallbacks += intersect_tri(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), best);
                    if (io.any_hit && best.prim != SOLRT_NO_HIT) {  // occlusion query: done at the first hit
                        tgrp.y = 0u;
                        grp = make_uint2(0u, 0u);
                        sp = 0;
                    }
                }
            }
        }
    }
}

}  // namespace solrt
