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
// The child-box test is the one of trace_bvh8 (bvh8_traverse.cuh), so the
// closest hit equals that of the per-ray loop.
#pragma once

#include "bvh8_traverse.cuh"

namespace solrt {

#ifndef SOLRT_BVH8_REFILL
#define SOLRT_BVH8_REFILL 16
#endif
#ifndef SOLRT_BVH8_NODE_MIN
#define SOLRT_BVH8_NODE_MIN 12
#endif

// Tests the 8 children of one node. Returns the hit internal children in
// visiting order (bit s ^ oct for slot s) and the hit leaf triangles
// (bit o of the node's triangle range).
SOLRT_D void bvh8_node_test(const uint4& w0, const uint4& w1, const uint4& w2, const uint4& w3, const uint4& w4,
                            float ox, float oy, float oz, float ix, float iy, float iz, bool negx, bool negy,
                            bool negz, uint32_t oct, float tmin, float tmax, uint32_t& hit_inner,
                            uint32_t& hit_tri) {
    const int ex = (int)(int8_t)(w0.w & 0xffu), ey = (int)(int8_t)((w0.w >> 8) & 0xffu),
              ez = (int)(int8_t)((w0.w >> 16) & 0xffu);
    const uint32_t imask = w0.w >> 24;
    const float sx = __uint_as_float((uint32_t)(ex + 127) << 23) * ix;
    const float sy = __uint_as_float((uint32_t)(ey + 127) << 23) * iy;
    const float sz = __uint_as_float((uint32_t)(ez + 127) << 23) * iz;
    // plane q is at t = (2^23 + q) * s + (a - 2^23 s): the biased byte
    // (byte_biased) needs no conversion. Rounding a - 2^23 s adds at most half
    // a grid step (in t) to each face, inside the one-step margin every face
    // has (grid_anchor); the rest is relative to |t| as in trace_bvh8.
    const float ax = fmaf(-8388608.0f, sx, (__uint_as_float(w0.x) - ox) * ix);
    const float ay = fmaf(-8388608.0f, sy, (__uint_as_float(w0.y) - oy) * iy);
    const float az = fmaf(-8388608.0f, sz, (__uint_as_float(w0.z) - oz) * iz);
    // near / far plane bytes per axis: lo is near for a positive direction
    const uint32_t nx0 = negx ? w3.z : w2.x, nx1 = negx ? w3.w : w2.y;
    const uint32_t fx0 = negx ? w2.x : w3.z, fx1 = negx ? w2.y : w3.w;
    const uint32_t ny0 = negy ? w4.x : w2.z, ny1 = negy ? w4.y : w2.w;
    const uint32_t fy0 = negy ? w2.z : w4.x, fy1 = negy ? w2.w : w4.y;
    const uint32_t nz0 = negz ? w4.z : w3.x, nz1 = negz ? w4.w : w3.y;
    const uint32_t fz0 = negz ? w3.x : w4.z, fz1 = negz ? w3.y : w4.w;
    hit_inner = 0;
    hit_tri = 0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const uint32_t k = (uint32_t)(s & 3);
        const uint32_t meta = ((s < 4 ? w1.z : w1.w) >> (8u * k)) & 0xffu;
        const float tnx = fmaf(byte_biased(s < 4 ? nx0 : nx1, k), sx, ax);
        const float tny = fmaf(byte_biased(s < 4 ? ny0 : ny1, k), sy, ay);
        const float tnz = fmaf(byte_biased(s < 4 ? nz0 : nz1, k), sz, az);
        const float tfx = fmaf(byte_biased(s < 4 ? fx0 : fx1, k), sx, ax);
        const float tfy = fmaf(byte_biased(s < 4 ? fy0 : fy1, k), sy, ay);
        const float tfz = fmaf(byte_biased(s < 4 ? fz0 : fz1, k), sz, az);
        const float tn = max3(tnx, tny, fmaxf(tnz, tmin));
        const float tf = min3(tfx, tfy, fminf(tfz, tmax));
        if (meta != 0u && tn <= tf * 1.0000153f) {
            if (imask & (1u << s)) hit_inner |= 1u << ((uint32_t)s ^ oct);
            else hit_tri |= (meta >> 5) << (meta & 31u);
        }
    }
}

template <class IO, bool kCount>
SOLRT_D void extend_bvh8_ww(const IO& io, uint32_t n, unsigned int* work, TraceCounters& cnt, uint32_t& ef) {
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    uint2 stack[SOLRT_BVH8_STACK];
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
                if ((grp.y >> 24) == 0u) grp = stack[--sp];
                const uint32_t j = (uint32_t)(__ffs(grp.y >> 24) - 1);
                grp.y &= ~(1u << (24u + j));
                const uint32_t s = j ^ oct;
                const uint32_t node = grp.x + (uint32_t)__popc(grp.y & ((1u << s) - 1u) & 0xffu);
                if (grp.y >> 24) {
                    if (sp < SOLRT_BVH8_STACK) stack[sp++] = grp;
                    else ef |= SOLRT_EFLAG_STACK;
                }
                grp = make_uint2(0u, 0u);
                if (--budget == 0u || node >= ts.node_count) {
                    ef |= SOLRT_EFLAG_INDEX;
                    sp = 0;
                } else {
                    const uint4* np = nodes + 5 * (size_t)node;
                    const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3),
                                w4 = __ldg(np + 4);
                    if (kCount) ++cnt.nodes;
                    uint32_t hi = 0, ht = 0;
                    bvh8_node_test(w0, w1, w2, w3, w4, r.ox, r.oy, r.oz, ix, iy, iz, negx, negy, negz, oct, r.tmin,
                                   best.t, hi, ht);
                    if (hi) grp = make_uint2(w1.x, (hi << 24) | (w0.w >> 24));
                    tgrp = make_uint2(w1.y, ht);
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
                }
            }
        }
    }
}

}  // namespace solrt
