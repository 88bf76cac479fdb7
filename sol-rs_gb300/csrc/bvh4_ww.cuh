// bvh4_ww.cuh — traversal of the 4-wide quantised BVH (64-byte nodes written
// by k_emit4 in bvh8_build.cu):
//   w0: anchor p.xyz (float) | exponents e.xyz (int8), internal mask (4 bits)
//   w1: child_base, tri_base, meta[0..3] (u8), qlo.x[0..3] (u8)
//   w2: qlo.y[0..3], qlo.z[0..3], qhi.x[0..3], qhi.y[0..3]
//   w3: qhi.z[0..3]
// A node is two 256-bit loads. The four child boxes are tested as in the
// 8-wide node (biased bytes folded into one FMA per plane, one grid step of
// margin on every face); hit internal children are sorted by entry distance,
// the nearest is visited next and the others are pushed far to near; hit leaf
// triangles are parked and tested in the leaf phase. The warp organisation
// (refill, node phase ended early when few lanes still have nodes, leaf
// phase) is that of bvh2_ww.cuh.
#pragma once

#include "bvh2_ww.cuh"
#include "bvh8_traverse.cuh"

namespace solrt {

// Tests the 4 children of a node. keys[i]: (entry distance bits & ~3) | slot
// for hit internal children, ~0 otherwise; hit_tri: hit leaf triangles
// (bit o of the node's triangle range).
SOLRT_D void bvh4_node_test(const float4& a, const float4& b, const float4& c, const float4& d, float ox, float oy,
                            float oz, float ix, float iy, float iz, bool negx, bool negy, bool negz, float tmin,
                            float tmax, uint32_t keys[4], uint32_t& hit_tri) {
    const uint32_t packed = __float_as_uint(a.w);
    const int ex = (int)(int8_t)(packed & 0xffu), ey = (int)(int8_t)((packed >> 8) & 0xffu),
              ez = (int)(int8_t)((packed >> 16) & 0xffu);
    const uint32_t imask = packed >> 24;
    const float sx = __uint_as_float((uint32_t)(ex + 127) << 23) * ix;
    const float sy = __uint_as_float((uint32_t)(ey + 127) << 23) * iy;
    const float sz = __uint_as_float((uint32_t)(ez + 127) << 23) * iz;
    // plane q at t = (2^23 + q) s + (a - 2^23 s), as in bvh8_node_test
    const float ax = fmaf(-8388608.0f, sx, (a.x - ox) * ix);
    const float ay = fmaf(-8388608.0f, sy, (a.y - oy) * iy);
    const float az = fmaf(-8388608.0f, sz, (a.z - oz) * iz);
    const uint32_t meta = __float_as_uint(b.z);
    const uint32_t lox = __float_as_uint(b.w), loy = __float_as_uint(c.x), loz = __float_as_uint(c.y);
    const uint32_t hix = __float_as_uint(c.z), hiy = __float_as_uint(c.w), hiz = __float_as_uint(d.x);
    const uint32_t nx = negx ? hix : lox, fx = negx ? lox : hix;
    const uint32_t ny = negy ? hiy : loy, fy = negy ? loy : hiy;
    const uint32_t nz = negz ? hiz : loz, fz = negz ? loz : hiz;
    hit_tri = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const uint32_t k = (uint32_t)s;
        const uint32_t m = (meta >> (8u * k)) & 0xffu;
        const float tn = max3(fmaf(byte_biased(nx, k), sx, ax), fmaf(byte_biased(ny, k), sy, ay),
                              fmaxf(fmaf(byte_biased(nz, k), sz, az), tmin));
        const float tf = min3(fmaf(byte_biased(fx, k), sx, ax), fmaf(byte_biased(fy, k), sy, ay),
                              fminf(fmaf(byte_biased(fz, k), sz, az), tmax));
        const bool hit = m != 0u && tn <= tf * 1.0000153f;
        const bool inner = (imask >> s) & 1u;
        keys[s] = hit && inner ? ((__float_as_uint(tn + 0.0f) & ~3u) | k) : 0xffffffffu;
        if (hit && !inner) hit_tri |= (m >> 5) << (m & 31u);
    }
}

SOLRT_D void sort4(uint32_t k[4]) {
    uint32_t a = min(k[0], k[1]), b = max(k[0], k[1]);
    uint32_t c = min(k[2], k[3]), d = max(k[2], k[3]);
    const uint32_t e = min(a, c), f = max(a, c);
    const uint32_t g = min(b, d), h = max(b, d);
    k[0] = e;
    k[1] = min(f, g);
    k[2] = max(f, g);
    k[3] = h;
}

template <class IO, bool kCount, int kBlock, int kSmem>
SOLRT_D void extend_bvh4_ww(const IO& io, uint32_t n, unsigned int* work, TraceCounters& cnt, uint32_t& ef) {
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    Bvh2Stack<kBlock, kSmem> stack;
    __shared__ int s_stack[(kSmem > 0 ? kSmem : 1) * kBlock];
    stack.sh = s_stack + threadIdx.x;
    int sp = 0;
    int node = kBvh2Sentinel;            // next 4-wide node to visit, or none
    uint2 tgrp = make_uint2(0u, 0u);     // parked triangles: (triangle base, hit bits)
    bool has = false;
    bool drained = false;
    uint32_t idx = 0, budget = 0;
    bool negx = false, negy = false, negz = false;
    RayWT r;
    TravScene ts{nullptr, nullptr, 0u, 0u};
    float ix = 0.0f, iy = 0.0f, iz = 0.0f;
    HitRec best{0.0f, SOLRT_NO_HIT, 0.0f, 0.0f};
    for (;;) {
        const bool idle = node == kBvh2Sentinel && tgrp.y == 0u;
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
                    const float bx = box_dir(d.x), by = box_dir(d.y), bz = box_dir(d.z);
                    ix = 1.0f / bx;
                    iy = 1.0f / by;
                    iz = 1.0f / bz;
                    negx = signbit(bx);
                    negy = signbit(by);
                    negz = signbit(bz);
                    best = HitRec{d.w, SOLRT_NO_HIT, 0.0f, 0.0f};
                    budget = 2u * (ts.node_count + ts.tri_count) + 64u;
                    stack.put(0, kBvh2Sentinel);
                    sp = 1;
                    tgrp = make_uint2(0u, 0u);
                    node = ts.tri_count ? 0 : kBvh2Sentinel;
                }
            }
        }
        if (!__any_sync(0xffffffffu, has)) {
            if (drained) break;
            continue;
        }
        // node phase
        for (;;) {
            const bool want = node != kBvh2Sentinel && tgrp.y == 0u;
            const uint32_t wb = __ballot_sync(0xffffffffu, want);
            if (wb == 0u) break;
            if (__popc(wb) < SOLRT_WW_NODE_MIN && __any_sync(0xffffffffu, tgrp.y != 0u)) break;
            if (want) {
                if (--budget == 0u || (uint32_t)node >= ts.node_count) {
                    ef |= SOLRT_EFLAG_INDEX;
                    node = kBvh2Sentinel;
                    sp = 1;
                } else {
                    const float4* np = ts.nodes + 4 * (size_t)node;
                    float4 w0, w1, w2, w3;
                    ldg_2x4(np, w0, w1);
                    ldg_2x4(np + 2, w2, w3);
                    if (kCount) ++cnt.nodes;
                    uint32_t keys[4], ht = 0;
                    bvh4_node_test(w0, w1, w2, w3, r.ox, r.oy, r.oz, ix, iy, iz, negx, negy, negz, r.tmin, best.t,
                                   keys, ht);
                    sort4(keys);
                    const uint32_t imask = __float_as_uint(w0.w) >> 24;
                    const uint32_t child_base = __float_as_uint(w1.x);
#pragma unroll
                    for (int q = 3; q >= 1; --q) {  // far to near
                        if (keys[q] != 0xffffffffu) {
                            const uint32_t s = keys[q] & 3u;
                            const int ch = (int)(child_base + (uint32_t)__popc(imask & ((1u << s) - 1u)));
                            if (sp <= SOLRT_BVH2_STACK) stack.put(sp++, ch);
                            else ef |= SOLRT_EFLAG_STACK;
                        }
                    }
                    if (keys[0] != 0xffffffffu) {
                        const uint32_t s = keys[0] & 3u;
                        node = (int)(child_base + (uint32_t)__popc(imask & ((1u << s) - 1u)));
                    } else {
                        node = stack.get(--sp);
                    }
                    tgrp = make_uint2(__float_as_uint(w1.y), ht);
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
                    node = kBvh2Sentinel;
                    sp = 1;
                } else {
                    const float4* tp = ts.tris + 3 * (size_t)ti;
                    if (kCount) ++cnt.tris;
                    cnt.fallbacks += intersect_tri(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), best);
                    if (io.any_hit && best.prim != SOLRT_NO_HIT) {  // occlusion query: done at the first hit
                        tgrp.y = 0u;
                        node = kBvh2Sentinel;
                        sp = 1;
                    }
                }
            }
        }
    }
}

// One ray, depth-first (nearest hit child first): the traversal of the
// per-pixel kernels.
SOLRT_D void trace_bvh4_ray(const TravScene& ts, float ox, float oy, float oz, float dx, float dy, float dz,
                            float tmin, float tmax, HitRec& best, TraceCounters& cnt, uint32_t& ef) {
    best = HitRec{tmax, SOLRT_NO_HIT, 0.0f, 0.0f};
    if (ts.tri_count == 0) return;
    const RayWT r = setup_ray(ox, oy, oz, dx, dy, dz, tmin);
    const float bx = box_dir(dx), by = box_dir(dy), bz = box_dir(dz);
    const float ix = 1.0f / bx, iy = 1.0f / by, iz = 1.0f / bz;
    const bool negx = signbit(bx), negy = signbit(by), negz = signbit(bz);
    int stack[SOLRT_BVH2_STACK + 1];
    stack[0] = kBvh2Sentinel;
    int sp = 1;
    int node = 0;
    uint32_t budget = 2u * (ts.node_count + ts.tri_count) + 64u;
    while (node != kBvh2Sentinel) {
        if (--budget == 0u || (uint32_t)node >= ts.node_count) {
            ef |= SOLRT_EFLAG_INDEX;
            return;
        }
        const float4* np = ts.nodes + 4 * (size_t)node;
        float4 w0, w1, w2, w3;
        ldg_2x4(np, w0, w1);
        ldg_2x4(np + 2, w2, w3);
        uint32_t keys[4], ht = 0;
        bvh4_node_test(w0, w1, w2, w3, ox, oy, oz, ix, iy, iz, negx, negy, negz, tmin, best.t, keys, ht);
        const uint32_t tri_base = __float_as_uint(w1.y);
        while (ht) {
            const uint32_t k = (uint32_t)(__ffs(ht) - 1);
            ht &= ht - 1u;
            const uint32_t ti = tri_base + k;
            if (ti >= ts.tri_count) {
                ef |= SOLRT_EFLAG_INDEX;
                return;
            }
            const float4* tp = ts.tris + 3 * (size_t)ti;
            cnt.fallbacks += intersect_tri(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), best);
        }
        sort4(keys);
        const uint32_t imask = __float_as_uint(w0.w) >> 24;
        const uint32_t child_base = __float_as_uint(w1.x);
        for (int q = 3; q >= 1; --q) {
            if (keys[q] != 0xffffffffu) {
                const uint32_t s = keys[q] & 3u;
                if (sp <= SOLRT_BVH2_STACK) stack[sp++] = (int)(child_base + (uint32_t)__popc(imask & ((1u << s) - 1u)));
                else ef |= SOLRT_EFLAG_STACK;
            }
        }
        if (keys[0] != 0xffffffffu) {
            const uint32_t s = keys[0] & 3u;
            node = (int)(child_base + (uint32_t)__popc(imask & ((1u << s) - 1u)));
        } else {
            node = stack[--sp];
        }
    }
}

}  // namespace solrt
