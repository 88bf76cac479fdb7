// bvh2_2l.cuh — traversal of two-level scenes (SOLRT_BVH2_TWO_LEVEL): a
// binary TLAS over instances whose leaves are sections, each with a binary
// BLAS over its object-space triangles. This is what traceRayEXT does with
// the reference's TLAS / BLAS pair (src/ray/acceleration.rs:308-467): the
// ray enters an instance through the instance's inverse transform, so one
// BLAS serves every frame whatever the instance transform.
//
// The object-space ray is (M o + m, M d) with M, m the rows of the inverse
// transform (transform_it transposed, src/ray/mod.rs:116), each component
// evaluated as ((m0 x + m1 y) + m2 z) + m3 without contraction; the ray
// parameter t is the same in both spaces, so closest hits of different
// instances compare directly. A "leave instance" marker on the traversal
// stack separates an instance's entries from the TLAS entries below them.
#pragma once

#include "bvh2_ww.cuh"

namespace solrt {

constexpr int kBvh2LeaveInstance = 0x7ffffffe;

// Instance entry k: rows 0-2 of the inverse transform, then (BLAS root, -, -, -).
SOLRT_D void instance_ray(const float4* inst, uint32_t k, float ox, float oy, float oz, float dx, float dy, float dz,
                          float& px, float& py, float& pz, float& qx, float& qy, float& qz, int& root) {
    const float4* e = inst + 4 * (size_t)k;
    const float4 r0 = __ldg(e), r1 = __ldg(e + 1), r2 = __ldg(e + 2);
    root = __float_as_int(__ldg(e + 3).x);
    px = r0.x * ox + r0.y * oy + r0.z * oz + r0.w;
    py = r1.x * ox + r1.y * oy + r1.z * oz + r1.w;
    pz = r2.x * ox + r2.y * oy + r2.z * oz + r2.w;
    qx = r0.x * dx + r0.y * dy + r0.z * dz;
    qy = r1.x * dx + r1.y * dy + r1.z * dz;
    qz = r2.x * dx + r2.y * dy + r2.z * dz;
}

// Warp-organised traversal of two-level scenes: the while-while loop of
// extend_bvh2_ww, where a TLAS leaf reached by a lane is entered at once
// (ray transformed, marker pushed, BLAS root next), a parked triangle leaf
// is tested before its lane leaves the instance, and the marker restores the
// world ray (reloaded from the queue).
template <class IO, bool kCount, int kBlock, int kSmem>
SOLRT_D void extend_bvh2_2l_ww(const IO& io, uint32_t n, unsigned int* work, TraceCounters& cnt, uint32_t& ef) {
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    Bvh2Stack<kBlock, kSmem> stack;
    __shared__ int s_stack[(kSmem > 0 ? kSmem : 1) * kBlock];
    stack.sh = s_stack + threadIdx.x;
    int sp = 0;
    int node = kBvh2Sentinel;  // TLAS or BLAS node (>= 0), leaf (< 0), marker, or sentinel
    int leaf = 0;              // parked triangle leaf (< 0) or none (>= 0)
    int inst = -1;             // instance being traversed, -1 = the TLAS
    bool has = false;
    bool drained = false;
    uint32_t idx = 0, budget = 0;
    RayWT r;
    TravScene ts{nullptr, nullptr, 0u, 0u};
    float ix = 0.0f, iy = 0.0f, iz = 0.0f, nox = 0.0f, noy = 0.0f, noz = 0.0f;
    float tmin = 0.0f;
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
                    tmin = o.w;
                    bvh2_ray_consts<false>(ts.nodes, o.x, o.y, o.z, d.x, d.y, d.z, ix, iy, iz, nox, noy, noz);
                    best = HitRec{d.w, SOLRT_NO_HIT, 0.0f, 0.0f};
                    budget = 2u * (ts.node_count + ts.tri_count + ts.tlas_count + ts.inst_count) + 64u;
                    stack.put(0, kBvh2Sentinel);
                    sp = 1;
                    inst = -1;
                    node = (ts.tlas_count && ts.tri_count) ? 0 : kBvh2Sentinel;
                    leaf = 0;
                }
            }
        }
        if (!__any_sync(0xffffffffu, has)) {
            if (drained) break;
            continue;
        }
        // node phase: inner nodes of either level, instance entries and exits
        for (;;) {
            const bool inner = (unsigned)node < (unsigned)kBvh2LeaveInstance;
            const bool enter = node < 0 && inst < 0;
            const bool leave = node == kBvh2LeaveInstance && leaf >= 0;
            const bool act = inner || enter || leave;
            const uint32_t b_act = __ballot_sync(0xffffffffu, act);
            const uint32_t b_leaf = __ballot_sync(0xffffffffu, leaf < 0);
            if ((b_act & ~b_leaf) == 0u) break;
#if SOLRT_WW_NODE_MIN > 0
            if (__popc(b_act) < SOLRT_WW_NODE_MIN && b_leaf) break;
#endif
            if (!act) continue;
            if (--budget == 0u) {
                ef |= SOLRT_EFLAG_INDEX;
                node = kBvh2Sentinel;
                leaf = 0;
                continue;
            }
            if (leave) {  // back to the TLAS: world ray again
                float4 o, d;
                io.load_ray(idx, o, d);
                bvh2_ray_consts<false>(ts.nodes, o.x, o.y, o.z, d.x, d.y, d.z, ix, iy, iz, nox, noy, noz);
                inst = -1;
                node = stack.get(--sp);
                continue;
            }
            if (enter) {
                const uint32_t k = (uint32_t)(~node);
                int root = -1;
                if (k < ts.inst_count) {
                    float4 o, d;
                    io.load_ray(idx, o, d);
                    float px, py, pz, qx, qy, qz;
                    instance_ray(ts.inst, k, o.x, o.y, o.z, d.x, d.y, d.z, px, py, pz, qx, qy, qz, root);
                    if (root >= 0 && (uint32_t)root < ts.node_count && sp <= SOLRT_BVH2_STACK) {
                        r = setup_ray(px, py, pz, qx, qy, qz, tmin);
                        bvh2_ray_consts<false>(ts.nodes, px, py, pz, qx, qy, qz, ix, iy, iz, nox, noy, noz);
                        stack.put(sp++, kBvh2LeaveInstance);
                        inst = (int)k;
                        node = root;
                        continue;
                    }
                }
                ef |= (root < 0 && k < ts.inst_count) ? 0u : SOLRT_EFLAG_INDEX;  // empty section: skip it
                node = stack.get(--sp);
                continue;
            }
            // inner node of the current level
            const float4* arr = inst < 0 ? ts.tlas : ts.nodes;
            const uint32_t cnt_nodes = inst < 0 ? ts.tlas_count : ts.node_count;
            if ((uint32_t)node >= cnt_nodes) {
                ef |= SOLRT_EFLAG_INDEX;
                node = kBvh2Sentinel;
                leaf = 0;
                continue;
            }
            if (kCount) ++cnt.nodes;
            float t0, t1;
            bool h0, h1;
            int c0, c1;
            bvh2_node_step<false>(arr, node, ix, iy, iz, nox, noy, noz, tmin, best.t, h0, t0, h1, t1, c0, c1);
            h1 = h1 && c1 != c0;  // a node whose two children are the same (one instance, one triangle)
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
            if (inst >= 0 && node < 0 && leaf >= 0) {  // park a triangle, keep descending
                leaf = node;
                node = stack.get(--sp);
            }
        }
        // leaf phase: triangles in the object space of the lane's instance
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
                        if (node < 0) node = stack.get(--sp);  // a second parked triangle
                    }
                }
            }
        }
    }
}

// One ray, plain depth-first loop over both levels (megakernel, debug and
// AO pipelines).
SOLRT_D void trace_bvh2_2l_ray(const TravScene& ts, float ox, float oy, float oz, float dx, float dy, float dz,
                               float tmin, float tmax, HitRec& best, TraceCounters& cnt, uint32_t& ef) {
    best = HitRec{tmax, SOLRT_NO_HIT, 0.0f, 0.0f};
    if (ts.tri_count == 0 || ts.tlas_count == 0) return;
    RayWT r;
    float ix, iy, iz, nox, noy, noz;
    bvh2_ray_consts<false>(ts.nodes, ox, oy, oz, dx, dy, dz, ix, iy, iz, nox, noy, noz);
    int stack[SOLRT_BVH2_STACK + 1];
    stack[0] = kBvh2Sentinel;
    int sp = 1;
    int node = 0;
    int inst = -1;
    uint32_t budget = 2u * (ts.node_count + ts.tri_count + ts.tlas_count + ts.inst_count) + 64u;
    while (node != kBvh2Sentinel) {
        if (--budget == 0u) {
            ef |= SOLRT_EFLAG_INDEX;
            return;
        }
        if (node == kBvh2LeaveInstance) {
            bvh2_ray_consts<false>(ts.nodes, ox, oy, oz, dx, dy, dz, ix, iy, iz, nox, noy, noz);
            inst = -1;
        } else if (node < 0 && inst < 0) {
            const uint32_t k = (uint32_t)(~node);
            if (k >= ts.inst_count) {
                ef |= SOLRT_EFLAG_INDEX;
                return;
            }
            float px, py, pz, qx, qy, qz;
            int root;
            instance_ray(ts.inst, k, ox, oy, oz, dx, dy, dz, px, py, pz, qx, qy, qz, root);
            if (root >= 0) {
                if ((uint32_t)root >= ts.node_count || sp > SOLRT_BVH2_STACK) {
                    ef |= SOLRT_EFLAG_INDEX;
                    return;
                }
                r = setup_ray(px, py, pz, qx, qy, qz, tmin);
                bvh2_ray_consts<false>(ts.nodes, px, py, pz, qx, qy, qz, ix, iy, iz, nox, noy, noz);
                stack[sp++] = kBvh2LeaveInstance;
                inst = (int)k;
                node = root;
                continue;
            }
        } else if (node < 0) {
            const uint32_t k = (uint32_t)(~node);
            if (k >= ts.tri_count) {
                ef |= SOLRT_EFLAG_INDEX;
                return;
            }
            const float4* tp = ts.tris + 3 * (size_t)k;
            cnt.fallbacks += intersect_tri(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), best);
        } else {
            const float4* arr = inst < 0 ? ts.tlas : ts.nodes;
            if ((uint32_t)node >= (inst < 0 ? ts.tlas_count : ts.node_count)) {
                ef |= SOLRT_EFLAG_INDEX;
                return;
            }
            float t0, t1;
            bool h0, h1;
            int c0, c1;
            bvh2_node_step<false>(arr, node, ix, iy, iz, nox, noy, noz, tmin, best.t, h0, t0, h1, t1, c0, c1);
            h1 = h1 && c1 != c0;
            if (h0 && h1) {
                const bool swap = t1 < t0;
                if (sp <= SOLRT_BVH2_STACK) stack[sp++] = swap ? c0 : c1;
                else ef |= SOLRT_EFLAG_STACK;
                node = swap ? c1 : c0;
                continue;
            }
            if (h0) { node = c0; continue; }
            if (h1) { node = c1; continue; }
        }
        node = stack[--sp];
    }
}

}  // namespace solrt
