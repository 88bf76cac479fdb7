// traverse.cuh — closest-hit queries on sm_103a: what traceRayEXT does on RT
// cores in the reference (assets/glsl/pathtrace.rgen:65-76, opaque rays,
// TRIANGLE_FACING_CULL_DISABLE from src/ray/acceleration.rs:337).
//
// Intersection: watertight ray-triangle test (Woop, Benthin, Wald, JCGT 2013)
// in FP32, with the three edge functions recomputed in FP64 when one of them
// is exactly zero (the products of two floats are exact in FP64, so the sign
// of each edge function is then exact). Closest hit = smaller t, ties go to
// the lower global triangle index, so the answer does not depend on the BVH
// or on traversal order. Box tests are conservative (NaN-ignoring min/max and
// a relative 2^-16 widening of the far distance) so that rounding never culls
// a box that holds the closest hit.
#pragma once

#include "device_math.cuh"

namespace solrt {

// Device view of a scene: the shading stream (world-space vertices, triangle
// index records, materials) and the traversal stream (BVH nodes, triangles in
// BVH leaf order).
struct DevScene {
    uint32_t tri_count;
    uint32_t bvh_kind;
    uint32_t node_count;
    const float4* vpos;       // world position per vertex (.w unused)
    const float4* vnrm;       // world normal (transform_it applied, unnormalised)
    const float4* vcol;       // vertex colour
    const uint4* tri_idx;     // (v0, v1, v2, material) per original triangle
    const float4* materials;  // solrt_material as 3 float4
    const float4* nodes;      // BVH2: 4 float4 per node; BVH8: 5 float4 per node
    const float4* tri_wt;     // 3 float4 per triangle in leaf order; p0.w = prim bits
};

struct HitRec {
    float t;
    uint32_t prim;
    float u, v;
};

struct RayWT {
    float ox, oy, oz;
    float tmin;
    int kx, ky, kz;
    float sx, sy, sz;
};

SOLRT_D float comp(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

SOLRT_D RayWT setup_ray(float ox, float oy, float oz, float dx, float dy, float dz, float tmin) {
    RayWT r;
    r.ox = ox; r.oy = oy; r.oz = oz; r.tmin = tmin;
    int kz = 0;
    if (fabsf(dy) > fabsf(comp(dx, dy, dz, kz))) kz = 1;
    if (fabsf(dz) > fabsf(comp(dx, dy, dz, kz))) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    const float dkz = comp(dx, dy, dz, kz);
    if (dkz < 0.0f) { const int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.sx = comp(dx, dy, dz, kx) / dkz;
    r.sy = comp(dx, dy, dz, ky) / dkz;
    r.sz = 1.0f / dkz;
    return r;
}

// One triangle; updates `best` on a closer hit (or an equal t with a lower
// index). Returns 1 when the FP64 fallback ran.
SOLRT_D uint32_t intersect_tri(const RayWT& r, float4 q0, float4 q1, float4 q2, HitRec& best) {
    const uint32_t prim = __float_as_uint(q0.w);
    const float Ax0 = q0.x - r.ox, Ay0 = q0.y - r.oy, Az0 = q0.z - r.oz;
    const float Bx0 = q1.x - r.ox, By0 = q1.y - r.oy, Bz0 = q1.z - r.oz;
    const float Cx0 = q2.x - r.ox, Cy0 = q2.y - r.oy, Cz0 = q2.z - r.oz;
    const float Akx = comp(Ax0, Ay0, Az0, r.kx), Aky = comp(Ax0, Ay0, Az0, r.ky), Akz = comp(Ax0, Ay0, Az0, r.kz);
    const float Bkx = comp(Bx0, By0, Bz0, r.kx), Bky = comp(Bx0, By0, Bz0, r.ky), Bkz = comp(Bx0, By0, Bz0, r.kz);
    const float Ckx = comp(Cx0, Cy0, Cz0, r.kx), Cky = comp(Cx0, Cy0, Cz0, r.ky), Ckz = comp(Cx0, Cy0, Cz0, r.kz);
    const float ax = Akx - r.sx * Akz, ay = Aky - r.sy * Akz;
    const float bx = Bkx - r.sx * Bkz, by = Bky - r.sy * Bkz;
    const float cx = Ckx - r.sx * Ckz, cy = Cky - r.sy * Ckz;
    float U = cx * by - cy * bx;
    float V = ax * cy - ay * cx;
    float W = bx * ay - by * ax;
    uint32_t fb = 0;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        fb = 1;
        U = __double2float_rn((double)cx * (double)by - (double)cy * (double)bx);
        V = __double2float_rn((double)ax * (double)cy - (double)ay * (double)cx);
        W = __double2float_rn((double)bx * (double)ay - (double)by * (double)ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return fb;
    const float det = (U + V) + W;
    if (det == 0.0f) return fb;
    const float az = r.sz * Akz, bz = r.sz * Bkz, cz = r.sz * Ckz;
    const float T = (U * az + V * bz) + W * cz;
    const float t = T / det;
    if (!(t > r.tmin)) return fb;
    if (t < best.t || (t == best.t && prim < best.prim)) {
        best.t = t;
        best.prim = prim;
        best.u = V / det;
        best.v = W / det;
    }
    return fb;
}

// NaN-propagating min / max (PTX min.NaN / max.NaN). A slab distance is NaN
// only for 0 * inf: the ray is parallel to the axis and lies in a box plane.
// Then both the near and the far distance of that axis become NaN and the
// NaN-ignoring fminf / fmaxf across axes drop the axis: a ray in the plane of
// a face is inside that slab for every t.
SOLRT_D float min_nan(float a, float b) {
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
SOLRT_D float max_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// Slab test of a float box; conservative (see file comment).
SOLRT_D bool slab(float lox, float hix, float loy, float hiy, float loz, float hiz, float ox, float oy, float oz,
                  float ix, float iy, float iz, float tmin, float tmax, float& tnear) {
    const float x0 = (lox - ox) * ix, x1 = (hix - ox) * ix;
    const float y0 = (loy - oy) * iy, y1 = (hiy - oy) * iy;
    const float z0 = (loz - oz) * iz, z1 = (hiz - oz) * iz;
    const float tn = fmaxf(fmaxf(fmaxf(min_nan(x0, x1), min_nan(y0, y1)), min_nan(z0, z1)), tmin);
    const float tf = fminf(fminf(fminf(max_nan(x0, x1), max_nan(y0, y1)), max_nan(z0, z1)), tmax);
    tnear = tn;
    return tn <= tf * 1.0000153f;
}

struct TraceCounters {
    uint32_t nodes;
    uint32_t tris;
    uint32_t fallbacks;
};

// BVH2 node (64 B): child boxes of the two children and their references.
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (ref0, ref1, -, -) as int bits: >= 0 internal node, < 0 leaf ~k
//        (triangle k of the leaf-ordered stream).
#ifndef SOLRT_BVH2_STACK
#define SOLRT_BVH2_STACK 64
#endif

template <bool kCount>
SOLRT_D void trace_bvh2(const DevScene& sc, float ox, float oy, float oz, float dx, float dy, float dz, float tmin,
                        float tmax, HitRec& best, TraceCounters& cnt, uint32_t& eflags) {
    best.t = tmax;
    best.prim = SOLRT_NO_HIT;
    best.u = 0.0f;
    best.v = 0.0f;
    if (sc.tri_count == 0) return;
    const RayWT r = setup_ray(ox, oy, oz, dx, dy, dz, tmin);
    const float ix = 1.0f / dx, iy = 1.0f / dy, iz = 1.0f / dz;
    int stack[SOLRT_BVH2_STACK];
    int sp = 0;
    int node = 0;
    // A valid BVH2 visits each node and leaf at most once; a longer walk
    // means a malformed hierarchy: flag it and stop instead of looping.
    uint32_t budget = 2u * (sc.node_count + sc.tri_count) + 64u;
    for (;;) {
        if (--budget == 0u) {
            eflags |= SOLRT_EFLAG_INDEX;
            break;
        }
        if (node >= 0) {
            if ((uint32_t)node >= sc.node_count) {
                eflags |= SOLRT_EFLAG_INDEX;
                break;
            }
            const float4* np = sc.nodes + 4 * (size_t)node;
            const float4 n0 = __ldg(np + 0), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
            const int4 n3 = __ldg(reinterpret_cast<const int4*>(np + 3));
            if (kCount) ++cnt.nodes;
            float t0, t1;
            const bool h0 = slab(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, ox, oy, oz, ix, iy, iz, tmin, best.t, t0);
            const bool h1 = slab(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, ox, oy, oz, ix, iy, iz, tmin, best.t, t1);
            if (h0 && h1) {
                int nearc = n3.x, farc = n3.y;
                if (t1 < t0) { nearc = n3.y; farc = n3.x; }
                if (sp < SOLRT_BVH2_STACK) stack[sp++] = farc;
                else eflags |= SOLRT_EFLAG_STACK;
                node = nearc;
                continue;
            }
            if (h0) { node = n3.x; continue; }
            if (h1) { node = n3.y; continue; }
        } else {
            const uint32_t k = (uint32_t)(~node);
            if (k < sc.tri_count) {
                const float4* tp = sc.tri_wt + 3 * (size_t)k;
                if (kCount) ++cnt.tris;
                cnt.fallbacks += intersect_tri(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), best);
            } else {
                eflags |= SOLRT_EFLAG_INDEX;
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
}

}  // namespace solrt
