// traverse.cuh — closest-hit queries on sm_103a: what traceRayEXT does on RT
// cores in the reference (assets/glsl/pathtrace.rgen:65-76, opaque rays,
// TRIANGLE_FACING_CULL_DISABLE from src/ray/acceleration.rs:337).
//
// Intersection: watertight ray-triangle test (Woop, Benthin, Wald, JCGT 2013)
// in FP32, with the three edge functions recomputed in FP64 when one of them
// is exactly zero (the products of two floats are exact in FP64, so the sign
// of each edge function is then exact). Closest hit = smaller t, ties go to
// the lower global triangle index, so the answer does not depend on the BVH
// or on traversal order. Box tests are conservative (see slab_fma and the
// 8-wide test in bvh8_traverse.cuh) so that rounding never culls a box that
// holds the closest hit.
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
    uint32_t tlas_count;      // SOLRT_BVH2_TWO_LEVEL: TLAS nodes (0: nothing to hit)
    uint32_t inst_count;      // SOLRT_BVH2_TWO_LEVEL: entries of `inst` (one per section)
    const float4* tlas;       // SOLRT_BVH2_TWO_LEVEL: BVH2 nodes over instances (leaf ~section)
    const float4* inst;       // SOLRT_BVH2_TWO_LEVEL: per section inverse-transform rows 0-2, BLAS root
    const float4* vpos;       // world position per vertex (.w unused): the BVH builds
    const float4* opos;       // object-space position per vertex: shading
    const float4* vnc;        // per vertex its object-space normal and its colour (2 float4, 32 B: one
                              // 256-bit load and one DRAM sector): shading
    const uint4* tri_idx;     // (v0, v1, v2, section) per original triangle
    const float4* sections;   // per section its solrt_instance as 9 float4: (id, ..), transform
                              // columns, transform_it columns (column-major)
    const uint32_t* sec_mat;  // material index per section
    const float4* materials;  // solrt_material as 3 float4
    const float4* nodes;      // BVH2: 4 float4 per node; BVH8: 5 float4 per node
    const float4* tri_wt;     // 3 float4 per triangle in leaf order; p0.w = prim bits
    // light tree of next-event estimation over the emissive triangles, three
    // float4 per inner node: (left box centre, squared half-diagonal), the
    // same for the right child, (left power, right power, left ref, right
    // ref as bits; ref >= 0 an inner node, < 0 the triangle ~ref); root 0
    const float4* lights;
    uint32_t light_count;     // leaves (emissive triangles)
    // per triangle: (levels << 27) | branch bits (bit l set: right child at
    // level l) of its leaf in the light tree, ~0u when it is not a light
    const uint32_t* tri_light;
};

// What the traversal needs of a scene (per ray: rays of one launch may belong
// to different scenes).
struct TravScene {
    const float4* nodes;
    const float4* tris;
    uint32_t node_count;
    uint32_t tri_count;
    const float4* tlas;   // two-level scenes only (see DevScene)
    const float4* inst;
    uint32_t tlas_count;
    uint32_t inst_count;
};

SOLRT_HD TravScene trav_scene(const DevScene& s) {
    return TravScene{s.nodes, s.tri_wt, s.node_count, s.tri_count, s.tlas, s.inst, s.tlas_count, s.inst_count};
}

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

// Two consecutive float4 from a 32-byte-aligned address. With
// SOLRT_NODE_V8 one 256-bit load (PTX ld.global.nc.v8.f32, sm_100 and
// later): half the L1 load instructions / wavefronts of two 128-bit loads.
#ifndef SOLRT_NODE_V8
#define SOLRT_NODE_V8 1
#endif
SOLRT_D void ldg_2x4(const float4* p, float4& a, float4& b) {
#if SOLRT_NODE_V8
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
#else
    a = __ldg(p);
    b = __ldg(p + 1);
#endif
}

// Three-input min / max (PTX ISA min.f32 / max.f32 with three sources).
SOLRT_D float max3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
SOLRT_D float min3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Direction component for box tests: components below 2^-100 (exact zeros
// included) become +-2^-100 (sign kept) so that 1/d and o/d stay finite for
// |o| < 2^27. Over t < 2^20 the tilt this gives a ray lying in a box plane is
// below 2^-80, the absolute part of the face widening, so such a ray stays
// inside the slab.
SOLRT_D float box_dir(float v) { return fabsf(v) < 0x1p-100f ? copysignf(0x1p-100f, v) : v; }

// Slab test in the form t = fma(plane, 1/d, -o/d) (one instruction per
// plane). Its rounding error relative to |o/d| is covered by the widening of
// every BVH2 child box by a relative 2^-21 at build time (widen_lo /
// widen_hi) plus the relative 2^-16 widening of the far distance.
SOLRT_D bool slab_fma(float lox, float hix, float loy, float hiy, float loz, float hiz, float ix, float iy,
                      float iz, float nox, float noy, float noz, float tmin, float tmax, float& tnear) {
    const float x0 = fmaf(lox, ix, nox), x1 = fmaf(hix, ix, nox);
    const float y0 = fmaf(loy, iy, noy), y1 = fmaf(hiy, iy, noy);
    const float z0 = fmaf(loz, iz, noz), z1 = fmaf(hiz, iz, noz);
    const float tn = fmaxf(max3(fminf(x0, x1), fminf(y0, y1), fminf(z0, z1)), tmin);
    const float tf = fminf(min3(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1)), tmax);
    tnear = tn;
    return tn <= tf * 1.0000153f;
}

// Both child boxes of a BVH2 node (n0: child 0 x/y planes, n1: child 1 x/y
// planes, n2: z planes of both) against one ray: the same arithmetic as two
// slab_fma calls. With SOLRT_SLAB_F32X2 the 12 plane distances are six
// packed two-lane FMAs (PTX fma.rn.f32x2, sm_100 and later; each lane is an
// ordinary correctly rounded fma).
#ifndef SOLRT_SLAB_F32X2
#define SOLRT_SLAB_F32X2 1
#endif
SOLRT_D float2 fma_x2(float a0, float a1, float b, float c) {
    float2 r;
#if SOLRT_SLAB_F32X2
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %4};\n\t"
        "mov.b64 rc, {%5, %5};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a0), "f"(a1), "f"(b), "f"(c));
#else
    r.x = fmaf(a0, b, c);
    r.y = fmaf(a1, b, c);
#endif
    return r;
}
SOLRT_D void slab2_fma(const float4& n0, const float4& n1, const float4& n2, float ix, float iy, float iz,
                       float nox, float noy, float noz, float tmin, float tmax, bool& h0, float& t0, bool& h1,
                       float& t1) {
    const float2 x0 = fma_x2(n0.x, n0.y, ix, nox), y0 = fma_x2(n0.z, n0.w, iy, noy);
    const float2 z0 = fma_x2(n2.x, n2.y, iz, noz);
    const float2 x1 = fma_x2(n1.x, n1.y, ix, nox), y1 = fma_x2(n1.z, n1.w, iy, noy);
    const float2 z1 = fma_x2(n2.z, n2.w, iz, noz);
    const float tn0 = fmaxf(max3(fminf(x0.x, x0.y), fminf(y0.x, y0.y), fminf(z0.x, z0.y)), tmin);
    const float tf0 = fminf(min3(fmaxf(x0.x, x0.y), fmaxf(y0.x, y0.y), fmaxf(z0.x, z0.y)), tmax);
    const float tn1 = fmaxf(max3(fminf(x1.x, x1.y), fminf(y1.x, y1.y), fminf(z1.x, z1.y)), tmin);
    const float tf1 = fminf(min3(fmaxf(x1.x, x1.y), fmaxf(y1.x, y1.y), fmaxf(z1.x, z1.y)), tmax);
    t0 = tn0;
    t1 = tn1;
    h0 = tn0 <= tf0 * 1.0000153f;
    h1 = tn1 <= tf1 * 1.0000153f;
}

// BVH2-q16 nodes (32 B): (ref0, ref1, c0.x, c0.y, c0.z, c1.x, c1.y, c1.z),
// each axis word holding the child's low plane in bits 0-15 and its high
// plane in bits 16-31, in units of the scene grid's cell from its origin G
// (a 32-byte header before node 0: G.xyz, c.x, c.y, c.z). The plane
// distance is t = fma(2^23 + q, s, a) with per-ray s = c / d and
// a = (G - o) / d - 2^23 s; 2^23 + q is q placed in the mantissa of 2^23
// (exact, one byte permute). The build quantises outward with two cells of
// margin, which covers the rounding of a and s (see the grid rules there).
// Direction components below 2^-80 are replaced by +-2^-80 for these tests
// (2^23 s stays finite for cells up to 2^23).
SOLRT_D float box_dir_q16(float v) { return fabsf(v) < 0x1p-80f ? copysignf(0x1p-80f, v) : v; }
SOLRT_D float q16_lo(uint32_t w) { return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7410u)); }
SOLRT_D float q16_hi(uint32_t w) { return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7432u)); }

SOLRT_D void q16_ray(const float4* header, float ox, float oy, float oz, float dx, float dy, float dz, float& sx,
                     float& sy, float& sz, float& ax, float& ay, float& az) {
    float4 g0, g1;
    ldg_2x4(header, g0, g1);
    const float jx = 1.0f / box_dir_q16(dx), jy = 1.0f / box_dir_q16(dy), jz = 1.0f / box_dir_q16(dz);
    sx = g0.w * jx;
    sy = g1.x * jy;
    sz = g1.y * jz;
    ax = fmaf(-8388608.0f, sx, fmaf(g0.x, jx, -(ox * jx)));
    ay = fmaf(-8388608.0f, sy, fmaf(g0.y, jy, -(oy * jy)));
    az = fmaf(-8388608.0f, sz, fmaf(g0.z, jz, -(oz * jz)));
}

// Both child boxes of a BVH2-q16 node (a, b: its two halves) against one
// ray; the outputs of slab2_fma.
SOLRT_D void slab2_q16(const float4& a, const float4& b, float sx, float sy, float sz, float ax, float ay, float az,
                       float tmin, float tmax, bool& h0, float& t0, bool& h1, float& t1) {
    const uint32_t c0x = __float_as_uint(a.z), c0y = __float_as_uint(a.w), c0z = __float_as_uint(b.x);
    const uint32_t c1x = __float_as_uint(b.y), c1y = __float_as_uint(b.z), c1z = __float_as_uint(b.w);
    const float2 x0 = fma_x2(q16_lo(c0x), q16_hi(c0x), sx, ax), y0 = fma_x2(q16_lo(c0y), q16_hi(c0y), sy, ay);
    const float2 z0 = fma_x2(q16_lo(c0z), q16_hi(c0z), sz, az);
    const float2 x1 = fma_x2(q16_lo(c1x), q16_hi(c1x), sx, ax), y1 = fma_x2(q16_lo(c1y), q16_hi(c1y), sy, ay);
    const float2 z1 = fma_x2(q16_lo(c1z), q16_hi(c1z), sz, az);
    const float tn0 = fmaxf(max3(fminf(x0.x, x0.y), fminf(y0.x, y0.y), fminf(z0.x, z0.y)), tmin);
    const float tf0 = fminf(min3(fmaxf(x0.x, x0.y), fmaxf(y0.x, y0.y), fmaxf(z0.x, z0.y)), tmax);
    const float tn1 = fmaxf(max3(fminf(x1.x, x1.y), fminf(y1.x, y1.y), fminf(z1.x, z1.y)), tmin);
    const float tf1 = fminf(min3(fmaxf(x1.x, x1.y), fmaxf(y1.x, y1.y), fmaxf(z1.x, z1.y)), tmax);
    t0 = tn0;
    t1 = tn1;
    h0 = tn0 <= tf0 * 1.0000153f;
    h1 = tn1 <= tf1 * 1.0000153f;
}

// Outward widening of a box face by a relative 2^-21 (about 4 ulp) plus an
// absolute 2^-80 (which matters only near 0).
SOLRT_HD float widen_lo(float v) { return (v - fabsf(v) * 0x1p-21f) - 0x1p-80f; }
SOLRT_HD float widen_hi(float v) { return (v + fabsf(v) * 0x1p-21f) + 0x1p-80f; }

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

}  // namespace solrt
