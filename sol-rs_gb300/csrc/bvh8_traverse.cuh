// bvh8_traverse.cuh — traversal of the 8-wide quantised BVH (bvh8.cuh).
//
// Stack of node groups (child base index, pending-child hit bits, internal
// mask), after the compressed-wide-BVH traversal of Ylitie, Karras and Laine
// (HPG 2017): a node test produces one 8-bit mask of hit internal children,
// stored in visiting order (bit s ^ octant for slot s, so slots are visited
// roughly near to far), and a 24-bit mask of hit leaf triangles, which are
// tested right away so that the closest distance shrinks early.
//
// Child box planes are decoded as p + q * 2^e from 8-bit q. The distance to
// a plane is fma(2^23 + q, 2^e / d, (p - o) / d - 2^23 * 2^e / d): the build
// keeps every face (the anchor plane q = 0 included: it sits one step below
// the node's box) at least one grid step away from the child's triangles,
// which bounds the rounding error of that form well inside the margin, and
// the relative 2^-16 widening of the far distance covers the rest. Zero
// direction components are replaced by box_dir for these tests only (the
// triangle test uses the exact direction). SOLRT_BVH8_F32 nodes hold the
// child boxes in FP32 and use the binary BVH's slab test instead.
#pragma once

#include "traverse.cuh"

namespace solrt {

#ifndef SOLRT_BVH8_STACK
#define SOLRT_BVH8_STACK 32
#endif

// byte k of `word` as the float 2^23 + byte, exactly.
SOLRT_D float byte_biased(uint32_t word, uint32_t k) {
    return __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7440u | k));
}

// 8-bit mask of the non-empty slots of a node from its meta bytes (m0:
// slots 0-3, m1: slots 4-7): a slot is used iff one of its meta bits 5-7 is
// set (internal children 0b001xxxxx, leaves (2^k - 1) << 5 with k >= 1).
// Bit 7 of each byte collects bits 5-7, moves to bit 0, and one multiply
// gathers the four byte bits into bits 24-27.
SOLRT_D uint32_t bvh8_used_mask(uint32_t m0, uint32_t m1) {
    const uint32_t v0 = ((m0 | (m0 << 1) | (m0 << 2)) >> 7) & 0x01010101u;
    const uint32_t v1 = ((m1 | (m1 << 1) | (m1 << 2)) >> 7) & 0x01010101u;
    return ((v0 * 0x01020408u) >> 24) | (((v1 * 0x01020408u) >> 24) << 4);
}

// Bit s of an 8-bit slot mask moved to bit s ^ oct (visiting order).
SOLRT_D uint32_t octant_order(uint32_t x, uint32_t oct) {
    if (oct & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
    if (oct & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
    if (oct & 4u) x = ((x & 0x0Fu) << 4) | ((x >> 4) & 0x0Fu);
    return x;
}

// Two lanes of a*b, each correctly rounded (PTX mul.rn.f32x2, sm_100 and
// later; see fma_x2).
SOLRT_D float2 mul_x2(float a0, float a1, float b) {
    float2 r;
#if SOLRT_SLAB_F32X2
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %4};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a0), "f"(a1), "f"(b));
#else
    r.x = a0 * b;
    r.y = a1 * b;
#endif
    return r;
}

// Tests the 8 children of one node. Returns the hit internal children in
// visiting order (bit s ^ oct for slot s) and the hit leaf triangles
// (bit o of the node's triangle range).
// Children are tested in pairs: each plane distance of two neighbouring
// slots is one packed two-lane FMA (every lane the same correctly rounded
// fma as a scalar one), and the far distances are widened in pairs, so the
// hit decisions are those of one child at a time. The 8-bit hit mask is
// then cut to the used slots, split into internal children (put in
// visiting order once per node) and leaves (only the hit leaf slots read
// their meta byte).
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
    uint32_t hit = 0;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const uint32_t k0 = (uint32_t)((2 * p) & 3), k1 = k0 + 1u;
        const uint32_t nxw = p < 2 ? nx0 : nx1, nyw = p < 2 ? ny0 : ny1, nzw = p < 2 ? nz0 : nz1;
        const uint32_t fxw = p < 2 ? fx0 : fx1, fyw = p < 2 ? fy0 : fy1, fzw = p < 2 ? fz0 : fz1;
        const float2 tnx = fma_x2(byte_biased(nxw, k0), byte_biased(nxw, k1), sx, ax);
        const float2 tny = fma_x2(byte_biased(nyw, k0), byte_biased(nyw, k1), sy, ay);
        const float2 tnz = fma_x2(byte_biased(nzw, k0), byte_biased(nzw, k1), sz, az);
        const float2 tfx = fma_x2(byte_biased(fxw, k0), byte_biased(fxw, k1), sx, ax);
        const float2 tfy = fma_x2(byte_biased(fyw, k0), byte_biased(fyw, k1), sy, ay);
        const float2 tfz = fma_x2(byte_biased(fzw, k0), byte_biased(fzw, k1), sz, az);
        const float tn0 = max3(tnx.x, tny.x, fmaxf(tnz.x, tmin)), tn1 = max3(tnx.y, tny.y, fmaxf(tnz.y, tmin));
        const float2 tf = mul_x2(min3(tfx.x, tfy.x, fminf(tfz.x, tmax)), min3(tfx.y, tfy.y, fminf(tfz.y, tmax)),
                                 1.0000153f);
        if (tn0 <= tf.x) hit |= 1u << (2 * p);
        if (tn1 <= tf.y) hit |= 2u << (2 * p);
    }
    hit &= bvh8_used_mask(w1.z, w1.w);
    hit_inner = octant_order(hit & imask, oct);
    hit_tri = 0;
    for (uint32_t leaves = hit & ~imask; leaves; leaves &= leaves - 1u) {
        const uint32_t s = (uint32_t)(__ffs(leaves) - 1);
        const uint32_t meta = __byte_perm(w1.z, w1.w, s) & 0xffu;
        hit_tri |= (meta >> 5) << (meta & 31u);
    }
}

// The same outputs for a full-precision node (SOLRT_BVH8_F32, 224 B at np):
// the slab test of the binary BVH (fma(plane, 1/d, -o/d) against child boxes
// widened at build time) on 8 children, one axis at a time.
SOLRT_D void bvh8f_node_test(const float4* np, float ix, float iy, float iz, float nox, float noy, float noz,
                             uint32_t oct, float tmin, float tmax, uint32_t& hit_inner, uint32_t& hit_tri,
                             uint32_t& child_base, uint32_t& tri_base, uint32_t& imask) {
    float4 h0, h1;
    ldg_2x4(np, h0, h1);
    child_base = __float_as_uint(h0.x);
    tri_base = __float_as_uint(h0.y);
    const uint32_t meta0 = __float_as_uint(h0.z), meta1 = __float_as_uint(h0.w);
    imask = __float_as_uint(h1.x);
    float tn[8], tf[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        tn[s] = tmin;
        tf[s] = tmax;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float4 l0, l1, u0, u1;
        ldg_2x4(np + 2 + 4 * a, l0, l1);
        ldg_2x4(np + 4 + 4 * a, u0, u1);
        const float inv = a == 0 ? ix : (a == 1 ? iy : iz);
        const float no = a == 0 ? nox : (a == 1 ? noy : noz);
        const float lo[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
        const float hi[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const float t0 = fmaf(lo[s], inv, no), t1 = fmaf(hi[s], inv, no);
            tn[s] = fmaxf(tn[s], fminf(t0, t1));
            tf[s] = fminf(tf[s], fmaxf(t0, t1));
        }
    }
    hit_inner = 0;
    hit_tri = 0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const uint32_t meta = ((s < 4 ? meta0 : meta1) >> (8u * (uint32_t)(s & 3))) & 0xffu;
        if (meta != 0u && tn[s] <= tf[s] * 1.0000153f) {
            if (imask & (1u << s)) hit_inner |= 1u << ((uint32_t)s ^ oct);
            else hit_tri |= (meta >> 5) << (meta & 31u);
        }
    }
}

template <bool kCount, bool kF32 = false>
SOLRT_D void trace_bvh8(const TravScene& sc, float ox, float oy, float oz, float dx, float dy, float dz, float tmin,
                        float tmax, HitRec& best, TraceCounters& cnt, uint32_t& eflags) {
    best.t = tmax;
    best.prim = SOLRT_NO_HIT;
    best.u = 0.0f;
    best.v = 0.0f;
    if (sc.tri_count == 0) return;
    const RayWT r = setup_ray(ox, oy, oz, dx, dy, dz, tmin);
    const float bx = box_dir(dx), by = box_dir(dy), bz = box_dir(dz);
    const float ix = 1.0f / bx, iy = 1.0f / by, iz = 1.0f / bz;
    const float nox = -(ox * ix), noy = -(oy * iy), noz = -(oz * iz);
    const bool negx = signbit(bx), negy = signbit(by), negz = signbit(bz);
    const uint32_t oct = (negx ? 1u : 0u) | (negy ? 2u : 0u) | (negz ? 4u : 0u);
    const uint4* nodes = reinterpret_cast<const uint4*>(sc.nodes);

    uint2 stack[SOLRT_BVH8_STACK];
    int sp = 0;
    uint2 group = make_uint2(0u, 0u);  // (child base, pending hit bits << 24 | internal mask)
    uint32_t node = 0;
    uint32_t budget = 2u * (sc.node_count + sc.tri_count) + 64u;
    for (;;) {
        if (--budget == 0u || node >= sc.node_count) {
            eflags |= SOLRT_EFLAG_INDEX;
            break;
        }
        if (kCount) ++cnt.nodes;
        uint32_t hit_inner = 0, hit_tri = 0, child_base = 0, tri_base = 0, imask = 0;
        if (kF32) {
            bvh8f_node_test(sc.nodes + 14 * (size_t)node, ix, iy, iz, nox, noy, noz, oct, tmin, best.t, hit_inner,
                            hit_tri, child_base, tri_base, imask);
        } else {
            const uint4* np = nodes + 5 * (size_t)node;
            const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3),
                        w4 = __ldg(np + 4);
            bvh8_node_test(w0, w1, w2, w3, w4, ox, oy, oz, ix, iy, iz, negx, negy, negz, oct, tmin, best.t,
                           hit_inner, hit_tri);
            child_base = w1.x;
            tri_base = w1.y;
            imask = w0.w >> 24;
        }
        while (hit_tri) {
            const uint32_t k = (uint32_t)(__ffs(hit_tri) - 1);
            hit_tri &= hit_tri - 1u;
            const uint32_t ti = tri_base + k;
            if (ti < sc.tri_count) {
                const float4* tp = sc.tris + 3 * (size_t)ti;
                if (kCount) ++cnt.tris;
                cnt.fallbacks += intersect_tri(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), best);
            } else {
                eflags |= SOLRT_EFLAG_INDEX;
            }
        }
        if (hit_inner) {
            if (group.y >> 24) {
                if (sp < SOLRT_BVH8_STACK) stack[sp++] = group;
                else eflags |= SOLRT_EFLAG_STACK;
            }
            group = make_uint2(child_base, (hit_inner << 24) | imask);
        }
        if ((group.y >> 24) == 0u) {
            if (sp == 0) break;
            group = stack[--sp];
        }
        const uint32_t j = (uint32_t)(__ffs(group.y >> 24) - 1);
        group.y &= ~(1u << (24u + j));
        const uint32_t s = j ^ oct;
        node = group.x + (uint32_t)__popc(group.y & ((1u << s) - 1u) & 0xffu);
    }
}

}  // namespace solrt
