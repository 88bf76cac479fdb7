// oracle.cpp — CPU oracle of the solrt path tracer. TEST INFRASTRUCTURE ONLY.
//
// Loaded (through ctypes) by the tests, the smoke check and the CPU-baseline
// leg of the benchmark, as the checker. Product code never links it.
//
// Scalar C++17, templated on the real type R (float for bit-exact parity with
// the device code, double for the converged FP64 reference images). Built
// with -ffp-contract=off so that every a*b+c is two rounded operations, which
// is what the device code does (nvcc -fmad=false). Each function cites the
// reference line it restates. Parity status is stated in oracle.h.

#include "oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// RNG (assets/glsl/sampling.glsl:18-42)
// ---------------------------------------------------------------------------

// 16 rounds of TEA on (val0, val1); sampling.glsl:18-32.
uint32_t tea(uint32_t val0, uint32_t val1) {
    uint32_t v0 = val0, v1 = val1, s0 = 0;
    for (int n = 0; n < 16; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

// LCG step + PCG RXS-M-XS output; sampling.glsl:35-42.
uint32_t pcg_word(uint32_t& rng) {
    rng = rng * 747796405u + 1u;
    uint32_t word = ((rng >> ((rng >> 28) + 4u)) ^ rng) * 277803737u;
    word = (word >> 22) ^ word;
    return word;
}

template <class R> R next_rand(uint32_t& rng);
template <> float next_rand<float>(uint32_t& rng) {
    return (float)pcg_word(rng) / 4294967295.0f;
}
template <> double next_rand<double>(uint32_t& rng) {
    return (double)pcg_word(rng) / 4294967295.0;
}

// ---------------------------------------------------------------------------
// sin / cos. The FP32 path uses one fixed polynomial evaluation shared (as a
// specification, not as code) with the device kernels so that secondary ray
// directions agree bit for bit: Cody-Waite reduction by pi/2 with a three-part
// split of pi/2 (8 + 12 + 24 significant bits), then the Taylor series of sin
// to x^9 and of cos to x^10 on |r| <= pi/4 (truncation < 2e-9), Horner order.
// The FP64 path uses the C library.
// ---------------------------------------------------------------------------

void sincos_poly(float x, float& s_out, float& c_out) {
    const float k = std::rint(x * 0x1.45f306p-1f);  // x * 2/pi
    float r = x - k * 0x1.92p+0f;                   // pi/2, bits 1-8
    r = r - k * 0x1.fb4p-12f;                       // pi/2, bits 9-20
    r = r - k * 0x1.4442d2p-24f;                    // pi/2, next 24 bits
    const float r2 = r * r;
    float ps = 0x1.71de3ap-19f;                     //  1/9!
    ps = ps * r2 + -0x1.a01a02p-13f;                // -1/7!
    ps = ps * r2 + 0x1.111112p-7f;                  //  1/5!
    ps = ps * r2 + -0x1.555556p-3f;                 // -1/3!
    const float s = r + (r * r2) * ps;
    float pc = -0x1.27e4fcp-22f;                    // -1/10!
    pc = pc * r2 + 0x1.a01a02p-16f;                 //  1/8!
    pc = pc * r2 + -0x1.6c16c2p-10f;                // -1/6!
    pc = pc * r2 + 0x1.555556p-5f;                  //  1/4!
    pc = pc * r2 + -0.5f;                           // -1/2!
    const float c = 1.0f + r2 * pc;
    const int q = ((int)k) & 3;
    switch (q) {
        case 0: s_out = s; c_out = c; break;
        case 1: s_out = c; c_out = -s; break;
        case 2: s_out = -s; c_out = -c; break;
        default: s_out = -c; c_out = s; break;
    }
}

template <class R> void sincos_r(R x, R& s, R& c);
template <> void sincos_r<float>(float x, float& s, float& c) { sincos_poly(x, s, c); }
template <> void sincos_r<double>(double x, double& s, double& c) {
    s = std::sin(x);
    c = std::cos(x);
}

// ---------------------------------------------------------------------------
// Small vector type with GLSL component-wise semantics. Every expression is
// written in the evaluation order of the GLSL source.
// ---------------------------------------------------------------------------

template <class R> struct V3 {
    R x, y, z;
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> R dot(V3<R> a, V3<R> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class R> R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> V3<R> normalize(V3<R> a) {
    const R l = length(a);
    return {a.x / l, a.y / l, a.z / l};
}
template <class R> R saturate(R x) { return std::min(std::max(x, R(0)), R(1)); }
template <class R> R glsl_sign(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }
// GLSL reflect(I, N) = I - 2 * dot(N, I) * N.
template <class R> V3<R> reflect(V3<R> i, V3<R> n) {
    const R k = R(2) * dot(n, i);
    return i - k * n;
}
// GLSL mix(x, y, a) = x * (1 - a) + y * a.
template <class R> V3<R> mix(V3<R> x, V3<R> y, R a) { return x * (R(1) - a) + y * a; }
template <class R> R smoothstep(R e0, R e1, R x) {
    R t = (x - e0) / (e1 - e0);
    t = std::min(std::max(t, R(0)), R(1));
    return (t * t) * (R(3) - R(2) * t);
}

// column-major mat4 (as float[16]) times (x, y, z, w), summed column by column.
template <class R> void mat4_mul(const float* m, R x, R y, R z, R w, R out[4]) {
    for (int r = 0; r < 4; ++r) {
        out[r] = ((R(m[0 + r]) * x + R(m[4 + r]) * y) + R(m[8 + r]) * z) + R(m[12 + r]) * w;
    }
}

template <class R> R two_pi();
template <> float two_pi<float>() { return 6.28318530718f; }
template <> double two_pi<double>() { return 6.28318530718; }

// ---------------------------------------------------------------------------
// Sampling (assets/glsl/sampling.glsl:52-96)
// ---------------------------------------------------------------------------

// sampling.glsl:52-64
template <class R> R fresnel_dielectric(V3<R> i, V3<R> m, R eta) {
    R result = R(1);
    const R cos_i = std::abs(dot(i, m));
    const R sin_o2 = (eta * eta) * (R(1) - cos_i * cos_i);
    if (sin_o2 <= R(1)) {
        const R cos_o = std::sqrt(saturate(R(1) - sin_o2));
        const R rs = (cos_i - eta * cos_o) / (cos_i + eta * cos_o);
        const R rp = (eta * cos_i - cos_o) / (eta * cos_i + cos_o);
        result = R(0.5) * (rs * rs + rp * rp);
    }
    return result;
}

// sampling.glsl:66-73 (branchless ONB, Duff et al. 2017)
template <class R> void onb(V3<R> n, V3<R>& u, V3<R>& v) {
    const R s = n.z < R(0) ? R(-1) : R(1);
    const R a = R(-1) / (s + n.z);
    const R b = n.x * n.y * a;
    u = V3<R>{R(1) + s * n.x * n.x * a, s * b, -s * n.x};
    v = V3<R>{b, s + n.y * n.y * a, -n.y};
}

// sampling.glsl:75-84
template <class R> V3<R> align_to_direction(V3<R> n, R cos_t, R phi) {
    const R sin_t = std::sqrt(saturate(R(1) - cos_t * cos_t));
    V3<R> u, v;
    onb(n, u, v);
    R sp, cp;
    sincos_r(phi, sp, cp);
    return (u * cp + v * sp) * sin_t + n * cos_t;
}

// sampling.glsl:86-90
template <class R> V3<R> sample_ggx(V3<R> n, R xi0, R xi1, R alpha2) {
    const R cos_t = std::sqrt(saturate((R(1) - xi0) / (xi0 * (alpha2 - R(1)) + R(1))));
    return align_to_direction(n, cos_t, xi1 * two_pi<R>());
}

// sampling.glsl:92-96
template <class R> V3<R> sample_cosine(V3<R> n, R xi0, R xi1) {
    const R cos_t = std::sqrt(xi0);
    return align_to_direction(n, cos_t, xi1 * two_pi<R>());
}

// pathtrace.rmiss:8-21 plus the gradient sky.
template <class R> V3<R> miss_color(V3<R> dir, uint32_t mode) {
    if (mode == SOLRT_MISS_REF_SKY) {
        const V3<R> wi = normalize(dir);
        const R t = smoothstep(R(0.35f), R(0.65f), R(0.5f) * (wi.y + R(1)));
        const V3<R> sky = mix(V3<R>{R(0.58f), R(0.45f), R(0.25f)}, V3<R>{R(0.3f), R(0.4f), R(0.5f)}, t);
        const V3<R> sun_dir = normalize(V3<R>{R(0), R(1), R(-0.25f)});
        const bool is_sun = dot(wi, sun_dir) > R(0.99f);
        return mix(sky, V3<R>{R(120), R(100), R(50)}, is_sun ? R(1) : R(0));
    }
    if (mode == SOLRT_MISS_GRADIENT) {
        const V3<R> wi = normalize(dir);
        const R t = R(0.5f) * (wi.y + R(1));
        return mix(V3<R>{R(1), R(1), R(1)}, V3<R>{R(0.5f), R(0.7f), R(1)}, t);
    }
    return V3<R>{R(0), R(0), R(0)};
}

// ---------------------------------------------------------------------------
// Scene
// ---------------------------------------------------------------------------

struct TriW {
    V3<float> p[3];   // world-space positions (intersection)
    V3<float> n[3];   // world-space (unnormalised) normals (export)
    V3<float> c[3];   // vertex colours
    V3<float> op[3];  // object-space positions and normals (shading)
    V3<float> on[3];
    uint32_t mat;
    uint32_t sec;     // section
};

struct Box {
    float lo[3], hi[3];
};

}  // namespace

struct oracle_scene {
    std::vector<TriW> tris;
    std::vector<solrt_material> mats;
    // two-level mode (SOLRT_BVH2_TWO_LEVEL): object-space triangles, each
    // section's triangle range and the rows 0-2 of its inverse transform
    // (transform_it transposed)
    bool two_level = false;
    std::vector<TriW> obj;
    std::vector<uint32_t> sec_first, sec_count;
    std::vector<std::array<float, 12>> minv;
    // per section its instance's transform and transform_it (column-major)
    std::vector<std::array<float, 16>> sec_t, sec_tit;
    // LBVH
    std::vector<uint32_t> order;         // sorted position -> triangle
    std::vector<uint32_t> morton;        // sorted codes
    std::vector<uint32_t> child;         // 2 per internal node
    std::vector<Box> node_box;           // per internal node
    std::vector<Box> leaf_box;           // per sorted position
    // next-event estimation: light tree over the emissive triangles; each
    // inner node holds its two children's box centre, squared half-diagonal,
    // power and ref (>= 0 an inner node, < 0 the triangle ~ref)
    struct LightNode {
        float c[2][3], r2[2], power[2];
        int32_t ref[2];
    };
    std::vector<LightNode> light_tree;
    // per triangle: (levels << 27) | branch bits of its leaf, ~0u if not a light
    std::vector<uint32_t> tri_light;
};

namespace {

// src/ray/mod.rs:113-118 gives each section transform and transform_it;
// pathtrace.rchit:80-90 applies them to the interpolated normal and position.
// Here they are applied per vertex before interpolation (equal in exact
// arithmetic; the device upload does the same in the same order).
bool flatten(const solrt_scene_desc* d, oracle_scene* s) {
    static const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    s->mats.assign(d->materials, d->materials + d->material_count);
    for (uint32_t si = 0; si < d->section_count; ++si) {
        const solrt_section& sec = d->sections[si];
        if (sec.index_count % 3 != 0) return false;
        if ((uint64_t)sec.vertex_offset + sec.vertex_count > d->vertex_count) return false;
        if ((uint64_t)sec.index_offset + sec.index_count > d->index_count) return false;
        if (sec.material_index >= d->material_count) return false;
        const float* T = d->instances ? d->instances[si].transform : ident;
        const float* Tit = d->instances ? d->instances[si].transform_it : ident;
        s->sec_first.push_back((uint32_t)s->tris.size());
        s->sec_count.push_back(sec.index_count / 3);
        std::array<float, 12> mi;
        for (int k = 0; k < 12; ++k) mi[k] = Tit[k];  // row r of the transpose = Tit[4r .. 4r + 3]
        s->minv.push_back(mi);
        std::array<float, 16> t16, ti16;
        for (int k = 0; k < 16; ++k) {
            t16[k] = T[k];
            ti16[k] = Tit[k];
        }
        s->sec_t.push_back(t16);
        s->sec_tit.push_back(ti16);
        for (uint32_t t = 0; t < sec.index_count / 3; ++t) {
            TriW tw, to;
            for (int k = 0; k < 3; ++k) {
                const uint32_t li = d->indices[sec.index_offset + 3 * t + k];
                if (li >= sec.vertex_count) return false;
                const solrt_vertex& v = d->vertices[sec.vertex_offset + li];
                float o[4];
                mat4_mul<float>(T, v.pos[0], v.pos[1], v.pos[2], 1.0f, o);
                tw.p[k] = V3<float>{o[0], o[1], o[2]};
                to.p[k] = V3<float>{v.pos[0], v.pos[1], v.pos[2]};
                mat4_mul<float>(Tit, v.normal[0], v.normal[1], v.normal[2], 0.0f, o);
                tw.n[k] = V3<float>{o[0], o[1], o[2]};
                tw.op[k] = V3<float>{v.pos[0], v.pos[1], v.pos[2]};
                tw.on[k] = V3<float>{v.normal[0], v.normal[1], v.normal[2]};
                tw.c[k] = V3<float>{v.color[0], v.color[1], v.color[2]};
            }
            tw.mat = sec.material_index;
            tw.sec = si;
            s->tris.push_back(tw);
            to.mat = sec.material_index;
            s->obj.push_back(to);
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// LBVH (Karras 2012): 30-bit Morton codes of triangle centroids normalised to
// the centroid bounds, stable sort, radix-tree hierarchy, bottom-up boxes.
// ---------------------------------------------------------------------------

uint32_t expand_bits10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

uint32_t quantise10(float c, float lo, float ext) {
    if (!(ext > 0.0f)) return 0;
    const float f = ((c - lo) / ext) * 1024.0f;
    if (f >= 1023.0f) return 1023;
    if (!(f > 0.0f)) return 0;
    return (uint32_t)f;
}

int clz32(uint32_t x) { return x == 0 ? 32 : __builtin_clz(x); }

void build_lbvh(oracle_scene* s) {
    const uint32_t n = (uint32_t)s->tris.size();
    s->order.clear(); s->morton.clear(); s->child.clear(); s->node_box.clear(); s->leaf_box.clear();
    if (n == 0) return;
    std::vector<V3<float>> cen(n);
    float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < n; ++i) {
        const TriW& t = s->tris[i];
        cen[i] = V3<float>{((t.p[0].x + t.p[1].x) + t.p[2].x) / 3.0f,
                           ((t.p[0].y + t.p[1].y) + t.p[2].y) / 3.0f,
                           ((t.p[0].z + t.p[1].z) + t.p[2].z) / 3.0f};
        for (int a = 0; a < 3; ++a) {
            cmin[a] = std::min(cmin[a], cen[i][a]);
            cmax[a] = std::max(cmax[a], cen[i][a]);
        }
    }
    const float ext = std::max(std::max(cmax[0] - cmin[0], cmax[1] - cmin[1]), cmax[2] - cmin[2]);  // cubic cells
    std::vector<uint32_t> code(n);
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t qx = quantise10(cen[i].x, cmin[0], ext);
        const uint32_t qy = quantise10(cen[i].y, cmin[1], ext);
        const uint32_t qz = quantise10(cen[i].z, cmin[2], ext);
        code[i] = (expand_bits10(qx) << 2) | (expand_bits10(qy) << 1) | expand_bits10(qz);
    }
    s->order.resize(n);
    for (uint32_t i = 0; i < n; ++i) s->order[i] = i;
    std::stable_sort(s->order.begin(), s->order.end(),
                     [&](uint32_t a, uint32_t b) { return code[a] < code[b]; });
    s->morton.resize(n);
    for (uint32_t k = 0; k < n; ++k) s->morton[k] = code[s->order[k]];
    s->leaf_box.resize(n);
    for (uint32_t k = 0; k < n; ++k) {
        const TriW& t = s->tris[s->order[k]];
        for (int a = 0; a < 3; ++a) {
            s->leaf_box[k].lo[a] = std::min(std::min(t.p[0][a], t.p[1][a]), t.p[2][a]);
            s->leaf_box[k].hi[a] = std::max(std::max(t.p[0][a], t.p[1][a]), t.p[2][a]);
        }
    }
    if (n == 1) return;
    const uint32_t* k = s->morton.data();
    auto delta = [&](int64_t i, int64_t j) -> int {
        if (j < 0 || j > (int64_t)n - 1) return -1;
        const uint32_t a = k[i], b = k[j];
        if (a == b) return 32 + clz32((uint32_t)i ^ (uint32_t)j);
        return clz32(a ^ b);
    };
    s->child.assign(2 * (n - 1), 0);
    std::vector<uint32_t> parent_int(n - 1, 0xffffffffu), parent_leaf(n, 0xffffffffu);
    for (int64_t i = 0; i < (int64_t)n - 1; ++i) {
        const int d = (delta(i, i + 1) - delta(i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = delta(i, i - d);
        int64_t lmax = 2;
        while (delta(i, i + lmax * d) > dmin) lmax *= 2;
        int64_t l = 0;
        for (int64_t t = lmax / 2; t >= 1; t /= 2)
            if (delta(i, i + (l + t) * d) > dmin) l += t;
        const int64_t j = i + l * d;
        const int dnode = delta(i, j);
        int64_t sp = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (delta(i, i + (sp + t) * d) > dnode) sp += t;
        } while (t > 1);
        const int64_t gamma = i + sp * d + std::min(d, 0);
        const int64_t lo = std::min(i, j), hi = std::max(i, j);
        uint32_t left, right;
        if (lo == gamma) { left = 0x80000000u | (uint32_t)gamma; parent_leaf[gamma] = (uint32_t)i; }
        else { left = (uint32_t)gamma; parent_int[gamma] = (uint32_t)i; }
        if (hi == gamma + 1) { right = 0x80000000u | (uint32_t)(gamma + 1); parent_leaf[gamma + 1] = (uint32_t)i; }
        else { right = (uint32_t)(gamma + 1); parent_int[gamma + 1] = (uint32_t)i; }
        s->child[2 * i] = left;
        s->child[2 * i + 1] = right;
    }
    // bottom-up boxes: a node is complete when both children are.
    s->node_box.assign(n - 1, Box{});
    std::vector<uint8_t> arrived(n - 1, 0);
    auto box_of = [&](uint32_t ref) -> const Box& {
        return (ref & 0x80000000u) ? s->leaf_box[ref & 0x7fffffffu] : s->node_box[ref];
    };
    for (uint32_t leaf = 0; leaf < n; ++leaf) {
        uint32_t p = parent_leaf[leaf];
        while (p != 0xffffffffu) {
            if (++arrived[p] < 2) break;
            const Box& a = box_of(s->child[2 * p]);
            const Box& b = box_of(s->child[2 * p + 1]);
            for (int ax = 0; ax < 3; ++ax) {
                s->node_box[p].lo[ax] = std::min(a.lo[ax], b.lo[ax]);
                s->node_box[p].hi[ax] = std::max(a.hi[ax], b.hi[ax]);
            }
            p = parent_int[p];
        }
    }
}

// ---------------------------------------------------------------------------
// Watertight ray-triangle test (Woop, Benthin, Wald, JCGT 2013), no culling
// (TRIANGLE_FACING_CULL_DISABLE, src/ray/acceleration.rs:337). Zero edge
// functions are recomputed in FP64 (products of floats are exact there).
// Closest hit: smaller t, then lower global triangle index.
// ---------------------------------------------------------------------------

template <class R> struct RayWT {
    V3<R> o, d;
    R tmin;
    int kx, ky, kz;
    R sx, sy, sz;
};

template <class R> RayWT<R> setup_ray(V3<R> o, V3<R> d, R tmin) {
    RayWT<R> r;
    r.o = o; r.d = d; r.tmin = tmin;
    int kz = 0;
    if (std::abs(d.y) > std::abs(d[kz])) kz = 1;
    if (std::abs(d.z) > std::abs(d[kz])) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (d[kz] < R(0)) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.sx = d[kx] / d[kz];
    r.sy = d[ky] / d[kz];
    r.sz = R(1) / d[kz];
    return r;
}

template <class R> struct HitR {
    R t;
    uint32_t prim;
    R u, v;
};

template <class R>
inline void intersect_tri(const RayWT<R>& r, const TriW& tri, uint32_t prim, HitR<R>& best, uint64_t& fb) {
    const V3<R> p0{R(tri.p[0].x), R(tri.p[0].y), R(tri.p[0].z)};
    const V3<R> p1{R(tri.p[1].x), R(tri.p[1].y), R(tri.p[1].z)};
    const V3<R> p2{R(tri.p[2].x), R(tri.p[2].y), R(tri.p[2].z)};
    const V3<R> A = p0 - r.o, B = p1 - r.o, C = p2 - r.o;
    const R ax = A[r.kx] - r.sx * A[r.kz], ay = A[r.ky] - r.sy * A[r.kz];
    const R bx = B[r.kx] - r.sx * B[r.kz], by = B[r.ky] - r.sy * B[r.kz];
    const R cx = C[r.kx] - r.sx * C[r.kz], cy = C[r.ky] - r.sy * C[r.kz];
    R U = cx * by - cy * bx;
    R V = ax * cy - ay * cx;
    R W = bx * ay - by * ax;
    if (std::is_same<R, float>::value && (U == R(0) || V == R(0) || W == R(0))) {
        ++fb;
        U = (R)((double)cx * (double)by - (double)cy * (double)bx);
        V = (R)((double)ax * (double)cy - (double)ay * (double)cx);
        W = (R)((double)bx * (double)ay - (double)by * (double)ax);
    }
    if ((U < R(0) || V < R(0) || W < R(0)) && (U > R(0) || V > R(0) || W > R(0))) return;
    const R det = (U + V) + W;
    if (det == R(0)) return;
    const R az = r.sz * A[r.kz], bz = r.sz * B[r.kz], cz = r.sz * C[r.kz];
    const R T = (U * az + V * bz) + W * cz;
    const R t = T / det;
    if (!(t > r.tmin)) return;
    if (t < best.t || (t == best.t && prim < best.prim)) {
        best.t = t;
        best.prim = prim;
        best.u = V / det;
        best.v = W / det;
    }
}

// Slab test against a float box, conservative: the far distance is widened
// by a relative 2^-16 so rounding never culls a box that holds the hit. A
// slab distance is NaN only for 0 * inf (ray parallel to the axis, lying in
// a box plane): that axis then constrains nothing (NaN near and far, dropped
// by the NaN-ignoring fmax / fmin across axes).
template <class R> inline bool box_hit(const Box& b, V3<R> o, V3<R> inv, R tmin, R tmax, R& tnear) {
    R tn = tmin, tf = tmax;
    for (int a = 0; a < 3; ++a) {
        const R t0 = (R(b.lo[a]) - o[a]) * inv[a];
        const R t1 = (R(b.hi[a]) - o[a]) * inv[a];
        const bool nan = std::isnan(t0) || std::isnan(t1);
        const R lo = nan ? t0 + t1 : std::fmin(t0, t1), hi = nan ? t0 + t1 : std::fmax(t0, t1);
        tn = std::fmax(tn, lo);
        tf = std::fmin(tf, hi);
    }
    tnear = tn;
    return tn <= tf * R(1.0000153);
}

// Two-level scenes: every section's triangles in its object space, the ray
// entering through the section's inverse transform with the device's
// arithmetic (((m0 x + m1 y) + m2 z) + m3 per component, no contraction).
template <class R> HitR<R> closest_hit_two_level(const oracle_scene* s, V3<R> o, V3<R> d, R tmin, R tmax,
                                                 uint64_t& fb, uint64_t& nt) {
    HitR<R> best{tmax, SOLRT_NO_HIT, R(0), R(0)};
    for (size_t si = 0; si < s->sec_first.size(); ++si) {
        const uint32_t first = s->sec_first[si], cnt = s->sec_count[si];
        if (cnt == 0) continue;
        const float* m = s->minv[si].data();
        const V3<R> p{R(m[0]) * o.x + R(m[1]) * o.y + R(m[2]) * o.z + R(m[3]),
                      R(m[4]) * o.x + R(m[5]) * o.y + R(m[6]) * o.z + R(m[7]),
                      R(m[8]) * o.x + R(m[9]) * o.y + R(m[10]) * o.z + R(m[11])};
        const V3<R> q{R(m[0]) * d.x + R(m[1]) * d.y + R(m[2]) * d.z, R(m[4]) * d.x + R(m[5]) * d.y + R(m[6]) * d.z,
                      R(m[8]) * d.x + R(m[9]) * d.y + R(m[10]) * d.z};
        const RayWT<R> r = setup_ray(p, q, tmin);
        for (uint32_t i = 0; i < cnt; ++i) {
            ++nt;
            intersect_tri(r, s->obj[first + i], first + i, best, fb);
        }
    }
    return best;
}

template <class R> HitR<R> closest_hit(const oracle_scene* s, V3<R> o, V3<R> d, R tmin, R tmax,
                                       int mode, uint64_t& fb, uint64_t& nv, uint64_t& nt) {
    if (s->two_level) return closest_hit_two_level<R>(s, o, d, tmin, tmax, fb, nt);
    HitR<R> best{tmax, SOLRT_NO_HIT, R(0), R(0)};
    const RayWT<R> r = setup_ray(o, d, tmin);
    const uint32_t n = (uint32_t)s->tris.size();
    if (n == 0) return best;
    if (mode == 0 || n == 1) {
        for (uint32_t i = 0; i < n; ++i) { ++nt; intersect_tri(r, s->tris[i], i, best, fb); }
        return best;
    }
    const V3<R> inv{R(1) / d.x, R(1) / d.y, R(1) / d.z};
    // Depth-first, nearer child first; both child boxes are tested at the
    // parent. The stack holds at most one entry per level.
    uint32_t stack[256];
    int sp = 0;
    uint32_t cur = 0;
    for (;;) {
        if (cur & 0x80000000u) {
            const uint32_t k = cur & 0x7fffffffu;
            ++nt;
            intersect_tri(r, s->tris[s->order[k]], s->order[k], best, fb);
        } else {
            ++nv;
            const uint32_t a = s->child[2 * cur], b = s->child[2 * cur + 1];
            const Box& ba = (a & 0x80000000u) ? s->leaf_box[a & 0x7fffffffu] : s->node_box[a];
            const Box& bb = (b & 0x80000000u) ? s->leaf_box[b & 0x7fffffffu] : s->node_box[b];
            R ta, tb;
            const bool ha = box_hit(ba, o, inv, tmin, best.t, ta);
            const bool hb = box_hit(bb, o, inv, tmin, best.t, tb);
            if (ha && hb) {
                const bool swap = tb < ta;
                if (sp < 256) stack[sp++] = swap ? a : b;
                cur = swap ? b : a;
                continue;
            }
            if (ha) { cur = a; continue; }
            if (hb) { cur = b; continue; }
        }
        if (sp == 0) break;
        cur = stack[--sp];
    }
    return best;
}

// ---------------------------------------------------------------------------
// Path tracing (pathtrace.rgen:39-104, .rchit:56-113, .rmiss:8-21)
// ---------------------------------------------------------------------------

struct Counters {
    uint64_t seg = 0, paths = 0, fb = 0, nv = 0, nt = 0;
    uint64_t shadow = 0, unoccluded = 0;  // next-event estimation
};

// Shading normal and position of a hit (pathtrace.rchit:82-90,
// ao.rchit:66-75): object-space vertex normals and positions interpolated,
// then the section instance's transform_it (w = 0, normalised) and
// transform (w = 1).
template <class R> void hit_frame(const oracle_scene* s, const TriW& tri, R b0, R b1, R b2, V3<R>& normal,
                                  V3<R>& pos) {
    auto cv = [](V3<float> a) { return V3<R>{R(a.x), R(a.y), R(a.z)}; };
    const V3<R> n = cv(tri.on[0]) * b0 + cv(tri.on[1]) * b1 + cv(tri.on[2]) * b2;
    const V3<R> p = cv(tri.op[0]) * b0 + cv(tri.op[1]) * b1 + cv(tri.op[2]) * b2;
    R o[4];
    mat4_mul<R>(s->sec_tit[tri.sec].data(), n.x, n.y, n.z, R(0), o);
    normal = normalize(V3<R>{o[0], o[1], o[2]});
    mat4_mul<R>(s->sec_t[tri.sec].data(), p.x, p.y, p.z, R(1), o);
    pos = V3<R>{o[0], o[1], o[2]};
}

// Importance of child j of a light-tree node seen from x with normal n:
// power * cos_bound / max(d^2, r^2), d the distance to the child's box
// centre, r the half-diagonal, cos_bound the largest cosine between n and a
// direction into the child's bounding sphere (1 inside the sphere's
// half-angle beta, sin beta = r / d; else max(0, cos theta cos beta +
// sin theta sin beta)).
template <class R> R light_importance(const oracle_scene::LightNode& nd, int j, V3<R> x, V3<R> n) {
    const V3<R> dv{R(nd.c[j][0]) - x.x, R(nd.c[j][1]) - x.y, R(nd.c[j][2]) - x.z};
    const R d2 = dot(dv, dv), r2 = R(nd.r2[j]);
    R cb = R(1);
    if (d2 > r2) {
        const R ct = dot(n, dv) / std::sqrt(d2);
        const R sb2 = r2 / d2;
        const R cbeta = std::sqrt(R(1) - sb2);
        if (ct < cbeta) {
            const R st = std::sqrt(std::max(R(1) - ct * ct, R(0)));
            cb = std::max(ct * cbeta + st * std::sqrt(sb2), R(0));
        }
    }
    return (R(nd.power[j]) * cb) / std::max(d2, r2);
}

// Probability that the light-tree walk from x (normal n) picks the light of
// `code` (the products of the sampling walk in nee_term).
template <class R> R light_pick_prob(const oracle_scene* s, uint32_t code, V3<R> x, V3<R> n) {
    const uint32_t levels = code >> 27;
    uint32_t k = 0;
    R pick = R(1);
    for (uint32_t lv = 0; lv < levels; ++lv) {
        const oracle_scene::LightNode& nd = s->light_tree[k];
        const R wl = light_importance<R>(nd, 0, x, n), wr = light_importance<R>(nd, 1, x, n);
        const R pl = wl / (wl + wr);
        if (!(pl >= R(0) && pl <= R(1))) return R(0);
        const bool right = (code >> lv) & 1u;
        pick = right ? pick * (R(1) - pl) : pick * pl;
        const int32_t ref = nd.ref[right ? 1 : 0];
        if (ref < 0) break;
        k = (uint32_t)ref;
    }
    return pick;
}

// Power-heuristic weight of a sample whose technique has pdf p_this against
// one with pdf p_other: 1 / (1 + (p_other / p_this)^2).
template <class R> R mis_weight(R p_this, R p_other) {
    if (!(p_this > R(0))) return R(0);
    const R r = p_other / p_this;
    return R(1) / (R(1) + r * r);
}

// Next-event estimation at a diffuse vertex (SOLRT_INTEGRATOR_PATH_NEE, an
// estimator the reference does not have). Draws: l1 and l2 pick a uniform
// point on the light triangle (b0 = 1 - sqrt(l1), b1 = l2 sqrt(l1)), then
// one draw per light-tree level takes the left child with probability
// wl / (wl + wr) of the children's importances (p_pick the product of the
// choices). The shadow ray leaves from the continuation origin `no` towards
// the point with tmax 0.9999 of the distance. An unoccluded one returns
// thr * Le * (pb / pl) * w: pl = p_pick r^2 / (area cos_y) and pb = cos_x / pi
// are the solid-angle pdfs of the light pick and of the cosine BSDF sample
// (thr already holds the albedo), w = 1 / (1 + (pb / pl)^2) the power
// heuristic; the BSDF sample's emitter hit gets the complementary weight in
// trace_path. Emitters are two-sided.
template <class R> bool nee_term(const oracle_scene* s, V3<R> no, V3<R> n_o, V3<R> thr, R tmin, uint32_t& rng,
                                 Counters& cn, V3<R>& contrib) {
    const R l1 = next_rand<R>(rng);
    const R l2 = next_rand<R>(rng);
    if (s->light_tree.empty()) return false;
    uint32_t k = 0, prim = ~0u;
    R pick = R(1);
    for (int level = 0; level < 64; ++level) {
        const oracle_scene::LightNode& nd = s->light_tree[k];
        const R wl = light_importance<R>(nd, 0, no, n_o), wr = light_importance<R>(nd, 1, no, n_o);
        const R pl = wl / (wl + wr);
        if (!(pl >= R(0) && pl <= R(1))) return false;
        const R ul = next_rand<R>(rng);
        int32_t ref;
        if (ul < pl) {
            ref = nd.ref[0];
            pick = pick * pl;
        } else {
            ref = nd.ref[1];
            pick = pick * (R(1) - pl);
        }
        if (ref < 0) {
            prim = (uint32_t)~ref;
            break;
        }
        k = (uint32_t)ref;
    }
    if (prim == ~0u || !(pick > R(0))) return false;
    const TriW& tri = s->tris[prim];
    auto cv = [](V3<float> a) { return V3<R>{R(a.x), R(a.y), R(a.z)}; };
    const V3<R> p0 = cv(tri.p[0]), p1 = cv(tri.p[1]), p2 = cv(tri.p[2]);
    const R su = std::sqrt(l1);
    const R b0 = R(1) - su, b1 = l2 * su;
    const R b2 = (R(1) - b0) - b1;
    const V3<R> y = p0 * b0 + p1 * b1 + p2 * b2;
    const V3<R> e1 = p1 - p0, e2 = p2 - p0;
    const V3<R> ng{e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
    const R a2 = length(ng);
    const V3<R> w = y - no;
    const R d2 = dot(w, w);
    if (!(a2 > R(0)) || !(d2 > R(0))) return false;
    const R dist = std::sqrt(d2);
    const V3<R> wl{w.x / dist, w.y / dist, w.z / dist};
    const R cx = dot(n_o, wl);
    const R cy = std::abs(dot(ng, wl)) / a2;
    const R tmax = dist * R(0.9999f);
    if (!(cx > R(0)) || !(cy > R(0)) || !(tmax > tmin)) return false;
    const float* le = s->mats[tri.mat].emissive;
    // solid-angle pdfs of this direction: light pick, cosine BSDF sample
    const R pl = (pick * d2) / ((R(0.5f) * a2) * cy);
    const R pb = cx / R(3.14159265f);
    if (!(pl > R(0))) return false;
    const R wgt = (pb / pl) * mis_weight<R>(pl, pb);
    ++cn.shadow;
    uint64_t nv = 0, nt = 0, fb = 0;
    const HitR<R> h = closest_hit<R>(s, no, wl, tmin, tmax, 1, fb, nv, nt);
    if (h.prim != SOLRT_NO_HIT) return false;
    ++cn.unoccluded;
    contrib = (thr * V3<R>{R(le[0]), R(le[1]), R(le[2])}) * wgt;
    return true;
}

template <class R> V3<R> trace_path(const oracle_scene* s, const solrt_render_params* p, V3<R> o,
                                    V3<R> d, R tmin, R tmax, uint32_t& rng, Counters& cn) {
    V3<R> acc{R(1), R(1), R(1)};
    uint32_t depth = 0;
    const bool nee = p->integrator == SOLRT_INTEGRATOR_PATH_NEE;
    V3<R> nee_sum{R(0), R(0), R(0)};  // shadow terms in bounce order, then the path's end
    R pdf_prev = R(0);                 // solid-angle pdf of the current ray's BSDF sample
    V3<R> n_prev{R(0), R(0), R(0)};    // oriented normal of the vertex it left
    for (;;) {
        const HitR<R> h = closest_hit<R>(s, o, d, tmin, tmax, 1, cn.fb, cn.nv, cn.nt);
        ++cn.seg;
        if (h.prim == SOLRT_NO_HIT) {                       // pathtrace.rmiss
            acc = acc * miss_color<R>(d, p->miss_mode);
            break;
        }
        const TriW& tri = s->tris[h.prim];                  // pathtrace.rchit
        const solrt_material& m = s->mats[tri.mat];
        if (m.emissive[0] >= 1.0f || m.emissive[1] >= 1.0f || m.emissive[2] >= 1.0f) {
            acc = acc * V3<R>{R(m.emissive[0]), R(m.emissive[1]), R(m.emissive[2])};
            if (nee && depth > 0) {  // power heuristic against next-event estimation
                const uint32_t code = s->tri_light.empty() ? ~0u : s->tri_light[h.prim];
                R pl = R(0);
                if (code != ~0u) {
                    auto cw = [](V3<float> a) { return V3<R>{R(a.x), R(a.y), R(a.z)}; };
                    const V3<R> e1 = cw(tri.p[1]) - cw(tri.p[0]), e2 = cw(tri.p[2]) - cw(tri.p[0]);
                    const V3<R> ng{e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
                    const R a2 = length(ng);
                    const R cy = std::abs(dot(ng, d)) / a2;
                    const R pick = light_pick_prob<R>(s, code, o, n_prev);
                    pl = (pick * (h.t * h.t)) / ((R(0.5f) * a2) * cy);
                }
                acc = acc * mis_weight<R>(pdf_prev, pl);
            }
            break;
        }
        const R b1 = h.u, b2 = h.v;
        const R b0 = (R(1) - b1) - b2;
        auto cv = [](V3<float> a) { return V3<R>{R(a.x), R(a.y), R(a.z)}; };
        V3<R> normal, pos;
        hit_frame<R>(s, tri, b0, b1, b2, normal, pos);
        const V3<R> vcol = cv(tri.c[0]) * b0 + cv(tri.c[1]) * b1 + cv(tri.c[2]) * b2;
        const V3<R> wi = normalize(d);
        const V3<R> n_o = normal * glsl_sign(dot(normal, -wi));
        const R alpha2 = R(m.roughness) * R(m.roughness);
        const R xi0 = next_rand<R>(rng);
        const R xi1 = next_rand<R>(rng);
        const R rnd = next_rand<R>(rng);
        const V3<R> base{R(m.base_color[0]), R(m.base_color[1]), R(m.base_color[2])};
        o = pos + R(0.0001f) * n_o;
        V3<R> hv;
        if (p->material_mode == SOLRT_MATERIAL_LAMBERT) {
            d = sample_cosine(n_o, xi0, xi1);
            hv = base * vcol;
            pdf_prev = dot(n_o, d) / R(3.14159265f);
            n_prev = n_o;
        } else if (rnd < R(m.metallic)) {
            d = sample_ggx(reflect(d, n_o), xi0, xi1, alpha2);
            hv = base * vcol;
        } else {
            const V3<R> mh = sample_ggx(n_o, xi0, xi1, alpha2);
            if (rnd < fresnel_dielectric(n_o, mh, R(1.0f / 1.5f))) {
                d = reflect(d, mh);
                hv = V3<R>{R(1), R(1), R(1)};
            } else {
                d = sample_cosine(n_o, xi0, xi1);
                hv = base * vcol;
            }
        }
        ++depth;
        acc = acc * hv;                                     // pathtrace.rgen:77
        if (depth > p->max_bounces) {                       // pathtrace.rgen:81-84
            acc = V3<R>{R(0), R(0), R(0)};
            break;
        }
        V3<R> c;
        if (nee && nee_term<R>(s, o, n_o, acc, tmin, rng, cn, c)) nee_sum = nee_sum + c;
    }
    return nee ? nee_sum + acc : acc;
}

template <class R> struct Cam {
    const solrt_camera* c;
};

// Camera ray of pathtrace.rgen:52-60.
template <class R> void camera_ray(const solrt_camera* cam, uint32_t x, uint32_t y, uint32_t W, uint32_t H,
                                   uint32_t& rng, V3<R>& o, V3<R>& d, R& tmin) {
    const R j0 = next_rand<R>(rng);
    const R j1 = next_rand<R>(rng);
    const R px = R(x) + j0, py = R(y) + j1;
    const R ux = px / R(W), uy = py / R(H);
    const R dx = ux * R(2) - R(1), dy = uy * R(2) - R(1);
    R org[4], tgt[4], dir[4];
    mat4_mul<R>(cam->view_inverse, R(0), R(0), R(0), R(1), org);
    mat4_mul<R>(cam->projection_inverse, dx, dy, R(1), R(1), tgt);
    const V3<R> tn = normalize(V3<R>{tgt[0], tgt[1], tgt[2]});
    mat4_mul<R>(cam->view_inverse, tn.x, tn.y, tn.z, R(0), dir);
    o = V3<R>{org[0], org[1], org[2]};
    d = V3<R>{dir[0], dir[1], dir[2]};
    tmin = std::max(R(1), length(o)) * R(1e-3f);            // pathtrace.rgen:35
}

inline uint32_t sample_seed(const solrt_render_params* p, uint32_t pix, uint32_t s) {
    uint32_t rng = tea(pix, p->frame * p->spp + s);
    if (p->seed != 0) rng ^= tea(p->seed, p->job_id);
    return rng;
}

template <class R> bool finite3(V3<R> c) {
    return std::isfinite(c.x) && std::isfinite(c.y) && std::isfinite(c.z);
}

float gamma_f(float c, float power) { return std::pow(c, 1.0f / power); }

uint8_t to_unorm8(float c) {
    const float cl = std::min(std::max(c, 0.0f), 1.0f);
    return (uint8_t)(cl * 255.0f + 0.5f);
}

template <class R>
void render_pixel(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p, uint32_t x,
                  uint32_t y, float* accum, float* ksum, float* kcomp, uint8_t* rgba8, float* samples_out,
                  Counters& cn) {
    const uint32_t W = p->width, H = p->height, pix = x + y * W;
    const R tmax = p->tmax > 0.0f ? R(p->tmax) : R(10000.0f);
    uint32_t rng = tea(pix, p->frame);                     // pathtrace.rgen:47
    V3<R> sum{R(0), R(0), R(0)};
    V3<R> kc{R(0), R(0), R(0)};
    V3<R> ks{R(0), R(0), R(0)};
    R kn = R(0);
    if (ksum) {
        ks = V3<R>{R(ksum[4 * pix]), R(ksum[4 * pix + 1]), R(ksum[4 * pix + 2])};
        kn = R(ksum[4 * pix + 3]);
        kc = V3<R>{R(kcomp[4 * pix]), R(kcomp[4 * pix + 1]), R(kcomp[4 * pix + 2])};
    }
    for (uint32_t si = 0; si < p->spp; ++si) {              // pathtrace.rgen:49
        if (p->rng_mode == SOLRT_RNG_PER_SAMPLE) rng = sample_seed(p, pix, si);
        V3<R> o, d;
        R tmin;
        camera_ray<R>(cam, x, y, W, H, rng, o, d, tmin);
        ++cn.paths;
        const V3<R> c = trace_path<R>(s, p, o, d, tmin, tmax, rng, cn);
        if (samples_out) {
            float* so = samples_out + 4 * ((size_t)pix * p->spp + si);
            so[0] = (float)c.x; so[1] = (float)c.y; so[2] = (float)c.z; so[3] = 1.0f;
        }
        if (p->accum_mode == SOLRT_ACCUM_KAHAN) {
            if (finite3(c)) {
                const V3<R> yv = c - kc;
                const V3<R> t = ks + yv;
                kc = (t - ks) - yv;
                ks = t;
                kn = kn + R(1);
            }
        } else {
            sum = sum + c;                                  // pathtrace.rgen:86
        }
    }
    if (samples_out) return;
    V3<R> out;
    const V3<R> old{R(accum[4 * pix]), R(accum[4 * pix + 1]), R(accum[4 * pix + 2])};
    if (p->accum_mode == SOLRT_ACCUM_KAHAN) {
        ksum[4 * pix] = (float)ks.x; ksum[4 * pix + 1] = (float)ks.y; ksum[4 * pix + 2] = (float)ks.z;
        ksum[4 * pix + 3] = (float)kn;
        kcomp[4 * pix] = (float)kc.x; kcomp[4 * pix + 1] = (float)kc.y; kcomp[4 * pix + 2] = (float)kc.z;
        kcomp[4 * pix + 3] = 0.0f;
        out = kn > R(0) ? V3<R>{ks.x / kn, ks.y / kn, ks.z / kn} : old;
    } else {
        const V3<R> mean = (R(1) / R(p->spp)) * sum;        // pathtrace.rgen:88
        const R alpha = R(1) / R((uint32_t)(p->frame + 1u - p->accum_start_frame));
        out = mix(old, mean, alpha);                        // pathtrace.rgen:89-92
        if (std::isnan(out.x) || std::isnan(out.y) || std::isnan(out.z)) out = old;
        if (std::isinf(out.x) || std::isinf(out.y) || std::isinf(out.z)) out = old;
    }
    const float of[3] = {(float)out.x, (float)out.y, (float)out.z};
    accum[4 * pix] = of[0]; accum[4 * pix + 1] = of[1]; accum[4 * pix + 2] = of[2]; accum[4 * pix + 3] = 1.0f;
    for (int c = 0; c < 3; ++c) rgba8[4 * pix + c] = to_unorm8(gamma_f(of[c], 2.2f));  // pathtrace.rgen:102-103
    rgba8[4 * pix + 3] = 255;
}

// debug.rgen:18-36 + debug.rchit:9-13 + debug.rmiss: one ray through the
// pixel centre; barycentrics of the hit or the ray direction, stored as is.
template <class R>
void render_pixel_debug(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p, uint32_t x,
                        uint32_t y, float* accum, uint8_t* rgba8, Counters& cn) {
    const uint32_t W = p->width, H = p->height, pix = x + y * W;
    const R px = R(x) + R(0.5f), py = R(y) + R(0.5f);
    const R ux = px / R(W), uy = py / R(H);
    const R dx = ux * R(2) - R(1), dy = uy * R(2) - R(1);
    R org[4], tgt[4], dir[4];
    mat4_mul<R>(cam->view_inverse, R(0), R(0), R(0), R(1), org);
    mat4_mul<R>(cam->projection_inverse, dx, dy, R(1), R(1), tgt);
    const V3<R> tn = normalize(V3<R>{tgt[0], tgt[1], tgt[2]});
    mat4_mul<R>(cam->view_inverse, tn.x, tn.y, tn.z, R(0), dir);
    const HitR<R> h = closest_hit<R>(s, V3<R>{org[0], org[1], org[2]}, V3<R>{dir[0], dir[1], dir[2]}, R(0.001f),
                                     R(1000.0f), 1, cn.fb, cn.nv, cn.nt);
    ++cn.seg;
    ++cn.paths;
    float v[3] = {(float)dir[0], (float)dir[1], (float)dir[2]};
    if (h.prim != SOLRT_NO_HIT) {
        v[0] = (float)((R(1) - h.u) - h.v);
        v[1] = (float)h.u;
        v[2] = (float)h.v;
    }
    for (int c = 0; c < 3; ++c) {
        accum[4 * pix + c] = v[c];
        rgba8[4 * pix + c] = to_unorm8(v[c]);
    }
    accum[4 * pix + 3] = 0.0f;
    rgba8[4 * pix + 3] = 0;
}

// ao.rgen:37-83 + ao.rchit:53-88 + ao.rmiss. `spp` samples of at most
// `max_bounces` + 1 hits; every hit after the first is one occlusion.
template <class R>
void render_pixel_ao(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p, uint32_t x,
                     uint32_t y, float* accum, uint8_t* rgba8, const uint8_t* noise, uint32_t nw, uint32_t nh,
                     Counters& cn) {
    const uint32_t W = p->width, H = p->height, pix = x + y * W;
    uint32_t rng = tea(pix, p->frame);                              // ao.rgen:49
    const R max_samples = R(p->max_bounces);
    V3<R> ao{R(0), R(0), R(0)};
    for (uint32_t i = 0; i < p->spp; ++i) {
        V3<R> o, d;
        R tmin;
        camera_ray<R>(cam, x, y, W, H, rng, o, d, tmin);           // ao.rgen:52-61 + preparePayload
        R tmax = R(10000.0f);
        ++cn.paths;
        R hv = R(0);
        uint32_t depth = 0;
        for (;;) {
            const HitR<R> h = closest_hit<R>(s, o, d, tmin, tmax, 1, cn.fb, cn.nv, cn.nt);
            ++cn.seg;
            if (h.prim == SOLRT_NO_HIT) break;                      // ao.rmiss: done
            const TriW& tri = s->tris[h.prim];
            const R b1 = h.u, b2 = h.v;
            const R b0 = (R(1) - b1) - b2;
            V3<R> normal, pos;
            hit_frame<R>(s, tri, b0, b1, b2, normal, pos);
            const V3<R> no = pos + R(0.00001f) * d;                 // ao.rchit:78
            // getBlueRand2(depth + depth * sampleId) (ao.rchit:43-49)
            const uint32_t bi = depth + depth * i;
            const R r0 = next_rand<R>(rng);
            const R r1 = next_rand<R>(rng);
            const R tw = R(nw), th = R(nh);
            R cx = R(x) + r0 * tw, cy = R(y) + r1 * th;
            cx = cx - tw * std::floor(cx / tw);                     // GLSL mod
            cy = cy - th * std::floor(cy / th);
            int ix = (int)cx, iy = (int)cy;
            ix = std::min(std::max(ix, 0), (int)nw - 1);
            iy = std::min(std::max(iy, 0), (int)nh - 1);
            const uint8_t* t = noise + 4 * ((size_t)iy * nw + ix);
            const R blue[4] = {R((float)t[0] / 255.0f), R((float)t[1] / 255.0f), R((float)t[2] / 255.0f),
                               R((float)t[3] / 255.0f)};
            const R xi0 = blue[bi % 4], xi1 = blue[(bi + 1) % 4];
            const V3<R> hit_n = normal * glsl_sign(dot(-d, normal));
            d = sample_cosine(hit_n, xi0, xi1);
            o = no;
            tmin = R(0.001f);
            tmax = R(10.0f);
            if (depth > 0) hv = hv + R(1);
            ++depth;
            if (depth > p->max_bounces) break;                      // ao.rgen:75
        }
        ao = ao + (R(1) / max_samples) * V3<R>{hv, hv, hv};        // ao.rgen:77
    }
    const R n = R(p->spp);
    V3<R> color = V3<R>{R(1) - ao.x / n, R(1) - ao.y / n, R(1) - ao.z / n};
    const R a = R(1) / R((uint32_t)(p->frame - p->accum_start_frame + 1u));
    const V3<R> old{R(accum[4 * pix]), R(accum[4 * pix + 1]), R(accum[4 * pix + 2])};
    color = mix(old, color, a);                                     // ao.rgen:79-82
    const float of[3] = {(float)color.x, (float)color.y, (float)color.z};
    for (int c = 0; c < 3; ++c) {
        accum[4 * pix + c] = of[c];
        rgba8[4 * pix + c] = to_unorm8(of[c]);
    }
    accum[4 * pix + 3] = 1.0f;
    rgba8[4 * pix + 3] = 255;
}

template <class F> void parallel_for(uint32_t n, int threads, F&& f) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (threads == 1 || n < 2) {
        for (uint32_t i = 0; i < n; ++i) f(i, 0);
        return;
    }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&, t]() {
            for (;;) {
                const uint32_t i = next.fetch_add(1);
                if (i >= n) break;
                f(i, t);
            }
        });
    }
    for (auto& th : pool) th.join();
}

int resolve_threads(int threads) {
    return threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
}

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------

// Light tree of next-event estimation: the emissive triangles (any emissive
// channel >= 1, pathtrace.rchit:75-80; zero-area ones left out) sorted by
// the 30-bit Morton code of their centroid ((p0 + p1) + p2) / 3 in the
// centroids' bounds (ties by triangle index), ranges split at their middle;
// a child's box is the union of its children's (a triangle's: its own), its
// power left + right (a triangle's: area * ((Le.r + Le.g) + Le.b)), its
// centre (min + max) / 2 and squared half-diagonal from (max - min) / 2. One
// light: a root whose two refs are that light and whose right power is 0.
void light_sphere(const float mn[3], const float mx[3], float c[3], float& r2) {
    float h[3];
    for (int k = 0; k < 3; ++k) {
        c[k] = (mn[k] + mx[k]) * 0.5f;
        h[k] = (mx[k] - mn[k]) * 0.5f;
    }
    r2 = (h[0] * h[0] + h[1] * h[1]) + h[2] * h[2];
}

int32_t light_node(oracle_scene* s, const std::vector<uint32_t>& order, const std::vector<float>& box,
                   const std::vector<float>& power, const std::vector<uint32_t>& prim, uint32_t b, uint32_t e,
                   float mn[3], float mx[3], float& pw, uint32_t bits, uint32_t level) {
    if (e - b == 1) {
        const uint32_t k = order[b];
        for (int c = 0; c < 3; ++c) {
            mn[c] = box[6 * k + c];
            mx[c] = box[6 * k + 3 + c];
        }
        pw = power[k];
        s->tri_light[prim[k]] = (level << 27) | bits;
        return ~(int32_t)prim[k];
    }
    const uint32_t idx = (uint32_t)s->light_tree.size();
    s->light_tree.push_back(oracle_scene::LightNode{});
    const uint32_t m = b + (e - b) / 2;
    float cmn[2][3], cmx[2][3], cp[2] = {0.0f, 0.0f};
    int32_t ref[2];
    ref[0] = light_node(s, order, box, power, prim, b, m, cmn[0], cmx[0], cp[0], bits, level + 1);
    ref[1] = light_node(s, order, box, power, prim, m, e, cmn[1], cmx[1], cp[1], bits | (1u << level), level + 1);
    oracle_scene::LightNode nd{};
    for (int j = 0; j < 2; ++j) {
        light_sphere(cmn[j], cmx[j], nd.c[j], nd.r2[j]);
        nd.power[j] = cp[j];
        nd.ref[j] = ref[j];
    }
    for (int c = 0; c < 3; ++c) {
        mn[c] = std::min(cmn[0][c], cmn[1][c]);
        mx[c] = std::max(cmx[0][c], cmx[1][c]);
    }
    pw = cp[0] + cp[1];
    s->light_tree[idx] = nd;
    return (int32_t)idx;
}

void build_light_tree(oracle_scene* s) {
    std::vector<uint32_t> prim;
    std::vector<float> box, power, cen;
    for (uint32_t t = 0; t < (uint32_t)s->tris.size(); ++t) {
        const TriW& tr = s->tris[t];
        const solrt_material& m = s->mats[tr.mat];
        if (!(m.emissive[0] >= 1.0f || m.emissive[1] >= 1.0f || m.emissive[2] >= 1.0f)) continue;
        const V3<float> e1 = tr.p[1] - tr.p[0], e2 = tr.p[2] - tr.p[0];
        const float nx = e1.y * e2.z - e1.z * e2.y, ny = e1.z * e2.x - e1.x * e2.z, nz = e1.x * e2.y - e1.y * e2.x;
        const float area = 0.5f * std::sqrt((nx * nx + ny * ny) + nz * nz);
        const float pw = area * ((m.emissive[0] + m.emissive[1]) + m.emissive[2]);
        if (!(area > 0.0f) || !(pw > 0.0f) || !std::isfinite(pw)) continue;
        prim.push_back(t);
        const float v[3][3] = {{tr.p[0].x, tr.p[0].y, tr.p[0].z}, {tr.p[1].x, tr.p[1].y, tr.p[1].z},
                               {tr.p[2].x, tr.p[2].y, tr.p[2].z}};
        float lo[3], hi[3];
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(std::min(v[0][k], v[1][k]), v[2][k]);
            hi[k] = std::max(std::max(v[0][k], v[1][k]), v[2][k]);
            cen.push_back(((v[0][k] + v[1][k]) + v[2][k]) / 3.0f);
        }
        box.insert(box.end(), lo, lo + 3);
        box.insert(box.end(), hi, hi + 3);
        power.push_back(pw);
    }
    const uint32_t n = std::min<uint32_t>((uint32_t)prim.size(), 1u << 26);  // codes hold 27 levels
    if (n == 0) return;
    s->tri_light.assign(s->tris.size(), ~0u);
    float cmin[3] = {cen[0], cen[1], cen[2]}, cmax[3] = {cen[0], cen[1], cen[2]};
    for (uint32_t i = 1; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            cmin[k] = std::min(cmin[k], cen[3 * i + k]);
            cmax[k] = std::max(cmax[k], cen[3 * i + k]);
        }
    std::vector<std::pair<uint32_t, uint32_t>> key(n);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t code = 0;
        for (int k = 0; k < 3; ++k) {
            const float ext = cmax[k] - cmin[k];
            const float f = ext > 0.0f ? (cen[3 * i + k] - cmin[k]) / ext : 0.0f;
            code |= expand_bits10((uint32_t)std::min(std::max(f * 1023.0f, 0.0f), 1023.0f)) << (2 - k);
        }
        key[i] = {code, i};
    }
    std::sort(key.begin(), key.end());
    std::vector<uint32_t> order(n);
    for (uint32_t i = 0; i < n; ++i) order[i] = key[i].second;
    float mn[3], mx[3], pw = 0.0f;
    s->light_tree.reserve((size_t)n);
    const int32_t root = light_node(s, order, box, power, prim, 0, n, mn, mx, pw, 0u, 0u);
    if (root < 0) {  // one light
        s->tri_light[prim[0]] = 1u << 27;
        oracle_scene::LightNode nd{};
        for (int j = 0; j < 2; ++j) {
            light_sphere(mn, mx, nd.c[j], nd.r2[j]);
            nd.ref[j] = root;
        }
        nd.power[0] = pw;
        nd.power[1] = 0.0f;
        s->light_tree.push_back(nd);
    }
}

extern "C" {

oracle_scene* oracle_scene_create(const solrt_scene_desc* desc) {
    if (!desc) return nullptr;
    oracle_scene* s = new oracle_scene();
    if (!flatten(desc, s)) {
        delete s;
        return nullptr;
    }
    build_lbvh(s);
    build_light_tree(s);
    return s;
}

void oracle_scene_destroy(oracle_scene* s) { delete s; }

int oracle_closest_hit(const void* scene, const float* o, const float* d, float tmin, float tmax, uint32_t* prim,
                       float* u, float* v) {
    const oracle_scene* s = static_cast<const oracle_scene*>(scene);
    uint64_t fb = 0, nv = 0, nt = 0;
    const HitR<float> h = closest_hit<float>(s, V3<float>{o[0], o[1], o[2]}, V3<float>{d[0], d[1], d[2]}, tmin,
                                             tmax, 1, fb, nv, nt);
    if (h.prim == SOLRT_NO_HIT) return 0;
    *prim = h.prim;
    *u = h.u;
    *v = h.v;
    return 1;
}

void oracle_scene_set_two_level(oracle_scene* s, int on) {
    if (s) s->two_level = on != 0;
}

uint32_t oracle_scene_tri_count(const oracle_scene* s) { return (uint32_t)s->tris.size(); }

int oracle_scene_export_world(const oracle_scene* s, float* tw, uint32_t* tm) {
    for (size_t i = 0; i < s->tris.size(); ++i) {
        const TriW& t = s->tris[i];
        float* o = tw + 36 * i;
        for (int k = 0; k < 3; ++k) {
            o[12 * k + 0] = t.p[k].x; o[12 * k + 1] = t.p[k].y; o[12 * k + 2] = t.p[k].z; o[12 * k + 3] = 0;
            o[12 * k + 4] = t.n[k].x; o[12 * k + 5] = t.n[k].y; o[12 * k + 6] = t.n[k].z; o[12 * k + 7] = 0;
            o[12 * k + 8] = t.c[k].x; o[12 * k + 9] = t.c[k].y; o[12 * k + 10] = t.c[k].z; o[12 * k + 11] = 0;
        }
        if (tm) tm[i] = t.mat;
    }
    return 0;
}

uint32_t oracle_bvh_export(const oracle_scene* s, uint32_t* child_refs, float* boxes, uint32_t* order,
                           uint32_t* morton) {
    const uint32_t n = (uint32_t)s->tris.size();
    const uint32_t ni = n > 1 ? n - 1 : 0;
    for (uint32_t i = 0; i < ni; ++i) {
        if (child_refs) { child_refs[2 * i] = s->child[2 * i]; child_refs[2 * i + 1] = s->child[2 * i + 1]; }
        if (boxes) {
            for (int a = 0; a < 3; ++a) {
                boxes[6 * i + a] = s->node_box[i].lo[a];
                boxes[6 * i + 3 + a] = s->node_box[i].hi[a];
            }
        }
    }
    for (uint32_t k = 0; k < n; ++k) {
        if (order) order[k] = s->order[k];
        if (morton) morton[k] = s->morton[k];
    }
    return ni;
}

int oracle_trace(const oracle_scene* s, const solrt_ray* rays, uint32_t n, solrt_hit* hits, int mode,
                 int threads, uint64_t* fp64_fallbacks) {
    threads = resolve_threads(threads);
    std::vector<uint64_t> fb(threads, 0);
    const uint32_t chunk = 1024;
    const uint32_t nchunks = (n + chunk - 1) / chunk;
    parallel_for(nchunks, threads, [&](uint32_t c, int t) {
        uint64_t nv = 0, nt = 0;
        for (uint32_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) {
            const solrt_ray& r = rays[i];
            const HitR<float> h = closest_hit<float>(s, V3<float>{r.origin[0], r.origin[1], r.origin[2]},
                                                     V3<float>{r.dir[0], r.dir[1], r.dir[2]}, r.tmin, r.tmax,
                                                     mode, fb[t], nv, nt);
            hits[i].t = h.prim == SOLRT_NO_HIT ? r.tmax : h.t;
            hits[i].prim = h.prim;
            hits[i].u = h.u;
            hits[i].v = h.v;
        }
    });
    if (fp64_fallbacks) {
        uint64_t tot = 0;
        for (uint64_t v : fb) tot += v;
        *fp64_fallbacks = tot;
    }
    return 0;
}

static int render_impl(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p, float* accum,
                       float* ksum, float* kcomp, uint8_t* rgba8, float* samples_out, int precision,
                       int threads, uint32_t row_begin, uint32_t row_end, oracle_render_stats* stats,
                       const uint8_t* noise = nullptr, uint32_t nw = 0, uint32_t nh = 0) {
    if (!s || !cam || !p || p->width == 0 || p->height == 0 || p->spp == 0) return 1;
    if (!samples_out && (!accum || !rgba8)) return 1;
    if (p->integrator > SOLRT_INTEGRATOR_PATH_NEE) return 1;
    if (p->integrator == SOLRT_INTEGRATOR_PATH_NEE && p->material_mode != SOLRT_MATERIAL_LAMBERT) return 1;
    const bool path = p->integrator == SOLRT_INTEGRATOR_PATH || p->integrator == SOLRT_INTEGRATOR_PATH_NEE;
    if (!path && samples_out) return 1;
    if (p->integrator == SOLRT_INTEGRATOR_AO && (!noise || nw == 0 || nh == 0 || p->max_bounces == 0)) return 1;
    if (!samples_out && p->accum_mode == SOLRT_ACCUM_KAHAN && (!ksum || !kcomp)) return 1;
    if (row_end <= row_begin) { row_begin = 0; row_end = p->height; }
    row_end = std::min(row_end, p->height);
    threads = resolve_threads(threads);
    std::vector<Counters> cn(threads);
    // work items are runs of up to 64 pixels of a row, so that a band of a
    // few rows still keeps every thread busy (pixels are independent)
    const uint32_t rows = row_end - row_begin;
    const uint32_t runs = (p->width + 63u) / 64u;
    parallel_for(rows * runs, threads, [&](uint32_t item, int t) {
        const uint32_t y = row_begin + item / runs;
        const uint32_t x0 = (item % runs) * 64u, x1 = std::min(p->width, x0 + 64u);
        for (uint32_t x = x0; x < x1; ++x) {
            if (p->integrator == SOLRT_INTEGRATOR_DEBUG) {
                if (precision == 64) render_pixel_debug<double>(s, cam, p, x, y, accum, rgba8, cn[t]);
                else render_pixel_debug<float>(s, cam, p, x, y, accum, rgba8, cn[t]);
            } else if (p->integrator == SOLRT_INTEGRATOR_AO) {
                if (precision == 64) render_pixel_ao<double>(s, cam, p, x, y, accum, rgba8, noise, nw, nh, cn[t]);
                else render_pixel_ao<float>(s, cam, p, x, y, accum, rgba8, noise, nw, nh, cn[t]);
            } else if (precision == 64) {
                render_pixel<double>(s, cam, p, x, y, accum, ksum, kcomp, rgba8, samples_out, cn[t]);
            } else {
                render_pixel<float>(s, cam, p, x, y, accum, ksum, kcomp, rgba8, samples_out, cn[t]);
            }
        }
    });
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        for (const Counters& c : cn) {
            stats->segments += c.seg;
            stats->paths += c.paths;
            stats->fp64_fallbacks += c.fb;
            stats->node_visits += c.nv;
            stats->tri_tests += c.nt;
            stats->shadow_segments += c.shadow;
            stats->shadow_unoccluded += c.unoccluded;
        }
    }
    return 0;
}

int oracle_render(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p, float* accum,
                  float* kahan_sum, float* kahan_comp, uint8_t* rgba8, int precision, int threads,
                  uint32_t row_begin, uint32_t row_end, oracle_render_stats* stats) {
    return render_impl(s, cam, p, accum, kahan_sum, kahan_comp, rgba8, nullptr, precision, threads, row_begin,
                       row_end, stats);
}

int oracle_render_ex(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p, float* accum,
                     float* kahan_sum, float* kahan_comp, uint8_t* rgba8, int precision, int threads,
                     uint32_t row_begin, uint32_t row_end, oracle_render_stats* stats, const uint8_t* blue_noise,
                     uint32_t noise_w, uint32_t noise_h) {
    return render_impl(s, cam, p, accum, kahan_sum, kahan_comp, rgba8, nullptr, precision, threads, row_begin,
                       row_end, stats, blue_noise, noise_w, noise_h);
}

int oracle_render_samples(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p,
                          float* out, int precision, int threads) {
    return render_impl(s, cam, p, nullptr, nullptr, nullptr, nullptr, out, precision, threads, 0, 0, nullptr);
}

uint32_t oracle_tea(uint32_t a, uint32_t b) { return tea(a, b); }
float oracle_next_rand(uint32_t* state) { return next_rand<float>(*state); }
void oracle_sincos(float x, float* s, float* c) { sincos_poly(x, *s, *c); }

void oracle_sample_ggx(const float n[3], float xi0, float xi1, float alpha2, float out[3]) {
    const V3<float> r = sample_ggx(V3<float>{n[0], n[1], n[2]}, xi0, xi1, alpha2);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void oracle_sample_cosine(const float n[3], float xi0, float xi1, float out[3]) {
    const V3<float> r = sample_cosine(V3<float>{n[0], n[1], n[2]}, xi0, xi1);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
float oracle_fresnel(const float i[3], const float m[3], float eta) {
    return fresnel_dielectric(V3<float>{i[0], i[1], i[2]}, V3<float>{m[0], m[1], m[2]}, eta);
}
void oracle_onb(const float n[3], float u[3], float v[3]) {
    V3<float> a, b;
    onb(V3<float>{n[0], n[1], n[2]}, a, b);
    u[0] = a.x; u[1] = a.y; u[2] = a.z;
    v[0] = b.x; v[1] = b.y; v[2] = b.z;
}
float oracle_gamma(float c, float power) { return gamma_f(c, power); }
void oracle_miss(const float dir[3], uint32_t mode, float out[3]) {
    const V3<float> r = miss_color<float>(V3<float>{dir[0], dir[1], dir[2]}, mode);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

// glam Mat4::look_at_rh / perspective_rh (src/scene/camera.rs:98-106), in
// FP64, rounded to FP32; inverses by cofactor expansion in FP64.
static void inv4(const double* m, double* o) {
    double inv[16];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    const double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    for (int i = 0; i < 16; ++i) o[i] = inv[i] / det;
}

void oracle_camera_look_at(const float eye[3], const float center[3], const float up[3], float vfov_deg,
                           float aspect, float znear, float zfar, solrt_camera* out) {
    double f[3] = {(double)center[0] - eye[0], (double)center[1] - eye[1], (double)center[2] - eye[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& v : f) v /= fl;
    double s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    for (double& v : s) v /= sl;
    const double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    const double e[3] = {eye[0], eye[1], eye[2]};
    const double view[16] = {s[0], u[0], -f[0], 0, s[1], u[1], -f[1], 0, s[2], u[2], -f[2], 0,
                             -(s[0] * e[0] + s[1] * e[1] + s[2] * e[2]),
                             -(u[0] * e[0] + u[1] * e[1] + u[2] * e[2]),
                             (f[0] * e[0] + f[1] * e[1] + f[2] * e[2]), 1};
    const double fov = (double)vfov_deg * 3.14159265358979323846 / 180.0;
    const double h = 1.0 / std::tan(0.5 * fov);
    const double w = h / (double)aspect;
    const double r = (double)zfar / ((double)znear - (double)zfar);
    const double proj[16] = {w, 0, 0, 0, 0, h, 0, 0, 0, 0, r, -1, 0, 0, r * znear, 0};
    double vi[16], pi[16];
    inv4(view, vi);
    inv4(proj, pi);
    for (int i = 0; i < 16; ++i) {
        out->view[i] = (float)view[i];
        out->view_inverse[i] = (float)vi[i];
        out->projection[i] = (float)proj[i];
        out->projection_inverse[i] = (float)pi[i];
    }
}

}  // extern "C"
