// path_ops.cuh — the per-path operations of the pathtrace shaders, shared by
// the wavefront kernels (one stage per launch) and the per-pixel megakernel
// (the reference's structure: one thread loops over samples and bounces).
#pragma once

#include "internal.h"

namespace solrt {

// RNG state of sample s of pixel pix (pathtrace.rgen:47 for REF_STREAM's
// first sample; later REF_STREAM samples continue the previous state).
SOLRT_D uint32_t sample_seed(const DevJob& J, uint32_t pix, uint32_t s, uint32_t prev) {
    if (J.rng_mode == SOLRT_RNG_PER_SAMPLE) {
        uint32_t rng = tea(pix, J.frame * J.spp + s);
        if (J.seed != 0) rng ^= tea(J.seed, J.job_id);
        return rng;
    }
    return s == 0 ? tea(pix, J.frame) : prev;
}

// pathtrace.rgen:52-60: jitter, NDC, origin and direction through the
// inverse matrices; tmin of preparePayload (rgen:35).
SOLRT_D void camera_ray(const DevJob& J, uint32_t pix, uint32_t& rng, float4& o_tmin, float4& d_tmax) {
    const uint32_t x = pix % J.width, y = pix / J.width;
    const float j0 = next_rand(rng);
    const float j1 = next_rand(rng);
    const float px = __uint2float_rn(x) + j0, py = __uint2float_rn(y) + j1;
    const float ux = px / __uint2float_rn(J.width), uy = py / __uint2float_rn(J.height);
    const float dx = ux * 2.0f - 1.0f, dy = uy * 2.0f - 1.0f;
    float org[4], tgt[4], dir[4];
    mat4_mul(J.vinv, 0.0f, 0.0f, 0.0f, 1.0f, org);
    mat4_mul(J.pinv, dx, dy, 1.0f, 1.0f, tgt);
    const f3 tn = normalize(f3{tgt[0], tgt[1], tgt[2]});
    mat4_mul(J.vinv, tn.x, tn.y, tn.z, 0.0f, dir);
    const float tmin = glsl_max(1.0f, length(f3{org[0], org[1], org[2]})) * 1e-3f;
    o_tmin = make_float4(org[0], org[1], org[2], tmin);
    d_tmax = make_float4(dir[0], dir[1], dir[2], J.tmax);
}

// Column-major mat4 (4 float4 columns at m) times (x, y, z, w), per row
// ((c0 x + c1 y) + c2 z) + c3 w: GLSL's mat4 * vec4 in the order the oracle
// and the reference's shaders compiled as C++ use.
SOLRT_D f3 mat4_xyz(const float4* m, float x, float y, float z, float w) {
    const float4 c0 = __ldg(m), c1 = __ldg(m + 1), c2 = __ldg(m + 2), c3 = __ldg(m + 3);
    return f3{((c0.x * x + c1.x * y) + c2.x * z) + c3.x * w, ((c0.y * x + c1.y * y) + c2.y * z) + c3.y * w,
              ((c0.z * x + c1.z * y) + c2.z * z) + c3.z * w};
}

// Shading normal and position of a hit as pathtrace.rchit:82-90 (and
// ao.rchit:66-75) compute them: object-space vertex normals and positions
// interpolated with the barycentrics, then the section instance's
// transform_it (normal, w = 0, normalised) and transform (position, w = 1).
// `vcol`, when given, receives the interpolated vertex colour (rchit:87),
// which each vertex's 256-bit normal load brings along.
SOLRT_D void hit_frame(const DevScene& sc, uint4 ti, float b0, float b1, float b2, f3& normal, f3& pos,
                       f3* vcol = nullptr) {
    float4 n0, n1, n2, c0, c1, c2;
    ldg_2x4(sc.vnc + 2 * (size_t)ti.x, n0, c0);
    ldg_2x4(sc.vnc + 2 * (size_t)ti.y, n1, c1);
    ldg_2x4(sc.vnc + 2 * (size_t)ti.z, n2, c2);
    const float4 p0 = __ldg(sc.opos + ti.x), p1 = __ldg(sc.opos + ti.y), p2 = __ldg(sc.opos + ti.z);
    if (vcol) *vcol = f3{c0.x, c0.y, c0.z} * b0 + f3{c1.x, c1.y, c1.z} * b1 + f3{c2.x, c2.y, c2.z} * b2;
    const f3 n = f3{n0.x, n0.y, n0.z} * b0 + f3{n1.x, n1.y, n1.z} * b1 + f3{n2.x, n2.y, n2.z} * b2;
    const f3 p = f3{p0.x, p0.y, p0.z} * b0 + f3{p1.x, p1.y, p1.z} * b1 + f3{p2.x, p2.y, p2.z} * b2;
    const float4* inst = sc.sections + 9 * (size_t)ti.w;  // (id, ..), transform, transform_it
    normal = normalize(mat4_xyz(inst + 5, n.x, n.y, n.z, 0.0f));
    pos = mat4_xyz(inst + 1, p.x, p.y, p.z, 1.0f);
}

// One closest-hit or miss step (pathtrace.rchit:56-113, pathtrace.rmiss:8-21
// and pathtrace.rgen:77-84). h = (t, prim bits, u, v). Updates the path
// throughput `acc`, the rng state and the depth; returns true when the path
// continues with the ray (o_next, d_next).
SOLRT_D float light_pick_prob(const DevScene& sc, uint32_t code, f3 x, f3 n);
SOLRT_D float mis_weight(float p_this, float p_other);

// kNee (jobs of SOLRT_INTEGRATOR_PATH_NEE; compiled out otherwise): an
// emitter hit after a bounce is weighted
// by the power heuristic against next-event estimation (`prev`: oriented
// normal of the vertex this ray left and the solid-angle pdf of its BSDF
// sample); `n_out` and `prev_out`, when given, receive the oriented shading
// normal of a continuing path and (that normal, the pdf of its new
// direction).
template <bool kNee = false>
SOLRT_D bool shade_step(const DevJob& J, float4 o, float4 d, float4 h, f3& acc, uint32_t& rng, uint32_t& depth,
                        float4& o_next, float4& d_next, uint32_t& ef, f3* n_out = nullptr,
                        float4 prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f), float4* prev_out = nullptr) {
    const DevScene& sc = J.sc;
    const f3 dir{d.x, d.y, d.z};
    const uint32_t prim = __float_as_uint(h.y);
    if (prim == SOLRT_NO_HIT || prim >= sc.tri_count) {
        if (prim != SOLRT_NO_HIT) ef |= SOLRT_EFLAG_INDEX;
        acc = acc * miss_color(dir, J.miss_mode);                           // rmiss:8-21
        return false;
    }
    const uint4 ti = __ldg(sc.tri_idx + prim);                               // rchit:63-73
    const uint32_t mat = __ldg(sc.sec_mat + ti.w);                           // rchit:71
    const float4 m0 = __ldg(sc.materials + 3 * mat);
    const float4 m1 = __ldg(sc.materials + 3 * mat + 1);
    const float4 m2 = __ldg(sc.materials + 3 * mat + 2);
    if (m1.x >= 1.0f || m1.y >= 1.0f || m1.z >= 1.0f) {                      // rchit:75-80
        acc = acc * f3{m1.x, m1.y, m1.z};
        if (kNee && J.integrator == SOLRT_INTEGRATOR_PATH_NEE && depth > 0u) {
            // the light pdf of this hit: pick probability from the ray's
            // origin times distance^2 / (area cos_y)
            const uint32_t code = sc.tri_light ? __ldg(sc.tri_light + prim) : ~0u;
            float pl = 0.0f;
            if (code != ~0u) {
                const float4 a = __ldg(sc.vpos + ti.x), b = __ldg(sc.vpos + ti.y), c = __ldg(sc.vpos + ti.z);
                const f3 e1{b.x - a.x, b.y - a.y, b.z - a.z}, e2{c.x - a.x, c.y - a.y, c.z - a.z};
                const f3 ng{e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
                const float a2 = length(ng);
                const float cy = fabsf(dot(ng, dir)) / a2;
                const float pick = light_pick_prob(sc, code, f3{o.x, o.y, o.z}, f3{prev.x, prev.y, prev.z});
                pl = (pick * (h.x * h.x)) / ((0.5f * a2) * cy);
            }
            acc = acc * mis_weight(prev.w, pl);
        }
        return false;
    }
    const float b1 = h.z, b2 = h.w;
    const float b0 = (1.0f - b1) - b2;                                       // rchit:82
    f3 normal, pos, vcol;
    hit_frame(sc, ti, b0, b1, b2, normal, pos, &vcol);                       // rchit:82-90
    const f3 wi = normalize(dir);                                            // rchit:94-95
    const f3 n_o = normal * glsl_sign(dot(normal, -wi));
    const float alpha2 = m2.y * m2.y;
    const float xi0 = next_rand(rng);                                        // rchit:97-98
    const float xi1 = next_rand(rng);
    const float rnd = next_rand(rng);
    const f3 base_c{m0.x, m0.y, m0.z};
    const f3 no = pos + 1e-4f * n_o;                                         // rchit:100
    f3 nd, hv;
    if (J.material_mode == SOLRT_MATERIAL_LAMBERT) {
        nd = sample_cosine(n_o, xi0, xi1);
        hv = base_c * vcol;
    } else if (rnd < m2.x) {                                                 // rchit:101-104
        nd = sample_ggx(reflect(dir, n_o), xi0, xi1, alpha2);
        hv = base_c * vcol;
    } else {
        const f3 mh = sample_ggx(n_o, xi0, xi1, alpha2);                     // rchit:106-114
        if (rnd < fresnel_dielectric(n_o, mh, 1.0f / 1.5f)) {
            nd = reflect(dir, mh);
            hv = f3{1.0f, 1.0f, 1.0f};
        } else {
            nd = sample_cosine(n_o, xi0, xi1);
            hv = base_c * vcol;
        }
    }
    depth = depth + 1u;                                                      // rchit:116
    acc = acc * hv;                                                          // rgen:77
    if (depth > J.max_bounces) {                                             // rgen:81-84
        acc = f3{0.0f, 0.0f, 0.0f};
        return false;
    }
    o_next = make_float4(no.x, no.y, no.z, o.w);
    d_next = make_float4(nd.x, nd.y, nd.z, d.w);
    if (kNee && n_out) *n_out = n_o;
    if (kNee && prev_out) *prev_out = make_float4(n_o.x, n_o.y, n_o.z, dot(n_o, nd) / 3.14159265f);
    return true;
}

// Importance of a light-tree child seen from x with normal n:
// power * cos_bound / max(d^2, r^2), d the distance to the child's box
// centre, r its half-diagonal (s = (centre, r^2)), cos_bound the largest
// cosine between n and a direction into the child's bounding sphere:
// 1 when the angle theta to the centre is within the sphere's half-angle
// beta (sin beta = r / d), else max(0, cos(theta - beta)) =
// max(0, cos theta cos beta + sin theta sin beta). Square roots only, so
// the host and the device agree bit for bit.
SOLRT_D float light_importance(float4 s, float power, f3 x, f3 n) {
    const f3 dv{s.x - x.x, s.y - x.y, s.z - x.z};
    const float d2 = dot(dv, dv);
    float cb = 1.0f;
    if (d2 > s.w) {
        const float ct = dot(n, dv) / sqrtf(d2);
        const float sb2 = s.w / d2;
        const float cbeta = sqrtf(1.0f - sb2);
        if (ct < cbeta) {
            const float st = sqrtf(glsl_max(1.0f - ct * ct, 0.0f));
            cb = glsl_max(ct * cbeta + st * sqrtf(sb2), 0.0f);
        }
    }
    return (power * cb) / glsl_max(d2, s.w);
}

// Probability that the light-tree walk from x (normal n) picks the light of
// `code` (the same products as the sampling walk of nee_sample).
SOLRT_D float light_pick_prob(const DevScene& sc, uint32_t code, f3 x, f3 n) {
    const uint32_t levels = code >> 27;
    uint32_t k = 0;
    float pick = 1.0f;
    for (uint32_t lv = 0; lv < levels; ++lv) {
        const float4* nd = sc.lights + 3 * (size_t)k;
        const float4 sl = __ldg(nd), sr = __ldg(nd + 1), pc = __ldg(nd + 2);
        const float wl = light_importance(sl, pc.x, x, n), wr = light_importance(sr, pc.y, x, n);
        const float pl = wl / (wl + wr);
        if (!(pl >= 0.0f && pl <= 1.0f)) return 0.0f;
        const bool right = (code >> lv) & 1u;
        pick = right ? pick * (1.0f - pl) : pick * pl;
        const int ref = __float_as_int(right ? pc.w : pc.z);
        if (ref < 0) break;
        k = (uint32_t)ref;
    }
    return pick;
}

// Power-heuristic weight of a sample whose technique has pdf p_this against
// one with pdf p_other: 1 / (1 + (p_other / p_this)^2).
SOLRT_D float mis_weight(float p_this, float p_other) {
    if (!(p_this > 0.0f)) return 0.0f;
    const float r = p_other / p_this;
    return 1.0f / (1.0f + r * r);
}

// Next-event estimation at a diffuse vertex of SOLRT_INTEGRATOR_PATH_NEE (an
// estimator the reference does not have). Draws: l1 and l2 pick a uniform
// point on the light triangle (b0 = 1 - sqrt(l1), b1 = l2 sqrt(l1)); then
// one draw per light-tree level takes the left child with probability
// wl / (wl + wr) of the children's importances, so near and bright lights
// are picked more often; p_pick is the product of the choices. `no` is the
// continuation origin (hit + 1e-4 n_o), `thr` the throughput after the
// vertex's albedo. Returns true with the shadow ray (so, sd: unit
// direction, tmax 0.9999 of the distance) and the radiance it adds when
// unoccluded: thr * Le * (pb / pl) * w, with the solid-angle pdfs
// pl = p_pick r^2 / (area cos_y) of the light pick and pb = cos_x / pi of the
// cosine BSDF sample, and w = 1 / (1 + (pb / pl)^2) the power heuristic
// (the BSDF sample's emitter hit gets the complementary weight in
// shade_step). Area of the triangle's current world vertices; emitters are
// two-sided, as hits on them are (rchit:75-80).
SOLRT_D bool nee_sample(const DevScene& sc, f3 no, f3 n_o, f3 thr, float tmin, uint32_t& rng, float4& so,
                        float4& sd, f3& contrib) {
    const float l1 = next_rand(rng);
    const float l2 = next_rand(rng);
    if (sc.light_count == 0u) return false;
    uint32_t k = 0, prim = ~0u;
    float pick = 1.0f;
    for (int level = 0; level < 64; ++level) {
        const float4* nd = sc.lights + 3 * (size_t)k;
        const float4 sl = __ldg(nd), sr = __ldg(nd + 1), pc = __ldg(nd + 2);
        const float wl = light_importance(sl, pc.x, no, n_o), wr = light_importance(sr, pc.y, no, n_o);
        const float pl = wl / (wl + wr);
        if (!(pl >= 0.0f && pl <= 1.0f)) return false;
        const float ul = next_rand(rng);
        int ref;
        if (ul < pl) {
            ref = __float_as_int(pc.z);
            pick = pick * pl;
        } else {
            ref = __float_as_int(pc.w);
            pick = pick * (1.0f - pl);
        }
        if (ref < 0) {
            prim = (uint32_t)~ref;
            break;
        }
        k = (uint32_t)ref;
    }
    if (prim >= sc.tri_count || !(pick > 0.0f)) return false;
    const uint4 ti = __ldg(sc.tri_idx + prim);
    const float4 a = __ldg(sc.vpos + ti.x), b = __ldg(sc.vpos + ti.y), c = __ldg(sc.vpos + ti.z);
    const f3 p0{a.x, a.y, a.z}, p1{b.x, b.y, b.z}, p2{c.x, c.y, c.z};
    const float su = sqrtf(l1);
    const float b0 = 1.0f - su, b1 = l2 * su;
    const float b2 = (1.0f - b0) - b1;
    const f3 y = p0 * b0 + p1 * b1 + p2 * b2;
    const f3 e1 = p1 - p0, e2 = p2 - p0;
    const f3 ng{e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
    const float a2 = length(ng);  // twice the area
    const f3 w = y - no;
    const float d2 = dot(w, w);
    if (!(a2 > 0.0f) || !(d2 > 0.0f)) return false;
    const float dist = sqrtf(d2);
    const f3 wl{w.x / dist, w.y / dist, w.z / dist};
    const float cx = dot(n_o, wl);
    const float cy = fabsf(dot(ng, wl)) / a2;
    const float tmax = dist * 0.9999f;
    if (!(cx > 0.0f) || !(cy > 0.0f) || !(tmax > tmin)) return false;
    const float4 le = __ldg(sc.materials + 3 * __ldg(sc.sec_mat + ti.w) + 1);
    // solid-angle pdfs of this direction: light pick, cosine BSDF sample
    const float pl = (pick * d2) / ((0.5f * a2) * cy);
    const float pb = cx / 3.14159265f;
    if (!(pl > 0.0f)) return false;
    const float wgt = (pb / pl) * mis_weight(pl, pb);  // BRDF cos / pdf, MIS-weighted
    contrib = (thr * f3{le.x, le.y, le.z}) * wgt;
    so = make_float4(no.x, no.y, no.z, tmin);
    sd = make_float4(wl.x, wl.y, wl.z, tmax);
    return true;
}

// Per-pixel sample sums (rgen:86) and the Kahan variant.
SOLRT_D void add_sample(f3& s, float4 c) { s = s + f3{c.x, c.y, c.z}; }
SOLRT_D void add_sample_kahan(f3& ks, f3& kc, float& kn, float4 c) {
    if (isfinite(c.x) && isfinite(c.y) && isfinite(c.z)) {
        const f3 yv = f3{c.x, c.y, c.z} - kc;
        const f3 t = ks + yv;
        kc = (t - ks) - yv;
        ks = t;
        kn = kn + 1.0f;
    }
}

// ---------------------------------------------------------------------------
// Stage bodies shared by the one-stage-per-launch kernels (pathtrace.cu) and
// the cooperative one-launch batch (coop.cu). `Ld` loads what an earlier
// stage wrote: plain loads when stages are separate launches, loads through
// L2 (ld.global.cg) when they are phases of one launch, where this SM's L1
// may still hold lines from before another SM's writes.
// ---------------------------------------------------------------------------
struct LdPlain {
    template <class T> SOLRT_D static T ld(const T* p) { return *p; }
};
struct LdL2 {
    template <class T> SOLRT_D static T ld(const T* p) { return __ldcg(p); }
};

// Largest index i in [0, n) with key(i) <= v (key increasing, key(0) = 0).
template <class F>
SOLRT_D uint32_t find_last_le(uint32_t n, uint32_t v, F key) {
    uint32_t lo = 0, hi = n;  // invariant: key(lo) <= v, answer in [lo, hi)
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (key(mid) <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Zeroes the frame sample sum of pixel t of the batch's pixel space (running
// mix jobs).
SOLRT_D void begin_pixel(const DevJob* jobs, const uint32_t* job_pix, uint32_t njobs, uint32_t t) {
    const uint32_t j = find_last_le(njobs, t, [&](uint32_t i) { return job_pix[i]; });
    const DevJob& J = jobs[j];
    if (J.accum_mode != SOLRT_ACCUM_KAHAN) J.fsum[t - job_pix[j]] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// Camera ray of path slot i of a pass (rgen:47-61) into queue q.
template <class Ld>
SOLRT_D void generate_path(const DevJob* jobs, const DevItem* items, uint32_t nitems, uint32_t i, const PathQueue& q,
                           float4* rad) {
    const DevItem it = items[find_last_le(nitems, i, [&](uint32_t t) { return items[t].path_base; })];
    const DevJob& J = jobs[it.job];
    const uint32_t local = i - it.path_base;
    const uint32_t lp = local / it.k, j = local - lp * it.k;
    const uint32_t pix = it.pix0 + lp, s = it.s0 + j;
    uint32_t rng = sample_seed(J, pix, s, J.rng_mode == SOLRT_RNG_REF_STREAM && s > 0 ? Ld::ld(J.rng_state + pix) : 0u);
    float4 o, d;
    camera_ray(J, pix, rng, o, d);
    q.o_tmin[i] = o;
    q.d_tmax[i] = d;
    q.thr_rng[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(rng));
    q.meta[i] = make_uint2(i, it.job << kDepthBits);
    if (J.integrator == SOLRT_INTEGRATOR_PATH_NEE) rad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // sums shadow terms
}

// Adds the pass's samples of pass pixel t to its pixel's sums, in sample
// order (rgen:86).
template <class Ld>
SOLRT_D void accumulate_pixel(const DevJob* jobs, const DevItem* items, uint32_t nitems, uint32_t t,
                              const float4* rad) {
    const DevItem it = items[find_last_le(nitems, t, [&](uint32_t i) { return items[i].pix_base; })];
    const DevJob& J = jobs[it.job];
    const uint32_t lp = t - it.pix_base;
    const uint32_t pix = it.pix0 + lp;
    const float4* r = rad + it.path_base + (size_t)lp * it.k;
    if (J.accum_mode == SOLRT_ACCUM_KAHAN) {
        const float4 s4 = Ld::ld(J.ksum + pix), c4 = Ld::ld(J.kcomp + pix);
        f3 ks{s4.x, s4.y, s4.z}, kc{c4.x, c4.y, c4.z};
        float kn = s4.w;
        for (uint32_t j = 0; j < it.k; ++j) add_sample_kahan(ks, kc, kn, Ld::ld(r + j));
        J.ksum[pix] = make_float4(ks.x, ks.y, ks.z, kn);
        J.kcomp[pix] = make_float4(kc.x, kc.y, kc.z, 0.0f);
    } else {
        const float4 s4 = Ld::ld(J.fsum + pix);
        f3 s{s4.x, s4.y, s4.z};
        for (uint32_t j = 0; j < it.k; ++j) add_sample(s, Ld::ld(r + j));
        J.fsum[pix] = make_float4(s.x, s.y, s.z, 0.0f);
    }
    if (J.sq) {  // squared sample sums of the stopping rule (samples the sums above keep)
        float q = Ld::ld(J.sq + pix);
        for (uint32_t j = 0; j < it.k; ++j) {
            const float4 c = Ld::ld(r + j);
            if (J.accum_mode != SOLRT_ACCUM_KAHAN || (isfinite(c.x) && isfinite(c.y) && isfinite(c.z)))
                q = q + (c.x * c.x + c.y * c.y + c.z * c.z);
        }
        J.sq[pix] = q;
    }
}

SOLRT_D unsigned char to_unorm8(float c) {
    const float cl = glsl_min(glsl_max(c, 0.0f), 1.0f);
    return (unsigned char)(cl * 255.0f + 0.5f);
}

// rgen:88-103 (REF_MIX) or the Kahan mean, for pixel t of the batch's pixel
// space.
template <class Ld>
SOLRT_D void finalize_pixel(const DevJob* jobs, const uint32_t* job_pix, uint32_t njobs, uint32_t t) {
    const uint32_t j = find_last_le(njobs, t, [&](uint32_t i) { return job_pix[i]; });
    const DevJob& J = jobs[j];
    const uint32_t pix = t - job_pix[j];
    const float4 a = J.accum[pix];
    const f3 old{a.x, a.y, a.z};
    f3 out;
    if (J.accum_mode == SOLRT_ACCUM_KAHAN) {
        const float4 s = Ld::ld(J.ksum + pix);
        out = s.w > 0.0f ? f3{s.x / s.w, s.y / s.w, s.z / s.w} : old;
    } else {
        const float4 s = Ld::ld(J.fsum + pix);
        const float inv = 1.0f / __uint2float_rn(J.spp);
        const f3 mean = inv * f3{s.x, s.y, s.z};
        const float alpha = 1.0f / __uint2float_rn(J.frame + 1u - J.start);
        out = mix(old, mean, alpha);
        if (isnan(out.x) || isnan(out.y) || isnan(out.z)) out = old;
        if (isinf(out.x) || isinf(out.y) || isinf(out.z)) out = old;
    }
    J.accum[pix] = make_float4(out.x, out.y, out.z, 1.0f);
    const float g = 1.0f / 2.2f;
    J.rgba8[pix] = make_uchar4(to_unorm8(powf(out.x, g)), to_unorm8(powf(out.y, g)), to_unorm8(powf(out.z, g)), 255);
}

}  // namespace solrt
