// pathtrace.cu — wavefront restatement of the 5-pathtrace shaders.
//
// The reference runs one raygen invocation per pixel that loops over 8
// samples and up to maxBounces+1 traceRayEXT calls, each resuming in the
// closest-hit or miss shader (assets/glsl/pathtrace.rgen:39-104,
// pathtrace.rchit:56-113, pathtrace.rmiss:8-21). Here the loop is split into
// stages over structure-of-arrays queues in HBM:
//
//   generate  camera rays for (pixel, sample) pairs of one pass  (rgen:47-61)
//   extend    closest hit per queued ray                          (trace.cu)
//   shade     miss / emissive / scatter; survivors are appended to the next
//             queue with one atomic per warp (ballot compaction)  (rchit, rmiss)
//   accumulate per-pixel sums of the pass's path radiance, in sample order
//   finalize  mean, running mix with NaN/Inf guard, gamma, RGBA8  (rgen:86-103)
//
// Every path writes its radiance to its own slot and the per-pixel sum runs
// in sample order, so the result does not depend on queue order: it equals a
// sequential per-pixel evaluation bit for bit.
#include <algorithm>

#include "internal.h"

namespace solrt {

int extend_blocks_per_sm(uint32_t kind, bool counters);

namespace {

struct GenParams {
    float vinv[16];
    float pinv[16];
    uint32_t width, height, spp, frame, seed, job_id, rng_mode;
    uint32_t pix0, npix, s0, k;
    float tmax;
};

struct ShadeParams {
    uint32_t max_bounces, miss_mode, material_mode, rng_mode;
    uint32_t pix0, k, capacity;
};

__global__ void k_generate(GenParams g, PathQueue q, unsigned int* __restrict__ count0,
                           const uint32_t* __restrict__ rng_state, DevStats* stats) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t P = g.npix * g.k;
    if (i == 0) {
        *count0 = P;
        atomicAdd(&stats->paths, (unsigned long long)P);
    }
    if (i >= P) return;
    const uint32_t lp = i / g.k, j = i - lp * g.k;
    const uint32_t pix = g.pix0 + lp, s = g.s0 + j;
    const uint32_t x = pix % g.width, y = pix / g.width;
    uint32_t rng;
    if (g.rng_mode == SOLRT_RNG_PER_SAMPLE) {
        rng = tea(pix, g.frame * g.spp + s);
        if (g.seed != 0) rng ^= tea(g.seed, g.job_id);
    } else {
        rng = s == 0 ? tea(pix, g.frame) : rng_state[pix];   // rgen:47
    }
    // rgen:52-58: jitter, NDC, origin and direction through the inverse matrices
    const float j0 = next_rand(rng);
    const float j1 = next_rand(rng);
    const float px = __uint2float_rn(x) + j0, py = __uint2float_rn(y) + j1;
    const float ux = px / __uint2float_rn(g.width), uy = py / __uint2float_rn(g.height);
    const float dx = ux * 2.0f - 1.0f, dy = uy * 2.0f - 1.0f;
    float org[4], tgt[4], dir[4];
    mat4_mul(g.vinv, 0.0f, 0.0f, 0.0f, 1.0f, org);
    mat4_mul(g.pinv, dx, dy, 1.0f, 1.0f, tgt);
    const f3 tn = normalize(f3{tgt[0], tgt[1], tgt[2]});
    mat4_mul(g.vinv, tn.x, tn.y, tn.z, 0.0f, dir);
    const float tmin = glsl_max(1.0f, length(f3{org[0], org[1], org[2]})) * 1e-3f;  // rgen:35
    q.o_tmin[i] = make_float4(org[0], org[1], org[2], tmin);
    q.d_tmax[i] = make_float4(dir[0], dir[1], dir[2], g.tmax);
    q.thr_rng[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(rng));
    q.meta[i] = make_uint2(i, 0u);
}

__global__ void __launch_bounds__(256) k_shade(DevScene sc, ShadeParams sp, PathQueue qin,
                                               const float4* __restrict__ hits,
                                               const unsigned int* __restrict__ count_in, PathQueue qout,
                                               unsigned int* __restrict__ count_out, float4* __restrict__ rad,
                                               uint32_t* __restrict__ rng_state, DevStats* stats) {
    const unsigned int n = *count_in;
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    const uint32_t warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t ef = 0;
    for (uint32_t base = warp_global * 32u; base < n; base += warps * 32u) {
        const uint32_t i = base + lane;
        bool alive = false;
        float4 out_o = make_float4(0, 0, 0, 0), out_d = make_float4(0, 0, 0, 0), out_t = make_float4(0, 0, 0, 0);
        uint2 m = make_uint2(0, 0);
        if (i < n) {
            const float4 o = qin.o_tmin[i], d = qin.d_tmax[i], tr = qin.thr_rng[i];
            m = qin.meta[i];
            const float4 h = hits[i];
            uint32_t rng = __float_as_uint(tr.w);
            f3 acc{tr.x, tr.y, tr.z};
            const f3 dir{d.x, d.y, d.z};
            const uint32_t prim = __float_as_uint(h.y);
            bool done = true;
            if (prim == SOLRT_NO_HIT || prim >= sc.tri_count) {
                if (prim != SOLRT_NO_HIT) ef |= SOLRT_EFLAG_INDEX;
                acc = acc * miss_color(dir, sp.miss_mode);                      // rmiss:8-21
            } else {
                const uint4 ti = __ldg(sc.tri_idx + prim);                       // rchit:63-73
                const float4 m0 = __ldg(sc.materials + 3 * ti.w);
                const float4 m1 = __ldg(sc.materials + 3 * ti.w + 1);
                const float4 m2 = __ldg(sc.materials + 3 * ti.w + 2);
                if (m1.x >= 1.0f || m1.y >= 1.0f || m1.z >= 1.0f) {              // rchit:75-80
                    acc = acc * f3{m1.x, m1.y, m1.z};
                } else {
                    const float b1 = h.z, b2 = h.w;
                    const float b0 = (1.0f - b1) - b2;                           // rchit:82
                    const float4 n0 = __ldg(sc.vnrm + ti.x), n1 = __ldg(sc.vnrm + ti.y), n2 = __ldg(sc.vnrm + ti.z);
                    const float4 p0 = __ldg(sc.vpos + ti.x), p1 = __ldg(sc.vpos + ti.y), p2 = __ldg(sc.vpos + ti.z);
                    const float4 c0 = __ldg(sc.vcol + ti.x), c1 = __ldg(sc.vcol + ti.y), c2 = __ldg(sc.vcol + ti.z);
                    f3 normal = f3{n0.x, n0.y, n0.z} * b0 + f3{n1.x, n1.y, n1.z} * b1 + f3{n2.x, n2.y, n2.z} * b2;
                    normal = normalize(normal);                                  // rchit:84-86
                    const f3 pos = f3{p0.x, p0.y, p0.z} * b0 + f3{p1.x, p1.y, p1.z} * b1 + f3{p2.x, p2.y, p2.z} * b2;
                    const f3 vcol = f3{c0.x, c0.y, c0.z} * b0 + f3{c1.x, c1.y, c1.z} * b1 + f3{c2.x, c2.y, c2.z} * b2;
                    const f3 wi = normalize(dir);                                // rchit:94-95
                    const f3 n_o = normal * glsl_sign(dot(normal, -wi));
                    const float alpha2 = m2.y * m2.y;
                    const float xi0 = next_rand(rng);                            // rchit:97-98
                    const float xi1 = next_rand(rng);
                    const float rnd = next_rand(rng);
                    const f3 base_c{m0.x, m0.y, m0.z};
                    const f3 no = pos + 1e-4f * n_o;                             // rchit:100
                    f3 nd, hv;
                    if (sp.material_mode == SOLRT_MATERIAL_LAMBERT) {
                        nd = sample_cosine(n_o, xi0, xi1);
                        hv = base_c * vcol;
                    } else if (rnd < m2.x) {                                     // rchit:101-104
                        nd = sample_ggx(reflect(dir, n_o), xi0, xi1, alpha2);
                        hv = base_c * vcol;
                    } else {
                        const f3 mh = sample_ggx(n_o, xi0, xi1, alpha2);         // rchit:106-114
                        if (rnd < fresnel_dielectric(n_o, mh, 1.0f / 1.5f)) {
                            nd = reflect(dir, mh);
                            hv = f3{1.0f, 1.0f, 1.0f};
                        } else {
                            nd = sample_cosine(n_o, xi0, xi1);
                            hv = base_c * vcol;
                        }
                    }
                    const uint32_t depth = m.y + 1u;                             // rchit:116
                    acc = acc * hv;                                              // rgen:77
                    if (depth > sp.max_bounces) {                                // rgen:81-84
                        acc = f3{0.0f, 0.0f, 0.0f};
                    } else {
                        done = false;
                        out_o = make_float4(no.x, no.y, no.z, o.w);
                        out_d = make_float4(nd.x, nd.y, nd.z, d.w);
                        out_t = make_float4(acc.x, acc.y, acc.z, __uint_as_float(rng));
                        m.y = depth;
                    }
                }
            }
            if (done) {
                rad[m.x] = make_float4(acc.x, acc.y, acc.z, 0.0f);
                if (sp.rng_mode == SOLRT_RNG_REF_STREAM) rng_state[sp.pix0 + m.x / sp.k] = rng;
            } else {
                alive = true;
            }
        }
        const uint32_t mask = __ballot_sync(0xffffffffu, alive);
        if (mask) {
            const int leader = __ffs(mask) - 1;
            uint32_t pos0 = 0;
            if (lane == leader) pos0 = atomicAdd(count_out, (unsigned int)__popc(mask));
            pos0 = __shfl_sync(0xffffffffu, pos0, leader);
            if (alive) {
                const uint32_t pos = pos0 + __popc(mask & lane_lt);
                if (pos < sp.capacity) {
                    qout.o_tmin[pos] = out_o;
                    qout.d_tmax[pos] = out_d;
                    qout.thr_rng[pos] = out_t;
                    qout.meta[pos] = m;
                } else {
                    ef |= SOLRT_EFLAG_QUEUE;
                }
            }
        }
    }
    if (ef) atomicOr(&stats->eflags, ef);
}

// Per-pixel sums of one pass, samples in order (rgen:86).
__global__ void k_accumulate(const float4* __restrict__ rad, uint32_t pix0, uint32_t npix, uint32_t k,
                             uint32_t accum_mode, float4* __restrict__ fsum, float4* __restrict__ ksum,
                             float4* __restrict__ kcomp) {
    const uint32_t lp = blockIdx.x * blockDim.x + threadIdx.x;
    if (lp >= npix) return;
    const uint32_t pix = pix0 + lp;
    if (accum_mode == SOLRT_ACCUM_KAHAN) {
        const float4 s4 = ksum[pix], c4 = kcomp[pix];
        f3 ks{s4.x, s4.y, s4.z}, kc{c4.x, c4.y, c4.z};
        float kn = s4.w;
        for (uint32_t j = 0; j < k; ++j) {
            const float4 c = rad[(size_t)lp * k + j];
            if (isfinite(c.x) && isfinite(c.y) && isfinite(c.z)) {
                const f3 yv = f3{c.x, c.y, c.z} - kc;
                const f3 t = ks + yv;
                kc = (t - ks) - yv;
                ks = t;
                kn = kn + 1.0f;
            }
        }
        ksum[pix] = make_float4(ks.x, ks.y, ks.z, kn);
        kcomp[pix] = make_float4(kc.x, kc.y, kc.z, 0.0f);
    } else {
        const float4 s4 = fsum[pix];
        f3 s{s4.x, s4.y, s4.z};
        for (uint32_t j = 0; j < k; ++j) {
            const float4 c = rad[(size_t)lp * k + j];
            s = s + f3{c.x, c.y, c.z};
        }
        fsum[pix] = make_float4(s.x, s.y, s.z, 0.0f);
    }
}

__device__ __forceinline__ unsigned char to_unorm8(float c) {
    const float cl = glsl_min(glsl_max(c, 0.0f), 1.0f);
    return (unsigned char)(cl * 255.0f + 0.5f);
}

// rgen:88-103 (REF_MIX) or the Kahan mean.
__global__ void k_finalize(uint32_t npix, uint32_t spp, uint32_t frame, uint32_t start, uint32_t accum_mode,
                           const float4* __restrict__ fsum, const float4* __restrict__ ksum,
                           float4* __restrict__ accum, uchar4* __restrict__ rgba8) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    const float4 a = accum[pix];
    const f3 old{a.x, a.y, a.z};
    f3 out;
    if (accum_mode == SOLRT_ACCUM_KAHAN) {
        const float4 s = ksum[pix];
        out = s.w > 0.0f ? f3{s.x / s.w, s.y / s.w, s.z / s.w} : old;
    } else {
        const float4 s = fsum[pix];
        const float inv = 1.0f / __uint2float_rn(spp);
        const f3 mean = inv * f3{s.x, s.y, s.z};
        const float alpha = 1.0f / __uint2float_rn(frame + 1u - start);
        out = mix(old, mean, alpha);
        if (isnan(out.x) || isnan(out.y) || isnan(out.z)) out = old;
        if (isinf(out.x) || isinf(out.y) || isinf(out.z)) out = old;
    }
    accum[pix] = make_float4(out.x, out.y, out.z, 1.0f);
    const float g = 1.0f / 2.2f;
    rgba8[pix] = make_uchar4(to_unorm8(powf(out.x, g)), to_unorm8(powf(out.y, g)), to_unorm8(powf(out.z, g)), 255);
}

// Known-answer kernels for the unit functions.
__global__ void k_debug_unit(uint32_t op, uint32_t n, const uint32_t* a, const uint32_t* b, const float* in,
                             uint32_t* out_u, float* out_f) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (op == 1) {
        if (i != 0) return;
        uint32_t st = a[0];
        for (uint32_t k = 0; k < b[0]; ++k) out_f[k] = next_rand(st);
        out_u[0] = st;
        return;
    }
    if (i >= n) return;
    const float* v = in + 8 * (size_t)i;
    if (op == 0) {
        out_u[i] = tea(a[i], b[i]);
    } else if (op == 2) {
        float s, c;
        sincos_poly(in[i], s, c);
        out_f[2 * i] = s;
        out_f[2 * i + 1] = c;
    } else if (op == 3) {
        const f3 r = sample_ggx(f3{v[0], v[1], v[2]}, v[3], v[4], v[5]);
        out_f[3 * i] = r.x; out_f[3 * i + 1] = r.y; out_f[3 * i + 2] = r.z;
    } else if (op == 4) {
        const f3 r = sample_cosine(f3{v[0], v[1], v[2]}, v[3], v[4]);
        out_f[3 * i] = r.x; out_f[3 * i + 1] = r.y; out_f[3 * i + 2] = r.z;
    } else if (op == 5) {
        out_f[i] = fresnel_dielectric(f3{v[0], v[1], v[2]}, f3{v[3], v[4], v[5]}, v[6]);
    } else if (op == 6) {
        const f3 r = miss_color(f3{v[0], v[1], v[2]}, a[i]);
        out_f[3 * i] = r.x; out_f[3 * i + 1] = r.y; out_f[3 * i + 2] = r.z;
    } else if (op == 7) {
        out_f[i] = powf(in[i], 1.0f / 2.2f);
    }
}

inline uint32_t cdiv(uint64_t a, uint32_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

solrt_status render_frame(Context& ctx, const Scene& sc, const solrt_camera& cam, const solrt_render_params& p,
                          Image& img) {
    cudaStream_t st = ctx.stream;
    const uint32_t npix = p.width * p.height;
    const bool ref_stream = p.rng_mode == SOLRT_RNG_REF_STREAM;
    const uint32_t cap = ctx.capacity;
    uint32_t k, chunk;
    if (ref_stream) {
        k = 1;
        chunk = std::min(npix, cap);
    } else if (npix <= cap) {
        k = std::max(1u, std::min(p.spp, cap / npix));
        chunk = npix;
    } else {
        k = 1;
        chunk = cap;
    }
    GenParams g;
    std::copy(cam.view_inverse, cam.view_inverse + 16, g.vinv);
    std::copy(cam.projection_inverse, cam.projection_inverse + 16, g.pinv);
    g.width = p.width;
    g.height = p.height;
    g.spp = p.spp;
    g.frame = p.frame;
    g.seed = p.seed;
    g.job_id = p.job_id;
    g.rng_mode = p.rng_mode;
    g.tmax = p.tmax > 0.0f ? p.tmax : 10000.0f;
    ShadeParams sp;
    sp.max_bounces = p.max_bounces;
    sp.miss_mode = p.miss_mode;
    sp.material_mode = p.material_mode;
    sp.rng_mode = p.rng_mode;
    sp.capacity = cap;
    const DevScene dsc = sc.view();
    DevStats* stats = ctx.stats.as<DevStats>();
    PassCtl* ctl = ctx.ctl.as<PassCtl>();
    const size_t ctl_bytes = sizeof(unsigned int) * (p.max_bounces + 2);
    const int shade_grid = ctx.sm_count * 8;

    SOLRT_CUDA(cudaEventRecord(ctx.ev0, st));
    if (p.accum_mode != SOLRT_ACCUM_KAHAN) SOLRT_CUDA(cudaMemsetAsync(img.frame_sum.ptr, 0, img.frame_sum.bytes, st));
    for (uint32_t s0 = 0; s0 < p.spp; s0 += k) {
        const uint32_t kk = std::min(k, p.spp - s0);
        for (uint32_t pix0 = 0; pix0 < npix; pix0 += chunk) {
            const uint32_t np = std::min(chunk, npix - pix0);
            SOLRT_CUDA(cudaMemsetAsync(ctl->count, 0, ctl_bytes, st));
            SOLRT_CUDA(cudaMemsetAsync(ctl->work, 0, ctl_bytes, st));
            g.pix0 = pix0;
            g.npix = np;
            g.s0 = s0;
            g.k = kk;
            sp.pix0 = pix0;
            sp.k = kk;
            k_generate<<<cdiv((uint64_t)np * kk, 256), 256, 0, st>>>(g, ctx.queue(0), ctl->count,
                                                                    img.rng_state.as<uint32_t>(), stats);
            ++ctx.launches;
            for (uint32_t b = 0; b <= p.max_bounces; ++b) {
                const PathQueue qin = ctx.queue(b & 1), qout = ctx.queue((b + 1) & 1);
                const int te = ctx.timing_begin(0);
                SOLRT_TRY(launch_extend(ctx, sc, qin, ctx.hits.as<float4>(), ctl->count + b, ctl->work + b, cap));
                ctx.timing_end(te);
                const int ts = ctx.timing_begin(1);
                k_shade<<<shade_grid, 256, 0, st>>>(dsc, sp, qin, ctx.hits.as<float4>(), ctl->count + b, qout,
                                                    ctl->count + b + 1, ctx.rad.as<float4>(),
                                                    img.rng_state.as<uint32_t>(), stats);
                ctx.timing_end(ts);
                ++ctx.launches;
            }
            k_accumulate<<<cdiv(np, 256), 256, 0, st>>>(ctx.rad.as<float4>(), pix0, np, kk, p.accum_mode,
                                                        img.frame_sum.as<float4>(), img.ksum.as<float4>(),
                                                        img.kcomp.as<float4>());
            ++ctx.launches;
        }
    }
    k_finalize<<<cdiv(npix, 256), 256, 0, st>>>(npix, p.spp, p.frame, p.accum_start_frame, p.accum_mode,
                                                img.frame_sum.as<float4>(), img.ksum.as<float4>(),
                                                img.accum.as<float4>(), img.rgba8.as<uchar4>());
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    SOLRT_CUDA(cudaEventRecord(ctx.ev1, st));
    return SOLRT_OK;
}

solrt_status debug_unit(Context& ctx, uint32_t op, uint32_t n, const uint32_t* a, const uint32_t* b,
                        const float* in_f32, uint32_t* out_u32, float* out_f32) {
    if (op > 7) {
        set_error("unknown debug op %u", op);
        return SOLRT_ERR_INVALID;
    }
    const size_t nu = op == 1 ? 1 : n;
    const size_t nf = op == 1 ? (b ? b[0] : 0) : (size_t)n * 3;
    DeviceBuffer da, db, din, dou, dof;
    cudaStream_t st = ctx.stream;
    SOLRT_TRY(da.alloc(4 * std::max<size_t>(nu, 1)));
    SOLRT_TRY(db.alloc(4 * std::max<size_t>(nu, 1)));
    SOLRT_TRY(din.alloc(32 * std::max<size_t>(n, 1)));
    SOLRT_TRY(dou.alloc(4 * std::max<size_t>(nu, 1)));
    SOLRT_TRY(dof.alloc(4 * std::max<size_t>(nf, 1)));
    if (a) SOLRT_CUDA(cudaMemcpyAsync(da.ptr, a, 4 * nu, cudaMemcpyHostToDevice, st));
    if (b) SOLRT_CUDA(cudaMemcpyAsync(db.ptr, b, 4 * nu, cudaMemcpyHostToDevice, st));
    if (in_f32) {
        const size_t nin = (op == 2 || op == 7) ? n : (size_t)n * 8;
        SOLRT_CUDA(cudaMemcpyAsync(din.ptr, in_f32, 4 * nin, cudaMemcpyHostToDevice, st));
    }
    k_debug_unit<<<cdiv(std::max<uint32_t>(n, 1), 128), 128, 0, st>>>(op, n, da.as<uint32_t>(), db.as<uint32_t>(),
                                                                      din.as<float>(), dou.as<uint32_t>(),
                                                                      dof.as<float>());
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    if (out_u32) SOLRT_CUDA(cudaMemcpyAsync(out_u32, dou.ptr, 4 * nu, cudaMemcpyDeviceToHost, st));
    if (out_f32) {
        const size_t nout = op == 1 ? nf : (op == 2 ? 2 * (size_t)n : ((op == 5 || op == 7) ? n : 3 * (size_t)n));
        SOLRT_CUDA(cudaMemcpyAsync(out_f32, dof.ptr, 4 * nout, cudaMemcpyDeviceToHost, st));
    }
    SOLRT_CUDA(cudaStreamSynchronize(st));
    return SOLRT_OK;
}

}  // namespace solrt
