// pathtrace.cu — wavefront restatement of the 5-pathtrace shaders, for one
// job (solrt_render) or a batch of jobs over many scenes (solrt_batch_*).
//
// The reference runs one raygen invocation per pixel that loops over 8
// samples and up to maxBounces+1 traceRayEXT calls, each resuming in the
// closest-hit or miss shader (assets/glsl/pathtrace.rgen:39-104,
// pathtrace.rchit:56-113, pathtrace.rmiss:8-21). Here the loop is split into
// stages over structure-of-arrays queues in HBM:
//
//   generate  camera rays for the (pixel, sample) pairs of a pass (rgen:47-61)
//   extend    closest hit per queued ray                           (trace.cu)
//   shade     miss / emissive / scatter; survivors are appended to the next
//             queue with one atomic per warp (ballot compaction)   (rchit, rmiss)
//   accumulate per-pixel sums of the pass's path radiance, in sample order
//   finalize  mean, running mix with NaN/Inf guard, gamma, RGBA8   (rgen:86-103)
//
// A pass is a list of work items (job, pixel range, sample range) whose
// paths fit the queues. Items of different jobs share a pass: each path
// carries its job in its meta word and reads that job's scene and
// parameters. Every path writes its radiance to its own slot and per-pixel
// sums run in sample order, so a job's image does not depend on queue order
// or on the other jobs: it equals a sequential per-pixel evaluation bit for
// bit.
#include <algorithm>

#include "bvh2_2l.cuh"
#include "bvh2_ww.cuh"
#include "bvh4_ww.cuh"
#include "bvh8_traverse.cuh"
#include "internal.h"
#include "path_ops.cuh"

namespace solrt {

namespace {

__global__ void k_generate(const DevJob* __restrict__ jobs, const DevItem* __restrict__ items, uint32_t nitems,
                           uint32_t P, PathQueue q, unsigned int* __restrict__ count0, DevStats* stats,
                           float4* __restrict__ rad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        *count0 = P;
        atomicAdd(&stats->paths, (unsigned long long)P);
    }
    if (i >= P) return;
    generate_path<LdPlain>(jobs, items, nitems, i, q, rad);
}

// kNee: the variant for passes with SOLRT_INTEGRATOR_PATH_NEE jobs (shadow
// queue, MIS state); plain passes run the variant without that code.
// Resident 256-thread shade blocks per SM asked of the register allocator:
// 4 (64 registers, a few spilled) against 3 at 74 / 96 registers: soup
// shade 12.92 -> 12.66 ms per frame, next-event-estimation shade on the
// tunnel 1133 -> 837 ms (its light-tree walk is load-latency bound).
#ifndef SOLRT_SHADE_MINB
#define SOLRT_SHADE_MINB 4
#endif
// 1: in the plain variant the continuing paths of a block's 256 slots take
// their queue positions with one atomic per block (two barriers per step);
// 0, and the next-event-estimation variant: one atomic per warp. Atomics on
// the one queue counter are serialised at its L2 slice (about 1.5 G warp
// atomics per second on GB300 when nothing else runs) and a 64-spp soup
// frame makes 10M of them: per block, the soup's shade stage takes 12.5
// instead of 12.5-16.3 ms per frame (the higher figure on some boxes). The
// NEE variant, bound by the latency of its light-tree walks, loses 9 % to
// the barriers, so it keeps the warp atomics.
#ifndef SOLRT_SHADE_BLOCK_COMPACT
#define SOLRT_SHADE_BLOCK_COMPACT 1
#endif
// 1: with block compaction, a block's continuing paths are written grouped
// by the octant of their new direction (octant-major, then warp and lane),
// so that the extend kernel's warps, which take consecutive queue slots, get
// rays of one or two octants; same images (queue order changes no result).
// Measured: extend -0.4 / -0.5 %, shade +3 / +5 % (soup / tunnel frame), no
// gain: the pixel-ordered queue is about as coherent.
#ifndef SOLRT_SHADE_OCTANT_SORT
#define SOLRT_SHADE_OCTANT_SORT 0
#endif
template <bool kNee>
__global__ void __launch_bounds__(256, SOLRT_SHADE_MINB)
    k_shade(const DevJob* __restrict__ jobs, const DevItem* __restrict__ items, uint32_t nitems, PathQueue qin,
            const float4* __restrict__ hits, const unsigned int* __restrict__ count_in, PathQueue qout,
            unsigned int* __restrict__ count_out, uint32_t capacity, float4* __restrict__ rad, DevStats* stats,
            PathQueue qs, unsigned int* __restrict__ count_s) {
    const unsigned int n = *count_in;
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    constexpr bool kBlock = SOLRT_SHADE_BLOCK_COMPACT && !kNee;
    // kBlock: a block-uniform loop, slots [base, base + 256) per block and
    // step; else a warp-uniform one, 32 slots per warp and step
    __shared__ uint32_t s_cnt[8], s_pre[8], s_base;
    __shared__ uint32_t s_cnt8[SOLRT_SHADE_OCTANT_SORT ? 64 : 1], s_pre8[SOLRT_SHADE_OCTANT_SORT ? 64 : 1];
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t start = kBlock ? blockIdx.x * blockDim.x : ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32u;
    const uint32_t stride = kBlock ? gridDim.x * blockDim.x : ((gridDim.x * blockDim.x) >> 5) * 32u;
    const uint32_t off = kBlock ? threadIdx.x : (uint32_t)lane;
    uint32_t ef = 0;
    for (uint32_t base = start; base < n; base += stride) {
        const uint32_t i = base + off;
        bool alive = false, shadow = false;
        float4 out_o = make_float4(0, 0, 0, 0), out_d = make_float4(0, 0, 0, 0), out_t = make_float4(0, 0, 0, 0);
        float4 s_o = make_float4(0, 0, 0, 0), s_d = make_float4(0, 0, 0, 0), s_c = make_float4(0, 0, 0, 0);
        float4 out_prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        bool out_nee = false;
        uint2 m = make_uint2(0, 0);
        if (i < n) {
            const float4 o = qin.o_tmin[i], d = qin.d_tmax[i], tr = qin.thr_rng[i];
            m = qin.meta[i];
            const uint32_t job = m.y >> kDepthBits;
            const DevJob& J = jobs[job];
            const bool nee = kNee && J.integrator == SOLRT_INTEGRATOR_PATH_NEE && qs.o_tmin != nullptr;
            uint32_t rng = __float_as_uint(tr.w);
            uint32_t depth = m.y & kDepthMask;
            f3 acc{tr.x, tr.y, tr.z};
            f3 n_o{0.0f, 0.0f, 0.0f};
            const float4 prev = nee && depth > 0u ? qin.prev[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (shade_step<kNee>(J, o, d, hits[i], acc, rng, depth, out_o, out_d, ef, &n_o, prev, &out_prev)) {
                alive = true;
                if (nee) {
                    out_nee = true;
                    f3 cn;
                    shadow = nee_sample(J.sc, f3{out_o.x, out_o.y, out_o.z}, n_o, acc, o.w, rng, s_o, s_d, cn);
                    s_c = make_float4(cn.x, cn.y, cn.z, 0.0f);
                }
                out_t = make_float4(acc.x, acc.y, acc.z, __uint_as_float(rng));
                m.y = (job << kDepthBits) | depth;
            } else {
                if (nee) {  // after this path's earlier shadow terms (resolved in bounce order)
                    const float4 r = rad[m.x];
                    rad[m.x] = make_float4(r.x + acc.x, r.y + acc.y, r.z + acc.z, 0.0f);
                } else {
                    rad[m.x] = make_float4(acc.x, acc.y, acc.z, 0.0f);
                }
                if (J.rng_mode == SOLRT_RNG_REF_STREAM) {
                    const DevItem it = items[find_last_le(nitems, m.x, [&](uint32_t t) { return items[t].path_base; })];
                    J.rng_state[it.pix0 + (m.x - it.path_base) / it.k] = rng;
                }
            }
        }
        const uint32_t mask = __ballot_sync(0xffffffffu, alive);
        const uint32_t smask = kNee ? __ballot_sync(0xffffffffu, shadow) : 0u;
        uint32_t same = 0, oct = 0;  // octant sort: the lanes of this warp with this lane's octant
        if constexpr (kBlock && SOLRT_SHADE_OCTANT_SORT) {
            oct = (out_d.x < 0.0f ? 1u : 0u) | (out_d.y < 0.0f ? 2u : 0u) | (out_d.z < 0.0f ? 4u : 0u);
#pragma unroll
            for (uint32_t o = 0; o < 8u; ++o) {
                const uint32_t bo = __ballot_sync(0xffffffffu, alive && oct == o);
                if (lane == 0) s_cnt8[o * 8u + warp] = (uint32_t)__popc(bo);
                if (oct == o) same = bo;
            }
            __syncthreads();
            if (threadIdx.x < 32) {  // exclusive scan of the 64 counts (octant-major), two per lane
                const uint32_t a0 = s_cnt8[2 * lane], a1 = s_cnt8[2 * lane + 1];
                uint32_t x = a0 + a1;
#pragma unroll
                for (int dd = 1; dd < 32; dd <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, x, dd);
                    if (lane >= dd) x += y;
                }
                const uint32_t excl = x - (a0 + a1);
                s_pre8[2 * lane] = excl;
                s_pre8[2 * lane + 1] = excl + a0;
                const uint32_t total = __shfl_sync(0xffffffffu, x, 31);
                if (lane == 0) s_base = total ? atomicAdd(count_out, total) : 0u;
            }
            __syncthreads();
        } else if constexpr (kBlock) {
            if (lane == 0) s_cnt[warp] = (uint32_t)__popc(mask);
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t t = 0;
                for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) {
                    s_pre[w] = t;
                    t += s_cnt[w];
                }
                s_base = t ? atomicAdd(count_out, t) : 0u;
            }
            __syncthreads();
        }
        if (mask) {
            uint32_t pos0 = 0;
            if constexpr (kBlock) {
                pos0 = s_base + s_pre[warp];
            } else {
                const int leader = __ffs(mask) - 1;
                if (lane == leader) pos0 = atomicAdd(count_out, (unsigned int)__popc(mask));
                pos0 = __shfl_sync(0xffffffffu, pos0, leader);
            }
            if (alive) {
                const uint32_t pos = (kBlock && SOLRT_SHADE_OCTANT_SORT)
                                         ? s_base + s_pre8[oct * 8u + warp] + (uint32_t)__popc(same & lane_lt)
                                         : pos0 + __popc(mask & lane_lt);
                if (pos < capacity) {
                    qout.o_tmin[pos] = out_o;
                    qout.d_tmax[pos] = out_d;
                    qout.thr_rng[pos] = out_t;
                    qout.meta[pos] = m;
                    if (out_nee) qout.prev[pos] = out_prev;
                } else {
                    ef |= SOLRT_EFLAG_QUEUE;
                }
            }
        }
        if (smask) {
            const int leader = __ffs(smask) - 1;
            uint32_t pos0 = 0;
            if (lane == leader) pos0 = atomicAdd(count_s, (unsigned int)__popc(smask));
            pos0 = __shfl_sync(0xffffffffu, pos0, leader);
            if (shadow) {
                const uint32_t pos = pos0 + __popc(smask & lane_lt);
                if (pos < capacity) {
                    qs.o_tmin[pos] = s_o;
                    qs.d_tmax[pos] = s_d;
                    qs.thr_rng[pos] = s_c;
                    qs.meta[pos] = m;
                } else {
                    ef |= SOLRT_EFLAG_QUEUE;
                }
            }
        }
    }
    if (ef) atomicOr(&stats->eflags, ef);
}

// Adds the contribution of every shadow ray that reached its light to its
// path's slot (one shadow ray per path and bounce, so no two threads share a
// slot). Counts them into the shadow stats block.
__global__ void __launch_bounds__(256) k_shadow_resolve(PathQueue qs, const float4* __restrict__ hits,
                                                        const unsigned int* __restrict__ count_s,
                                                        float4* __restrict__ rad, DevStats* sstats) {
    const unsigned int n = *count_s;
    uint32_t reached = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (__float_as_uint(hits[i].y) != SOLRT_NO_HIT) continue;
        const float4 c = qs.thr_rng[i];
        const uint32_t slot = qs.meta[i].x;
        const float4 r = rad[slot];
        rad[slot] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.0f);
        ++reached;
    }
    const uint32_t w = __reduce_add_sync(0xffffffffu, reached);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&sstats->unoccluded, (unsigned long long)w);
}

// Per-pixel sums of one pass, samples in order (rgen:86).
__global__ void k_accumulate(const DevJob* __restrict__ jobs, const DevItem* __restrict__ items, uint32_t nitems,
                             uint32_t pixels, const float4* __restrict__ rad) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= pixels) return;
    accumulate_pixel<LdPlain>(jobs, items, nitems, t, rad);
}

// Per job, the sum over its pixels of the variance of the pixel mean summed
// over RGB: with n samples (Kahan mode: the finite ones it kept), sums S_c
// and squared sums Q = sum of r^2 + g^2 + b^2, the unbiased sample variance
// summed over channels is (Q - sum_c S_c^2 / n) / (n - 1), and the mean's is
// that over n. A non-finite pixel makes the job's sum infinite.
__global__ void k_rmse_estimate(const DevJob* __restrict__ jobs, const uint32_t* __restrict__ job_pix,
                                const uint32_t* __restrict__ nsamp, uint32_t njobs, uint32_t pixels,
                                double* __restrict__ sums) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = t < pixels;
    const uint32_t j = in ? find_last_le(njobs, t, [&](uint32_t i) { return job_pix[i]; }) : 0u;
    double v = 0.0;
    if (in) {
        const DevJob& J = jobs[j];
        const uint32_t pix = t - job_pix[j];
        const float4 s = J.accum_mode == SOLRT_ACCUM_KAHAN ? J.ksum[pix] : J.fsum[pix];
        const double n = J.accum_mode == SOLRT_ACCUM_KAHAN ? (double)s.w : (double)nsamp[j];
        const double q = (double)J.sq[pix];
        const double ss = (double)s.x * s.x + (double)s.y * s.y + (double)s.z * s.z;
        if (!isfinite(ss) || !isfinite(q)) v = __longlong_as_double(0x7ff0000000000000LL);
        else if (n >= 2.0) v = fmax(q - ss / n, 0.0) / (n - 1.0) / n;
        else v = __longlong_as_double(0x7ff0000000000000LL);
    }
    // warps whose lanes share one job add once; others lane by lane
    const uint32_t first = __shfl_sync(0xffffffffu, j, 0);
    if (__all_sync(0xffffffffu, !in || j == first)) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(sums + first, v);
    } else if (in) {
        atomicAdd(sums + j, v);
    }
}

// The reference's structure (pathtrace.rgen:39-104): one thread per pixel
// loops over its samples and their bounces, tracing each segment itself.
// Same arithmetic as the wavefront stages, so the same image; used as the
// plain kernel the wavefront and the batched path are measured against.
// Minimum resident 128-thread blocks per SM asked of the register allocator
// for the megakernel. 8 (64 registers, ~100 B of spills) against the
// unconstrained 128 registers: 1099 vs 682 Mrays/s on the 1M-triangle soup
// (6: 914, 10: 1106, 12: 1062, 16: 890): the per-pixel loop is latency-bound
// and needs the warps.
#ifndef SOLRT_MEGA_MINB
#define SOLRT_MEGA_MINB 8
#endif
__device__ __forceinline__ void flush_stats(DevStats* stats, uint32_t segs, uint32_t paths, uint32_t fb,
                                            uint32_t ef) {
    const uint32_t wsegs = __reduce_add_sync(0xffffffffu, segs);
    const uint32_t wpaths = __reduce_add_sync(0xffffffffu, paths);
    const uint32_t wfb = __reduce_add_sync(0xffffffffu, fb);
    const uint32_t wef = __reduce_or_sync(0xffffffffu, ef);
    if ((threadIdx.x & 31) == 0) {
        if (wsegs) atomicAdd(&stats->segments, (unsigned long long)wsegs);
        if (wpaths) atomicAdd(&stats->paths, (unsigned long long)wpaths);
        if (wfb) atomicAdd(&stats->fp64_fallbacks, (unsigned long long)wfb);
        if (wef) atomicOr(&stats->eflags, wef);
    }
}

// All samples of pixel `pix` of job J, each path traced and shaded to its
// end by this thread; the pixel's sums are written once (the body of
// k_megakernel's per-pixel loop, for the persistent batch launch).
template <int KIND>
__device__ __forceinline__ void mega_pixel(const DevJob& J, uint32_t pix, uint32_t& segs, TraceCounters& cnt,
                                           uint32_t& ef) {
    const TravScene ts = trav_scene(J.sc);
    f3 s{0.0f, 0.0f, 0.0f}, ks{0.0f, 0.0f, 0.0f}, kc{0.0f, 0.0f, 0.0f};
    float kn = 0.0f;
    if (J.accum_mode == SOLRT_ACCUM_KAHAN) {
        const float4 s4 = J.ksum[pix], c4 = J.kcomp[pix];
        ks = f3{s4.x, s4.y, s4.z};
        kc = f3{c4.x, c4.y, c4.z};
        kn = s4.w;
    }
    uint32_t rng = 0;
    for (uint32_t smp = 0; smp < J.spp; ++smp) {
        rng = sample_seed(J, pix, smp, rng);
        float4 o, d;
        camera_ray(J, pix, rng, o, d);
        f3 acc{1.0f, 1.0f, 1.0f};
        uint32_t depth = 0;
        for (;;) {
            HitRec h;
            if (KIND == SOLRT_BVH8_Q8) trace_bvh8<false>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
            else if (KIND == SOLRT_BVH8_F32) trace_bvh8<false, true>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
            else if (KIND == SOLRT_BVH4_Q8) trace_bvh4_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
            else if (KIND == SOLRT_BVH2_Q16) trace_bvh2_ray<true>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
            else if (KIND == SOLRT_BVH2_TWO_LEVEL) trace_bvh2_2l_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
            else trace_bvh2_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
            ++segs;
            float4 on, dn;
            if (!shade_step(J, o, d, make_float4(h.t, __uint_as_float(h.prim), h.u, h.v), acc, rng, depth, on, dn,
                            ef))
                break;
            o = on;
            d = dn;
        }
        const float4 c = make_float4(acc.x, acc.y, acc.z, 0.0f);
        if (J.accum_mode == SOLRT_ACCUM_KAHAN) add_sample_kahan(ks, kc, kn, c);
        else add_sample(s, c);
    }
    if (J.accum_mode == SOLRT_ACCUM_KAHAN) {
        J.ksum[pix] = make_float4(ks.x, ks.y, ks.z, kn);
        J.kcomp[pix] = make_float4(kc.x, kc.y, kc.z, 0.0f);
    } else {
        J.fsum[pix] = make_float4(s.x, s.y, s.z, 0.0f);
    }
}

template <int KIND>
__global__ void __launch_bounds__(128, SOLRT_MEGA_MINB) k_megakernel(const DevJob* __restrict__ job, DevStats* stats) {
    const DevJob& J = *job;
    const uint32_t npix = J.width * J.height;
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t segs = 0, fb_ef[2] = {0, 0};
    TraceCounters cnt{0, 0, 0};
    if (pix < npix) {
        const TravScene ts = trav_scene(J.sc);
        f3 s{0.0f, 0.0f, 0.0f}, ks{0.0f, 0.0f, 0.0f}, kc{0.0f, 0.0f, 0.0f};
        float kn = 0.0f;
        if (J.accum_mode == SOLRT_ACCUM_KAHAN) {
            const float4 s4 = J.ksum[pix], c4 = J.kcomp[pix];
            ks = f3{s4.x, s4.y, s4.z};
            kc = f3{c4.x, c4.y, c4.z};
            kn = s4.w;
        }
        uint32_t rng = 0;
        for (uint32_t smp = 0; smp < J.spp; ++smp) {
            rng = sample_seed(J, pix, smp, rng);
            float4 o, d;
            camera_ray(J, pix, rng, o, d);
            f3 acc{1.0f, 1.0f, 1.0f};
            uint32_t depth = 0;
            for (;;) {
                HitRec h;
                if (KIND == SOLRT_BVH8_Q8) trace_bvh8<false>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, fb_ef[1]);
                else if (KIND == SOLRT_BVH8_F32) trace_bvh8<false, true>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, fb_ef[1]);
                else if (KIND == SOLRT_BVH4_Q8) trace_bvh4_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, fb_ef[1]);
                else if (KIND == SOLRT_BVH2_Q16) trace_bvh2_ray<true>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, fb_ef[1]);
                else if (KIND == SOLRT_BVH2_TWO_LEVEL) trace_bvh2_2l_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, fb_ef[1]);
                else trace_bvh2_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, fb_ef[1]);
                ++segs;
                float4 on, dn;
                if (!shade_step(J, o, d, make_float4(h.t, __uint_as_float(h.prim), h.u, h.v), acc, rng, depth, on,
                                dn, fb_ef[1]))
                    break;
                o = on;
                d = dn;
            }
            const float4 c = make_float4(acc.x, acc.y, acc.z, 0.0f);
            if (J.accum_mode == SOLRT_ACCUM_KAHAN) add_sample_kahan(ks, kc, kn, c);
            else add_sample(s, c);
        }
        if (J.accum_mode == SOLRT_ACCUM_KAHAN) {
            J.ksum[pix] = make_float4(ks.x, ks.y, ks.z, kn);
            J.kcomp[pix] = make_float4(kc.x, kc.y, kc.z, 0.0f);
        } else {
            J.fsum[pix] = make_float4(s.x, s.y, s.z, 0.0f);
        }
    }
    const uint32_t wsegs = __reduce_add_sync(0xffffffffu, segs);
    const uint32_t wfb = __reduce_add_sync(0xffffffffu, cnt.fallbacks);
    const uint32_t wef = __reduce_or_sync(0xffffffffu, fb_ef[1]);
    const uint32_t wpaths = __reduce_add_sync(0xffffffffu, pix < npix ? J.spp : 0u);
    if ((threadIdx.x & 31) == 0) {
        if (wsegs) atomicAdd(&stats->segments, (unsigned long long)wsegs);
        if (wpaths) atomicAdd(&stats->paths, (unsigned long long)wpaths);
        if (wfb) atomicAdd(&stats->fp64_fallbacks, (unsigned long long)wfb);
        if (wef) atomicOr(&stats->eflags, wef);
    }
}

// The persistent multi-scene launch: one grid of (SMs x resident blocks)
// whose warps take 32 consecutive pixels of the batch's pixel space (all
// jobs, job after job) from an atomic work counter until it passes the end;
// each lane renders all samples of its pixel (mega_pixel). No thread waits
// on another, so nothing needs a bounded wait.
template <int KIND>
__global__ void __launch_bounds__(128, SOLRT_MEGA_MINB)
    k_megakernel_batch(const DevJob* __restrict__ jobs, const uint32_t* __restrict__ job_pix, uint32_t njobs,
                       uint32_t total_pix, unsigned int* __restrict__ work, DevStats* stats) {
    const int lane = threadIdx.x & 31;
    uint32_t segs = 0, paths = 0, ef = 0;
    TraceCounters cnt{0, 0, 0};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total_pix) break;
        const uint32_t t = base + (uint32_t)lane;
        if (t < total_pix) {
            const uint32_t j = find_last_le(njobs, t, [&](uint32_t i) { return job_pix[i]; });
            mega_pixel<KIND>(jobs[j], t - job_pix[j], segs, cnt, ef);
            paths += jobs[j].spp;
        }
        __syncwarp();
    }
    flush_stats(stats, segs, paths, cnt.fallbacks, ef);
}

// ---------------------------------------------------------------------------
// Next-event estimation in the per-pixel structure (KERNEL_MEGA renders and
// SOLRT_BATCH_PERSISTENT batches with SOLRT_INTEGRATOR_PATH_NEE jobs): the
// same estimator as the wavefront's shadow queue, one path at a time.
// ---------------------------------------------------------------------------

// Closest hit of one ray with the kind's per-ray loop.
template <int KIND>
SOLRT_D void trace_one(const TravScene& ts, const float4& o, const float4& d, HitRec& h, TraceCounters& cnt,
                       uint32_t& ef) {
    if (KIND == SOLRT_BVH8_Q8) trace_bvh8<false>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
    else if (KIND == SOLRT_BVH8_F32) trace_bvh8<false, true>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
    else if (KIND == SOLRT_BVH4_Q8) trace_bvh4_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
    else if (KIND == SOLRT_BVH2_Q16) trace_bvh2_ray<true>(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
    else if (KIND == SOLRT_BVH2_TWO_LEVEL) trace_bvh2_2l_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
    else trace_bvh2_ray(ts, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, h, cnt, ef);
}

// Per-thread counts of the per-pixel NEE kernels.
struct MegaCounts {
    uint32_t segs = 0, paths = 0, shadow = 0, unoccluded = 0, ef = 0;
    TraceCounters cnt{0, 0, 0}, scnt{0, 0, 0};  // path / shadow-ray traversals
};

// One path to its end: at each continuing vertex of a NEE job the shadow
// ray of k_shade<true> (same draws, same order) is traced at once; closest-
// hit traversal gives the same occlusion answer as the wavefront's any-hit
// one. The sample is (0 + unoccluded shadow terms in bounce order) + the end
// term, as the wavefront's radiance slot sums them.
template <int KIND>
SOLRT_D f3 mega_path_nee(const DevJob& J, const TravScene& ts, float4 o, float4 d, uint32_t& rng, MegaCounts& mc) {
    const bool nee = J.integrator == SOLRT_INTEGRATOR_PATH_NEE;
    f3 acc{1.0f, 1.0f, 1.0f}, rsum{0.0f, 0.0f, 0.0f};
    uint32_t depth = 0;
    float4 prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (;;) {
        HitRec h;
        trace_one<KIND>(ts, o, d, h, mc.cnt, mc.ef);
        ++mc.segs;
        float4 on, dn, prev_out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        f3 n_o{0.0f, 0.0f, 0.0f};
        const float4 pv = nee && depth > 0u ? prev : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (!shade_step<true>(J, o, d, make_float4(h.t, __uint_as_float(h.prim), h.u, h.v), acc, rng, depth, on, dn,
                              mc.ef, &n_o, pv, &prev_out))
            break;
        if (nee) {
            float4 so, sd;
            f3 cn;
            if (nee_sample(J.sc, f3{on.x, on.y, on.z}, n_o, acc, o.w, rng, so, sd, cn)) {
                HitRec sh;
                trace_one<KIND>(ts, so, sd, sh, mc.scnt, mc.ef);
                ++mc.shadow;
                if (sh.prim == SOLRT_NO_HIT) {
                    rsum = rsum + cn;
                    ++mc.unoccluded;
                }
            }
            prev = prev_out;
        }
        o = on;
        d = dn;
    }
    return nee ? rsum + acc : acc;
}

// All samples of pixel `pix` of job J with mega_path_nee; the pixel's sums
// are written once.
template <int KIND>
SOLRT_D void mega_pixel_nee(const DevJob& J, uint32_t pix, MegaCounts& mc) {
    const TravScene ts = trav_scene(J.sc);
    f3 s{0.0f, 0.0f, 0.0f}, ks{0.0f, 0.0f, 0.0f}, kc{0.0f, 0.0f, 0.0f};
    float kn = 0.0f;
    if (J.accum_mode == SOLRT_ACCUM_KAHAN) {
        const float4 s4 = J.ksum[pix], c4 = J.kcomp[pix];
        ks = f3{s4.x, s4.y, s4.z};
        kc = f3{c4.x, c4.y, c4.z};
        kn = s4.w;
    }
    uint32_t rng = 0;
    for (uint32_t smp = 0; smp < J.spp; ++smp) {
        rng = sample_seed(J, pix, smp, rng);
        float4 o, d;
        camera_ray(J, pix, rng, o, d);
        const f3 v = mega_path_nee<KIND>(J, ts, o, d, rng, mc);
        const float4 c = make_float4(v.x, v.y, v.z, 0.0f);
        if (J.accum_mode == SOLRT_ACCUM_KAHAN) add_sample_kahan(ks, kc, kn, c);
        else add_sample(s, c);
    }
    mc.paths += J.spp;
    if (J.accum_mode == SOLRT_ACCUM_KAHAN) {
        J.ksum[pix] = make_float4(ks.x, ks.y, ks.z, kn);
        J.kcomp[pix] = make_float4(kc.x, kc.y, kc.z, 0.0f);
    } else {
        J.fsum[pix] = make_float4(s.x, s.y, s.z, 0.0f);
    }
}

// Path segments into stats[0], shadow rays into stats[1] (the split of the
// wavefront's launches).
SOLRT_D void flush_mega_counts(DevStats* stats, const MegaCounts& mc) {
    flush_stats(stats, mc.segs, mc.paths, mc.cnt.fallbacks, mc.ef);
    const uint32_t ws = __reduce_add_sync(0xffffffffu, mc.shadow);
    const uint32_t wu = __reduce_add_sync(0xffffffffu, mc.unoccluded);
    const uint32_t wf = __reduce_add_sync(0xffffffffu, mc.scnt.fallbacks);
    if ((threadIdx.x & 31) == 0) {
        if (ws) atomicAdd(&stats[1].segments, (unsigned long long)ws);
        if (wu) atomicAdd(&stats[1].unoccluded, (unsigned long long)wu);
        if (wf) atomicAdd(&stats[1].fp64_fallbacks, (unsigned long long)wf);
    }
}

// k_megakernel for a NEE job: one thread per pixel.
template <int KIND>
__global__ void __launch_bounds__(128, SOLRT_MEGA_MINB) k_megakernel_nee(const DevJob* __restrict__ job,
                                                                        DevStats* stats) {
    const DevJob& J = *job;
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    MegaCounts mc;
    if (pix < J.width * J.height) mega_pixel_nee<KIND>(J, pix, mc);
    flush_mega_counts(stats, mc);
}

// k_megakernel_batch for batches with NEE jobs (every job of the batch runs
// through mega_pixel_nee; a job without NEE gets the plain estimator's
// image there too).
template <int KIND>
__global__ void __launch_bounds__(128, SOLRT_MEGA_MINB)
    k_megakernel_batch_nee(const DevJob* __restrict__ jobs, const uint32_t* __restrict__ job_pix, uint32_t njobs,
                           uint32_t total_pix, unsigned int* __restrict__ work, DevStats* stats) {
    const int lane = threadIdx.x & 31;
    MegaCounts mc;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total_pix) break;
        const uint32_t t = base + (uint32_t)lane;
        if (t < total_pix) {
            const uint32_t j = find_last_le(njobs, t, [&](uint32_t i) { return job_pix[i]; });
            mega_pixel_nee<KIND>(jobs[j], t - job_pix[j], mc);
        }
        __syncwarp();
    }
    flush_mega_counts(stats, mc);
}

// Zeroes the per-frame sample sums of running-mix jobs.
__global__ void k_begin(const DevJob* __restrict__ jobs, const uint32_t* __restrict__ job_pix, uint32_t njobs,
                        uint32_t pixels) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= pixels) return;
    begin_pixel(jobs, job_pix, njobs, t);
}

// ---------------------------------------------------------------------------
// Sibling integrators over the same traversal (one thread per pixel, the
// structure of their ray-generation shaders).
// ---------------------------------------------------------------------------

// Primary direction of debug.rgen:20-27 / ao.rgen:56-61 for pixel position
// (px, py): origin and direction through the inverse matrices.
__device__ __forceinline__ void pixel_ray(const DevJob& J, float px, float py, float org[4], float dir[4]) {
    const float ux = px / __uint2float_rn(J.width), uy = py / __uint2float_rn(J.height);
    const float dx = ux * 2.0f - 1.0f, dy = uy * 2.0f - 1.0f;
    float tgt[4];
    mat4_mul(J.vinv, 0.0f, 0.0f, 0.0f, 1.0f, org);
    mat4_mul(J.pinv, dx, dy, 1.0f, 1.0f, tgt);
    const f3 tn = normalize(f3{tgt[0], tgt[1], tgt[2]});
    mat4_mul(J.vinv, tn.x, tn.y, tn.z, 0.0f, dir);
}

template <int KIND>
__device__ __forceinline__ void trace_one(const TravScene& ts, float ox, float oy, float oz, float dx, float dy,
                                          float dz, float tmin, float tmax, HitRec& h, TraceCounters& cnt,
                                          uint32_t& ef) {
    if (KIND == SOLRT_BVH8_Q8) trace_bvh8<false>(ts, ox, oy, oz, dx, dy, dz, tmin, tmax, h, cnt, ef);
    else if (KIND == SOLRT_BVH8_F32) trace_bvh8<false, true>(ts, ox, oy, oz, dx, dy, dz, tmin, tmax, h, cnt, ef);
    else if (KIND == SOLRT_BVH4_Q8) trace_bvh4_ray(ts, ox, oy, oz, dx, dy, dz, tmin, tmax, h, cnt, ef);
    else if (KIND == SOLRT_BVH2_Q16) trace_bvh2_ray<true>(ts, ox, oy, oz, dx, dy, dz, tmin, tmax, h, cnt, ef);
    else if (KIND == SOLRT_BVH2_TWO_LEVEL) trace_bvh2_2l_ray(ts, ox, oy, oz, dx, dy, dz, tmin, tmax, h, cnt, ef);
    else trace_bvh2_ray(ts, ox, oy, oz, dx, dy, dz, tmin, tmax, h, cnt, ef);
}

// debug.rgen:18-36, debug.rchit:9-13, debug.rmiss: barycentrics of the
// primary hit through the pixel centre, else the ray direction; stored
// without accumulation (imageStore of vec4(hitValue, 0)).
template <int KIND>
__global__ void __launch_bounds__(128) k_debug(const DevJob* __restrict__ job, DevStats* stats) {
    const DevJob& J = *job;
    const uint32_t npix = J.width * J.height;
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t segs = 0, ef = 0;
    TraceCounters cnt{0, 0, 0};
    if (pix < npix) {
        const TravScene ts = trav_scene(J.sc);
        const uint32_t x = pix % J.width, y = pix / J.width;
        float org[4], dir[4];
        pixel_ray(J, __uint2float_rn(x) + 0.5f, __uint2float_rn(y) + 0.5f, org, dir);
        HitRec h;
        trace_one<KIND>(ts, org[0], org[1], org[2], dir[0], dir[1], dir[2], 0.001f, 1000.0f, h, cnt, ef);
        ++segs;
        float4 v = make_float4(dir[0], dir[1], dir[2], 0.0f);
        if (h.prim != SOLRT_NO_HIT) v = make_float4((1.0f - h.u) - h.v, h.u, h.v, 0.0f);
        J.accum[pix] = v;
        J.rgba8[pix] = make_uchar4(to_unorm8(v.x), to_unorm8(v.y), to_unorm8(v.z), 0);
    }
    flush_stats(stats, segs, pix < npix ? 1u : 0u, cnt.fallbacks, ef);
}

// ao.rgen:37-83, ao.rchit:53-88, ao.rmiss: `spp` jittered samples; each
// follows cosine-weighted rays (directions from the blue-noise texture)
// until a miss or max_bounces + 1 hits, counting every hit after the first.
// Minimum resident 128-thread AO blocks per SM asked of the register
// allocator: 8 (64 registers) against the unconstrained 96: 1083 vs 801
// Mrays/s for the AO pipeline on the 1M-triangle soup at 1920x1080 (same
// image), latency-bound like the megakernel.
#ifndef SOLRT_AO_MINB
#define SOLRT_AO_MINB 8
#endif
template <int KIND>
__global__ void __launch_bounds__(128, SOLRT_AO_MINB) k_ao(const DevJob* __restrict__ job, DevStats* stats) {
    const DevJob& J = *job;
    const uint32_t npix = J.width * J.height;
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t segs = 0, ef = 0;
    TraceCounters cnt{0, 0, 0};
    if (pix < npix) {
        const DevScene& sc = J.sc;
        const TravScene ts = trav_scene(sc);
        const uint32_t x = pix % J.width, y = pix / J.width;
        uint32_t rng = tea(pix, J.frame);                                     // ao.rgen:49
        const float max_samples = __uint2float_rn(J.max_bounces);
        const float tw = __uint2float_rn(J.noise_w), th = __uint2float_rn(J.noise_h);
        f3 ao{0.0f, 0.0f, 0.0f};
        for (uint32_t i = 0; i < J.spp; ++i) {
            const float j0 = next_rand(rng);                                  // nextRand2 (ao.rgen:53)
            const float j1 = next_rand(rng);
            float org[4], dir[4];
            pixel_ray(J, __uint2float_rn(x) + j0, __uint2float_rn(y) + j1, org, dir);
            f3 o{org[0], org[1], org[2]}, d{dir[0], dir[1], dir[2]};
            float tmin = glsl_max(1.0f, length(o)) * 1e-3f, tmax = 10000.0f;  // preparePayload
            float hv = 0.0f;
            uint32_t depth = 0;
            for (;;) {
                HitRec h;
                trace_one<KIND>(ts, o.x, o.y, o.z, d.x, d.y, d.z, tmin, tmax, h, cnt, ef);
                ++segs;
                if (h.prim == SOLRT_NO_HIT) break;                            // ao.rmiss
                if (h.prim >= sc.tri_count) {
                    ef |= SOLRT_EFLAG_INDEX;
                    break;
                }
                const uint4 ti = __ldg(sc.tri_idx + h.prim);
                const float b1 = h.u, b2 = h.v;
                const float b0 = (1.0f - b1) - b2;
                f3 normal, pos;
                hit_frame(sc, ti, b0, b1, b2, normal, pos);                   // ao.rchit:66-75
                const f3 no = pos + 0.00001f * d;                             // ao.rchit:78
                // getBlueRand2(depth + depth * sampleId) (ao.rchit:43-49)
                const uint32_t bi = depth + depth * i;
                const float r0 = next_rand(rng);
                const float r1 = next_rand(rng);
                float cx = __uint2float_rn(x) + r0 * tw, cy = __uint2float_rn(y) + r1 * th;
                cx = cx - tw * floorf(cx / tw);                               // GLSL mod
                cy = cy - th * floorf(cy / th);
                const int ix = min(max((int)cx, 0), (int)J.noise_w - 1);
                const int iy = min(max((int)cy, 0), (int)J.noise_h - 1);
                const uchar4 t = __ldg(J.noise + (size_t)iy * J.noise_w + ix);
                const float blue[4] = {__uint2float_rn(t.x) / 255.0f, __uint2float_rn(t.y) / 255.0f,
                                       __uint2float_rn(t.z) / 255.0f, __uint2float_rn(t.w) / 255.0f};
                const f3 hit_n = normal * glsl_sign(dot(-d, normal));
                d = sample_cosine(hit_n, blue[bi % 4], blue[(bi + 1) % 4]);
                o = no;
                tmin = 0.001f;
                tmax = 10.0f;
                if (depth > 0) hv = hv + 1.0f;
                ++depth;
                if (depth > J.max_bounces) break;                             // ao.rgen:75
            }
            ao = ao + (1.0f / max_samples) * f3{hv, hv, hv};                  // ao.rgen:77
        }
        const float n = __uint2float_rn(J.spp);
        f3 color{1.0f - ao.x / n, 1.0f - ao.y / n, 1.0f - ao.z / n};
        const float a = 1.0f / __uint2float_rn(J.frame - J.start + 1u);      // ao.rgen:79-82
        const float4 old = J.accum[pix];
        color = mix(f3{old.x, old.y, old.z}, color, a);
        J.accum[pix] = make_float4(color.x, color.y, color.z, 1.0f);
        J.rgba8[pix] = make_uchar4(to_unorm8(color.x), to_unorm8(color.y), to_unorm8(color.z), 255);
    }
    flush_stats(stats, segs, pix < npix ? J.spp : 0u, cnt.fallbacks, ef);
}

// rgen:88-103 (REF_MIX) or the Kahan mean, for every pixel of every job.
__global__ void k_finalize(const DevJob* __restrict__ jobs, const uint32_t* __restrict__ job_pix, uint32_t njobs,
                           uint32_t pixels) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= pixels) return;
    finalize_pixel<LdPlain>(jobs, job_pix, njobs, t);
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

solrt_status check_params(const Context& ctx, const Scene& sc, const Image& img, const solrt_render_params& p) {
    if (sc.ctx != &ctx || img.ctx != &ctx) { set_error("objects belong to another context"); return SOLRT_ERR_INVALID; }
    if (p.width != img.width || p.height != img.height) { set_error("params size differs from the image"); return SOLRT_ERR_INVALID; }
    if (p.spp < 1) { set_error("spp must be >= 1"); return SOLRT_ERR_INVALID; }
    if (p.max_bounces > SOLRT_MAX_BOUNCES) { set_error("max_bounces > 1024"); return SOLRT_ERR_INVALID; }
    if (p.accum_mode != img.accum_mode) { set_error("accum_mode differs from the image"); return SOLRT_ERR_INVALID; }
    if (p.miss_mode > SOLRT_MISS_GRADIENT || p.material_mode > SOLRT_MATERIAL_LAMBERT || p.rng_mode > SOLRT_RNG_PER_SAMPLE) {
        set_error("bad miss, material or rng mode");
        return SOLRT_ERR_INVALID;
    }
    if (p.accum_mode != SOLRT_ACCUM_KAHAN && p.frame + 1u - p.accum_start_frame == 0u) {
        set_error("frame + 1 - accum_start_frame is zero");
        return SOLRT_ERR_INVALID;
    }
    if (!(p.tmax >= 0.0f)) { set_error("tmax must be >= 0"); return SOLRT_ERR_INVALID; }
    if (p.kernel > SOLRT_KERNEL_MEGA) { set_error("unknown kernel"); return SOLRT_ERR_INVALID; }
    if (p.integrator > SOLRT_INTEGRATOR_PATH_NEE) { set_error("unknown integrator"); return SOLRT_ERR_INVALID; }
    if (p.integrator == SOLRT_INTEGRATOR_PATH_NEE && p.material_mode != SOLRT_MATERIAL_LAMBERT) {
        set_error("next-event estimation needs material_mode SOLRT_MATERIAL_LAMBERT");
        return SOLRT_ERR_INVALID;
    }
    if (p.integrator == SOLRT_INTEGRATOR_AO) {
        if (!ctx.blue_noise.ptr) { set_error("the AO integrator needs solrt_context_set_blue_noise"); return SOLRT_ERR_INVALID; }
        if (p.max_bounces < 1) { set_error("the AO integrator needs max_bounces >= 1"); return SOLRT_ERR_INVALID; }
        if (p.frame + 1u - p.accum_start_frame == 0u) { set_error("frame + 1 - accum_start_frame is zero"); return SOLRT_ERR_INVALID; }
    }
    return SOLRT_OK;
}

DevJob make_job(const Scene& sc, const Image& img, const solrt_camera& cam, const solrt_render_params& p) {
    DevJob J{};
    J.sc = sc.view();
    std::copy(cam.view_inverse, cam.view_inverse + 16, J.vinv);
    std::copy(cam.projection_inverse, cam.projection_inverse + 16, J.pinv);
    J.width = p.width;
    J.height = p.height;
    J.spp = p.spp;
    J.frame = p.frame;
    J.start = p.accum_start_frame;
    J.seed = p.seed;
    J.job_id = p.job_id;
    J.rng_mode = p.rng_mode;
    J.miss_mode = p.miss_mode;
    J.material_mode = p.material_mode;
    J.max_bounces = p.max_bounces;
    J.accum_mode = p.accum_mode;
    J.integrator = p.integrator;
    J.tmax = p.tmax > 0.0f ? p.tmax : 10000.0f;
    J.accum = img.accum.as<float4>();
    J.rgba8 = img.rgba8.as<uchar4>();
    J.fsum = img.frame_sum.as<float4>();
    J.ksum = img.ksum.as<float4>();
    J.kcomp = img.kcomp.as<float4>();
    J.rng_state = img.rng_state.as<uint32_t>();
    return J;
}

// One pass: generate, (extend, shade) x bounces, accumulate.
solrt_status issue_pass(Context& ctx, uint32_t kind, const DevJob* dj, const DevItem* items, const PassPlan& pp,
                        bool record_timing) {
    cudaStream_t st = ctx.stream;
    DevStats* stats = ctx.stats.as<DevStats>();
    PassCtl* ctl = ctx.ctl.as<PassCtl>();
    const size_t ctl_bytes = sizeof(unsigned int) * (pp.bounces + 1);
    SOLRT_CUDA(cudaMemsetAsync(ctl->count, 0, ctl_bytes, st));
    SOLRT_CUDA(cudaMemsetAsync(ctl->work, 0, ctl_bytes, st));
    if (pp.nee) {
        if (!ctx.q_o[2].ptr) { set_error("shadow queue not allocated"); return SOLRT_ERR_INVALID; }
        SOLRT_CUDA(cudaMemsetAsync(ctl->scount, 0, ctl_bytes, st));
        SOLRT_CUDA(cudaMemsetAsync(ctl->swork, 0, ctl_bytes, st));
    }
    const int tg = record_timing ? ctx.timing_begin(2) : -1;
    k_generate<<<cdiv(pp.paths, 256), 256, 0, st>>>(dj, items, pp.item_count, pp.paths, ctx.queue(0), ctl->count,
                                                    stats, ctx.rad.as<float4>());
    ctx.timing_end(tg);
    ++ctx.launches;
    const int shade_grid = ctx.sm_count * 8;
    for (uint32_t bnc = 0; bnc < pp.bounces; ++bnc) {
        const PathQueue qin = ctx.queue(bnc & 1), qout = ctx.queue((bnc + 1) & 1);
        const int te = record_timing ? ctx.timing_begin(0) : -1;
        SOLRT_TRY(launch_extend(ctx, kind, dj, qin, ctx.hits.as<float4>(), ctl->count + bnc, ctl->work + bnc));
        ctx.timing_end(te);
        const int ts = record_timing ? ctx.timing_begin(1) : -1;
        if (pp.nee)
            k_shade<true><<<shade_grid, 256, 0, st>>>(dj, items, pp.item_count, qin, ctx.hits.as<float4>(),
                                                      ctl->count + bnc, qout, ctl->count + bnc + 1, ctx.capacity,
                                                      ctx.rad.as<float4>(), stats, ctx.queue(2), ctl->scount + bnc);
        else
            k_shade<false><<<shade_grid, 256, 0, st>>>(dj, items, pp.item_count, qin, ctx.hits.as<float4>(),
                                                       ctl->count + bnc, qout, ctl->count + bnc + 1, ctx.capacity,
                                                       ctx.rad.as<float4>(), stats, PathQueue{}, ctl->scount + bnc);
        ctx.timing_end(ts);
        ++ctx.launches;
        if (pp.nee && bnc + 1 < pp.bounces) {  // shadow rays of this bounce (none at the last: depth > max)
            const int tx = record_timing ? ctx.timing_begin(0) : -1;
            SOLRT_TRY(launch_extend(ctx, kind, dj, ctx.queue(2), ctx.hits.as<float4>(), ctl->scount + bnc,
                                    ctl->swork + bnc, stats + 1, true));
            ctx.timing_end(tx);
            const int tr = record_timing ? ctx.timing_begin(1) : -1;
            k_shadow_resolve<<<shade_grid, 256, 0, st>>>(ctx.queue(2), ctx.hits.as<float4>(), ctl->scount + bnc,
                                                         ctx.rad.as<float4>(), stats + 1);
            ctx.timing_end(tr);
            ++ctx.launches;
        }
    }
    const int ta = record_timing ? ctx.timing_begin(3) : -1;
    k_accumulate<<<cdiv(pp.pixels, 256), 256, 0, st>>>(dj, items, pp.item_count, pp.pixels, ctx.rad.as<float4>());
    ctx.timing_end(ta);
    ++ctx.launches;
    return SOLRT_OK;
}

// Issues the batch's launches on the context stream.
// The persistent launch of a SOLRT_BATCH_PERSISTENT batch: a grid of (SMs x
// resident blocks) of k_megakernel_batch over the batch's pixels.
template <int KIND>
void launch_mega_batch(Context& ctx, const DevJob* dj, const uint32_t* jp, uint32_t njobs, uint32_t total_pix,
                       unsigned int* work, bool nee) {
    auto kern = nee ? k_megakernel_batch_nee<KIND> : k_megakernel_batch<KIND>;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0);
    const uint32_t grid = std::min<uint32_t>((uint32_t)ctx.sm_count * (uint32_t)std::max(per_sm, 1),
                                             cdiv(total_pix, 128u));
    kern<<<grid, 128, 0, ctx.stream>>>(dj, jp, njobs, total_pix, work, ctx.stats.as<DevStats>());
}

solrt_status batch_issue(Batch& b, bool record_timing) {
    Context& ctx = *b.ctx;
    cudaStream_t st = ctx.stream;
    const DevJob* dj = b.d_jobs.as<DevJob>();
    const DevItem* di = b.d_items.as<DevItem>();
    const uint32_t* jp = b.d_job_pix.as<uint32_t>();
    const uint32_t njobs = (uint32_t)b.jobs.size();
    const uint32_t total_pix = b.job_pix_base[njobs];
    if (b.flags & SOLRT_BATCH_PERSISTENT) {
        unsigned int* work = ctx.trace_work.as<unsigned int>();
        SOLRT_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned int), st));
        const int tm = record_timing ? ctx.timing_begin(0) : -1;  // traversal and shading in one launch
        bool nee = false;
        for (const DevJob& J : b.jobs) nee = nee || J.integrator == SOLRT_INTEGRATOR_PATH_NEE;
        if (b.kind == SOLRT_BVH8_Q8) launch_mega_batch<SOLRT_BVH8_Q8>(ctx, dj, jp, njobs, total_pix, work, nee);
        else if (b.kind == SOLRT_BVH4_Q8) launch_mega_batch<SOLRT_BVH4_Q8>(ctx, dj, jp, njobs, total_pix, work, nee);
        else if (b.kind == SOLRT_BVH8_F32) launch_mega_batch<SOLRT_BVH8_F32>(ctx, dj, jp, njobs, total_pix, work, nee);
        else if (b.kind == SOLRT_BVH2_Q16) launch_mega_batch<SOLRT_BVH2_Q16>(ctx, dj, jp, njobs, total_pix, work, nee);
        else if (b.kind == SOLRT_BVH2_TWO_LEVEL)
            launch_mega_batch<SOLRT_BVH2_TWO_LEVEL>(ctx, dj, jp, njobs, total_pix, work, nee);
        else launch_mega_batch<SOLRT_BVH2>(ctx, dj, jp, njobs, total_pix, work, nee);
        ctx.timing_end(tm);
        const int tf = record_timing ? ctx.timing_begin(3) : -1;
        k_finalize<<<cdiv(total_pix, 256), 256, 0, st>>>(dj, jp, njobs, total_pix);
        ctx.timing_end(tf);
        ctx.launches += 2;
        SOLRT_CUDA(cudaGetLastError());
        return SOLRT_OK;
    }
    if (b.flags & SOLRT_BATCH_COOPERATIVE) {
        const int tm = record_timing ? ctx.timing_begin(0) : -1;  // every stage in one launch
        bool nee = false;
        for (const PassPlan& pp : b.passes) nee = nee || pp.nee;
        SOLRT_TRY(launch_batch_coop(ctx, b.kind, dj, di, b.d_passes.as<PassPlan>(), (uint32_t)b.passes.size(),
                                    b.coop_stride, jp, njobs, total_pix, b.d_coop.ptr, nee));
        ctx.timing_end(tm);
        SOLRT_CUDA(cudaGetLastError());
        return SOLRT_OK;
    }
    const int tb = record_timing ? ctx.timing_begin(3) : -1;
    k_begin<<<cdiv(total_pix, 256), 256, 0, st>>>(dj, jp, njobs, total_pix);
    ctx.timing_end(tb);
    ++ctx.launches;
    for (const PassPlan& pp : b.passes) SOLRT_TRY(issue_pass(ctx, b.kind, dj, di + pp.item_begin, pp, record_timing));
    const int tf = record_timing ? ctx.timing_begin(3) : -1;
    k_finalize<<<cdiv(total_pix, 256), 256, 0, st>>>(dj, jp, njobs, total_pix);
    ctx.timing_end(tf);
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}

}  // namespace

// Plans passes for `jobs` and uploads the job table and the work items.
solrt_status batch_plan(Context& ctx, const solrt_job* jobs, uint32_t n, uint32_t flags, Batch& b) {
    if (n == 0 || !jobs) { set_error("empty batch"); return SOLRT_ERR_INVALID; }
    if (n > (1u << (32 - kDepthBits))) { set_error("too many jobs in one batch"); return SOLRT_ERR_CAPACITY; }
    b.ctx = &ctx;
    b.flags = flags;
    if (jobs != b.src.data()) b.src.assign(jobs, jobs + n);
    b.total_paths = 0;
    b.jobs.clear();
    b.items.clear();
    b.passes.clear();
    b.job_pix_base.assign(1, 0u);
    const uint32_t cap = ctx.tune.pass_paths ? std::min(ctx.tune.pass_paths, ctx.capacity) : ctx.capacity;
    for (uint32_t j = 0; j < n; ++j) {
        const solrt_job& jb = jobs[j];
        if (!jb.scene || !jb.image) { set_error("job %u: null scene or image", j); return SOLRT_ERR_INVALID; }
        const Scene& sc = *static_cast<const Scene*>(reinterpret_cast<const void*>(jb.scene));
        const Image& img = *static_cast<const Image*>(reinterpret_cast<const void*>(jb.image));
        SOLRT_TRY(check_params(ctx, sc, img, jb.params));
        if (jb.params.kernel != SOLRT_KERNEL_WAVEFRONT) { set_error("job %u: batches run the wavefront kernel", j); return SOLRT_ERR_INVALID; }
        if (jb.params.integrator != SOLRT_INTEGRATOR_PATH && jb.params.integrator != SOLRT_INTEGRATOR_PATH_NEE) {
            set_error("job %u: batches run the path integrators", j);
            return SOLRT_ERR_INVALID;
        }
        if (jb.params.integrator == SOLRT_INTEGRATOR_PATH_NEE) SOLRT_TRY(ensure_shadow_queue(ctx));
        if (j == 0) b.kind = sc.info.kind;
        if (sc.info.kind != b.kind) { set_error("job %u: all scenes of a batch need the same BVH kind", j); return SOLRT_ERR_INVALID; }
        b.jobs.push_back(make_job(sc, img, jb.camera, jb.params));
        const uint64_t np = (uint64_t)jb.params.width * jb.params.height;
        if (b.job_pix_base.back() + np >= (1ull << 31)) { set_error("batch has too many pixels"); return SOLRT_ERR_CAPACITY; }
        b.job_pix_base.push_back(b.job_pix_base.back() + (uint32_t)np);
    }
    if (flags & SOLRT_BATCH_PERSISTENT) {  // no passes: one launch over all pixels
        for (const DevJob& J : b.jobs) b.total_paths += (uint64_t)J.width * J.height * J.spp;
        SOLRT_TRY(b.d_jobs.alloc(sizeof(DevJob) * b.jobs.size()));
        SOLRT_TRY(b.d_items.alloc(sizeof(DevItem)));
        SOLRT_TRY(b.d_job_pix.alloc(sizeof(uint32_t) * b.job_pix_base.size()));
        SOLRT_CUDA(cudaMemcpyAsync(b.d_jobs.ptr, b.jobs.data(), sizeof(DevJob) * b.jobs.size(), cudaMemcpyHostToDevice,
                                   ctx.stream));
        SOLRT_CUDA(cudaMemcpyAsync(b.d_job_pix.ptr, b.job_pix_base.data(), sizeof(uint32_t) * b.job_pix_base.size(),
                                   cudaMemcpyHostToDevice, ctx.stream));
        return SOLRT_OK;
    }
    // work items, round-robin over jobs so that passes mix jobs
    struct Chunk { uint32_t job, pix0, npix, k, spp; };
    std::vector<Chunk> chunks;
    for (uint32_t j = 0; j < n; ++j) {
        const DevJob& J = b.jobs[j];
        const uint32_t np = J.width * J.height;
        const uint32_t k = J.rng_mode == SOLRT_RNG_REF_STREAM ? 1u : std::max(1u, std::min(J.spp, cap / std::max(np, 1u)));
        for (uint32_t p0 = 0; p0 < np; p0 += cap) chunks.push_back(Chunk{j, p0, std::min(cap, np - p0), k, J.spp});
    }
    // Passes are filled first fit: round r of every chunk (its samples
    // [r k, r k + k)), largest items first, goes to the first pass after the
    // pass of the chunk's round r - 1 that has room, so a pixel's samples are
    // still accumulated in order and passes run close to the capacity.
    struct Bin {
        PassPlan plan;
        std::vector<DevItem> items;
    };
    std::vector<Bin> bins;
    std::vector<int64_t> last(chunks.size(), -1);
    std::vector<uint32_t> live;
    for (uint32_t round = 0;; ++round) {
        live.clear();
        for (uint32_t c = 0; c < (uint32_t)chunks.size(); ++c)
            if ((uint64_t)round * chunks[c].k < chunks[c].spp) live.push_back(c);
        if (live.empty()) break;
        auto paths_of = [&](uint32_t c) {
            const uint32_t s0 = round * chunks[c].k;
            return (uint64_t)chunks[c].npix * std::min(chunks[c].k, chunks[c].spp - s0);
        };
        std::stable_sort(live.begin(), live.end(), [&](uint32_t a, uint32_t b2) { return paths_of(a) > paths_of(b2); });
        for (uint32_t c : live) {
            const Chunk& ch = chunks[c];
            const uint32_t s0 = round * ch.k;
            const uint64_t paths = paths_of(c);
            size_t p = (size_t)(last[c] + 1);
            while (p < bins.size() && bins[p].plan.paths + paths > cap) ++p;
            if (p == bins.size()) bins.push_back(Bin{PassPlan{0, 0, 0, 0, 0}, {}});
            Bin& bn = bins[p];
            DevItem it{ch.job, ch.pix0, ch.npix, s0, std::min(ch.k, ch.spp - s0), bn.plan.paths, bn.plan.pixels, 0};
            bn.items.push_back(it);
            bn.plan.item_count += 1;
            bn.plan.paths += (uint32_t)paths;
            bn.plan.pixels += it.npix;
            bn.plan.bounces = std::max(bn.plan.bounces, b.jobs[it.job].max_bounces + 1u);
            if (b.jobs[it.job].integrator == SOLRT_INTEGRATOR_PATH_NEE) bn.plan.nee = 1u;
            b.total_paths += paths;
            last[c] = (int64_t)p;
        }
    }
    for (Bin& bn : bins) {
        bn.plan.item_begin = (uint32_t)b.items.size();
        b.items.insert(b.items.end(), bn.items.begin(), bn.items.end());
        b.passes.push_back(bn.plan);
    }
    SOLRT_TRY(b.d_jobs.alloc(sizeof(DevJob) * b.jobs.size()));
    SOLRT_TRY(b.d_items.alloc(sizeof(DevItem) * b.items.size()));
    SOLRT_TRY(b.d_job_pix.alloc(sizeof(uint32_t) * b.job_pix_base.size()));
    cudaStream_t st = ctx.stream;
    SOLRT_CUDA(cudaMemcpyAsync(b.d_jobs.ptr, b.jobs.data(), sizeof(DevJob) * b.jobs.size(), cudaMemcpyHostToDevice, st));
    SOLRT_CUDA(cudaMemcpyAsync(b.d_items.ptr, b.items.data(), sizeof(DevItem) * b.items.size(), cudaMemcpyHostToDevice, st));
    SOLRT_CUDA(cudaMemcpyAsync(b.d_job_pix.ptr, b.job_pix_base.data(), sizeof(uint32_t) * b.job_pix_base.size(),
                               cudaMemcpyHostToDevice, st));
    if (flags & SOLRT_BATCH_COOPERATIVE) {
        int coop = 0;
        SOLRT_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx.device));
        if (!coop) { set_error("the device has no cooperative launches"); return SOLRT_ERR_DEVICE; }
        b.coop_stride = 2;
        for (const PassPlan& pp : b.passes) b.coop_stride = std::max(b.coop_stride, pp.bounces + 2u);
        SOLRT_TRY(b.d_passes.alloc(sizeof(PassPlan) * b.passes.size()));
        SOLRT_TRY(b.d_coop.alloc(coop_buffer_bytes((uint32_t)b.passes.size(), b.coop_stride)));
        SOLRT_CUDA(cudaMemcpyAsync(b.d_passes.ptr, b.passes.data(), sizeof(PassPlan) * b.passes.size(),
                                   cudaMemcpyHostToDevice, st));
    }
    return SOLRT_OK;
}

// Replaces cameras / frames / seeds (the plan's structure must not change).
solrt_status batch_set_jobs(Batch& b, const solrt_job* jobs) {
    for (size_t j = 0; j < b.jobs.size(); ++j) {
        const solrt_job& jb = jobs[j];
        const Scene& sc = *static_cast<const Scene*>(reinterpret_cast<const void*>(jb.scene));
        const Image& img = *static_cast<const Image*>(reinterpret_cast<const void*>(jb.image));
        SOLRT_TRY(check_params(*b.ctx, sc, img, jb.params));
        const DevJob nj = make_job(sc, img, jb.camera, jb.params);
        const DevJob& oj = b.jobs[j];
        if (nj.width != oj.width || nj.height != oj.height || nj.spp != oj.spp || nj.max_bounces != oj.max_bounces ||
            nj.rng_mode != oj.rng_mode || nj.accum_mode != oj.accum_mode || sc.info.kind != b.kind) {
            set_error("job %zu changed size, spp, bounces or modes: plan a new batch", j);
            return SOLRT_ERR_INVALID;
        }
        b.jobs[j] = nj;
        b.src[j] = jb;
    }
    SOLRT_CUDA(cudaMemcpyAsync(b.d_jobs.ptr, b.jobs.data(), sizeof(DevJob) * b.jobs.size(), cudaMemcpyHostToDevice,
                               b.ctx->stream));
    return SOLRT_OK;
}

solrt_status batch_launch(Batch& b) {
    Context& ctx = *b.ctx;
    cudaGetLastError();  // launch errors below must be this call's own
    if (!(b.flags & SOLRT_BATCH_GRAPH)) {
        SOLRT_CUDA(cudaEventRecord(ctx.ev0, ctx.stream));
        SOLRT_TRY(batch_issue(b, true));
        SOLRT_CUDA(cudaEventRecord(ctx.ev1, ctx.stream));
        return SOLRT_OK;
    }
    if (!b.exec) {
        const uint64_t launches0 = ctx.launches;
        SOLRT_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
        const solrt_status s = batch_issue(b, false);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx.stream, &g);
        if (s != SOLRT_OK) {
            if (g) cudaGraphDestroy(g);
            return s;
        }
        SOLRT_CUDA(e);
        b.graph = g;
        SOLRT_CUDA(cudaGraphInstantiate(&b.exec, b.graph, 0));
        b.graph_launches = ctx.launches - launches0;
        ctx.launches = launches0;
    }
    SOLRT_CUDA(cudaEventRecord(ctx.ev0, ctx.stream));
    SOLRT_CUDA(cudaGraphLaunch(b.exec, ctx.stream));
    SOLRT_CUDA(cudaEventRecord(ctx.ev1, ctx.stream));
    ctx.launches += b.graph_launches;
    return SOLRT_OK;
}

// Coordinate search over the extend launch shape, then the pass size; each
// candidate re-plans the batch (a new CUDA graph) and is timed on its best of
// two launches after a warm-up.
solrt_status batch_autotune(Batch& b, solrt_tune_result* out) {
    Context& ctx = *b.ctx;
    const TuneConfig initial = ctx.tune;
    const std::vector<solrt_job> src = b.src;
    // candidates are timed on at most kTuneJobs jobs spread over the batch
    constexpr size_t kTuneJobs = 32;
    std::vector<solrt_job> sample;
    if (src.size() <= kTuneJobs) {
        sample = src;
    } else {
        for (size_t i = 0; i < kTuneJobs; ++i) sample.push_back(src[i * src.size() / kTuneJobs]);
    }
    Batch tb;
    uint32_t candidates = 0;
    auto measure = [&](const TuneConfig& cfg, float* ms) -> solrt_status {
        ctx.tune = cfg;
        if (tb.exec) { cudaGraphExecDestroy(tb.exec); tb.exec = nullptr; }
        if (tb.graph) { cudaGraphDestroy(tb.graph); tb.graph = nullptr; }
        SOLRT_TRY(batch_plan(ctx, sample.data(), (uint32_t)sample.size(), b.flags, tb));
        float best = 0.0f;
        for (int r = 0; r < 3; ++r) {
            SOLRT_TRY(batch_launch(tb));
            SOLRT_CUDA(cudaEventSynchronize(ctx.ev1));
            float t = 0.0f;
            SOLRT_CUDA(cudaEventElapsedTime(&t, ctx.ev0, ctx.ev1));
            if (r == 1 || (r > 1 && t < best)) best = t;
        }
        ++candidates;
        *ms = best;
        return SOLRT_OK;
    };
    auto run = [&]() -> solrt_status {
        float initial_ms = 0.0f;
        SOLRT_TRY(measure(initial, &initial_ms));
        TuneConfig best = initial;
        float best_ms = initial_ms;
        const uint32_t smems[2] = {16u, 32u};
        const uint32_t blocks[3] = {64u, 128u, 256u};
        // a cooperative batch's kernel has one launch shape: only the pass size is tuned
        const uint32_t nblocks = (b.flags & SOLRT_BATCH_COOPERATIVE) ? 0u : 3u;
        for (uint32_t bi = 0; bi < nblocks; ++bi) {
            const uint32_t bl = blocks[bi];
            for (uint32_t sm : smems) {
                if ((b.kind == SOLRT_BVH8_Q8 || b.kind == SOLRT_BVH8_F32) && sm != initial.smem) continue;  // no shared stack
                TuneConfig c = initial;
                c.block = bl;
                c.smem = sm;
                if (c.block == initial.block && c.smem == initial.smem) continue;
                float ms = 0.0f;
                SOLRT_TRY(measure(c, &ms));
                if (ms < best_ms) { best_ms = ms; best = c; }
            }
        }
        const uint32_t cap = ctx.capacity;
        const uint32_t passes[3] = {std::max(1u, cap / 4u), std::max(1u, cap / 2u), 0u};
        const TuneConfig shape = best;
        for (uint32_t pp : passes) {
            TuneConfig c = shape;
            c.pass_paths = pp;
            if (c.pass_paths == shape.pass_paths) continue;
            float ms = 0.0f;
            SOLRT_TRY(measure(c, &ms));
            if (ms < best_ms) { best_ms = ms; best = c; }
        }
        ctx.tune = best;  // the whole batch, re-planned with the winner
        if (b.exec) { cudaGraphExecDestroy(b.exec); b.exec = nullptr; }
        if (b.graph) { cudaGraphDestroy(b.graph); b.graph = nullptr; }
        SOLRT_TRY(batch_plan(ctx, src.data(), (uint32_t)src.size(), b.flags, b));
        if (out) {
            out->best.block_size = best.block;
            out->best.smem_stack = best.smem;
            out->best.pass_paths = best.pass_paths;
            out->best.reserved = 0;
            out->best_ms = best_ms;
            out->initial_ms = initial_ms;
            out->candidates = candidates;
            out->reserved = 0;
        }
        return SOLRT_OK;
    };
    const solrt_status s = run();
    if (s != SOLRT_OK) {  // back to the configuration the call started from
        ctx.tune = initial;
        if (b.exec) { cudaGraphExecDestroy(b.exec); b.exec = nullptr; }
        if (b.graph) { cudaGraphDestroy(b.graph); b.graph = nullptr; }
        batch_plan(ctx, src.data(), (uint32_t)src.size(), b.flags, b);
    }
    return s;
}

solrt_status batch_apply_tune(Batch& b, const TuneConfig& cfg) {
    Context& ctx = *b.ctx;
    const TuneConfig initial = ctx.tune;
    const std::vector<solrt_job> src = b.src;
    ctx.tune = cfg;
    if (b.exec) { cudaGraphExecDestroy(b.exec); b.exec = nullptr; }
    if (b.graph) { cudaGraphDestroy(b.graph); b.graph = nullptr; }
    const solrt_status s = batch_plan(ctx, src.data(), (uint32_t)src.size(), b.flags, b);
    if (s != SOLRT_OK) {  // back to the plan the call started from
        ctx.tune = initial;
        batch_plan(ctx, src.data(), (uint32_t)src.size(), b.flags, b);
    }
    return s;
}

// One serving tick: uploads the active jobs and this tick's items, runs one
// pass, then finalizes the jobs listed in `fin` (their last samples were in
// this pass). Asynchronous on the context stream.
solrt_status serve_tick(Context& ctx, TickBuffers& tb, uint32_t kind, const std::vector<DevJob>& jobs,
                        const std::vector<DevItem>& items, const PassPlan& pp, const std::vector<DevJob>& fin) {
    cudaStream_t st = ctx.stream;
    cudaGetLastError();
    SOLRT_TRY(tb.jobs.alloc(sizeof(DevJob) * std::max<size_t>(jobs.size(), 1)));
    SOLRT_TRY(tb.items.alloc(sizeof(DevItem) * std::max<size_t>(items.size(), 1)));
    SOLRT_CUDA(cudaMemcpyAsync(tb.jobs.ptr, jobs.data(), sizeof(DevJob) * jobs.size(), cudaMemcpyHostToDevice, st));
    SOLRT_CUDA(cudaMemcpyAsync(tb.items.ptr, items.data(), sizeof(DevItem) * items.size(), cudaMemcpyHostToDevice, st));
    if (pp.item_count) SOLRT_TRY(issue_pass(ctx, kind, tb.jobs.as<DevJob>(), tb.items.as<DevItem>(), pp, false));
    if (!fin.empty()) {
        std::vector<uint32_t> pix(1, 0u);
        for (const DevJob& J : fin) pix.push_back(pix.back() + J.width * J.height);
        SOLRT_TRY(tb.fin_jobs.alloc(sizeof(DevJob) * fin.size()));
        SOLRT_TRY(tb.fin_pix.alloc(sizeof(uint32_t) * pix.size()));
        SOLRT_CUDA(cudaMemcpyAsync(tb.fin_jobs.ptr, fin.data(), sizeof(DevJob) * fin.size(), cudaMemcpyHostToDevice, st));
        SOLRT_CUDA(cudaMemcpyAsync(tb.fin_pix.ptr, pix.data(), sizeof(uint32_t) * pix.size(), cudaMemcpyHostToDevice, st));
        k_finalize<<<cdiv(pix.back(), 256), 256, 0, st>>>(tb.fin_jobs.as<DevJob>(), tb.fin_pix.as<uint32_t>(),
                                                          (uint32_t)fin.size(), pix.back());
        ++ctx.launches;
    }
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}

solrt_status estimate_rmse(Context& ctx, TickBuffers& tb, const std::vector<DevJob>& jobs,
                           const std::vector<uint32_t>& n, std::vector<double>& out) {
    out.assign(jobs.size(), 0.0);
    if (jobs.empty()) return SOLRT_OK;
    cudaStream_t st = ctx.stream;
    std::vector<uint32_t> pix(1, 0u);
    for (const DevJob& J : jobs) pix.push_back(pix.back() + J.width * J.height);
    SOLRT_TRY(tb.est_jobs.alloc(sizeof(DevJob) * jobs.size()));
    SOLRT_TRY(tb.est_pix.alloc(sizeof(uint32_t) * pix.size()));
    SOLRT_TRY(tb.est_n.alloc(sizeof(uint32_t) * n.size()));
    SOLRT_TRY(tb.est_sum.alloc(sizeof(double) * jobs.size()));
    cudaGetLastError();
    SOLRT_CUDA(cudaMemcpyAsync(tb.est_jobs.ptr, jobs.data(), sizeof(DevJob) * jobs.size(), cudaMemcpyHostToDevice, st));
    SOLRT_CUDA(cudaMemcpyAsync(tb.est_pix.ptr, pix.data(), sizeof(uint32_t) * pix.size(), cudaMemcpyHostToDevice, st));
    SOLRT_CUDA(cudaMemcpyAsync(tb.est_n.ptr, n.data(), sizeof(uint32_t) * n.size(), cudaMemcpyHostToDevice, st));
    SOLRT_CUDA(cudaMemsetAsync(tb.est_sum.ptr, 0, sizeof(double) * jobs.size(), st));
    k_rmse_estimate<<<cdiv(pix.back(), 256), 256, 0, st>>>(tb.est_jobs.as<DevJob>(), tb.est_pix.as<uint32_t>(),
                                                           tb.est_n.as<uint32_t>(), (uint32_t)jobs.size(), pix.back(),
                                                           tb.est_sum.as<double>());
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    SOLRT_CUDA(cudaMemcpyAsync(out.data(), tb.est_sum.ptr, sizeof(double) * jobs.size(), cudaMemcpyDeviceToHost, st));
    SOLRT_CUDA(cudaStreamSynchronize(st));
    return SOLRT_OK;
}

DevJob job_for(const Scene& sc, const Image& img, const solrt_camera& cam, const solrt_render_params& p) {
    return make_job(sc, img, cam, p);
}

solrt_status check_job(const Context& ctx, const Scene& sc, const Image& img, const solrt_render_params& p) {
    if (p.integrator != SOLRT_INTEGRATOR_PATH && p.integrator != SOLRT_INTEGRATOR_PATH_NEE) {
        set_error("the server runs the path integrators");
        return SOLRT_ERR_INVALID;
    }
    return check_params(ctx, sc, img, p);
}

solrt_status ensure_shadow_queue(Context& ctx) {
    const size_t C = ctx.capacity;
    SOLRT_TRY(ctx.q_o[2].alloc(16 * C));
    SOLRT_TRY(ctx.q_d[2].alloc(16 * C));
    SOLRT_TRY(ctx.q_thr[2].alloc(16 * C));
    SOLRT_TRY(ctx.q_meta[2].alloc(8 * C));
    SOLRT_TRY(ctx.q_prev[0].alloc(16 * C));
    SOLRT_TRY(ctx.q_prev[1].alloc(16 * C));
    return SOLRT_OK;
}

// DEBUG / AO: one per-pixel launch over a one-job table.
static solrt_status render_sibling(Context& ctx, const Scene& sc, const solrt_camera& cam,
                                   const solrt_render_params& p, Image& img) {
    SOLRT_TRY(check_params(ctx, sc, img, p));
    DevJob J = make_job(sc, img, cam, p);
    J.integrator = p.integrator;
    J.noise = ctx.blue_noise.as<uchar4>();
    J.noise_w = ctx.noise_w;
    J.noise_h = ctx.noise_h;
    cudaGetLastError();
    SOLRT_TRY(ctx.sibling_job.alloc(sizeof(DevJob)));
    SOLRT_CUDA(cudaMemcpyAsync(ctx.sibling_job.ptr, &J, sizeof(DevJob), cudaMemcpyHostToDevice, ctx.stream));
    const uint32_t npix = p.width * p.height;
    const DevJob* dj = ctx.sibling_job.as<DevJob>();
    DevStats* stats = ctx.stats.as<DevStats>();
    SOLRT_CUDA(cudaEventRecord(ctx.ev0, ctx.stream));
    const uint32_t kind = sc.info.kind;
    if (p.integrator == SOLRT_INTEGRATOR_DEBUG) {
        if (kind == SOLRT_BVH8_Q8) k_debug<SOLRT_BVH8_Q8><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else if (kind == SOLRT_BVH4_Q8) k_debug<SOLRT_BVH4_Q8><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else if (kind == SOLRT_BVH8_F32) k_debug<SOLRT_BVH8_F32><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else if (kind == SOLRT_BVH2_Q16) k_debug<SOLRT_BVH2_Q16><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else if (kind == SOLRT_BVH2_TWO_LEVEL) k_debug<SOLRT_BVH2_TWO_LEVEL><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else k_debug<SOLRT_BVH2><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
    } else {
        if (kind == SOLRT_BVH8_Q8) k_ao<SOLRT_BVH8_Q8><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else if (kind == SOLRT_BVH4_Q8) k_ao<SOLRT_BVH4_Q8><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else if (kind == SOLRT_BVH8_F32) k_ao<SOLRT_BVH8_F32><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else if (kind == SOLRT_BVH2_Q16) k_ao<SOLRT_BVH2_Q16><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else if (kind == SOLRT_BVH2_TWO_LEVEL) k_ao<SOLRT_BVH2_TWO_LEVEL><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
        else k_ao<SOLRT_BVH2><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(dj, stats);
    }
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    SOLRT_CUDA(cudaEventRecord(ctx.ev1, ctx.stream));
    return SOLRT_OK;
}

solrt_status render_frame(Context& ctx, const Scene& sc, const solrt_camera& cam, const solrt_render_params& p,
                          Image& img) {
    if (p.integrator != SOLRT_INTEGRATOR_PATH && p.integrator != SOLRT_INTEGRATOR_PATH_NEE)
        return render_sibling(ctx, sc, cam, p, img);
    solrt_job jb;
    jb.scene = reinterpret_cast<solrt_scene*>(const_cast<Scene*>(&sc));
    jb.image = reinterpret_cast<solrt_image*>(&img);
    jb.camera = cam;
    jb.params = p;
    jb.params.kernel = SOLRT_KERNEL_WAVEFRONT;
    SOLRT_TRY(batch_plan(ctx, &jb, 1, 0, ctx.single));
    if (p.kernel != SOLRT_KERNEL_MEGA) return batch_launch(ctx.single);
    // per-pixel megakernel + the shared finalize
    Batch& b = ctx.single;
    cudaGetLastError();
    const uint32_t npix = p.width * p.height;
    SOLRT_CUDA(cudaEventRecord(ctx.ev0, ctx.stream));
    const DevJob* dj = b.d_jobs.as<DevJob>();
    DevStats* dst = ctx.stats.as<DevStats>();
    const uint32_t g = cdiv(npix, 128);
    if (p.integrator == SOLRT_INTEGRATOR_PATH_NEE) {
        if (b.kind == SOLRT_BVH8_Q8) k_megakernel_nee<SOLRT_BVH8_Q8><<<g, 128, 0, ctx.stream>>>(dj, dst);
        else if (b.kind == SOLRT_BVH4_Q8) k_megakernel_nee<SOLRT_BVH4_Q8><<<g, 128, 0, ctx.stream>>>(dj, dst);
        else if (b.kind == SOLRT_BVH8_F32) k_megakernel_nee<SOLRT_BVH8_F32><<<g, 128, 0, ctx.stream>>>(dj, dst);
        else if (b.kind == SOLRT_BVH2_Q16) k_megakernel_nee<SOLRT_BVH2_Q16><<<g, 128, 0, ctx.stream>>>(dj, dst);
        else if (b.kind == SOLRT_BVH2_TWO_LEVEL)
            k_megakernel_nee<SOLRT_BVH2_TWO_LEVEL><<<g, 128, 0, ctx.stream>>>(dj, dst);
        else k_megakernel_nee<SOLRT_BVH2><<<g, 128, 0, ctx.stream>>>(dj, dst);
    } else if (b.kind == SOLRT_BVH8_Q8)
        k_megakernel<SOLRT_BVH8_Q8><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(b.d_jobs.as<DevJob>(), ctx.stats.as<DevStats>());
    else if (b.kind == SOLRT_BVH4_Q8)
        k_megakernel<SOLRT_BVH4_Q8><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(b.d_jobs.as<DevJob>(), ctx.stats.as<DevStats>());
    else if (b.kind == SOLRT_BVH8_F32)
        k_megakernel<SOLRT_BVH8_F32><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(b.d_jobs.as<DevJob>(), ctx.stats.as<DevStats>());
    else if (b.kind == SOLRT_BVH2_Q16)
        k_megakernel<SOLRT_BVH2_Q16><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(b.d_jobs.as<DevJob>(), ctx.stats.as<DevStats>());
    else if (b.kind == SOLRT_BVH2_TWO_LEVEL)
        k_megakernel<SOLRT_BVH2_TWO_LEVEL><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(b.d_jobs.as<DevJob>(), ctx.stats.as<DevStats>());
    else
        k_megakernel<SOLRT_BVH2><<<cdiv(npix, 128), 128, 0, ctx.stream>>>(b.d_jobs.as<DevJob>(), ctx.stats.as<DevStats>());
    k_finalize<<<cdiv(npix, 256), 256, 0, ctx.stream>>>(b.d_jobs.as<DevJob>(), b.d_job_pix.as<uint32_t>(), 1u, npix);
    ctx.launches += 2;
    SOLRT_CUDA(cudaGetLastError());
    SOLRT_CUDA(cudaEventRecord(ctx.ev1, ctx.stream));
    return SOLRT_OK;
}

solrt_status debug_unit(Context& ctx, uint32_t op, uint32_t n, const uint32_t* a, const uint32_t* b,
                        const float* in_f32, uint32_t* out_u32, float* out_f32) {
    if (op == 8) {  // bounded grid-barrier wait: in_f32[0] = seconds, out_u32[0] = error flags raised
        if (!in_f32 || !out_u32 || !(in_f32[0] > 0.0f && in_f32[0] <= 10.0f)) {
            set_error("debug op 8 needs a wait of (0, 10] seconds and an output word");
            return SOLRT_ERR_INVALID;
        }
        return coop_wait_test(ctx, in_f32[0], out_u32);
    }
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
