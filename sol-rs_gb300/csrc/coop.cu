// coop.cu — SOLRT_BATCH_COOPERATIVE: a whole batch step as one persistent
// wavefront launch.
//
// The wavefront stages of pathtrace.cu (generate, extend, shade, accumulate,
// finalize) normally run as one launch per stage and bounce, about 14 per
// pass. Here one cooperative grid of (SMs x resident blocks) runs every pass
// of the batch: the stages become phases of the same kernel, and the grid
// meets at a grid-wide barrier where a stage needs the previous one's output
// (after generate, after every extend and every shade). Within a phase the
// work is shared as in the separate kernels: extend warps take rays from the
// phase's atomic work counter (bvh2_ww.cuh and the other traversal loops,
// unchanged), the other phases stride over their paths or pixels. Results
// are those of the per-stage launches bit for bit: every path still writes
// its own slot, sums run in sample order.
//
// The cooperative launch makes every block resident at once, so a barrier
// is always reached; each wait is still bounded (clock64 budget): a block
// whose wait runs out raises an abort word that every other waiting block
// sees, sets SOLRT_EFLAG_TIMEOUT and returns, so a late or lost block ends
// the launch with SOLRT_ERR_TIMEOUT instead of a hang.
//
// Data written in one phase and read in a later one by another SM (queues,
// hits, path radiance, queue counts, pixel sums, REF_STREAM states) is read
// through L2 (ld.global.cg): the SM's L1 is not coherent with other SMs'
// writes within a launch. Scene data is read-only for the launch.
//
// Batches with next-event-estimation jobs run the kNee variant: after each
// shade phase (which also pushes shadow rays), an any-hit extend phase over
// the shadow queue and a resolve phase that adds the unoccluded shadow
// rays' terms to their paths, as issue_pass does with separate launches.
#include <algorithm>

#include "bvh2_2l.cuh"
#include "bvh2_ww.cuh"
#include "bvh4_ww.cuh"
#include "bvh8_ww.cuh"
#include "internal.h"
#include "path_ops.cuh"

namespace solrt {

namespace {

#ifndef SOLRT_COOP_BLOCK
#define SOLRT_COOP_BLOCK 128
#endif
// 1: the shade phase is a separate (not inlined) function. Inlined (0) is
// faster: 64 mixed jobs, 2768 against 2677 Mrays/s with both phases as
// calls (the per-stage launches: 2859).
#ifndef SOLRT_COOP_SHADE_CALL
#define SOLRT_COOP_SHADE_CALL 0
#endif
#if SOLRT_COOP_SHADE_CALL
#define SOLRT_COOP_SHADE_ATTR __device__ __noinline__
#else
#define SOLRT_COOP_SHADE_ATTR __device__ __forceinline__
#endif
// 1: the extend phase is a separate (not inlined) function (0: inlined)
#ifndef SOLRT_COOP_EXTEND_CALL
#define SOLRT_COOP_EXTEND_CALL 0
#endif
#if SOLRT_COOP_EXTEND_CALL
#define SOLRT_COOP_EXTEND_ATTR __device__ __noinline__
#else
#define SOLRT_COOP_EXTEND_ATTR __device__ __forceinline__
#endif
// Resident blocks per SM asked of the register allocator for the binary
// kinds (0: no constraint).
#ifndef SOLRT_COOP_MINB
#define SOLRT_COOP_MINB 8
#endif
constexpr int kCoopBlock = SOLRT_COOP_BLOCK;

// Barrier state at the start of the batch's cooperative buffer (zeroed
// before every launch), followed by the per-pass queue counts and work
// counters.
struct CoopSync {
    unsigned int arrive;  // blocks at the current barrier
    unsigned int gen;     // barriers completed in this launch
    unsigned int abort;   // a wait ran out: every block leaves
    unsigned int pad;
};

struct CoopArgs {
    const DevJob* jobs;
    const DevItem* items;
    const PassPlan* passes;
    uint32_t npasses;
    const uint32_t* job_pix;
    uint32_t njobs;
    uint32_t total_pix;
    PathQueue q0, q1;
    PathQueue qs;         // shadow rays (kNee)
    float4* hits;
    float4* rad;
    uint32_t capacity;
    CoopSync* sync;
    unsigned int* ctr;    // per pass: count, work, shadow count, shadow work (ctr_stride each, by bounce)
    uint32_t ctr_stride;
    DevStats* stats;
    long long wait_cycles;  // budget of one barrier wait in SM clock cycles
};

// Wavefront queue through L2 (QueueIO of trace.cu with ld.global.cg loads).
// kNee: any_hit is a run-time field, so that the closest-hit and the shadow
// (any-hit) phases share one instantiation of the traversal loop and its
// shared-memory stack.
template <bool kNee>
struct CoopIOT {
    const float4* o_tmin;
    const float4* d_tmax;
    const uint2* meta;
    const DevJob* jobs;
    float4* hits;
    bool any_hit;
    SOLRT_D void load(uint32_t i, float4& o, float4& d, TravScene& ts) const {
        o = __ldcg(o_tmin + i);
        d = __ldcg(d_tmax + i);
        const DevScene* s = &jobs[__ldcg(&meta[i].y) >> kDepthBits].sc;
        ts.nodes = s->nodes;
        ts.tris = s->tri_wt;
        ts.node_count = s->node_count;
        ts.tri_count = s->tri_count;
        ts.tlas = s->tlas;
        ts.inst = s->inst;
        ts.tlas_count = s->tlas_count;
        ts.inst_count = s->inst_count;
    }
    SOLRT_D void load_ray(uint32_t i, float4& o, float4& d) const {
        o = __ldcg(o_tmin + i);
        d = __ldcg(d_tmax + i);
    }
    SOLRT_D void store(uint32_t i, const HitRec& h) const {
        hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
    }
};
template <>
struct CoopIOT<false> {
    const float4* o_tmin;
    const float4* d_tmax;
    const uint2* meta;
    const DevJob* jobs;
    float4* hits;
    bool unused;
    static constexpr bool any_hit = false;
    SOLRT_D void load(uint32_t i, float4& o, float4& d, TravScene& ts) const {
        CoopIOT<true>{o_tmin, d_tmax, meta, jobs, hits, false}.load(i, o, d, ts);
    }
    SOLRT_D void load_ray(uint32_t i, float4& o, float4& d) const {
        o = __ldcg(o_tmin + i);
        d = __ldcg(d_tmax + i);
    }
    SOLRT_D void store(uint32_t i, const HitRec& h) const {
        hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
    }
};

SOLRT_D unsigned int ld_acquire(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Loop state of a block, in shared memory and volatile: the phases' inner
// loops then keep none of it in registers (each phase gets the whole
// register budget, as the separate kernels do), and thread 0 advances it
// inside the barriers, when no thread still reads the old values.
struct CoopCtl {
    uint32_t p;    // pass
    uint32_t b;    // bounce level within the pass
    uint32_t gen;  // barriers passed
    uint32_t ok;   // 0: the launch is being abandoned
    uint32_t fb;   // FP64 fallbacks of the block's traversals
    uint32_t ef;   // error flags of the block
    uint32_t sfb;  // FP64 fallbacks of its shadow-ray traversals (kNee)
    uint32_t unocc;  // shadow rays it found unoccluded (kNee)
};
enum CoopAdvance { kStay = 0, kNextBounce = 1, kNextPass = 2 };

// Grid-wide barrier with a bounded wait; `adv` moves the block's loop
// state on. Returns false when the launch is being abandoned (this block's
// wait ran out, or another block's did).
SOLRT_D bool coop_barrier(const CoopArgs& a, volatile CoopCtl& c, int adv) {
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const uint32_t target = c.gen + 1u;
        __threadfence();  // this block's writes before its arrival
        if (atomicAdd(&a.sync->arrive, 1u) == gridDim.x - 1u) {
            atomicExch(&a.sync->arrive, 0u);  // reset before the next barrier can start
            __threadfence();
            atomicExch(&a.sync->gen, target);
        } else {
            const long long t0 = clock64();
            while (ld_acquire(&a.sync->gen) != target) {
                if (ld_acquire(&a.sync->abort)) {
                    ok = 0;
                    break;
                }
                if (clock64() - t0 > a.wait_cycles) {
                    atomicExch(&a.sync->abort, 1u);
                    atomicOr(&a.stats->eflags, (unsigned int)SOLRT_EFLAG_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();  // other blocks' writes before this block's later loads
        c.gen = target;
        c.ok = (uint32_t)ok;
        if (adv == kNextBounce) {
            c.b = c.b + 1u;
        } else if (adv == kNextPass) {
            c.p = c.p + 1u;
            c.b = 0u;
        }
    }
    __syncthreads();
    return c.ok != 0u;
}

// The per-thread results of a phase into the block's totals.
SOLRT_D void coop_flush(volatile CoopCtl& c, uint32_t fb, uint32_t ef) {
    if (fb) atomicAdd(const_cast<uint32_t*>(&c.fb), fb);
    if (ef) atomicOr(const_cast<uint32_t*>(&c.ef), ef);
}

// The shade stage of k_shade (plain variant, block compaction) over the n
// paths of queue qin: survivors go to qout in block order, finished paths
// write their radiance slot.
// Returns the error flags (kept in a register in the loop).
SOLRT_COOP_SHADE_ATTR uint32_t coop_shade(const DevJob* jobs, const DevItem* items, uint32_t nitems,
                                          const PathQueue& qin, const float4* hits, uint32_t n,
                                          const PathQueue& qout, unsigned int* count_out, uint32_t capacity,
                                          float4* rad) {
    uint32_t ef = 0;
    __shared__ uint32_t s_cnt[kCoopBlock / 32], s_pre[kCoopBlock / 32], s_base;
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    const uint32_t warp = threadIdx.x >> 5;
    for (uint32_t base = blockIdx.x * kCoopBlock; base < n; base += gridDim.x * kCoopBlock) {
        const uint32_t i = base + threadIdx.x;
        bool alive = false;
        float4 out_o = make_float4(0, 0, 0, 0), out_d = make_float4(0, 0, 0, 0), out_t = make_float4(0, 0, 0, 0);
        uint2 m = make_uint2(0, 0);
        if (i < n) {
            const float4 o = __ldcg(qin.o_tmin + i), d = __ldcg(qin.d_tmax + i), tr = __ldcg(qin.thr_rng + i);
            m = __ldcg(qin.meta + i);
            const uint32_t job = m.y >> kDepthBits;
            const DevJob& J = jobs[job];
            uint32_t rng = __float_as_uint(tr.w);
            uint32_t depth = m.y & kDepthMask;
            f3 acc{tr.x, tr.y, tr.z};
            if (shade_step<false>(J, o, d, __ldcg(hits + i), acc, rng, depth, out_o, out_d, ef)) {
                alive = true;
                out_t = make_float4(acc.x, acc.y, acc.z, __uint_as_float(rng));
                m.y = (job << kDepthBits) | depth;
            } else {
                rad[m.x] = make_float4(acc.x, acc.y, acc.z, 0.0f);
                if (J.rng_mode == SOLRT_RNG_REF_STREAM) {
                    const DevItem it = items[find_last_le(nitems, m.x, [&](uint32_t t) { return items[t].path_base; })];
                    J.rng_state[it.pix0 + (m.x - it.path_base) / it.k] = rng;
                }
            }
        }
        const uint32_t mask = __ballot_sync(0xffffffffu, alive);
        if (lane == 0) s_cnt[warp] = (uint32_t)__popc(mask);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (uint32_t w = 0; w < (uint32_t)(kCoopBlock / 32); ++w) {
                s_pre[w] = t;
                t += s_cnt[w];
            }
            s_base = t ? atomicAdd(count_out, t) : 0u;
        }
        __syncthreads();
        if (alive) {
            const uint32_t pos = s_base + s_pre[warp] + (uint32_t)__popc(mask & lane_lt);
            if (pos < capacity) {
                qout.o_tmin[pos] = out_o;
                qout.d_tmax[pos] = out_d;
                qout.thr_rng[pos] = out_t;
                qout.meta[pos] = m;
            } else {
                ef |= SOLRT_EFLAG_QUEUE;
            }
        }
    }
    return ef;
}

// The shade stage of k_shade's next-event-estimation variant over the n
// paths of queue qin: survivors go to qout and their shadow rays to qs, both
// with one atomic per warp; a path that ends adds its term to its radiance
// slot after the shadow terms resolved so far. Returns the error flags.
SOLRT_COOP_SHADE_ATTR uint32_t coop_shade_nee(const DevJob* jobs, const DevItem* items, uint32_t nitems,
                                              const PathQueue& qin, const float4* hits, uint32_t n,
                                              const PathQueue& qout, unsigned int* count_out, uint32_t capacity,
                                              float4* rad, const PathQueue& qs, unsigned int* count_s) {
    uint32_t ef = 0;
    const int lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    const uint32_t start = ((blockIdx.x * kCoopBlock + threadIdx.x) >> 5) * 32u;
    const uint32_t stride = ((gridDim.x * kCoopBlock) >> 5) * 32u;
    for (uint32_t base = start; base < n; base += stride) {
        const uint32_t i = base + (uint32_t)lane;
        bool alive = false, shadow = false, out_nee = false;
        float4 out_o = make_float4(0, 0, 0, 0), out_d = make_float4(0, 0, 0, 0), out_t = make_float4(0, 0, 0, 0);
        float4 s_o = make_float4(0, 0, 0, 0), s_d = make_float4(0, 0, 0, 0), s_c = make_float4(0, 0, 0, 0);
        float4 out_prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        uint2 m = make_uint2(0, 0);
        if (i < n) {
            const float4 o = __ldcg(qin.o_tmin + i), d = __ldcg(qin.d_tmax + i), tr = __ldcg(qin.thr_rng + i);
            m = __ldcg(qin.meta + i);
            const uint32_t job = m.y >> kDepthBits;
            const DevJob& J = jobs[job];
            const bool nee = J.integrator == SOLRT_INTEGRATOR_PATH_NEE;
            uint32_t rng = __float_as_uint(tr.w);
            uint32_t depth = m.y & kDepthMask;
            f3 acc{tr.x, tr.y, tr.z};
            f3 n_o{0.0f, 0.0f, 0.0f};
            const float4 prev = nee && depth > 0u ? __ldcg(qin.prev + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (shade_step<true>(J, o, d, __ldcg(hits + i), acc, rng, depth, out_o, out_d, ef, &n_o, prev,
                                 &out_prev)) {
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
                    const float4 r = __ldcg(rad + m.x);
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
        const uint32_t smask = __ballot_sync(0xffffffffu, shadow);
        if (mask) {
            const int leader = __ffs(mask) - 1;
            uint32_t pos0 = 0;
            if (lane == leader) pos0 = atomicAdd(count_out, (unsigned int)__popc(mask));
            pos0 = __shfl_sync(0xffffffffu, pos0, leader);
            if (alive) {
                const uint32_t pos = pos0 + (uint32_t)__popc(mask & lane_lt);
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
                const uint32_t pos = pos0 + (uint32_t)__popc(smask & lane_lt);
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
    return ef;
}

// k_shadow_resolve over the ns shadow rays of qs: an unoccluded one adds its
// term to its path's slot (one shadow ray per path and bounce, so no two
// threads share a slot). Returns the unoccluded rays this thread resolved.
SOLRT_D uint32_t coop_resolve(const PathQueue& qs, const float4* hits, uint32_t ns, float4* rad) {
    uint32_t reached = 0;
    for (uint32_t i = blockIdx.x * kCoopBlock + threadIdx.x; i < ns; i += gridDim.x * kCoopBlock) {
        if (__float_as_uint(__ldcg(hits + i).y) != SOLRT_NO_HIT) continue;
        const float4 c = __ldcg(qs.thr_rng + i);
        const uint32_t slot = __ldcg(&qs.meta[i].x);
        const float4 r = __ldcg(rad + slot);
        rad[slot] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.0f);
        ++reached;
    }
    return reached;
}

// The closest hits of the n rays of queue q (the extend kernel's loop for
// the kind, 32 shared-memory stack slots for the binary kinds). Returns
// (FP64 fallbacks, error flags).
template <int KIND, bool kNee>
SOLRT_COOP_EXTEND_ATTR uint2 coop_extend(const CoopIOT<kNee>& io, uint32_t n, unsigned int* work) {
    using CoopIO = CoopIOT<kNee>;
    TraceCounters cnt{0, 0, 0};
    uint32_t ef = 0;
    if constexpr (KIND == SOLRT_BVH2) {
        extend_bvh2_ww<CoopIO, false, kCoopBlock, SOLRT_SMEM_STACK, false>(io, n, work, cnt, ef);
    } else if constexpr (KIND == SOLRT_BVH2_Q16) {
        extend_bvh2_ww<CoopIO, false, kCoopBlock, SOLRT_SMEM_STACK, true>(io, n, work, cnt, ef);
    } else if constexpr (KIND == SOLRT_BVH2_TWO_LEVEL) {
        extend_bvh2_2l_ww<CoopIO, false, kCoopBlock, SOLRT_SMEM_STACK>(io, n, work, cnt, ef);
    } else if constexpr (KIND == SOLRT_BVH4_Q8) {
        extend_bvh4_ww<CoopIO, false, kCoopBlock, SOLRT_SMEM_STACK>(io, n, work, cnt, ef);
    } else if constexpr (KIND == SOLRT_BVH8_F32) {
        extend_bvh8_ww<CoopIO, false, true, kCoopBlock, 0>(io, n, work, cnt, ef);
    } else {
        extend_bvh8_ww<CoopIO, false, false, kCoopBlock, 0>(io, n, work, cnt, ef);
    }
    return make_uint2(cnt.fallbacks, ef);
}

// Resident blocks per SM asked of the register allocator: 8 (64 registers,
// the extend and shade kernels' own budget) for the binary kinds, 7 (72,
// what the 8-wide extend kernel uses by itself) for the wide kinds.
template <int KIND>
constexpr int coop_min_blocks() {
    return (KIND == SOLRT_BVH8_Q8 || KIND == SOLRT_BVH8_F32 || KIND == SOLRT_BVH4_Q8) ? 7 : SOLRT_COOP_MINB;
}

template <int KIND, bool kNee>
__global__ void __launch_bounds__(kCoopBlock, (coop_min_blocks<KIND>())) k_batch_coop(const CoopArgs a) {
    volatile __shared__ CoopCtl c;
    if (threadIdx.x == 0) {
        c.p = 0u;
        c.b = 0u;
        c.gen = 0u;
        c.ok = 1u;
        c.fb = 0u;
        c.ef = 0u;
        c.sfb = 0u;
        c.unocc = 0u;
    }
    __syncthreads();
    // counters of pass p: count, work, shadow count, shadow work, by bounce
    auto counters = [&](uint32_t p) { return a.ctr + (size_t)p * 4u * a.ctr_stride; };
    for (uint32_t t = blockIdx.x * kCoopBlock + threadIdx.x; t < a.total_pix; t += gridDim.x * kCoopBlock)
        begin_pixel(a.jobs, a.job_pix, a.njobs, t);
    while (c.p < a.npasses) {
        {   // generate (in the phase of the previous pass's accumulate: it
            // writes queue 0, which accumulate does not read)
            const PassPlan pp = a.passes[c.p];
            const DevItem* items = a.items + pp.item_begin;
            for (uint32_t i = blockIdx.x * kCoopBlock + threadIdx.x; i < pp.paths; i += gridDim.x * kCoopBlock)
                generate_path<LdL2>(a.jobs, items, pp.item_count, i, a.q0, a.rad);
            if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.stats->paths, (unsigned long long)pp.paths);
        }
        if (!coop_barrier(a, c, kStay)) break;
        for (;;) {
            {   // extend of bounce level b
                const uint32_t p = c.p, b = c.b;
                if (b >= a.passes[p].bounces) break;
                unsigned int* count = counters(p);
                const uint32_t nq = b == 0 ? a.passes[p].paths : __ldcg(count + b);
                const uint32_t n = nq < a.capacity ? nq : a.capacity;
                if (n == 0) break;  // every block reads the same count: the exit is grid-uniform
                if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.stats->segments, (unsigned long long)n);
                const PathQueue& qin = (b & 1u) ? a.q1 : a.q0;
                const uint2 r = coop_extend<KIND, kNee>(
                    CoopIOT<kNee>{qin.o_tmin, qin.d_tmax, qin.meta, a.jobs, a.hits, false}, n,
                    count + a.ctr_stride + b);
                coop_flush(c, r.x, r.y);
            }
            if (!coop_barrier(a, c, kStay)) break;
            {   // shade of the same level: survivors into the other queue
                const uint32_t p = c.p, b = c.b;
                const PassPlan pp = a.passes[p];
                unsigned int* count = counters(p);
                const uint32_t nq = b == 0 ? pp.paths : __ldcg(count + b);
                const uint32_t n = nq < a.capacity ? nq : a.capacity;
                const PathQueue& qin = (b & 1u) ? a.q1 : a.q0;
                const PathQueue& qout = (b & 1u) ? a.q0 : a.q1;
                if constexpr (kNee)
                    coop_flush(c, 0u, coop_shade_nee(a.jobs, a.items + pp.item_begin, pp.item_count, qin, a.hits, n,
                                                     qout, count + b + 1, a.capacity, a.rad, a.qs,
                                                     count + 2u * a.ctr_stride + b));
                else
                    coop_flush(c, 0u, coop_shade(a.jobs, a.items + pp.item_begin, pp.item_count, qin, a.hits, n,
                                                 qout, count + b + 1, a.capacity, a.rad));
            }
            if constexpr (kNee) {  // shadow rays of this level (none at the last: depth > max)
                if (!coop_barrier(a, c, kStay)) break;
                const uint32_t p = c.p, b = c.b;
                unsigned int* count = counters(p);
                const uint32_t nq = b + 1u < a.passes[p].bounces ? __ldcg(count + 2u * a.ctr_stride + b) : 0u;
                const uint32_t ns = nq < a.capacity ? nq : a.capacity;
                if (ns) {
                    if (blockIdx.x == 0 && threadIdx.x == 0)
                        atomicAdd(&a.stats[1].segments, (unsigned long long)ns);
                    const uint2 r = coop_extend<KIND, kNee>(
                        CoopIOT<kNee>{a.qs.o_tmin, a.qs.d_tmax, a.qs.meta, a.jobs, a.hits, true}, ns,
                        count + 3u * a.ctr_stride + b);
                    if (r.x) atomicAdd(const_cast<uint32_t*>(&c.sfb), r.x);
                    if (r.y) atomicOr(const_cast<uint32_t*>(&c.ef), r.y);
                    if (!coop_barrier(a, c, kStay)) break;
                    const uint32_t u = coop_resolve(a.qs, a.hits, ns, a.rad);
                    if (u) atomicAdd(const_cast<uint32_t*>(&c.unocc), u);
                }
            }
            if (!coop_barrier(a, c, kNextBounce)) break;
        }
        if (!c.ok) break;
        {   // accumulate the pass; the next pass's generate follows in the same phase
            const PassPlan pp = a.passes[c.p];
            const DevItem* items = a.items + pp.item_begin;
            for (uint32_t t = blockIdx.x * kCoopBlock + threadIdx.x; t < pp.pixels; t += gridDim.x * kCoopBlock)
                accumulate_pixel<LdL2>(a.jobs, items, pp.item_count, t, a.rad);
        }
        __syncthreads();  // every thread is done with pass c.p
        if (threadIdx.x == 0) {
            c.p = c.p + 1u;
            c.b = 0u;
        }
        __syncthreads();
    }
    if (c.ok && coop_barrier(a, c, kStay))
        for (uint32_t t = blockIdx.x * kCoopBlock + threadIdx.x; t < a.total_pix; t += gridDim.x * kCoopBlock)
            finalize_pixel<LdL2>(a.jobs, a.job_pix, a.njobs, t);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (c.fb) atomicAdd(&a.stats->fp64_fallbacks, (unsigned long long)c.fb);
        if (c.ef) atomicOr(&a.stats->eflags, c.ef);
        if (kNee && c.sfb) atomicAdd(&a.stats[1].fp64_fallbacks, (unsigned long long)c.sfb);
        if (kNee && c.unocc) atomicAdd(&a.stats[1].unoccluded, (unsigned long long)c.unocc);
    }
}

// A test of the bounded wait: a cooperative grid in which block 0 never
// arrives at the barrier the others wait at; each waiting block must give up
// after `wait_cycles`, set SOLRT_EFLAG_TIMEOUT and return.
__global__ void k_coop_wait_test(const CoopArgs a) {
    volatile __shared__ CoopCtl c;
    if (blockIdx.x == 0) return;
    if (threadIdx.x == 0) {
        c.p = c.b = c.gen = c.fb = c.ef = 0u;
        c.ok = 1u;
    }
    coop_barrier(a, c, kStay);
}

template <int KIND>
solrt_status launch_kind(Context& ctx, const CoopArgs& args, bool nee) {
    auto kern = nee ? k_batch_coop<KIND, true> : k_batch_coop<KIND, false>;
    int per_sm = 0;
    SOLRT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCoopBlock, 0));
    if (per_sm < 1) {
        set_error("cooperative batch kernel does not fit an SM");
        return SOLRT_ERR_DEVICE;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(ctx.sm_count * per_sm));
    cfg.blockDim = dim3(kCoopBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = ctx.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SOLRT_CUDA(cudaLaunchKernelEx(&cfg, kern, args));
    return SOLRT_OK;
}

long long wait_budget_cycles(const Context& ctx, double seconds) {
    int khz = 0;
    if (cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, ctx.device) != cudaSuccess || khz <= 0) {
        cudaGetLastError();  // not this launch's error: fall back to 2.1 GHz
        khz = 2100000;
    }
    return (long long)((double)khz * 1e3 * seconds);
}

}  // namespace

size_t coop_buffer_bytes(uint32_t npasses, uint32_t stride) {
    return sizeof(CoopSync) + sizeof(unsigned int) * 4u * (size_t)npasses * stride;
}

solrt_status launch_batch_coop(Context& ctx, uint32_t kind, const DevJob* jobs, const DevItem* items,
                               const PassPlan* passes, uint32_t npasses, uint32_t ctr_stride, const uint32_t* job_pix,
                               uint32_t njobs, uint32_t total_pix, void* coop, bool nee) {
    SOLRT_CUDA(cudaMemsetAsync(coop, 0, coop_buffer_bytes(npasses, ctr_stride), ctx.stream));
    CoopArgs a;
    a.jobs = jobs;
    a.items = items;
    a.passes = passes;
    a.npasses = npasses;
    a.job_pix = job_pix;
    a.njobs = njobs;
    a.total_pix = total_pix;
    a.q0 = ctx.queue(0);
    a.q1 = ctx.queue(1);
    a.qs = ctx.queue(2);
    if (nee && !a.qs.o_tmin) {
        set_error("shadow queue not allocated");
        return SOLRT_ERR_INVALID;
    }
    a.hits = ctx.hits.as<float4>();
    a.rad = ctx.rad.as<float4>();
    a.capacity = ctx.capacity;
    a.sync = static_cast<CoopSync*>(coop);
    a.ctr = reinterpret_cast<unsigned int*>(static_cast<char*>(coop) + sizeof(CoopSync));
    a.ctr_stride = ctr_stride;
    a.stats = ctx.stats.as<DevStats>();
    a.wait_cycles = wait_budget_cycles(ctx, 4.0);
    if (kind == SOLRT_BVH8_Q8) SOLRT_TRY(launch_kind<SOLRT_BVH8_Q8>(ctx, a, nee));
    else if (kind == SOLRT_BVH4_Q8) SOLRT_TRY(launch_kind<SOLRT_BVH4_Q8>(ctx, a, nee));
    else if (kind == SOLRT_BVH8_F32) SOLRT_TRY(launch_kind<SOLRT_BVH8_F32>(ctx, a, nee));
    else if (kind == SOLRT_BVH2_Q16) SOLRT_TRY(launch_kind<SOLRT_BVH2_Q16>(ctx, a, nee));
    else if (kind == SOLRT_BVH2_TWO_LEVEL) SOLRT_TRY(launch_kind<SOLRT_BVH2_TWO_LEVEL>(ctx, a, nee));
    else SOLRT_TRY(launch_kind<SOLRT_BVH2>(ctx, a, nee));
    ++ctx.launches;
    return SOLRT_OK;
}

solrt_status coop_wait_test(Context& ctx, double seconds, uint32_t* eflags) {
    DeviceBuffer buf, st;
    SOLRT_TRY(buf.alloc(sizeof(CoopSync)));
    SOLRT_TRY(st.alloc(sizeof(DevStats)));
    SOLRT_CUDA(cudaMemsetAsync(buf.ptr, 0, sizeof(CoopSync), ctx.stream));
    SOLRT_CUDA(cudaMemsetAsync(st.ptr, 0, sizeof(DevStats), ctx.stream));
    CoopArgs a = {};
    a.sync = buf.as<CoopSync>();
    a.stats = st.as<DevStats>();
    a.wait_cycles = wait_budget_cycles(ctx, seconds);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)std::max(2, ctx.sm_count));
    cfg.blockDim = dim3(32);
    cfg.stream = ctx.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SOLRT_CUDA(cudaLaunchKernelEx(&cfg, k_coop_wait_test, a));
    ++ctx.launches;
    DevStats h{};
    SOLRT_CUDA(cudaMemcpyAsync(&h, st.ptr, sizeof(DevStats), cudaMemcpyDeviceToHost, ctx.stream));
    SOLRT_CUDA(cudaStreamSynchronize(ctx.stream));
    *eflags = h.eflags;
    return SOLRT_OK;
}

}  // namespace solrt
