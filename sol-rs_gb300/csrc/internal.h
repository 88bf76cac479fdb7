// internal.h — host-side objects behind the solrt C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/solrt.h"
#include "traverse.cuh"

namespace solrt {

void set_error(const char* fmt, ...);

// Returns from the calling function with SOLRT_ERR_DEVICE on a CUDA error.
#define SOLRT_CUDA(call)                                                              \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            ::solrt::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,             \
                               cudaGetErrorString(e_));                               \
            return e_ == cudaErrorMemoryAllocation ? SOLRT_ERR_OOM : SOLRT_ERR_DEVICE; \
        }                                                                             \
    } while (0)

#define SOLRT_TRY(expr)                          \
    do {                                         \
        solrt_status s_ = (expr);                \
        if (s_ != SOLRT_OK) return s_;           \
    } while (0)

// Owning device allocation.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    solrt_status alloc(size_t n) {
        if (n <= bytes && ptr) return SOLRT_OK;
        release();
        if (n == 0) return SOLRT_OK;
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e != cudaSuccess) {
            ptr = nullptr;
            set_error("cudaMalloc(%zu): %s", n, cudaGetErrorString(e));
            return SOLRT_ERR_OOM;
        }
        bytes = n;
        return SOLRT_OK;
    }
    template <class T> T* as() const { return reinterpret_cast<T*>(ptr); }
    // Takes over `o`'s allocation (releasing this one's).
    void adopt(DeviceBuffer& o) {
        if (&o == this) return;
        release();
        ptr = o.ptr;
        bytes = o.bytes;
        o.ptr = nullptr;
        o.bytes = 0;
    }
};

// Statistics and error word kept on the device.
struct DevStats {
    unsigned long long segments;
    unsigned long long paths;
    unsigned long long node_visits;
    unsigned long long tri_tests;
    unsigned long long fp64_fallbacks;
    unsigned long long unoccluded;  // shadow rays that reached their light
    unsigned int eflags;
    unsigned int pad;
};

// Per-pass control block: queue lengths and work counters per bounce.
#define SOLRT_MAX_BOUNCES 1024
struct PassCtl {
    unsigned int count[SOLRT_MAX_BOUNCES + 2];
    unsigned int work[SOLRT_MAX_BOUNCES + 2];
    unsigned int scount[SOLRT_MAX_BOUNCES + 2];  // shadow queue per bounce
    unsigned int swork[SOLRT_MAX_BOUNCES + 2];
};

// Structure-of-arrays path queue (one wavefront).
struct PathQueue {
    float4* o_tmin;   // origin, tmin
    float4* d_tmax;   // direction, tmax
    float4* thr_rng;  // throughput, rng state (bits)
    uint2* meta;      // slot within the pass, job << kDepthBits | depth
    float4* prev;     // SOLRT_INTEGRATOR_PATH_NEE: normal of the vertex the ray left, pdf of its BSDF sample
};

// One job of a wavefront batch, as the device sees it.
struct DevJob {
    DevScene sc;
    float vinv[16];
    float pinv[16];
    uint32_t width, height, spp, frame, start, seed, job_id, rng_mode;
    uint32_t miss_mode, material_mode, max_bounces, accum_mode;
    float tmax;
    uint32_t integrator, noise_w, noise_h;
    const uchar4* noise;
    float4* accum;
    uchar4* rgba8;
    float4* fsum;
    float4* ksum;
    float4* kcomp;
    uint32_t* rng_state;
    // served jobs with a stopping rule: per pixel the sum over its samples of
    // r^2 + g^2 + b^2 (null otherwise)
    float* sq;
};

// A work item of one pass: samples [s0, s0 + k) of pixels [pix0, pix0 + npix)
// of one job. Its paths occupy slots [path_base, path_base + npix * k) of the
// pass (pixel-major), its pixels [pix_base, pix_base + npix) of the pass's
// pixel space.
struct DevItem {
    uint32_t job, pix0, npix, s0, k, path_base, pix_base, pad;
};

// The depth field of a path's meta word also carries its job.
constexpr uint32_t kDepthBits = 11;
constexpr uint32_t kDepthMask = (1u << kDepthBits) - 1u;

struct PassPlan {
    uint32_t item_begin, item_count;
    uint32_t paths, pixels;
    uint32_t bounces;  // extend/shade launches of the pass
    uint32_t nee = 0;  // a job of the pass uses SOLRT_INTEGRATOR_PATH_NEE
};

struct Context;

// A planned batch (also a single render: a batch of one job).
struct Batch {
    Context* ctx = nullptr;
    uint32_t flags = 0;
    uint32_t kind = 0;
    std::vector<DevJob> jobs;
    std::vector<DevItem> items;
    std::vector<PassPlan> passes;
    std::vector<uint32_t> job_pix_base;  // prefix of width*height over jobs (+ total)
    uint64_t total_paths = 0;
    uint64_t graph_launches = 0;
    DeviceBuffer d_jobs, d_items, d_job_pix;
    // SOLRT_BATCH_COOPERATIVE: the pass table on the device and the launch's
    // barrier word + per-pass queue counts (coop_buffer_bytes)
    DeviceBuffer d_passes, d_coop;
    uint32_t coop_stride = 0;  // counters per pass and kind (count, work, shadow count, shadow work): max bounces + 2
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<solrt_job> src;  // the jobs as given (re-planned by the autotuner)
    Batch() = default;
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;
    ~Batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

// Launch shape of the extend kernel and pass size of batches, chosen by
// solrt_context_set_tune or solrt_batch_autotune.
struct TuneConfig {
    uint32_t block = 128;      // threads per extend block: 64, 128 or 256
    uint32_t smem = 32;        // BVH2 traversal-stack slots in shared memory: 16 or 32
    uint32_t pass_paths = 0;   // paths per batch pass (0 = the path capacity)
};

struct Context {
    // The handle and every scene, image and batch created on the context hold
    // a reference; the context is freed when the last one goes, so objects
    // destroyed after solrt_context_destroy stay valid until then.
    int refs = 1;
    Batch single;  // plan of the last solrt_render call
    TuneConfig tune;
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    uint32_t capacity = 0;
    bool counters = false;
    uint32_t block_size = 0;
    // queues 0 and 1: paths of alternate bounces; queue 2: shadow rays of
    // SOLRT_INTEGRATOR_PATH_NEE (allocated when a render first needs it)
    DeviceBuffer q_o[3], q_d[3], q_thr[3], q_meta[3];
    DeviceBuffer q_prev[2];  // per path of queues 0 and 1, next-event estimation only
    DeviceBuffer hits, rad, ctl, stats, trace_work;
    DeviceBuffer blue_noise;  // RGBA8 texels of SOLRT_INTEGRATOR_AO
    DeviceBuffer sibling_job;  // one-job table of DEBUG / AO launches
    uint32_t noise_w = 0, noise_h = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint64_t launches = 0;
    double last_render_ms = 0.0;
    int extend_blocks_per_sm = 0;
    // stage timing (enable_timing): event pairs recorded around launches
    bool timing = false;
    struct TimedLaunch {
        cudaEvent_t start, end;
        int stage;  // 0 extend, 1 shade, 2 generate, 3 begin / accumulate / finalize
    };
    std::vector<TimedLaunch> timed;
    size_t timed_used = 0;
    double extend_ms = 0.0, shade_ms = 0.0, generate_ms = 0.0, accumulate_ms = 0.0;
    uint64_t extend_launches = 0, shade_launches = 0;
    // Records the start event of a timed launch of `stage`; returns its slot.
    int timing_begin(int stage) {
        if (!timing) return -1;
        if (timed_used == timed.size()) {
            TimedLaunch t{};
            if (cudaEventCreate(&t.start) != cudaSuccess || cudaEventCreate(&t.end) != cudaSuccess) return -1;
            timed.push_back(t);
        }
        timed[timed_used].stage = stage;
        cudaEventRecord(timed[timed_used].start, stream);
        return (int)timed_used++;
    }
    void timing_end(int slot) {
        if (slot >= 0) cudaEventRecord(timed[slot].end, stream);
    }
    // Adds the elapsed times of all recorded launches (stream must be idle).
    void timing_collect() {
        for (size_t i = 0; i < timed_used; ++i) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, timed[i].start, timed[i].end) == cudaSuccess) {
                if (timed[i].stage == 0) { extend_ms += ms; ++extend_launches; }
                else if (timed[i].stage == 1) { shade_ms += ms; ++shade_launches; }
                else if (timed[i].stage == 2) generate_ms += ms;
                else accumulate_ms += ms;
            }
        }
        timed_used = 0;
    }
    PathQueue queue(int i) const {
        return PathQueue{q_o[i].as<float4>(), q_d[i].as<float4>(), q_thr[i].as<float4>(), q_meta[i].as<uint2>(),
                         i < 2 ? q_prev[i].as<float4>() : nullptr};
    }
};

struct Scene {
    Context* ctx = nullptr;
    uint32_t tri_count = 0;
    uint32_t vertex_count = 0;
    uint32_t material_count = 0;
    // world positions (BVH builds), object-space positions and normals and
    // colours (shading), triangles (v0, v1, v2, section), materials, and per
    // section its material index
    DeviceBuffer vpos, tri_idx, materials, sec_mat;
    DeviceBuffer nodes, tri_wt;
    solrt_bvh_info info{};
    solrt_bvh_desc desc{};
    // Object-space positions / normals (float4 per vertex; shading reads
    // them and transforms by the section's instance, as pathtrace.rchit
    // does), the first vertex of each section, the instances (one per
    // section); SOLRT_BVH_DYNAMIC also keeps the BVH2 topology of the last
    // build (leaf order, children, parents, key ranges) for refits.
    bool dynamic = false;
    uint32_t section_count = 0;
    DeviceBuffer opos, vnc, vsec_start, instances;
    DeviceBuffer topo_order, topo_child, topo_par_int, topo_par_leaf, topo_range;
    // Host copies: each section's first triangle and triangle count, and the
    // staged instances (one per section).
    std::vector<uint32_t> sec_tri_first, sec_tri_count;
    std::vector<solrt_instance> inst_host;
    // SOLRT_BVH2_TWO_LEVEL: one BLAS per section over its object-space
    // triangles (concatenated in `nodes` / `tri_wt`), their object-space
    // root boxes (6 floats per section) and root nodes (-1: empty section),
    // and the TLAS over the instances with the instance table.
    std::vector<float> blas_box;
    std::vector<int32_t> blas_root;
    uint32_t blas_depth = 0, tlas_count = 0, tlas_depth = 0;
    DeviceBuffer tlas, inst_table;
    // light tree of next-event estimation (see DevScene::lights), built at
    // creation and by regenerate, and per triangle its light-tree code
    // (DevScene::tri_light); host copies of the candidates (emissive
    // triangles) and of what their power needs
    DeviceBuffer lights, tri_light;
    std::vector<uint32_t> light_cand_prim;
    std::vector<uint4> light_cand_tri;
    std::vector<uint32_t> light_sec_mat;
    std::vector<solrt_material> light_mats;
    uint32_t light_count = 0;
    DevScene view() const {
        DevScene d;
        d.tri_count = tri_count;
        d.bvh_kind = info.kind;
        d.node_count = info.node_count;
        const bool two = info.kind == SOLRT_BVH2_TWO_LEVEL;
        d.tlas_count = two ? tlas_count : 0u;
        d.inst_count = two ? section_count : 0u;
        d.tlas = two ? tlas.as<float4>() : nullptr;
        d.inst = two ? inst_table.as<float4>() : nullptr;
        d.vpos = vpos.as<float4>();
        d.opos = opos.as<float4>();
        d.vnc = vnc.as<float4>();
        d.tri_idx = tri_idx.as<uint4>();
        d.sections = instances.as<float4>();
        d.sec_mat = sec_mat.as<uint32_t>();
        d.materials = materials.as<float4>();
        d.nodes = nodes.as<float4>();
        d.tri_wt = tri_wt.as<float4>();
        d.lights = lights.as<float4>();
        d.tri_light = tri_light.as<uint32_t>();
        d.light_count = light_count;
        return d;
    }
};

struct Image {
    Context* ctx = nullptr;
    uint32_t width = 0, height = 0, accum_mode = 0;
    DeviceBuffer accum, rgba8, frame_sum, ksum, kcomp, rng_state;
};

// bvh_build.cu
solrt_status build_bvh(Context& ctx, Scene& sc, const solrt_bvh_desc& desc);
// Dynamic scenes: world-space vertices from object space and the staged
// instances, then a rebuild or a refit of the kept topology.
solrt_status regenerate_scene(Context& ctx, Scene& sc, uint32_t mode);

// trace.cu
solrt_status launch_trace_rays(Context& ctx, const Scene& sc, const solrt_ray* rays, uint32_t n, solrt_hit* hits);
// Extend for a batched queue: the scene of ray i is jobs[meta[i].y >> kDepthBits].sc.
// Closest hits of the `*count` rays of queue `q` (any_hit: some hit in
// (tmin, tmax), for occlusion queries); `st` (default: the context's first
// stats block) receives their segment and visit counts.
solrt_status launch_extend(Context& ctx, uint32_t kind, const DevJob* jobs, const PathQueue& q, float4* hits,
                           const unsigned int* count, unsigned int* work, DevStats* st = nullptr,
                           bool any_hit = false);
// Whether an extend kernel exists for this block size / shared stack slots.
bool extend_variant_ok(uint32_t block, uint32_t smem);

// coop.cu: SOLRT_BATCH_COOPERATIVE. Bytes of the barrier word and counters
// of a batch of `npasses` passes with `stride` counters per pass and kind.
size_t coop_buffer_bytes(uint32_t npasses, uint32_t stride);
// Zeroes `coop` (coop_buffer_bytes) and runs every pass of the batch in one
// cooperative launch on the context stream.
solrt_status launch_batch_coop(Context& ctx, uint32_t kind, const DevJob* jobs, const DevItem* items,
                               const PassPlan* passes, uint32_t npasses, uint32_t ctr_stride, const uint32_t* job_pix,
                               uint32_t njobs, uint32_t total_pix, void* coop, bool nee);
// A cooperative grid whose block 0 never reaches the barrier the others wait
// at, each wait bounded by `seconds`; returns the error flags it raised
// (SOLRT_EFLAG_TIMEOUT expected). Synchronises.
solrt_status coop_wait_test(Context& ctx, double seconds, uint32_t* eflags);

// pathtrace.cu
solrt_status batch_plan(Context& ctx, const solrt_job* jobs, uint32_t n, uint32_t flags, Batch& b);
solrt_status batch_autotune(Batch& b, solrt_tune_result* out);
// Sets the context's launch shape / pass size and re-plans the batch with it.
solrt_status batch_apply_tune(Batch& b, const TuneConfig& cfg);
solrt_status batch_set_jobs(Batch& b, const solrt_job* jobs);
solrt_status batch_launch(Batch& b);
solrt_status render_frame(Context& ctx, const Scene& sc, const solrt_camera& cam, const solrt_render_params& p,
                          Image& img);
struct TickBuffers {
    DeviceBuffer jobs, items, fin_jobs, fin_pix;
    DeviceBuffer est_jobs, est_pix, est_n, est_sum;  // convergence estimates
};

// Convergence estimates of served jobs: for job i (its DevJob with `sq`,
// n[i] samples per pixel so far) the sum over its pixels of the variance of
// the pixel mean summed over RGB; out[i] / (3 * pixels) is the estimated
// squared RMSE against the converged image (infinite when a pixel sum is
// not finite). Synchronises.
solrt_status estimate_rmse(Context& ctx, TickBuffers& tb, const std::vector<DevJob>& jobs,
                           const std::vector<uint32_t>& n, std::vector<double>& out);
solrt_status serve_tick(Context& ctx, TickBuffers& tb, uint32_t kind, const std::vector<DevJob>& jobs,
                        const std::vector<DevItem>& items, const PassPlan& pp, const std::vector<DevJob>& fin);
DevJob job_for(const Scene& sc, const Image& img, const solrt_camera& cam, const solrt_render_params& p);
solrt_status check_job(const Context& ctx, const Scene& sc, const Image& img, const solrt_render_params& p);
// Allocates the shadow-ray queue of SOLRT_INTEGRATOR_PATH_NEE (no-op once done).
solrt_status ensure_shadow_queue(Context& ctx);
// api.cpp: light tree of next-event estimation from world positions `pos`
// (upload_light_tree) or from the scene's current vertices (refresh).
solrt_status upload_light_tree(Scene& sc, const std::vector<float4>& pos, cudaStream_t st);
solrt_status refresh_light_tree(Context& ctx, Scene& sc);
solrt_status debug_unit(Context& ctx, uint32_t op, uint32_t n, const uint32_t* a, const uint32_t* b,
                        const float* in_f32, uint32_t* out_u32, float* out_f32);

}  // namespace solrt
