/*
 * solrt.h — C ABI of the GB300-native software path tracer.
 *
 * This library stands in for the `5-pathtrace` render path of sol-rs:
 *   - scene upload + acceleration-structure build
 *       replaces ray::SceneDescription::from_scene / from_meshes
 *       (src/ray/mod.rs:49-156) and BLAS::new / TLAS::new
 *       (src/ray/acceleration.rs:135-239, 344-400);
 *   - one render launch
 *       replaces the per-frame `render` of examples/5-pathtrace.rs:294-369:
 *       UBO SceneUniforms (:7-32), push constant accum_start_frame (:306-314),
 *       tlas_regenerate (:316) and ShaderBindingTable::cmd_trace_rays
 *       (src/ray/sbt.rs:167-180) running pathtrace.rgen / .rchit / .rmiss;
 *   - the RGBA32F accumulation image and RGBA8 render image
 *       (examples/5-pathtrace.rs:222-229) become device buffers read back by
 *       solrt_image_read.
 *
 * Conventions
 *   - Every function returns solrt_status (0 = ok). No exceptions cross it.
 *   - The caller owns host arrays; the library owns device objects until the
 *     matching *_destroy call.
 *   - A context owns one CUDA stream; calls on one context are serialised by
 *     the caller (one context per host thread). Server calls are thread-safe.
 *   - All device work of a context is asynchronous on its stream unless the
 *     function says it synchronises.
 *   - Plain-old-data structs mirror the reference's repr(C) Rust types and are
 *     pinned by static_assert in the implementation (64 / 48 / 144 bytes).
 */
#ifndef SOLRT_H
#define SOLRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: solrt_stats gained shadow_segments and shadow_unoccluded. */
#define SOLRT_ABI_VERSION 3u

typedef enum solrt_status {
    SOLRT_OK = 0,
    SOLRT_ERR_INVALID = 1,       /* bad argument, malformed scene */
    SOLRT_ERR_OOM = 2,           /* device or host allocation failed */
    SOLRT_ERR_DEVICE = 3,        /* CUDA error, or no usable device */
    SOLRT_ERR_TIMEOUT = 4,       /* a bounded wait ran out */
    SOLRT_ERR_CAPACITY = 5,      /* a fixed-capacity queue or stack overflowed */
    SOLRT_ERR_NOT_READY = 6,     /* job still running (server poll) */
    SOLRT_ERR_NOT_FOUND = 7,     /* unknown job / object */
    SOLRT_ERR_BUDGET = 8,        /* request larger than the memory budget */
    SOLRT_ERR_CANCELLED = 9      /* served job cancelled (solrt_server_cancel) */
} solrt_status;

/* ------------------------------------------------------------------------ */
/* Scene types                                                              */
/* ------------------------------------------------------------------------ */

/* ModelVertex (src/scene/mesh.rs:9-14): pos, color, normal, uv as vec4. 64 B. */
typedef struct solrt_vertex {
    float pos[4];
    float color[4];
    float normal[4];
    float uv[4];
} solrt_vertex;

/* MaterialInfo (src/scene/mod.rs:21-29). 48 B. */
typedef struct solrt_material {
    float base_color[4];
    float emissive[3];
    float padding0;
    float metallic;
    float roughness;
    float padding1;
    float padding2;
} solrt_material;

/* SceneInstance (src/ray/mod.rs:18-24): id, texture_offset, padding,
 * transform, transform_it (inverse-transpose). Column-major mat4. 144 B. */
typedef struct solrt_instance {
    uint32_t id;
    uint32_t texture_offset;
    float padding[2];
    float transform[16];
    float transform_it[16];
} solrt_instance;

/* PrimitiveSection + BufferPart (src/scene/mod.rs:31-44): one section is one
 * BLAS geometry and one instance in the reference (src/ray/mod.rs:78-134).
 * Indices of a section are relative to its vertex_offset, as the per-section
 * descriptors of the reference make them (src/scene/mod.rs:47-61). */
typedef struct solrt_section {
    uint32_t vertex_offset;
    uint32_t vertex_count;
    uint32_t index_offset;
    uint32_t index_count;     /* a multiple of 3 */
    uint32_t material_index;  /* into solrt_scene_desc.materials */
    uint32_t reserved;
} solrt_section;

/* Everything SceneDescription::from_meshes consumes. `instances` holds one
 * entry per section (transform + transform_it) or is NULL for identity. */
typedef struct solrt_scene_desc {
    const solrt_vertex* vertices;
    uint32_t vertex_count;
    uint32_t index_count;
    const uint32_t* indices;
    const solrt_section* sections;
    uint32_t section_count;
    uint32_t material_count;
    const solrt_material* materials;
    const solrt_instance* instances;
} solrt_scene_desc;

typedef enum solrt_bvh_kind {
    SOLRT_BVH2 = 0,     /* binary LBVH, FP32 child boxes, 64 B nodes */
    SOLRT_BVH8_Q8 = 1,  /* 8-wide, 8-bit quantised child boxes, 80 B nodes */
    SOLRT_BVH4_Q8 = 2,  /* 4-wide, 8-bit quantised child boxes, 64 B nodes */
    SOLRT_BVH8_F32 = 3, /* 8-wide, FP32 child boxes, 224 B nodes (the unquantised
                           reference point of SOLRT_BVH8_Q8) */
    SOLRT_BVH2_Q16 = 4, /* binary LBVH, child boxes as 16-bit planes of one
                           per-scene grid, 32 B nodes (same hits as SOLRT_BVH2) */
    SOLRT_BVH2_TWO_LEVEL = 5 /* one binary BLAS per section over its object-space
                           triangles, built once, and a binary TLAS over the
                           instances, rebuilt by solrt_scene_regenerate; rays
                           enter an instance through its inverse transform
                           (transform_it transposed), as the reference's
                           TLAS / BLAS pair does. Implies SOLRT_BVH_DYNAMIC */
} solrt_bvh_kind;

/* solrt_bvh_desc.flags */
#define SOLRT_BVH_DYNAMIC 1u  /* keep object-space geometry and the BVH topology on
                                 the device so solrt_scene_set_instances +
                                 solrt_scene_regenerate can move sections */
#define SOLRT_BVH_SAH 2u      /* BVH8 / BVH4 kinds: choose each wide node's children
                                 by the SAH-optimal collapse of the binary tree
                                 (dynamic program over the binary nodes) instead of
                                 opening the largest child first, from a binary
                                 tree restructured as below when leaf_max <= 1.
                                 BVH2 / BVH2-q16 kinds (and each BLAS of the
                                 two-level kind): restructure the LBVH toward
                                 the SAH by treelets of 7 leaves (three bottom-up
                                 rounds on the device; a longer build, fewer node
                                 visits). Same hits either way */

typedef struct solrt_bvh_desc {
    uint32_t kind;       /* solrt_bvh_kind */
    uint32_t leaf_max;   /* BVH8 / BVH4: max triangles per leaf child (1..3), 0 = 1 */
    uint32_t flags;      /* SOLRT_BVH_DYNAMIC (honoured by solrt_scene_create), SOLRT_BVH_SAH */
    uint32_t reserved;
} solrt_bvh_desc;

typedef struct solrt_bvh_info {
    uint32_t kind;
    uint32_t tri_count;
    uint32_t node_count;
    uint32_t depth;          /* levels on the longest root-to-leaf path */
    uint64_t node_bytes;
    uint64_t tri_bytes;      /* intersection stream, 48 B / triangle */
    uint64_t shade_bytes;    /* shading stream (vertices, indices, materials) */
    double build_ms;         /* device time of the last build */
} solrt_bvh_info;

/* ------------------------------------------------------------------------ */
/* Camera and per-launch parameters                                         */
/* ------------------------------------------------------------------------ */

/* The matrices of SceneUniforms (examples/5-pathtrace.rs:9-17) that the ray
 * generation reads. Column-major, as glam. */
typedef struct solrt_camera {
    float view[16];
    float view_inverse[16];
    float projection[16];
    float projection_inverse[16];
} solrt_camera;

typedef enum solrt_miss_mode {
    SOLRT_MISS_BLACK = 0,     /* pathtrace.rmiss with ENABLE_SKYLIGHT = 0 */
    SOLRT_MISS_REF_SKY = 1,   /* pathtrace.rmiss with ENABLE_SKYLIGHT = 1 (--sky) */
    SOLRT_MISS_GRADIENT = 2   /* mix((1,1,1),(0.5,0.7,1),0.5*(dir.y+1)) */
} solrt_miss_mode;

typedef enum solrt_material_mode {
    SOLRT_MATERIAL_REF = 0,     /* pathtrace.rchit: metallic GGX / Fresnel / cosine */
    SOLRT_MATERIAL_LAMBERT = 1  /* cosine-weighted diffuse only, same 3 draws */
} solrt_material_mode;

typedef enum solrt_accum_mode {
    SOLRT_ACCUM_REF_MIX = 0,    /* pathtrace.rgen:89-101 running mix */
    SOLRT_ACCUM_KAHAN = 1       /* Kahan-compensated per-pixel sample sums */
} solrt_accum_mode;

typedef enum solrt_rng_mode {
    /* One TEA-seeded stream per pixel per launch, samples drawn one after the
     * other: rng = tea(x + y*W, frame) (pathtrace.rgen:47-52). */
    SOLRT_RNG_REF_STREAM = 0,
    /* One stream per (pixel, sample): rng = tea(x + y*W, frame*spp + s),
     * xor tea(seed, job_id) when seed != 0. Samples run concurrently. */
    SOLRT_RNG_PER_SAMPLE = 1
} solrt_rng_mode;

typedef struct solrt_render_params {
    uint32_t width;
    uint32_t height;
    uint32_t spp;               /* samples per pixel per launch (reference: 8) */
    uint32_t max_bounces;       /* reference maxBounces = 32; <= 1024 */
    uint32_t frame;             /* SceneUniforms.frame.z (elapsed ticks) */
    uint32_t accum_start_frame; /* push constant of pathtrace.rgen */
    uint32_t seed;
    uint32_t job_id;
    uint32_t miss_mode;         /* solrt_miss_mode */
    uint32_t material_mode;     /* solrt_material_mode */
    uint32_t accum_mode;        /* solrt_accum_mode; must match the image */
    uint32_t rng_mode;          /* solrt_rng_mode */
    float tmax;                 /* 0 = reference 1e4 */
    uint32_t kernel;            /* solrt_kernel */
    uint32_t integrator;        /* solrt_integrator */
    uint32_t reserved;
} solrt_render_params;

/* What one launch computes per pixel. DEBUG and AO are the reference's
 * sibling ray-tracing pipelines over the same acceleration structure; they
 * run one thread per pixel (their shaders' structure), ignore `kernel`, and
 * are not accepted by batches or the server. */
typedef enum solrt_integrator {
    /* pathtrace.rgen / .rchit / .rmiss */
    SOLRT_INTEGRATOR_PATH = 0,
    /* debug.rgen / .rchit / .rmiss: one ray through each pixel centre
     * (tmin 0.001, tmax 1000); the image gets (1-u-v, u, v, 0) of the hit, or
     * the ray direction (x, y, z, 0) on a miss. No accumulation: the RGBA32F
     * image holds that value, the RGBA8 image its UNORM conversion. */
    SOLRT_INTEGRATOR_DEBUG = 1,
    /* ao.rgen / .rchit / .rmiss: `spp` jittered samples (reference 4), each
     * a chain of cosine-weighted rays along which every hit after the first
     * counts one occlusion, until a miss or `max_bounces` + 1 hits
     * (reference max_samples 4); directions from the blue-noise texture
     * set by solrt_context_set_blue_noise; colour = 1 - mean occlusion /
     * max_bounces, mixed into the image with 1 / (frame + 1 -
     * accum_start_frame) (ao.rgen:57-80). RGBA8 = UNORM of the colour. */
    SOLRT_INTEGRATOR_AO = 2,
    /* Path tracing with next-event estimation, an estimator the reference
     * does not have (it finds emitters only by hitting them). At every
     * diffuse vertex that continues the path, after the vertex's three
     * pathtrace.rchit draws, two draws pick a uniform point on an emissive
     * triangle that a walk down the scene's light tree chooses (one draw
     * per level, each child with probability proportional to its power
     * over its distance, bounded by the receiver's cosine); one shadow ray
     * per vertex goes through a second wavefront queue (or, in the
     * per-pixel kernel, is traced at once), and an unoccluded one adds its
     * light weighted by the power heuristic against the BSDF sample. An
     * emitter hit after a bounce adds its term with the complementary
     * weight; camera rays that hit an emitter and misses keep the
     * reference's terms. Same expected image as SOLRT_INTEGRATOR_PATH with
     * material_mode SOLRT_MATERIAL_LAMBERT, less noise under small lights.
     * Needs material_mode SOLRT_MATERIAL_LAMBERT; runs in both kernels, in
     * every batch mode and in the server. Shadow segments are counted in
     * solrt_stats.shadow_segments, not segments. */
    SOLRT_INTEGRATOR_PATH_NEE = 3
} solrt_integrator;

typedef enum solrt_kernel {
    /* generate / extend / shade stages over queues shared by all paths */
    SOLRT_KERNEL_WAVEFRONT = 0,
    /* the reference's structure (pathtrace.rgen:39-104): one thread per pixel
     * loops over its samples and bounces; same image, the plain kernel that
     * the wavefront and batches are measured against. Not for batches. */
    SOLRT_KERNEL_MEGA = 1
} solrt_kernel;

/* ------------------------------------------------------------------------ */
/* Rays for the ray-file (hit record) API                                   */
/* ------------------------------------------------------------------------ */

typedef struct solrt_ray {
    float origin[3];
    float tmin;
    float dir[3];
    float tmax;
} solrt_ray;

/* prim = global triangle index (section triangles are numbered in section
 * order) or SOLRT_NO_HIT; u, v = barycentrics of vertex 1 and 2 (the
 * hitAttributeEXT of pathtrace.rchit:58). */
typedef struct solrt_hit {
    float t;
    uint32_t prim;
    float u;
    float v;
} solrt_hit;

#define SOLRT_NO_HIT 0xffffffffu

typedef struct solrt_stats {
    uint64_t segments;        /* ray segments traced (primary + bounce) */
    uint64_t paths;           /* camera paths started */
    uint64_t node_visits;     /* only with counters enabled */
    uint64_t tri_tests;       /* only with counters enabled */
    uint64_t fp64_fallbacks;  /* watertight test edge functions recomputed in FP64 */
    uint64_t launches;        /* kernels launched by the library */
    uint32_t error_flags;     /* device error word (see solrt_error_bits) */
    uint32_t reserved;
    double render_ms;         /* device time of the last solrt_render */
    double extend_ms;         /* summed device time of extend launches (enable_timing) */
    double shade_ms;          /* summed device time of shade launches (enable_timing) */
    uint64_t extend_launches; /* launches timed into extend_ms */
    uint64_t shade_launches;  /* launches timed into shade_ms */
    double generate_ms;       /* camera-ray generation (enable_timing) */
    double accumulate_ms;     /* per-pixel sums, frame begin / finalize (enable_timing) */
    uint64_t shadow_segments; /* shadow rays traced (SOLRT_INTEGRATOR_PATH_NEE) */
    uint64_t shadow_unoccluded; /* of them, those that reached their light */
} solrt_stats;

typedef enum solrt_error_bits {
    SOLRT_EFLAG_STACK = 1u,       /* traversal stack overflow (ray dropped) */
    SOLRT_EFLAG_QUEUE = 2u,       /* wavefront queue overflow */
    SOLRT_EFLAG_INDEX = 4u,       /* out-of-range node / triangle index */
    SOLRT_EFLAG_TIMEOUT = 8u      /* a bounded device wait ran out */
} solrt_error_bits;

/* ------------------------------------------------------------------------ */
/* Opaque objects                                                           */
/* ------------------------------------------------------------------------ */

typedef struct solrt_context solrt_context;
typedef struct solrt_scene solrt_scene;
typedef struct solrt_image solrt_image;
typedef struct solrt_server solrt_server;

typedef struct solrt_context_desc {
    int device;                  /* CUDA ordinal */
    uint32_t path_capacity;      /* paths in flight per pass; 0 = default (32M, 4.8 GB of queues) */
    uint32_t enable_counters;    /* 1 = count node visits / triangle tests */
    uint32_t block_size;         /* extend kernel block size; 0 = default */
    uint32_t enable_timing;      /* 1 = CUDA-event timing of every extend / shade launch */
    uint32_t reserved[3];
} solrt_context_desc;

/* ------------------------------------------------------------------------ */
/* Functions                                                                */
/* ------------------------------------------------------------------------ */

uint32_t solrt_abi_version(void);
const char* solrt_status_string(solrt_status s);
/* Message of the last error on this host thread (never NULL). */
const char* solrt_last_error(void);

/* Context: CUDA device, stream, wavefront queues. Replaces the Vulkan Context
 * (src/context.rs:222-575) for this path. */
solrt_status solrt_context_create(const solrt_context_desc* desc, solrt_context** out);
solrt_status solrt_context_destroy(solrt_context* ctx);
solrt_status solrt_synchronize(solrt_context* ctx);
solrt_status solrt_get_stats(solrt_context* ctx, solrt_stats* out);
solrt_status solrt_reset_stats(solrt_context* ctx);
/* The CUDA stream (cudaStream_t) of the context, for callers that enqueue
 * their own work around the library's. */
void* solrt_context_stream(solrt_context* ctx);
/* Blue-noise texture of SOLRT_INTEGRATOR_AO: width x height RGBA8 UNORM
 * texels, row-major (the sampler2D of ao.rchit:39, loaded from
 * textures/HDR_RGBA_0.png by examples/4-ray-ao.rs:198-201). Copied. */
solrt_status solrt_context_set_blue_noise(solrt_context* ctx, const uint8_t* rgba8, uint32_t width,
                                          uint32_t height);

/* Scene: flattens sections to world space (transform, transform_it as in
 * pathtrace.rchit:80-86), uploads and builds the BVH. Synchronises.
 * Replaces SceneDescription::from_scene (src/ray/mod.rs:49-57). */
solrt_status solrt_scene_create(solrt_context* ctx, const solrt_scene_desc* desc,
                                const solrt_bvh_desc* bvh, solrt_scene** out);
solrt_status solrt_scene_destroy(solrt_scene* scene);
/* Rebuilds the BVH (kind may change). Synchronises. Replaces
 * SceneDescription::tlas_regenerate (src/ray/mod.rs:178-181). */
solrt_status solrt_scene_build_bvh(solrt_scene* scene, const solrt_bvh_desc* bvh);
solrt_status solrt_scene_bvh_info(solrt_scene* scene, solrt_bvh_info* out);
/* Copies the device BVH to host memory (for topology checks). `nodes` gets
 * node_bytes, `tris` gets tri_bytes; either may be NULL. Synchronises. */
solrt_status solrt_scene_bvh_export(solrt_scene* scene, void* nodes, size_t nodes_bytes,
                                    void* tris, size_t tris_bytes);
/* Device memory held by the scene, in bytes. */
solrt_status solrt_scene_bytes(solrt_scene* scene, uint64_t* out);

/* ---- per-frame instance transforms --------------------------------------
 * Replaces SceneDescription::blas_transform / blas_transforms (which set a
 * BLAS instance's transform and the SceneInstance transform + inverse
 * transpose, src/ray/mod.rs:162-176, SceneInstance::update_transform
 * src/ray/mod.rs:26-35) and tlas_regenerate (src/ray/mod.rs:178-181, called
 * every frame by examples/5-pathtrace.rs:316).
 *
 * The scene keeps its sections' object-space vertices on the device (scene
 * created with SOLRT_BVH_DYNAMIC). set_instances stores one instance per
 * section; regenerate transforms every vertex on the device with its
 * section's instance (the same arithmetic as solrt_scene_create's
 * flattening, so results equal a scene created with those instances) and
 * then rebuilds the BVH (REBUILD: identical to a fresh build) or refits the
 * boxes of the existing topology (REFIT: cheaper, same hits, BVH quality
 * degrades as sections move). Stream-ordered on the context stream. */
typedef enum solrt_regen_mode {
    SOLRT_REGEN_REBUILD = 0,
    SOLRT_REGEN_REFIT = 1
} solrt_regen_mode;

/* transform (column-major) -> instance with transform_it = inverse(T)^T
 * computed in FP64 and rounded; ERR_INVALID for a singular transform. */
solrt_status solrt_instance_from_transform(const float transform[16], uint32_t id, solrt_instance* out);
/* count must equal the scene's section count. */
solrt_status solrt_scene_set_instances(solrt_scene* scene, const solrt_instance* instances, uint32_t count);
solrt_status solrt_scene_regenerate(solrt_scene* scene, uint32_t mode);

/* Camera matrices (src/scene/camera.rs:98-106: look_at_rh, perspective_rh),
 * computed in FP64 and rounded to FP32. vfov in degrees. */
solrt_status solrt_camera_look_at(const float eye[3], const float center[3], const float up[3],
                                  float vfov_deg, float aspect, float znear, float zfar,
                                  solrt_camera* out);
/* Camera from a view matrix, as Camera::from_view (src/scene/camera.rs:73-94). */
solrt_status solrt_camera_from_view(const float view[16], float vfov_deg, float aspect,
                                    float znear, float zfar, solrt_camera* out);

/* Images: RGBA32F accumulation + RGBA8 render target (+ Kahan sums). */
solrt_status solrt_image_create(solrt_context* ctx, uint32_t width, uint32_t height,
                                uint32_t accum_mode, solrt_image** out);
solrt_status solrt_image_destroy(solrt_image* img);
solrt_status solrt_image_clear(solrt_image* img);
/* Synchronises; either pointer may be NULL. rgba32f: W*H*4 floats,
 * rgba8: W*H*4 bytes, row-major from pixel (0,0) = gl_LaunchIDEXT (0,0). */
solrt_status solrt_image_read(solrt_image* img, float* rgba32f, uint8_t* rgba8);
/* Device pointers of the images (float4 accumulation, uchar4 render). */
solrt_status solrt_image_device_ptrs(solrt_image* img, void** accum, void** rgba8);
/* Checkpoint / resume of the accumulation state (no counterpart in the
 * reference, whose images live only in VRAM): the RGBA32F accumulation
 * (W*H*4 floats) and, for KAHAN images, the compensated sums and
 * compensations (W*H*4 floats each; NULL for REF_MIX images). Restoring a
 * snapshot into an image of the same size and mode and rendering the next
 * frame index continues the accumulation bit for bit (the RGBA8 image is
 * written by the next render). Both synchronise. */
solrt_status solrt_image_snapshot(solrt_image* img, float* accum, float* kahan_sum, float* kahan_comp);
solrt_status solrt_image_restore(solrt_image* img, const float* accum, const float* kahan_sum,
                                 const float* kahan_comp);

/* One launch of the path tracer: spp samples for every pixel, accumulated
 * into `img`. Asynchronous on the context stream. */
solrt_status solrt_render(solrt_context* ctx, solrt_scene* scene, const solrt_camera* camera,
                          const solrt_render_params* params, solrt_image* img);

/* ------------------------------------------------------------------------ */
/* Batched rendering: many scenes, one wavefront                            */
/* ------------------------------------------------------------------------ */
/* No counterpart in the reference, which renders one scene per
 * ShaderBindingTable::cmd_trace_rays (src/ray/sbt.rs:167-180): this is the
 * batched mixed-scene workload built on the same per-job semantics. */

/* One render job: what one solrt_render call takes. */
typedef struct solrt_job {
    solrt_scene* scene;
    solrt_image* image;
    solrt_camera camera;
    solrt_render_params params;
} solrt_job;

typedef struct solrt_batch solrt_batch;

enum {
    SOLRT_BATCH_GRAPH = 1u,      /* capture the batch's launches once into a CUDA graph and replay it */
    /* one persistent launch per step instead of wavefront passes: warps take
     * 32 pixels at a time of all jobs' pixels from a device work counter and
     * each thread traces all samples of its pixel to the end (the per-pixel
     * structure of the reference's raygen loop; a next-event-estimation
     * job's shadow rays are traced at their vertices); same images. */
    SOLRT_BATCH_PERSISTENT = 2u,
    /* the wavefront passes of a step (generate, extend and shade per bounce,
     * accumulate, finalize) as phases of one cooperative launch: a grid of
     * (SMs x resident blocks) that meets at grid-wide barriers between
     * stages instead of one launch per stage (next-event-estimation jobs add
     * a shadow-ray extend and a resolve phase per bounce); same images. Each
     * barrier wait is bounded: a launch whose blocks do not all arrive ends
     * with SOLRT_ERR_TIMEOUT. Node / triangle counters are not gathered.
     * Not with SOLRT_BATCH_PERSISTENT. */
    SOLRT_BATCH_COOPERATIVE = 4u
};

/* Plans a batch: the paths of all jobs share the wavefront queues, each pass
 * mixes work items of several jobs, and every job's image is bit-identical
 * to rendering that job alone with solrt_render (each path depends only on
 * its own job; per-pixel sums run in sample order). All scenes must use the
 * same BVH kind; every job needs width * height <= the context's path
 * capacity. Synchronises. */
solrt_status solrt_batch_create(solrt_context* ctx, const solrt_job* jobs, uint32_t n, uint32_t flags,
                                solrt_batch** out);
/* New cameras / frames / seeds for the same jobs (same scenes, images,
 * sizes, spp, bounces and modes). */
solrt_status solrt_batch_update(solrt_batch* batch, const solrt_job* jobs);
/* Renders every job once (asynchronous on the context stream). */
solrt_status solrt_batch_launch(solrt_batch* batch);
solrt_status solrt_batch_destroy(solrt_batch* batch);
/* Passes, work items and bounce launches of the plan. */
solrt_status solrt_batch_info(solrt_batch* batch, uint32_t* passes, uint32_t* items, uint64_t* paths);

/* ---- launch tuning ---------------------------------------------------------
 * No counterpart in the reference (its launch shape is the driver's). The
 * extend kernel's block size and the number of BVH2 traversal-stack slots
 * kept in shared memory, and the number of paths per batch pass, change
 * speed only: images are identical for every setting. */
typedef struct solrt_tune_config {
    uint32_t block_size;   /* extend threads per block: 64, 128 or 256 */
    uint32_t smem_stack;   /* BVH2 stack slots per thread in shared memory: 16 or 32 */
    uint32_t pass_paths;   /* paths per batch pass, <= the path capacity; 0 = the capacity */
    uint32_t reserved;
} solrt_tune_config;

typedef struct solrt_tune_result {
    solrt_tune_config best;
    float best_ms;         /* one launch of the timed jobs with `best` */
    float initial_ms;      /* the same with the configuration the call started from */
    uint32_t candidates;   /* configurations timed */
    uint32_t reserved;
} solrt_tune_result;

solrt_status solrt_context_get_tune(solrt_context* ctx, solrt_tune_config* out);
/* Applies to later launches and plans (a batch already captured into a CUDA
 * graph keeps its launch shape until it is re-planned). */
solrt_status solrt_context_set_tune(solrt_context* ctx, const solrt_tune_config* cfg);
/* Times the batch (at most 32 of its jobs, spread over it) under each extend
 * block size x shared stack depth (not for SOLRT_BATCH_COOPERATIVE batches,
 * whose kernel has one launch shape), then under pass sizes of 1/4, 1/2 and
 * all of the path capacity with the best of those, keeps the fastest on the
 * context and re-plans the batch with it. Each candidate is launched three
 * times (one warm-up): REF_MIX images of the timed jobs hold the last
 * launch's frame afterwards, KAHAN images the sum of all of them (clear
 * them before rendering for real). */
solrt_status solrt_batch_autotune(solrt_batch* batch, solrt_tune_result* out);

/* ---- autotune cache ---------------------------------------------------------
 * The winner of solrt_batch_autotune kept in a small text file (one JSON
 * object per line: key, block_size, smem_stack, pass_paths, best_ms) so that
 * a later process with a batch of the same shape skips the timing. The key
 * names the GPU (name and SM count), the BVH kind, the context's path
 * capacity, the batch flags and the jobs' shapes (sizes, spp, bounces,
 * modes, triangle counts; a 64-bit hash of them), not the cameras. */
#define SOLRT_TUNE_KEY_MAX 256u
/* The batch's cache key, NUL-terminated, into key[0..key_bytes). */
solrt_status solrt_batch_tune_key(solrt_batch* batch, char* key, size_t key_bytes);
/* Host only. SOLRT_OK with the entry of `key`; SOLRT_ERR_NOT_FOUND when the
 * file or the key is missing (lines that do not parse, or hold a launch
 * shape no kernel exists for, are skipped). */
solrt_status solrt_tune_cache_lookup(const char* path, const char* key, solrt_tune_config* cfg, float* best_ms);
/* Host only. Adds or replaces the entry of `key` (the file is rewritten
 * through a temporary file and a rename, so readers never see half a
 * file; of two processes storing at once, the later rename wins and the
 * other's new entry is lost). Keys hold no quote, backslash or control
 * character. */
solrt_status solrt_tune_cache_store(const char* path, const char* key, const solrt_tune_config* cfg, float best_ms);
/* solrt_batch_autotune through the cache at `path`: when it holds the
 * batch's key, applies that configuration to the context and re-plans the
 * batch (no timing; out->candidates = 0, *hit = 1); otherwise autotunes and
 * stores the winner (*hit = 0). */
solrt_status solrt_batch_autotune_cached(solrt_batch* batch, const char* path, solrt_tune_result* out,
                                         uint32_t* hit);

/* ------------------------------------------------------------------------ */
/* Serving: continuous batching of render jobs                              */
/* ------------------------------------------------------------------------ */
/* No counterpart in the reference (an interactive single-window renderer):
 * the served-jobs workload, each job rendered as solrt_render renders it. */

typedef enum solrt_serve_policy {
    /* every active job gets an equal share of each tick's paths */
    SOLRT_SERVE_FAIR = 0,
    /* jobs with the least remaining work (pixels x samples left) first, each
     * taking as many of its remaining samples as the tick has room for:
     * short jobs finish in one tick while long ones wait */
    SOLRT_SERVE_SHORTEST_FIRST = 1
} solrt_serve_policy;

typedef struct solrt_server_desc {
    uint64_t memory_budget;   /* bytes of job images + scenes in use; 0 = 150 GB */
    /* paths per tick; 0 = adaptive: each tick is sized to about tick_ms of
     * device time at the rate measured over the previous ticks, between 1M
     * paths and the context's path capacity (the first tick: 8M) */
    uint32_t tick_paths;
    uint32_t policy;          /* solrt_serve_policy */
    /* host-side fault injection for tests: the next this-many admissions
     * fail as if their image allocation had failed (SOLRT_ERR_OOM) */
    uint32_t inject_alloc_failures;
    /* > 0: convergence stopping rule. After each tick, once a job has at
     * least stop_min_spp samples, its image's RMSE against the converged
     * image (the mean over all samples it could take) is estimated from the
     * per-pixel sample variance: sqrt(mean over pixels and RGB of
     * variance / samples). The job completes early, with the samples it has,
     * once the estimate is at most stop_rmse; otherwise it runs its spp.
     * The server keeps one float of squared sample sums per pixel for such
     * jobs. 0 = every job runs all of its spp. */
    float stop_rmse;
    uint32_t stop_min_spp;    /* samples before the first estimate; 0 = 4 */
    uint32_t tick_ms;         /* adaptive ticks: target device time per tick; 0 = 40 ms */
} solrt_server_desc;

typedef struct solrt_job_result {
    uint32_t status;          /* SOLRT_OK when done, SOLRT_ERR_NOT_READY before */
    uint32_t spp_done;        /* samples accumulated (below spp when the job stopped early) */
    uint64_t latency_ns;      /* submit -> last sample accumulated and image final */
    uint64_t queue_ns;        /* submit -> admitted */
    solrt_image* image;       /* owned by the server until released or evicted */
    float rmse_estimate;      /* last convergence estimate (stop_rmse > 0), else -1 */
    uint32_t stopped_early;   /* 1 when the stopping rule ended the job before its spp */
} solrt_job_result;

typedef struct solrt_server_stats {
    uint64_t submitted, admitted, completed, evicted;
    uint64_t ticks;
    uint64_t segments;
    uint32_t queue_depth;     /* submitted, not yet admitted */
    uint32_t active;          /* admitted, not yet complete */
    uint64_t bytes_in_use;
    double busy_ms;           /* device time of all ticks */
    uint64_t stopped_early;   /* jobs completed by the stopping rule */
    uint32_t tick_paths;      /* size of the last tick */
    uint32_t reserved;
} solrt_server_stats;

/* A serving thread owns the context's stream until solrt_server_destroy:
 * meanwhile no other render, trace or batch call may use that context (use
 * a second context). Each tick it admits waiting jobs in arrival order
 * while their image (and scene, when not already counted) fits the memory
 * budget, evicting the least recently completed unreleased results first;
 * then it runs one wavefront pass in which every active job advances by its
 * share of tick_paths (at least one sample; a job with more pixels than a
 * tick runs one sample per tick), and finalizes the jobs that reached their
 * spp (or, with stop_rmse, converged). A job's image equals solrt_render of
 * the same job alone with the samples it took (spp_done). */
solrt_status solrt_server_create(solrt_context* ctx, const solrt_server_desc* desc, solrt_server** out);
/* Queues a job: the server allocates its image (params.width x height). */
solrt_status solrt_server_submit(solrt_server* srv, solrt_scene* scene, const solrt_camera* camera,
                                 const solrt_render_params* params, uint64_t* ticket);
/* SOLRT_OK with the result when done; SOLRT_ERR_NOT_READY while queued or
 * running; SOLRT_ERR_NOT_FOUND for an unknown, released or evicted ticket. */
solrt_status solrt_server_poll(solrt_server* srv, uint64_t ticket, solrt_job_result* out);
/* Waits up to timeout_ms for the ticket (bounded wait). */
solrt_status solrt_server_wait(solrt_server* srv, uint64_t ticket, uint32_t timeout_ms, solrt_job_result* out);
/* Frees a completed job's image. */
solrt_status solrt_server_release(solrt_server* srv, uint64_t ticket);
/* Cancels a queued or running job: a queued job leaves the queue at once, a
 * running one after the tick in flight (a job whose last samples are in that
 * tick completes normally); its memory is freed and poll / wait then return
 * SOLRT_ERR_CANCELLED until it is released. SOLRT_ERR_INVALID for a job that
 * has already finished. */
solrt_status solrt_server_cancel(solrt_server* srv, uint64_t ticket);
/* The completion queue: tickets of jobs that reached their final state
 * (done, failed, cancelled) since the last call, oldest first, at most
 * `max` of them (the rest stay for the next call); *n = how many. A client
 * with thousands of jobs in flight fetches these and polls only them. The
 * queue holds the newest 2^20 tickets not yet fetched (older ones drop). */
solrt_status solrt_server_finished(solrt_server* srv, uint64_t* tickets, uint32_t max, uint32_t* n);
solrt_status solrt_server_get_stats(solrt_server* srv, solrt_server_stats* out);
/* Stops the serving thread (unfinished jobs are dropped) and frees images. */
solrt_status solrt_server_destroy(solrt_server* srv);

/* Closest-hit queries (one traceRayEXT each, opaque, no culling); n below
 * 2^31 (SOLRT_ERR_INVALID otherwise).
 * Host arrays; synchronises. */
solrt_status solrt_trace_rays(solrt_context* ctx, solrt_scene* scene, const solrt_ray* rays,
                              uint32_t n, solrt_hit* hits);
/* Device arrays; asynchronous on the context stream. */
solrt_status solrt_trace_rays_device(solrt_context* ctx, solrt_scene* scene,
                                     const solrt_ray* rays_dev, uint32_t n, solrt_hit* hits_dev);

/* Device-side unit functions for known-answer tests (host in, host out).
 * op: 0 = tea(a[i], b[i]) -> out_u32; 1 = nextRand sequence of length b[0]
 * from seed a[0] -> out_f32 + final state in out_u32[0]; 2 = sincos of
 * in_f32[i] -> out_f32[2i], out_f32[2i+1]; 3-7 = the sampling functions,
 * miss colour and gamma (see the tests); 8 = the bounded wait of the
 * cooperative batch's grid barrier: a cooperative grid in which one block
 * never arrives, each wait limited to in_f32[0] seconds (at most 10), its
 * error flags -> out_u32[0] (SOLRT_EFLAG_TIMEOUT when the waits gave up).
 * Synchronises. */
solrt_status solrt_debug_unit(solrt_context* ctx, uint32_t op, uint32_t n, const uint32_t* a,
                              const uint32_t* b, const float* in_f32, uint32_t* out_u32,
                              float* out_f32);

/* ------------------------------------------------------------------------ */
/* glTF 2.0 scene input                                                     */
/* ------------------------------------------------------------------------ */

typedef struct solrt_gltf solrt_gltf;

/* Reads a .gltf (JSON with external .bin or base64 data URIs) or .glb file
 * into host arrays, as load_scene does (src/scene/mod.rs:138-295): one
 * section per mesh primitive with its material; POSITION, NORMAL (default
 * 0,1,0), COLOR_0 (default 1,1,1,1), TEXCOORD_0 (default 0); u8/u16/u32
 * indices; every primitive of a mesh gets the mesh's global transform
 * (calc_mesh_global_transform, src/scene/mod.rs:124-136) and its
 * inverse-transpose. Primitives without a material use a default one
 * (base colour 1, metallic 1, roughness 1, as glTF specifies). */
solrt_status solrt_gltf_load(const char* path, solrt_gltf** out);
/* Scene description over the loaded arrays (valid until solrt_gltf_destroy). */
solrt_status solrt_gltf_scene_desc(const solrt_gltf* g, solrt_scene_desc* out);
/* The first perspective camera: its node matrix taken as the view matrix and
 * yfov taken in degrees, as Camera::from_view and update_persp do
 * (src/scene/camera.rs:73-106). SOLRT_ERR_NOT_FOUND when there is none. */
solrt_status solrt_gltf_camera(const solrt_gltf* g, float aspect, solrt_camera* out);
solrt_status solrt_gltf_destroy(solrt_gltf* g);

/* ------------------------------------------------------------------------ */
/* Allocation-free BVH build (no counterpart in the reference)              */
/* ------------------------------------------------------------------------ */

/* Largest triangle count solrt_bvh2_build_noalloc accepts. */
#define SOLRT_NOALLOC_MAX_TRIS 65536u

/* Builds the same BVH2 as solrt_scene_create / solrt_scene_build_bvh, for
 * callers that must not allocate device memory: a real-time frame loop that
 * rebuilds a moving mesh's hierarchy every frame cannot afford cudaMalloc /
 * cudaFree (they may synchronise the whole device and stall the frame), and
 * a plugin that is handed device buffers by its host application may have
 * no allocator of its own. The caller passes the inputs and outputs in
 * device memory; the library's temporary data (sort keys, hierarchy links,
 * boxes) lives in a fixed scratch array compiled into the library, about
 * 5.5 MB, which every GPU that loads the library holds until the process
 * exits.
 *
 *   vpos      float4 per vertex (world position in .xyz), 16-byte aligned
 *   tri_idx   uint4 per triangle (v0, v1, v2, material), 16-byte aligned;
 *             every vertex index must be below the number of float4 in
 *             vpos (the call takes no vertex count and cannot check them:
 *             an index past the end makes the build read out of bounds)
 *   nodes     output, 64 * max(tri_count - 1, 1) bytes (BVH2 node layout of
 *             solrt_scene_bvh_export)
 *   tris      output, 48 * tri_count bytes (triangles in leaf order)
 *   stream    cudaStream_t to run on (NULL = the legacy default stream)
 *
 * Work is queued on `stream` and the call returns without waiting. Up to
 * SOLRT_NOALLOC_MAX_TRIS triangles; more returns SOLRT_ERR_CAPACITY. Every
 * call looks up the scratch array's device address in the CUDA context
 * current at the call (cudaGetSymbolAddress, a host-side query; nothing is
 * cached, so a context created again after cudaDeviceReset, or a host
 * application's own context, gets its own address); make the first call
 * on a device before any stream capture, since that first lookup loads the
 * library's device code into the context. All calls share the one scratch array: calls
 * whose work overlaps on the GPU (different streams without ordering)
 * race and corrupt each other's result; order them on one stream or with
 * events. The call clears the parts of the scratch that must start at zero,
 * so leftovers of an earlier call do no harm. */
solrt_status solrt_bvh2_build_noalloc(const void* vpos, const void* tri_idx, uint32_t tri_count, void* nodes,
                                      size_t nodes_bytes, void* tris, size_t tris_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SOLRT_H */
