/*
 * oracle.h — CPU oracle of the solrt path tracer. TEST INFRASTRUCTURE ONLY.
 *
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark
 * load this library, and only as the checker: no product code links it.
 *
 * It restates, in scalar C++ templated on the real type (float / double):
 *   - assets/glsl/sampling.glsl:18-96   tea, nextRand, fresnelDielectric,
 *                                       buildOrthonormalBasis, alignToDirection,
 *                                       sampleGGXDistribution,
 *                                       sampleCosineWeightedHemisphere
 *   - assets/glsl/pathtrace.rgen:28-104 camera ray, sample loop, accumulation
 *   - assets/glsl/pathtrace.rchit:56-113 closest-hit shading
 *   - assets/glsl/pathtrace.rmiss:8-21  miss shading
 *   - assets/glsl/postprocess.glsl:38-41 gamma
 *   - src/ray/mod.rs:113-118            per-section transform / transform_it
 * plus what the reference delegates to the Vulkan driver and RT cores (no
 * source): a watertight ray-triangle test (Woop, Benthin, Wald 2013) with an
 * FP64 fallback on zero edge functions, closest-hit tie-break on the lower
 * global triangle index, a CPU LBVH (30-bit Morton, Karras 2012 hierarchy)
 * and brute force.
 *
 * Parity: sampling.glsl and postprocess.glsl are pinned against the
 * reference's own GLSL source compiled as C++ (golden vectors under
 * tests/golden), and the whole path against the reference's
 * pathtrace.rgen / .rchit / .rmiss compiled as C++ and run as a CPU
 * pipeline (oracle/ref_glsl; traceRayEXT answered by oracle_closest_hit):
 * equal images bit for bit. Unpinned only where the reference has no source
 * (the Vulkan driver's BVH and intersection, and its sin / cos).
 */
#ifndef SOLRT_ORACLE_H
#define SOLRT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/solrt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_scene oracle_scene;

typedef struct oracle_render_stats {
    uint64_t segments;
    uint64_t paths;
    uint64_t fp64_fallbacks;
    uint64_t node_visits;
    uint64_t tri_tests;
    uint64_t shadow_segments;    /* SOLRT_INTEGRATOR_PATH_NEE shadow rays */
    uint64_t shadow_unoccluded;  /* of them, those that reached their light */
} oracle_render_stats;

/* Flattens to world space and builds the CPU LBVH. NULL on error. */
oracle_scene* oracle_scene_create(const solrt_scene_desc* desc);
void oracle_scene_destroy(oracle_scene* s);
/* on != 0: closest hits as a two-level scene (SOLRT_BVH2_TWO_LEVEL): each
 * section's triangles in object space, the ray entering through the
 * section's inverse transform (brute force over sections and triangles). */
void oracle_scene_set_two_level(oracle_scene* s, int on);
/* Closest hit of one ray (the oracle's watertight traversal, FP32): 1 and
 * the triangle index (sections' order) with the barycentrics u, v of
 * vertices 1 and 2, or 0 for a miss. `scene` is an oracle_scene; the
 * signature is the one the reference-shader pipeline (oracle/ref_glsl) calls. */
int oracle_closest_hit(const void* scene, const float* o, const float* d, float tmin, float tmax, uint32_t* prim,
                       float* u, float* v);
uint32_t oracle_scene_tri_count(const oracle_scene* s);

/* World-space flattened geometry: per triangle 3 vertices x (pos, normal,
 * color) as float4 = 9 float4 (144 B) per triangle, and material index. */
int oracle_scene_export_world(const oracle_scene* s, float* tri_world, uint32_t* tri_material);

/* LBVH export. Internal node i (0..n-2): child refs (leaf = 0x80000000 | sorted
 * position), box lo/hi. order[k] = original triangle of sorted position k.
 * Returns the internal node count. */
uint32_t oracle_bvh_export(const oracle_scene* s, uint32_t* child_refs /* 2*(n-1) */,
                           float* boxes /* 6*(n-1): lo xyz, hi xyz */, uint32_t* order /* n */,
                           uint32_t* morton /* n, sorted */);

/* Closest hits. mode 0 = brute force, 1 = LBVH. threads 0 = all cores. */
int oracle_trace(const oracle_scene* s, const solrt_ray* rays, uint32_t n, solrt_hit* hits,
                 int mode, int threads, uint64_t* fp64_fallbacks);

/* One launch of the path tracer on the CPU. accum (W*H*4 floats) is read and
 * written (REF_MIX); kahan_sum / kahan_comp (W*H*4 floats each, .w of sum =
 * sample count) are read and written in KAHAN mode (else may be NULL);
 * rgba8 (W*H*4) is written. precision: 32 or 64. rows: if row_end > row_begin,
 * only rows [row_begin, row_end) are rendered (a bounded sample of the image).
 * Returns 0 on success. */
int oracle_render(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p,
                  float* accum, float* kahan_sum, float* kahan_comp, uint8_t* rgba8,
                  int precision, int threads, uint32_t row_begin, uint32_t row_end,
                  oracle_render_stats* stats);

/* oracle_render for every integrator (p->integrator): DEBUG and AO write
 * accum and rgba8 as the library does; AO needs the blue-noise texture
 * (noise_w x noise_h RGBA8 texels). */
int oracle_render_ex(const oracle_scene* s, const solrt_camera* cam, const solrt_render_params* p,
                     float* accum, float* kahan_sum, float* kahan_comp, uint8_t* rgba8,
                     int precision, int threads, uint32_t row_begin, uint32_t row_end,
                     oracle_render_stats* stats, const uint8_t* blue_noise, uint32_t noise_w,
                     uint32_t noise_h);

/* Per-path radiance of one launch, no accumulation: out[(pix*spp + s)*4]. */
int oracle_render_samples(const oracle_scene* s, const solrt_camera* cam,
                          const solrt_render_params* p, float* out, int precision, int threads);

/* Unit functions for known-answer tests. */
uint32_t oracle_tea(uint32_t a, uint32_t b);
float oracle_next_rand(uint32_t* state);
void oracle_sincos(float x, float* s, float* c);
/* sampling.glsl functions in FP32: out gets 3 floats. */
void oracle_sample_ggx(const float n[3], float xi0, float xi1, float alpha2, float out[3]);
void oracle_sample_cosine(const float n[3], float xi0, float xi1, float out[3]);
float oracle_fresnel(const float i[3], const float m[3], float eta);
void oracle_onb(const float n[3], float u[3], float v[3]);
float oracle_gamma(float c, float power);
void oracle_miss(const float dir[3], uint32_t mode, float out[3]);
void oracle_camera_look_at(const float eye[3], const float center[3], const float up[3],
                           float vfov_deg, float aspect, float znear, float zfar, solrt_camera* out);

#ifdef __cplusplus
}
#endif

#endif
