// ref_glsl.cpp — the reference's own shaders, mechanically rewritten to
// C++ by build_ref.py into oracle/_ref, behind a C ABI. TEST INFRASTRUCTURE
// ONLY: golden vectors of the sampling functions (sampling.glsl /
// postprocess.glsl), and the path's ray-tracing pipeline (pathtrace.rgen,
// .rchit, .rmiss) run on CPU threads, with traceRayEXT answered by the
// closest-hit function the caller passes (the oracle's watertight traversal:
// the reference leaves intersection to the driver).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "glsl_shim.h"
#include "solrt.h"

namespace glsl {
#include "payload.glsl.inc"

// the sampling / postprocess functions behind the golden vectors (C library
// sin / cos), in a namespace of their own so that calls on glsl:: vectors
// inside the pipeline namespaces find only those namespaces' copies
namespace golden {
#include "sampling.glsl.inc"
#include "postprocess.glsl.inc"
}

thread_local uvec3 gl_LaunchIDEXT;
thread_local uvec3 gl_LaunchSizeEXT;
thread_local int gl_InstanceID;
thread_local int gl_PrimitiveID;
thread_local vec3 gl_WorldRayOriginEXT;
thread_local vec3 gl_WorldRayDirectionEXT;
thread_local vec3 attribs;
thread_local Payload prd;
TraceFn g_trace = nullptr;

// each shader in its own namespace, with the shared sin / cos evaluation
// (the include guards of sampling.glsl / postprocess.glsl are reset so that
// every namespace compiles its own copy against those)
#define REF_PIPELINE_TRIG                                    \
    inline float sin(float x) { return poly_sin(x); }        \
    inline float cos(float x) { return poly_cos(x); }
#undef SAMPLING_GLSL
#undef POSTPROCESS_GLSL
namespace ref_rgen {
REF_PIPELINE_TRIG
#include "pathtrace.rgen.inc"
}
#undef SAMPLING_GLSL
#undef POSTPROCESS_GLSL
namespace ref_rchit {
REF_PIPELINE_TRIG
#include "pathtrace.rchit.inc"
}
#undef SAMPLING_GLSL
#undef POSTPROCESS_GLSL
namespace ref_rmiss {
REF_PIPELINE_TRIG
#include "pathtrace.rmiss.inc"
}
// the AO pipeline (examples/4-ray-ao.rs)
#undef SAMPLING_GLSL
namespace ref_ao_rgen {
REF_PIPELINE_TRIG
#include "ao.rgen.inc"
}
#undef SAMPLING_GLSL
namespace ref_ao_rchit {
REF_PIPELINE_TRIG
#include "ao.rchit.inc"
}
namespace ref_ao_rmiss {
#include "ao.rmiss.inc"
}
// the debug pipeline (examples/3-ray-debug.rs): its payload is one vec3
thread_local vec3 hitValue;
namespace ref_dbg_rgen {
#include "debug.rgen.inc"
}
namespace ref_dbg_rchit {
#include "debug.rchit.inc"
}
namespace ref_dbg_rmiss {
#include "debug.rmiss.inc"
}
}  // namespace glsl

#undef in

static_assert(sizeof(glsl::ref_rchit::ModelVertex) == sizeof(solrt_vertex), "ModelVertex layout");
static_assert(sizeof(glsl::ref_rchit::MaterialInfo) == sizeof(solrt_material), "MaterialInfo layout");
static_assert(sizeof(glsl::ref_rchit::SceneInstance) == sizeof(solrt_instance), "SceneInstance layout");

extern "C" {
// closest hit of (o, d) in [tmin, tmax]: 1 and the triangle (index in the
// scene's section order) with its barycentrics (u, v) of vertices 1 and 2,
// or 0 for a miss
typedef int (*ref_hit_fn)(const void* ctx, const float* o, const float* d, float tmin, float tmax, uint32_t* prim,
                          float* u, float* v);
}

namespace {

enum Pipeline { kPath, kAo, kDebug };

struct PathState {
    Pipeline pipeline = kPath;
    ref_hit_fn hit = nullptr;
    const void* hit_ctx = nullptr;
    std::vector<uint32_t> sec_first;  // first triangle of each section (+ total)
    std::atomic<uint64_t> rays{0};    // traceRayEXT calls
};
PathState* g_path = nullptr;

void trace_ray(glsl::vec3 o, float tmin, glsl::vec3 d, float tmax) {
    g_path->rays.fetch_add(1, std::memory_order_relaxed);
    glsl::gl_WorldRayOriginEXT = o;
    glsl::gl_WorldRayDirectionEXT = d;
    const float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
    uint32_t prim = 0;
    float u = 0.0f, v = 0.0f;
    if (g_path->hit(g_path->hit_ctx, of, df, tmin, tmax, &prim, &u, &v)) {
        const auto& f = g_path->sec_first;
        const size_t s = (size_t)(std::upper_bound(f.begin(), f.end(), prim) - f.begin()) - 1;
        glsl::gl_InstanceID = (int)s;
        glsl::gl_PrimitiveID = (int)(prim - f[s]);
        glsl::attribs = glsl::vec3{u, v, 0.0f};
        if (g_path->pipeline == kPath) glsl::ref_rchit::main();
        else if (g_path->pipeline == kAo) glsl::ref_ao_rchit::main();
        else glsl::ref_dbg_rchit::main();
    } else {
        if (g_path->pipeline == kPath) glsl::ref_rmiss::main();
        else if (g_path->pipeline == kAo) glsl::ref_ao_rmiss::main();
        else glsl::ref_dbg_rmiss::main();
    }
}

// The closest-hit shaders' buffers (pathtrace.rchit / ao.rchit bindings 3-6)
// from a scene description: instances (identity when absent, id = section),
// each section's vertices and u64 indices (src/scene/mod.rs:228-233), and
// each instance's material.
struct SceneBufs {
    std::vector<solrt_instance> inst;
    std::vector<const solrt_vertex*> verts;
    std::vector<std::vector<uint64_t>> idx64;
    std::vector<solrt_material> mats;
};

bool scene_bufs(const solrt_scene_desc* desc, SceneBufs& b, PathState& st) {
    static const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    const uint32_t S = desc->section_count;
    b.inst.resize(S);
    b.verts.resize(S);
    b.idx64.resize(S);
    b.mats.resize(S);
    uint32_t first = 0;
    for (uint32_t s = 0; s < S; ++s) {
        const solrt_section& sec = desc->sections[s];
        if (sec.material_index >= desc->material_count) return false;
        if (desc->instances) {
            b.inst[s] = desc->instances[s];
        } else {
            b.inst[s] = solrt_instance{};
            b.inst[s].id = s;
            std::memcpy(b.inst[s].transform, ident, sizeof(ident));
            std::memcpy(b.inst[s].transform_it, ident, sizeof(ident));
        }
        b.verts[s] = desc->vertices + sec.vertex_offset;
        b.idx64[s].assign(desc->indices + sec.index_offset, desc->indices + sec.index_offset + sec.index_count);
        b.mats[s] = desc->materials[sec.material_index];
        st.sec_first.push_back(first);
        first += sec.index_count / 3;
    }
    st.sec_first.push_back(first);
    return true;
}

// rgen main over rows [r0, r1) of a W x H launch on `threads` threads
template <class F>
void launch_rows(uint32_t width, uint32_t height, uint32_t r0, uint32_t r1, int threads, F rgen) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    threads = std::min<int>(threads, (int)(r1 - r0));
    auto rows = [&](int t) {
        for (uint32_t y = r0 + (uint32_t)t; y < r1; y += (uint32_t)threads) {
            for (uint32_t x = 0; x < width; ++x) {
                glsl::gl_LaunchIDEXT = glsl::uvec3{x, y, 0u};
                glsl::gl_LaunchSizeEXT = glsl::uvec3{width, height, 1u};
                rgen();
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(rows, t);
    rows(0);
    for (auto& th : pool) th.join();
}

glsl::mat4 to_mat4(const float* m) {
    glsl::mat4 r;
    for (int c = 0; c < 4; ++c) r.c[c] = glsl::vec4{m[4 * c], m[4 * c + 1], m[4 * c + 2], m[4 * c + 3]};
    return r;
}

}  // namespace

extern "C" {

uint32_t ref_tea(uint32_t a, uint32_t b) { return glsl::golden::tea(a, b); }

float ref_next_rand(uint32_t* state) {
    glsl::uint s = *state;
    const float r = glsl::golden::nextRand(s);
    *state = s;
    return r;
}

void ref_next_rand2(uint32_t* state, float out[2]) {
    glsl::uint s = *state;
    const glsl::vec2 r = glsl::golden::nextRand2(s);
    *state = s;
    out[0] = r.x;
    out[1] = r.y;
}

void ref_sample_ggx(const float n[3], float xi0, float xi1, float alpha2, float out[3]) {
    const glsl::vec3 r = glsl::golden::sampleGGXDistribution(glsl::vec3{n[0], n[1], n[2]}, glsl::vec2{xi0, xi1}, alpha2);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void ref_sample_cosine(const float n[3], float xi0, float xi1, float out[3]) {
    const glsl::vec3 r = glsl::golden::sampleCosineWeightedHemisphere(glsl::vec3{n[0], n[1], n[2]}, glsl::vec2{xi0, xi1});
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

float ref_fresnel(const float i[3], const float m[3], float eta) {
    return glsl::golden::fresnelDielectric(glsl::vec3{i[0], i[1], i[2]}, glsl::vec3{m[0], m[1], m[2]}, eta);
}

void ref_onb(const float n[3], float u[3], float v[3]) {
    glsl::vec3 a, b;
    glsl::golden::buildOrthonormalBasis(glsl::vec3{n[0], n[1], n[2]}, a, b);
    u[0] = a.x; u[1] = a.y; u[2] = a.z;
    v[0] = b.x; v[1] = b.y; v[2] = b.z;
}

// One launch of examples/5-pathtrace.rs: pathtrace.rgen over the pixels of
// rows [row_begin, row_end) of a W x H launch (all rows when row_end is 0;
// 8 samples, at most 32 bounces, as the shader fixes), with scene.frame.z =
// frame and push.accum_start_frame = accum_start; `accum` (RGBA32F, read and
// written) and `rgba8` are the two storage images (full W x H). sky sets the
// miss shader's ENABLE_SKYLIGHT. `rays` (optional) receives the number of
// traceRayEXT calls. Renders are not reentrant.
int ref_path_render(const solrt_scene_desc* desc, const float* view_inverse, const float* projection_inverse,
                    uint32_t width, uint32_t height, uint32_t frame, int32_t accum_start, int sky, float* accum,
                    uint8_t* rgba8, ref_hit_fn hit, const void* hit_ctx, int threads, uint32_t row_begin,
                    uint32_t row_end, uint64_t* rays) {
    using namespace glsl;
    if (!desc || !view_inverse || !projection_inverse || !accum || !rgba8 || !hit || width == 0 || height == 0)
        return 1;
    static const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    const uint32_t S = desc->section_count;
    PathState st;
    st.hit = hit;
    st.hit_ctx = hit_ctx;
    std::vector<ref_rchit::SceneInstance> inst(S);
    std::vector<ref_rchit::Vertices> verts(S);
    std::vector<std::vector<uint64_t>> idx64(S);
    std::vector<ref_rchit::Indices> idx(S);
    std::vector<ref_rchit::MatBuffer> mats(S);
    uint32_t first = 0;
    for (uint32_t s = 0; s < S; ++s) {
        const solrt_section& sec = desc->sections[s];
        if (sec.material_index >= desc->material_count) return 1;
        if (desc->instances) {
            std::memcpy(&inst[s], &desc->instances[s], sizeof(solrt_instance));
        } else {
            solrt_instance id{};
            id.id = s;
            std::memcpy(id.transform, ident, sizeof(ident));
            std::memcpy(id.transform_it, ident, sizeof(ident));
            std::memcpy(&inst[s], &id, sizeof(id));
        }
        verts[s].v = reinterpret_cast<const ref_rchit::ModelVertex*>(desc->vertices + sec.vertex_offset);
        idx64[s].assign(desc->indices + sec.index_offset, desc->indices + sec.index_offset + sec.index_count);
        idx[s].i = idx64[s].data();
        std::memcpy(&mats[s].mat, &desc->materials[sec.material_index], sizeof(solrt_material));
        st.sec_first.push_back(first);
        first += sec.index_count / 3;
    }
    st.sec_first.push_back(first);
    ref_rchit::scnDesc.i = inst.data();
    ref_rchit::vertices = verts.data();
    ref_rchit::indices = idx.data();
    ref_rchit::materials = mats.data();
    ref_rgen::scene.view_inverse = to_mat4(view_inverse);
    ref_rgen::scene.projection_inverse = to_mat4(projection_inverse);
    ref_rgen::scene.frame = uvec3{width, height, frame};
    ref_rgen::push.accum_start_frame = accum_start;
    ref_rgen::accumImage = image2D{accum, nullptr, (int)width};
    ref_rgen::renderImage = image2D{nullptr, rgba8, (int)width};
    ref_rmiss::ENABLE_SKYLIGHT = sky ? 1 : 0;
    g_path = &st;
    g_trace = trace_ray;
    if (row_end == 0 || row_end > height) row_end = height;
    if (row_begin >= row_end) return 1;
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    threads = std::min<int>(threads, (int)(row_end - row_begin));
    auto rows = [&](int t) {
        for (uint32_t y = row_begin + (uint32_t)t; y < row_end; y += (uint32_t)threads) {
            for (uint32_t x = 0; x < width; ++x) {
                gl_LaunchIDEXT = uvec3{x, y, 0u};
                gl_LaunchSizeEXT = uvec3{width, height, 1u};
                ref_rgen::main();
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(rows, t);
    rows(0);
    for (auto& th : pool) th.join();
    g_path = nullptr;
    if (rays) *rays = st.rays.load();
    return 0;
}

// One launch of examples/4-ray-ao.rs: ao.rgen (4 samples, at most 4 hits per
// sample, as the shader fixes) with ao.rchit / ao.rmiss over rows [row_begin,
// row_end) of a W x H launch (all rows when row_end is 0). `accum` is the
// RGBA32F render target the example allocates (4-ray-ao.rs:58), read and
// written; `noise` the RGBA8 blue-noise texture (nw x nh texels, rows as the
// loader uploads them).
int ref_ao_render(const solrt_scene_desc* desc, const float* view_inverse, const float* projection_inverse,
                  uint32_t width, uint32_t height, uint32_t frame, int32_t accum_start, const uint8_t* noise,
                  uint32_t nw, uint32_t nh, float* accum, ref_hit_fn hit, const void* hit_ctx, int threads,
                  uint32_t row_begin, uint32_t row_end, uint64_t* rays) {
    using namespace glsl;
    if (!desc || !view_inverse || !projection_inverse || !accum || !noise || !hit || width == 0 || height == 0 ||
        nw == 0 || nh == 0)
        return 1;
    PathState st;
    st.pipeline = kAo;
    st.hit = hit;
    st.hit_ctx = hit_ctx;
    SceneBufs b;
    if (!scene_bufs(desc, b, st)) return 1;
    const uint32_t S = desc->section_count;
    std::vector<ref_ao_rchit::SceneInstance> inst(S);
    std::vector<ref_ao_rchit::Vertices> verts(S);
    std::vector<ref_ao_rchit::Indices> idx(S);
    for (uint32_t s = 0; s < S; ++s) {
        std::memcpy(&inst[s], &b.inst[s], sizeof(solrt_instance));
        verts[s].v = reinterpret_cast<const ref_ao_rchit::ModelVertex*>(b.verts[s]);
        idx[s].i = b.idx64[s].data();
    }
    ref_ao_rchit::scnDesc.i = inst.data();
    ref_ao_rchit::vertices = verts.data();
    ref_ao_rchit::indices = idx.data();
    ref_ao_rchit::blueNoise = sampler2D{noise, (int)nw, (int)nh};
    ref_ao_rgen::scene.view_inverse = to_mat4(view_inverse);
    ref_ao_rgen::scene.projection_inverse = to_mat4(projection_inverse);
    ref_ao_rgen::scene.frame = uvec3{width, height, frame};
    ref_ao_rgen::push.accum_start_frame = accum_start;
    ref_ao_rgen::image = image2D{accum, nullptr, (int)width};
    if (row_end == 0 || row_end > height) row_end = height;
    if (row_begin >= row_end) return 1;
    g_path = &st;
    g_trace = trace_ray;
    launch_rows(width, height, row_begin, row_end, threads, [] { ref_ao_rgen::main(); });
    g_path = nullptr;
    if (rays) *rays = st.rays.load();
    return 0;
}

// One launch of examples/3-ray-debug.rs: debug.rgen / .rchit / .rmiss into
// the RGBA8 render target the example allocates (3-ray-debug.rs:54).
int ref_debug_render(const solrt_scene_desc* desc, const float* view_inverse, const float* projection_inverse,
                     uint32_t width, uint32_t height, uint8_t* rgba8, ref_hit_fn hit, const void* hit_ctx,
                     int threads) {
    using namespace glsl;
    if (!desc || !view_inverse || !projection_inverse || !rgba8 || !hit || width == 0 || height == 0) return 1;
    PathState st;
    st.pipeline = kDebug;
    st.hit = hit;
    st.hit_ctx = hit_ctx;
    SceneBufs b;
    if (!scene_bufs(desc, b, st)) return 1;
    ref_dbg_rgen::scene.view_inverse = to_mat4(view_inverse);
    ref_dbg_rgen::scene.projection_inverse = to_mat4(projection_inverse);
    ref_dbg_rgen::scene.frame = uvec3{width, height, 0u};
    ref_dbg_rgen::image = image2D{nullptr, rgba8, (int)width};
    g_path = &st;
    g_trace = trace_ray;
    launch_rows(width, height, 0, height, threads, [] { ref_dbg_rgen::main(); });
    g_path = nullptr;
    return 0;
}

void ref_gamma(const float c[3], float power, float out[3]) {
    const glsl::vec3 r = glsl::golden::gammaCorrect(glsl::vec3{c[0], c[1], c[2]}, power);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void ref_tonemap_uncharted2(const float c[3], float out[3]) {
    const glsl::vec3 r = glsl::golden::tonemapUncharted2(glsl::vec3{c[0], c[1], c[2]});
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void ref_tonemap_aces(const float c[3], float out[3]) {
    const glsl::vec3 r = glsl::golden::ACESFilm(glsl::vec3{c[0], c[1], c[2]});
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

}  // extern "C"
