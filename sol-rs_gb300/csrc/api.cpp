// api.cpp — the C ABI of include/solrt.h.
//
// Host-side counterpart of the reference's per-path Rust objects:
//   solrt_context  ~ the Vulkan Context + queue (src/context.rs:222-575)
//   solrt_scene    ~ SceneDescription (src/ray/mod.rs:38-156): sections are
//                    flattened to world space with each section's transform
//                    and transform_it, uploaded, and an LBVH replaces the
//                    driver-built BLAS/TLAS
//   solrt_image    ~ the accumulation (RGBA32F) and render (RGBA8) images of
//                    examples/5-pathtrace.rs:222-229
//   solrt_render   ~ one `render` frame of examples/5-pathtrace.rs:294-369
// Errors are status codes with a per-thread message instead of the
// reference's panics (unwrap/expect).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "internal.h"

static_assert(sizeof(solrt_vertex) == 64, "ModelVertex is 64 bytes (src/scene/mesh.rs:9-14)");
static_assert(sizeof(solrt_material) == 48, "MaterialInfo is 48 bytes (src/scene/mod.rs:21-29)");
static_assert(sizeof(solrt_instance) == 144, "SceneInstance is 144 bytes (src/ray/mod.rs:18-24)");
static_assert(sizeof(solrt_ray) == 32, "solrt_ray is two float4");
static_assert(sizeof(solrt_hit) == 16, "solrt_hit is one float4");
static_assert(sizeof(solrt_camera) == 256, "four mat4");
static_assert(sizeof(solrt_server_desc) == 32 && sizeof(solrt_job_result) == 40 && sizeof(solrt_server_stats) == 88,
              "server structs (mirrored by the Python binding)");

struct solrt_context : solrt::Context {};
struct solrt_scene : solrt::Scene {};
struct solrt_image : solrt::Image {};
struct solrt_batch : solrt::Batch {};

namespace solrt {

namespace {
thread_local std::string g_last_error;
}

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

namespace {

#define CHECK_ARG(cond, msg)                         \
    do {                                             \
        if (!(cond)) {                               \
            ::solrt::set_error("%s", msg);           \
            return SOLRT_ERR_INVALID;                \
        }                                            \
    } while (0)

solrt_status check_device_flags(Context& ctx) {
    // block 0: path segments; block 1: shadow rays
    unsigned int fl[2] = {0u, 0u};
    DevStats* st = ctx.stats.as<DevStats>();
    for (int k = 0; k < 2; ++k)
        SOLRT_CUDA(cudaMemcpyAsync(&fl[k], &st[k].eflags, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx.stream));
    SOLRT_CUDA(cudaStreamSynchronize(ctx.stream));
    const unsigned int flags = fl[0] | fl[1];
    if (flags == 0) return SOLRT_OK;
    for (int k = 0; k < 2; ++k) SOLRT_CUDA(cudaMemsetAsync(&st[k].eflags, 0, sizeof(unsigned int), ctx.stream));
    SOLRT_CUDA(cudaStreamSynchronize(ctx.stream));
    set_error("device error flags 0x%x (1 stack overflow, 2 queue overflow, 4 bad index, 8 timeout)", flags);
    if (flags & SOLRT_EFLAG_TIMEOUT) return SOLRT_ERR_TIMEOUT;
    if (flags & SOLRT_EFLAG_INDEX) return SOLRT_ERR_DEVICE;
    return SOLRT_ERR_CAPACITY;
}

// glam-equivalent matrix maths in FP64 (src/scene/camera.rs:98-106).
void inverse4(const double* m, double* o, bool* ok) {
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
    *ok = det != 0.0 && std::isfinite(det);
    for (int i = 0; i < 16; ++i) o[i] = *ok ? inv[i] / det : 0.0;
}

solrt_status fill_camera(const double view[16], float vfov_deg, float aspect, float znear, float zfar,
                         solrt_camera* out) {
    CHECK_ARG(out, "null camera");
    CHECK_ARG(vfov_deg > 0.0f && vfov_deg < 180.0f, "vfov must be in (0, 180) degrees");
    CHECK_ARG(aspect > 0.0f && znear > 0.0f && zfar > znear, "bad aspect or depth range");
    // Mat4::perspective_rh(vfov.to_radians(), aspect, near, far)
    const double fov = (double)vfov_deg * 3.14159265358979323846 / 180.0;
    const double h = 1.0 / std::tan(0.5 * fov);
    const double w = h / (double)aspect;
    const double r = (double)zfar / ((double)znear - (double)zfar);
    const double proj[16] = {w, 0, 0, 0, 0, h, 0, 0, 0, 0, r, -1, 0, 0, r * znear, 0};
    double vi[16], pi[16];
    bool ok1 = false, ok2 = false;
    inverse4(view, vi, &ok1);
    inverse4(proj, pi, &ok2);
    CHECK_ARG(ok1 && ok2, "singular camera matrix");
    for (int i = 0; i < 16; ++i) {
        out->view[i] = (float)view[i];
        out->view_inverse[i] = (float)vi[i];
        out->projection[i] = (float)proj[i];
        out->projection_inverse[i] = (float)pi[i];
    }
    return SOLRT_OK;
}

std::mutex g_refs_mutex;

// Light tree of next-event estimation over the emissive triangles (emissive
// as pathtrace.rchit:75-80 decides it: any emissive channel >= 1; zero-area
// triangles cannot be hit and are left out). Lights sorted by the 30-bit
// Morton code of their centroid in the centroids' bounds (ties by triangle
// index), split at the middle of each range, so the tree is balanced. Each
// inner node holds both children, three float4: (left box centre, left
// squared half-diagonal), the same for the right child, (left power, right
// power, left ref, right ref as bits); a ref >= 0 is an inner node, < 0 the
// triangle ~ref. A leaf's power is area * ((Le.r + Le.g) + Le.b), a node's
// the sum left + right. One light: a root whose two refs are that light and
// whose right power is 0. Per light its code: (levels << 27) | branch bits
// (bit l set: right child at level l).
struct LightBuild {
    std::vector<uint32_t> prim, code;
    std::vector<float> lo, hi, power;  // per light: box (3 + 3), power
    std::vector<float4> nodes;
    static float4 sphere(const float mn[3], const float mx[3]) {
        const float hx = (mx[0] - mn[0]) * 0.5f, hy = (mx[1] - mn[1]) * 0.5f, hz = (mx[2] - mn[2]) * 0.5f;
        return make_float4((mn[0] + mx[0]) * 0.5f, (mn[1] + mx[1]) * 0.5f, (mn[2] + mx[2]) * 0.5f,
                           (hx * hx + hy * hy) + hz * hz);
    }
    static float as_float(int32_t v) {
        float f;
        std::memcpy(&f, &v, 4);
        return f;
    }
    int32_t build(const std::vector<uint32_t>& order, uint32_t b, uint32_t e, float bmin[3], float bmax[3],
                  float& pw, uint32_t bits, uint32_t level) {
        if (e - b == 1) {
            const uint32_t k = order[b];
            for (int c = 0; c < 3; ++c) {
                bmin[c] = lo[3 * k + c];
                bmax[c] = hi[3 * k + c];
            }
            pw = power[k];
            code[k] = (level << 27) | bits;
            return ~(int32_t)prim[k];
        }
        const uint32_t idx = (uint32_t)(nodes.size() / 3);
        nodes.resize(nodes.size() + 3);
        const uint32_t m = b + (e - b) / 2;
        float amin[3], amax[3], cmin[3], cmax[3], pa = 0.0f, pc = 0.0f;
        const int32_t l = build(order, b, m, amin, amax, pa, bits, level + 1);
        const int32_t r = build(order, m, e, cmin, cmax, pc, bits | (1u << level), level + 1);
        nodes[3 * idx] = sphere(amin, amax);
        nodes[3 * idx + 1] = sphere(cmin, cmax);
        nodes[3 * idx + 2] = make_float4(pa, pc, as_float(l), as_float(r));
        for (int c = 0; c < 3; ++c) {
            bmin[c] = std::min(amin[c], cmin[c]);
            bmax[c] = std::max(amax[c], cmax[c]);
        }
        pw = pa + pc;
        return (int32_t)idx;
    }
};

uint32_t expand10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// Tree over the candidates (emissive triangles in triangle order: their
// index and (v0, v1, v2, section)) at world positions `pos`; `tri_code`
// gets one code per triangle of the scene (`tri_count`).
std::vector<float4> build_light_tree(const std::vector<float4>& pos, const std::vector<uint32_t>& cand_prim,
                                     const std::vector<uint4>& cand_tri, const std::vector<uint32_t>& sec_mat,
                                     const std::vector<solrt_material>& mats, size_t tri_count, uint32_t& count,
                                     std::vector<uint32_t>& tri_code) {
    LightBuild lb;
    std::vector<float> cen;
    for (size_t ci = 0; ci < cand_tri.size(); ++ci) {
        const uint4 tr = cand_tri[ci];
        const solrt_material& m = mats[sec_mat[tr.w]];
        const float4 a = pos[tr.x], b = pos[tr.y], c = pos[tr.z];
        const float e1x = b.x - a.x, e1y = b.y - a.y, e1z = b.z - a.z;
        const float e2x = c.x - a.x, e2y = c.y - a.y, e2z = c.z - a.z;
        const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
        const float area = 0.5f * std::sqrt((nx * nx + ny * ny) + nz * nz);
        const float pw = area * ((m.emissive[0] + m.emissive[1]) + m.emissive[2]);
        if (!(area > 0.0f) || !(pw > 0.0f) || !std::isfinite(pw)) continue;
        lb.prim.push_back(cand_prim[ci]);
        const float v[3][3] = {{a.x, a.y, a.z}, {b.x, b.y, b.z}, {c.x, c.y, c.z}};
        for (int k = 0; k < 3; ++k) {
            lb.lo.push_back(std::min(std::min(v[0][k], v[1][k]), v[2][k]));
            lb.hi.push_back(std::max(std::max(v[0][k], v[1][k]), v[2][k]));
            cen.push_back(((v[0][k] + v[1][k]) + v[2][k]) / 3.0f);
        }
        lb.power.push_back(pw);
    }
    const uint32_t n = std::min<uint32_t>((uint32_t)lb.prim.size(), 1u << 26);  // codes hold 27 levels
    count = n;
    tri_code.assign(tri_count, ~0u);
    if (n == 0) return {};
    lb.code.assign(n, 0u);
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
            const uint32_t q = (uint32_t)std::min(std::max(f * 1023.0f, 0.0f), 1023.0f);
            code |= expand10(q) << (2 - k);
        }
        key[i] = {code, i};
    }
    std::sort(key.begin(), key.end());
    std::vector<uint32_t> order(n);
    for (uint32_t i = 0; i < n; ++i) order[i] = key[i].second;
    float bmin[3], bmax[3], pw = 0.0f;
    lb.nodes.reserve(3 * (size_t)n);
    const int32_t root = lb.build(order, 0, n, bmin, bmax, pw, 0u, 0u);
    if (root < 0) {  // one light
        const float4 sp = LightBuild::sphere(bmin, bmax);
        lb.nodes = {sp, sp, make_float4(pw, 0.0f, LightBuild::as_float(root), LightBuild::as_float(root))};
        lb.code[0] = 1u << 27;
    }
    tri_code.assign(tri_count, ~0u);
    for (uint32_t k = 0; k < n; ++k) tri_code[lb.prim[k]] = lb.code[k];
    return lb.nodes;
}

}  // namespace

solrt_status upload_light_tree(Scene& sc, const std::vector<float4>& pos, cudaStream_t st) {
    uint32_t count = 0;
    std::vector<uint32_t> tri_code;
    const std::vector<float4> nodes = build_light_tree(pos, sc.light_cand_prim, sc.light_cand_tri, sc.light_sec_mat,
                                                       sc.light_mats, sc.tri_count, count, tri_code);
    if (cudaMemcpyAsync(sc.tri_light.ptr, tri_code.data(), 4 * tri_code.size(), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        (!nodes.empty() && cudaMemcpyAsync(sc.lights.ptr, nodes.data(), sizeof(float4) * nodes.size(),
                                           cudaMemcpyHostToDevice, st) != cudaSuccess) ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("light tree upload failed");
        return SOLRT_ERR_DEVICE;
    }
    sc.light_count = count;
    return SOLRT_OK;
}

// Rebuilds the light tree from the scene's current world vertices (after
// instances moved), as a fresh scene with those positions would build it.
solrt_status refresh_light_tree(Context& ctx, Scene& sc) {
    if (sc.light_cand_prim.empty()) return SOLRT_OK;
    std::vector<float4> pos(sc.vertex_count);
    SOLRT_CUDA(cudaMemcpyAsync(pos.data(), sc.vpos.ptr, sizeof(float4) * pos.size(), cudaMemcpyDeviceToHost,
                               ctx.stream));
    SOLRT_CUDA(cudaStreamSynchronize(ctx.stream));
    return upload_light_tree(sc, pos, ctx.stream);
}

}  // namespace solrt

using namespace solrt;

// Reference counting of contexts (see Context::refs).
static void context_retain(solrt_context* c) {
    std::lock_guard<std::mutex> lock(g_refs_mutex);
    ++c->refs;
}

static void context_release(solrt_context* c) {
    {
        std::lock_guard<std::mutex> lock(g_refs_mutex);
        if (--c->refs > 0) return;
    }
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (auto& t : c->timed) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.end);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    cudaGetLastError();
    delete c;
}

extern "C" {

uint32_t solrt_abi_version(void) { return SOLRT_ABI_VERSION; }

const char* solrt_status_string(solrt_status s) {
    switch (s) {
        case SOLRT_OK: return "ok";
        case SOLRT_ERR_INVALID: return "invalid argument";
        case SOLRT_ERR_OOM: return "out of memory";
        case SOLRT_ERR_DEVICE: return "device error";
        case SOLRT_ERR_TIMEOUT: return "timeout";
        case SOLRT_ERR_CAPACITY: return "capacity exceeded";
        case SOLRT_ERR_NOT_READY: return "not ready";
        case SOLRT_ERR_NOT_FOUND: return "not found";
        case SOLRT_ERR_BUDGET: return "over memory budget";
        case SOLRT_ERR_CANCELLED: return "cancelled";
    }
    return "unknown status";
}

const char* solrt_last_error(void) { return g_last_error.c_str(); }

solrt_status solrt_context_create(const solrt_context_desc* desc, solrt_context** out) {
    CHECK_ARG(out, "null output");
    *out = nullptr;
    solrt_context_desc d{};
    if (desc) d = *desc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return SOLRT_ERR_DEVICE;
    }
    CHECK_ARG(d.device >= 0 && d.device < ndev, "device ordinal out of range");
    SOLRT_CUDA(cudaSetDevice(d.device));
    cudaDeviceProp prop;
    SOLRT_CUDA(cudaGetDeviceProperties(&prop, d.device));
    if (prop.major * 10 + prop.minor != 103) {
        set_error("solrt is built for sm_103a (GB300); device %d is sm_%d%d", d.device, prop.major, prop.minor);
        return SOLRT_ERR_DEVICE;
    }
    solrt_context* c = new (std::nothrow) solrt_context();
    if (!c) return SOLRT_ERR_OOM;
    c->device = d.device;
    c->sm_count = prop.multiProcessorCount;
    c->capacity = d.path_capacity ? d.path_capacity : (32u << 20);
    c->counters = d.enable_counters != 0;
    c->block_size = d.block_size;
    if (d.block_size) {
        if (!extend_variant_ok(d.block_size, c->tune.smem)) {
            set_error("block_size must be 64, 128 or 256");
            delete c;
            return SOLRT_ERR_INVALID;
        }
        c->tune.block = d.block_size;
    }
    c->timing = d.enable_timing != 0;
    auto fail = [&](solrt_status s) {
        solrt_context_destroy(c);
        return s;
    };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        return fail(SOLRT_ERR_DEVICE);
    }
    if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
        set_error("cudaEventCreate failed");
        return fail(SOLRT_ERR_DEVICE);
    }
    const size_t C = c->capacity;
    for (int i = 0; i < 2; ++i) {
        solrt_status s;
        if ((s = c->q_o[i].alloc(16 * C)) != SOLRT_OK) return fail(s);
        if ((s = c->q_d[i].alloc(16 * C)) != SOLRT_OK) return fail(s);
        if ((s = c->q_thr[i].alloc(16 * C)) != SOLRT_OK) return fail(s);
        if ((s = c->q_meta[i].alloc(8 * C)) != SOLRT_OK) return fail(s);
    }
    solrt_status s;
    if ((s = c->hits.alloc(16 * C)) != SOLRT_OK) return fail(s);
    if ((s = c->rad.alloc(16 * C)) != SOLRT_OK) return fail(s);
    if ((s = c->ctl.alloc(sizeof(PassCtl))) != SOLRT_OK) return fail(s);
    if ((s = c->stats.alloc(2 * sizeof(DevStats))) != SOLRT_OK) return fail(s);
    if ((s = c->trace_work.alloc(sizeof(unsigned int))) != SOLRT_OK) return fail(s);
    if (cudaMemset(c->ctl.ptr, 0, sizeof(PassCtl)) != cudaSuccess ||
        cudaMemset(c->stats.ptr, 0, 2 * sizeof(DevStats)) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {
        set_error("device initialisation failed");
        return fail(SOLRT_ERR_DEVICE);
    }
    *out = c;
    return SOLRT_OK;
}

solrt_status solrt_context_destroy(solrt_context* ctx) {
    if (!ctx) return SOLRT_OK;
    context_release(ctx);
    return SOLRT_OK;
}

void* solrt_context_stream(solrt_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

solrt_status solrt_context_set_blue_noise(solrt_context* ctx, const uint8_t* rgba8, uint32_t width,
                                          uint32_t height) {
    CHECK_ARG(ctx && rgba8, "null argument");
    CHECK_ARG(width > 0 && height > 0 && (uint64_t)width * height <= (1ull << 26), "bad texture size");
    SOLRT_CUDA(cudaSetDevice(ctx->device));
    SOLRT_CUDA(cudaStreamSynchronize(ctx->stream));  // launches in flight may read the old texture
    SOLRT_TRY(ctx->blue_noise.alloc(4ull * width * height));
    SOLRT_CUDA(cudaMemcpyAsync(ctx->blue_noise.ptr, rgba8, 4ull * width * height, cudaMemcpyHostToDevice,
                               ctx->stream));
    SOLRT_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->noise_w = width;
    ctx->noise_h = height;
    return SOLRT_OK;
}

solrt_status solrt_synchronize(solrt_context* ctx) {
    CHECK_ARG(ctx, "null context");
    SOLRT_CUDA(cudaStreamSynchronize(ctx->stream));
    return check_device_flags(*ctx);
}

solrt_status solrt_get_stats(solrt_context* ctx, solrt_stats* out) {
    CHECK_ARG(ctx && out, "null argument");
    DevStats d2[2];
    SOLRT_CUDA(cudaMemcpyAsync(d2, ctx->stats.ptr, sizeof(d2), cudaMemcpyDeviceToHost, ctx->stream));
    const DevStats& d = d2[0];
    SOLRT_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->timing_collect();
    std::memset(out, 0, sizeof(*out));
    out->extend_ms = ctx->extend_ms;
    out->shade_ms = ctx->shade_ms;
    out->extend_launches = ctx->extend_launches;
    out->shade_launches = ctx->shade_launches;
    out->generate_ms = ctx->generate_ms;
    out->accumulate_ms = ctx->accumulate_ms;
    out->segments = d.segments;
    out->paths = d.paths;
    out->node_visits = d.node_visits;
    out->tri_tests = d.tri_tests;
    out->fp64_fallbacks = d.fp64_fallbacks;
    out->launches = ctx->launches;
    out->error_flags = d.eflags | d2[1].eflags;
    out->shadow_segments = d2[1].segments;
    out->shadow_unoccluded = d2[1].unoccluded;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) out->render_ms = ms;
    cudaGetLastError();
    return SOLRT_OK;
}

solrt_status solrt_reset_stats(solrt_context* ctx) {
    CHECK_ARG(ctx, "null context");
    SOLRT_CUDA(cudaMemsetAsync(ctx->stats.ptr, 0, 2 * sizeof(DevStats), ctx->stream));
    SOLRT_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->timing_collect();
    ctx->launches = 0;
    ctx->extend_ms = ctx->shade_ms = ctx->generate_ms = ctx->accumulate_ms = 0.0;
    ctx->extend_launches = ctx->shade_launches = 0;
    return SOLRT_OK;
}

solrt_status solrt_scene_create(solrt_context* ctx, const solrt_scene_desc* d, const solrt_bvh_desc* bvh,
                                solrt_scene** out) {
    CHECK_ARG(ctx && d && out, "null argument");
    *out = nullptr;
    CHECK_ARG(d->section_count == 0 || d->sections, "sections missing");
    CHECK_ARG(d->vertex_count == 0 || d->vertices, "vertices missing");
    CHECK_ARG(d->index_count == 0 || d->indices, "indices missing");
    CHECK_ARG(d->material_count == 0 || d->materials, "materials missing");
    static const float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    // flatten: world-space vertices per section, then triangles
    uint64_t nv = 0, nt = 0;
    for (uint32_t s = 0; s < d->section_count; ++s) {
        const solrt_section& sec = d->sections[s];
        if (sec.index_count % 3 != 0 || (uint64_t)sec.vertex_offset + sec.vertex_count > d->vertex_count ||
            (uint64_t)sec.index_offset + sec.index_count > d->index_count || sec.material_index >= d->material_count) {
            set_error("malformed section %u", s);
            return SOLRT_ERR_INVALID;
        }
        nv += sec.vertex_count;
        nt += sec.index_count / 3;
    }
    CHECK_ARG(nv < (1ull << 31) && nt < (1ull << 31), "scene too large");
    // two-level scenes take instances, as dynamic ones do
    const bool dynamic = bvh && ((bvh->flags & SOLRT_BVH_DYNAMIC) || bvh->kind == SOLRT_BVH2_TWO_LEVEL);
    // world positions for the BVH; object-space positions and normals for
    // shading, which interpolates them and then applies the section's
    // transform / transform_it (pathtrace.rchit:80-90)
    std::vector<float4> pos(nv), opos(nv), vnc(2 * nv);  // vnc: (normal, colour) per vertex
    std::vector<uint32_t> vsec_start(d->section_count), sec_mat(d->section_count);
    std::vector<solrt_instance> inst(d->section_count);
    std::vector<uint32_t> sec_first(d->section_count), sec_count(d->section_count);
    std::vector<uint4> tri(nt);
    uint64_t vb = 0, tb = 0;
    for (uint32_t s = 0; s < d->section_count; ++s) {
        const solrt_section& sec = d->sections[s];
        const float* T = d->instances ? d->instances[s].transform : ident;
        const float* Tit = d->instances ? d->instances[s].transform_it : ident;
        if (d->instances) {
            inst[s] = d->instances[s];
        } else {
            inst[s] = solrt_instance{};
            inst[s].id = s;
            std::memcpy(inst[s].transform, ident, sizeof(ident));
            std::memcpy(inst[s].transform_it, ident, sizeof(ident));
        }
        sec_first[s] = (uint32_t)tb;
        sec_count[s] = sec.index_count / 3;
        sec_mat[s] = sec.material_index;
        vsec_start[s] = (uint32_t)vb;
        (void)Tit;
        for (uint32_t v = 0; v < sec.vertex_count; ++v) {
            const solrt_vertex& in = d->vertices[sec.vertex_offset + v];
            opos[vb + v] = make_float4(in.pos[0], in.pos[1], in.pos[2], 0.0f);
            vnc[2 * (vb + v)] = make_float4(in.normal[0], in.normal[1], in.normal[2], 0.0f);
            float o[4];
            mat4_mul(T, in.pos[0], in.pos[1], in.pos[2], 1.0f, o);       // the BVH's world positions
            pos[vb + v] = make_float4(o[0], o[1], o[2], 0.0f);
            vnc[2 * (vb + v) + 1] = make_float4(in.color[0], in.color[1], in.color[2], 0.0f);
        }
        for (uint32_t t = 0; t < sec.index_count / 3; ++t) {
            uint32_t id[3];
            for (int k = 0; k < 3; ++k) {
                id[k] = d->indices[sec.index_offset + 3 * t + k];
                if (id[k] >= sec.vertex_count) {
                    set_error("section %u triangle %u: index %u >= vertex_count %u", s, t, id[k], sec.vertex_count);
                    return SOLRT_ERR_INVALID;
                }
            }
            tri[tb + t] = make_uint4((uint32_t)(vb + id[0]), (uint32_t)(vb + id[1]), (uint32_t)(vb + id[2]), s);
        }
        vb += sec.vertex_count;
        tb += sec.index_count / 3;
    }
    solrt_scene* sc = new (std::nothrow) solrt_scene();
    if (!sc) return SOLRT_ERR_OOM;
    sc->ctx = ctx;
    sc->tri_count = (uint32_t)nt;
    sc->vertex_count = (uint32_t)nv;
    sc->material_count = d->material_count;
    auto fail = [&](solrt_status s) {
        delete sc;
        return s;
    };
    cudaStream_t st = ctx->stream;
    solrt_status s;
    const size_t ns = d->section_count;
    if ((s = sc->vpos.alloc(16 * nv)) || (s = sc->opos.alloc(16 * nv)) || (s = sc->vnc.alloc(32 * nv)) ||
        (s = sc->tri_idx.alloc(16 * nt)) ||
        (s = sc->materials.alloc(48 * (size_t)d->material_count)) || (s = sc->sec_mat.alloc(4 * ns)) ||
        (s = sc->vsec_start.alloc(4 * ns)) || (s = sc->instances.alloc(sizeof(solrt_instance) * ns)))
        return fail(s);
    if (nv) {
        if (cudaMemcpyAsync(sc->vpos.ptr, pos.data(), 16 * nv, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(sc->opos.ptr, opos.data(), 16 * nv, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(sc->vnc.ptr, vnc.data(), 32 * nv, cudaMemcpyHostToDevice, st) != cudaSuccess) {
            set_error("scene upload failed");
            return fail(SOLRT_ERR_DEVICE);
        }
    }
    if (ns && (cudaMemcpyAsync(sc->sec_mat.ptr, sec_mat.data(), 4 * ns, cudaMemcpyHostToDevice, st) != cudaSuccess ||
               cudaMemcpyAsync(sc->vsec_start.ptr, vsec_start.data(), 4 * ns, cudaMemcpyHostToDevice, st) !=
                   cudaSuccess ||
               cudaMemcpyAsync(sc->instances.ptr, inst.data(), sizeof(solrt_instance) * ns, cudaMemcpyHostToDevice,
                               st) != cudaSuccess)) {
        set_error("scene upload failed");
        return fail(SOLRT_ERR_DEVICE);
    }
    if (nt && cudaMemcpyAsync(sc->tri_idx.ptr, tri.data(), 16 * nt, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        set_error("scene upload failed");
        return fail(SOLRT_ERR_DEVICE);
    }
    if (d->material_count &&
        cudaMemcpyAsync(sc->materials.ptr, d->materials, 48 * (size_t)d->material_count, cudaMemcpyHostToDevice,
                        st) != cudaSuccess) {
        set_error("scene upload failed");
        return fail(SOLRT_ERR_DEVICE);
    }
    // light tree of next-event estimation over the emissive triangles (world
    // positions at creation; rebuilt by solrt_scene_regenerate), buffers
    // sized for every candidate so that rebuilds keep their addresses
    for (uint64_t t = 0; t < nt; ++t) {
        const solrt_material& m = d->materials[sec_mat[tri[t].w]];
        if (m.emissive[0] >= 1.0f || m.emissive[1] >= 1.0f || m.emissive[2] >= 1.0f) {
            sc->light_cand_prim.push_back((uint32_t)t);
            sc->light_cand_tri.push_back(tri[t]);
        }
    }
    if (!sc->light_cand_prim.empty()) {
        sc->light_sec_mat = sec_mat;
        sc->light_mats.assign(d->materials, d->materials + d->material_count);
        if ((s = sc->tri_light.alloc(4 * (size_t)nt)) != SOLRT_OK ||
            (s = sc->lights.alloc(3 * sizeof(float4) * sc->light_cand_prim.size())) != SOLRT_OK)
            return fail(s);
        if ((s = upload_light_tree(*sc, pos, st)) != SOLRT_OK) return fail(s);
    }
    sc->section_count = d->section_count;
    sc->sec_tri_first = std::move(sec_first);
    sc->sec_tri_count = std::move(sec_count);
    sc->inst_host = inst;
    sc->dynamic = dynamic;
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("scene upload failed");
        return fail(SOLRT_ERR_DEVICE);
    }
    solrt_bvh_desc bd{};
    if (bvh) bd = *bvh;
    if ((s = solrt_scene_build_bvh(sc, &bd)) != SOLRT_OK) return fail(s);
    context_retain(ctx);
    *out = sc;
    return SOLRT_OK;
}

solrt_status solrt_scene_destroy(solrt_scene* scene) {
    if (!scene) return SOLRT_OK;
    solrt_context* c = static_cast<solrt_context*>(scene->ctx);
    cudaStreamSynchronize(c->stream);
    delete scene;
    context_release(c);
    return SOLRT_OK;
}

solrt_status solrt_scene_build_bvh(solrt_scene* scene, const solrt_bvh_desc* bvh) {
    CHECK_ARG(scene && bvh, "null argument");
    CHECK_ARG(bvh->kind <= SOLRT_BVH2_TWO_LEVEL, "unknown BVH kind");
    CHECK_ARG(bvh->leaf_max <= 3, "leaf_max must be 0..3");
    CHECK_ARG((bvh->flags & ~(SOLRT_BVH_DYNAMIC | SOLRT_BVH_SAH)) == 0, "unknown BVH flags");
    SOLRT_CUDA(cudaSetDevice(scene->ctx->device));
    return build_bvh(*scene->ctx, *scene, *bvh);
}

solrt_status solrt_scene_bvh_info(solrt_scene* scene, solrt_bvh_info* out) {
    CHECK_ARG(scene && out, "null argument");
    *out = scene->info;
    return SOLRT_OK;
}

solrt_status solrt_scene_bvh_export(solrt_scene* scene, void* nodes, size_t nodes_bytes, void* tris,
                                    size_t tris_bytes) {
    CHECK_ARG(scene, "null scene");
    cudaStream_t st = scene->ctx->stream;
    if (nodes) {
        CHECK_ARG(nodes_bytes >= scene->info.node_bytes, "node buffer too small");
        if (scene->info.node_bytes)
            SOLRT_CUDA(cudaMemcpyAsync(nodes, scene->nodes.ptr, scene->info.node_bytes, cudaMemcpyDeviceToHost, st));
    }
    if (tris) {
        CHECK_ARG(tris_bytes >= scene->info.tri_bytes, "triangle buffer too small");
        if (scene->info.tri_bytes)
            SOLRT_CUDA(cudaMemcpyAsync(tris, scene->tri_wt.ptr, scene->info.tri_bytes, cudaMemcpyDeviceToHost, st));
    }
    SOLRT_CUDA(cudaStreamSynchronize(st));
    return SOLRT_OK;
}

solrt_status solrt_scene_bytes(solrt_scene* scene, uint64_t* out) {
    CHECK_ARG(scene && out, "null argument");
    *out = scene->vpos.bytes + scene->opos.bytes + scene->vnc.bytes + scene->tri_idx.bytes +
           scene->materials.bytes + scene->sec_mat.bytes + scene->nodes.bytes + scene->tri_wt.bytes +
           scene->vsec_start.bytes + scene->instances.bytes + scene->topo_order.bytes + scene->topo_child.bytes +
           scene->topo_par_int.bytes + scene->topo_par_leaf.bytes + scene->topo_range.bytes + scene->tlas.bytes +
           scene->inst_table.bytes + scene->lights.bytes + scene->tri_light.bytes;
    return SOLRT_OK;
}

solrt_status solrt_instance_from_transform(const float transform[16], uint32_t id, solrt_instance* out) {
    CHECK_ARG(transform && out, "null argument");
    // SceneInstance::update_transform: transform_it = inverse(T)^T
    // (src/ray/mod.rs:27-30), in FP64 and rounded once
    double m[16], inv[16];
    for (int i = 0; i < 16; ++i) m[i] = transform[i];
    bool ok = false;
    inverse4(m, inv, &ok);
    CHECK_ARG(ok, "singular instance transform");
    *out = solrt_instance{};
    out->id = id;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            out->transform[c * 4 + r] = transform[c * 4 + r];
            out->transform_it[c * 4 + r] = (float)inv[r * 4 + c];
        }
    return SOLRT_OK;
}

solrt_status solrt_scene_set_instances(solrt_scene* scene, const solrt_instance* instances, uint32_t count) {
    CHECK_ARG(scene && instances, "null argument");
    CHECK_ARG(scene->dynamic, "scene was not created with SOLRT_BVH_DYNAMIC");
    CHECK_ARG(count == scene->section_count, "instance count must equal the section count");
    if (count == 0) return SOLRT_OK;
    SOLRT_CUDA(cudaSetDevice(scene->ctx->device));
    // pageable source: the call returns once the host array has been staged
    SOLRT_CUDA(cudaMemcpyAsync(scene->instances.ptr, instances, sizeof(solrt_instance) * count,
                               cudaMemcpyHostToDevice, scene->ctx->stream));
    scene->inst_host.assign(instances, instances + count);  // the two-level TLAS is built from these
    return SOLRT_OK;
}

solrt_status solrt_scene_regenerate(solrt_scene* scene, uint32_t mode) {
    CHECK_ARG(scene, "null scene");
    CHECK_ARG(scene->dynamic, "scene was not created with SOLRT_BVH_DYNAMIC");
    CHECK_ARG(mode == SOLRT_REGEN_REBUILD || mode == SOLRT_REGEN_REFIT, "unknown regenerate mode");
    SOLRT_CUDA(cudaSetDevice(scene->ctx->device));
    SOLRT_TRY(regenerate_scene(*scene->ctx, *scene, mode));
    return refresh_light_tree(*scene->ctx, *scene);
}

solrt_status solrt_camera_look_at(const float eye[3], const float center[3], const float up[3], float vfov_deg,
                                  float aspect, float znear, float zfar, solrt_camera* out) {
    CHECK_ARG(eye && center && up && out, "null argument");
    // Mat4::look_at_rh(eye, center, up) = look_to_rh(eye, center - eye, up)
    double f[3] = {(double)center[0] - eye[0], (double)center[1] - eye[1], (double)center[2] - eye[2]};
    const double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    CHECK_ARG(fl > 0.0, "eye equals center");
    for (double& v : f) v /= fl;
    double s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    const double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    CHECK_ARG(sl > 0.0, "up is parallel to the view direction");
    for (double& v : s) v /= sl;
    const double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    const double e[3] = {eye[0], eye[1], eye[2]};
    const double view[16] = {s[0], u[0], -f[0], 0, s[1], u[1], -f[1], 0, s[2], u[2], -f[2], 0,
                             -(s[0] * e[0] + s[1] * e[1] + s[2] * e[2]),
                             -(u[0] * e[0] + u[1] * e[1] + u[2] * e[2]),
                             (f[0] * e[0] + f[1] * e[1] + f[2] * e[2]), 1};
    return fill_camera(view, vfov_deg, aspect, znear, zfar, out);
}

solrt_status solrt_camera_from_view(const float view[16], float vfov_deg, float aspect, float znear, float zfar,
                                    solrt_camera* out) {
    CHECK_ARG(view && out, "null argument");
    double v[16];
    for (int i = 0; i < 16; ++i) v[i] = view[i];
    return fill_camera(v, vfov_deg, aspect, znear, zfar, out);
}

solrt_status solrt_image_create(solrt_context* ctx, uint32_t width, uint32_t height, uint32_t accum_mode,
                                solrt_image** out) {
    CHECK_ARG(ctx && out, "null argument");
    *out = nullptr;
    CHECK_ARG(width > 0 && height > 0 && (uint64_t)width * height < (1ull << 31), "bad image size");
    CHECK_ARG(accum_mode == SOLRT_ACCUM_REF_MIX || accum_mode == SOLRT_ACCUM_KAHAN, "bad accumulation mode");
    solrt_image* img = new (std::nothrow) solrt_image();
    if (!img) return SOLRT_ERR_OOM;
    img->ctx = ctx;
    img->width = width;
    img->height = height;
    img->accum_mode = accum_mode;
    const size_t np = (size_t)width * height;
    solrt_status s;
    if ((s = img->accum.alloc(16 * np)) || (s = img->rgba8.alloc(4 * np)) || (s = img->frame_sum.alloc(16 * np)) ||
        (s = img->rng_state.alloc(4 * np))) {
        delete img;
        return s;
    }
    if (accum_mode == SOLRT_ACCUM_KAHAN) {
        if ((s = img->ksum.alloc(16 * np)) || (s = img->kcomp.alloc(16 * np))) {
            delete img;
            return s;
        }
    }
    context_retain(ctx);
    *out = img;
    return solrt_image_clear(img);
}

solrt_status solrt_image_destroy(solrt_image* img) {
    if (!img) return SOLRT_OK;
    solrt_context* c = static_cast<solrt_context*>(img->ctx);
    cudaStreamSynchronize(c->stream);
    delete img;
    context_release(c);
    return SOLRT_OK;
}

solrt_status solrt_image_clear(solrt_image* img) {
    CHECK_ARG(img, "null image");
    cudaStream_t st = img->ctx->stream;
    for (DeviceBuffer* b : {&img->accum, &img->rgba8, &img->frame_sum, &img->ksum, &img->kcomp, &img->rng_state})
        if (b->ptr) SOLRT_CUDA(cudaMemsetAsync(b->ptr, 0, b->bytes, st));
    SOLRT_CUDA(cudaStreamSynchronize(st));
    return SOLRT_OK;
}

solrt_status solrt_image_read(solrt_image* img, float* rgba32f, uint8_t* rgba8) {
    CHECK_ARG(img, "null image");
    cudaStream_t st = img->ctx->stream;
    const size_t np = (size_t)img->width * img->height;
    if (rgba32f) SOLRT_CUDA(cudaMemcpyAsync(rgba32f, img->accum.ptr, 16 * np, cudaMemcpyDeviceToHost, st));
    if (rgba8) SOLRT_CUDA(cudaMemcpyAsync(rgba8, img->rgba8.ptr, 4 * np, cudaMemcpyDeviceToHost, st));
    SOLRT_CUDA(cudaStreamSynchronize(st));
    return check_device_flags(*img->ctx);
}

solrt_status solrt_image_snapshot(solrt_image* img, float* accum, float* kahan_sum, float* kahan_comp) {
    CHECK_ARG(img && accum, "null argument");
    const bool kahan = img->accum_mode == SOLRT_ACCUM_KAHAN;
    CHECK_ARG(!kahan || (kahan_sum && kahan_comp), "a KAHAN image needs its sums and compensations");
    cudaStream_t st = img->ctx->stream;
    const size_t bytes = 16 * (size_t)img->width * img->height;
    SOLRT_CUDA(cudaMemcpyAsync(accum, img->accum.ptr, bytes, cudaMemcpyDeviceToHost, st));
    if (kahan) {
        SOLRT_CUDA(cudaMemcpyAsync(kahan_sum, img->ksum.ptr, bytes, cudaMemcpyDeviceToHost, st));
        SOLRT_CUDA(cudaMemcpyAsync(kahan_comp, img->kcomp.ptr, bytes, cudaMemcpyDeviceToHost, st));
    }
    SOLRT_CUDA(cudaStreamSynchronize(st));
    return check_device_flags(*img->ctx);
}

solrt_status solrt_image_restore(solrt_image* img, const float* accum, const float* kahan_sum,
                                 const float* kahan_comp) {
    CHECK_ARG(img && accum, "null argument");
    const bool kahan = img->accum_mode == SOLRT_ACCUM_KAHAN;
    CHECK_ARG(!kahan || (kahan_sum && kahan_comp), "a KAHAN image needs its sums and compensations");
    cudaStream_t st = img->ctx->stream;
    const size_t bytes = 16 * (size_t)img->width * img->height;
    SOLRT_CUDA(cudaMemcpyAsync(img->accum.ptr, accum, bytes, cudaMemcpyHostToDevice, st));
    if (kahan) {
        SOLRT_CUDA(cudaMemcpyAsync(img->ksum.ptr, kahan_sum, bytes, cudaMemcpyHostToDevice, st));
        SOLRT_CUDA(cudaMemcpyAsync(img->kcomp.ptr, kahan_comp, bytes, cudaMemcpyHostToDevice, st));
    }
    SOLRT_CUDA(cudaStreamSynchronize(st));
    return SOLRT_OK;
}

solrt_status solrt_image_device_ptrs(solrt_image* img, void** accum, void** rgba8) {
    CHECK_ARG(img, "null image");
    if (accum) *accum = img->accum.ptr;
    if (rgba8) *rgba8 = img->rgba8.ptr;
    return SOLRT_OK;
}

solrt_status solrt_render(solrt_context* ctx, solrt_scene* scene, const solrt_camera* camera,
                          const solrt_render_params* p, solrt_image* img) {
    CHECK_ARG(ctx && scene && camera && p && img, "null argument");
    CHECK_ARG(scene->ctx == ctx && img->ctx == ctx, "objects belong to another context");
    CHECK_ARG(p->width == img->width && p->height == img->height, "params size differs from the image");
    CHECK_ARG(p->spp >= 1, "spp must be >= 1");
    CHECK_ARG(p->max_bounces <= SOLRT_MAX_BOUNCES, "max_bounces > 1024");
    CHECK_ARG(p->accum_mode == img->accum_mode, "accum_mode differs from the image");
    CHECK_ARG(p->miss_mode <= SOLRT_MISS_GRADIENT, "bad miss mode");
    CHECK_ARG(p->material_mode <= SOLRT_MATERIAL_LAMBERT, "bad material mode");
    CHECK_ARG(p->rng_mode <= SOLRT_RNG_PER_SAMPLE, "bad rng mode");
    CHECK_ARG(p->accum_mode == SOLRT_ACCUM_KAHAN || p->frame + 1u - p->accum_start_frame != 0u,
              "frame + 1 - accum_start_frame is zero");
    CHECK_ARG(p->tmax >= 0.0f, "tmax must be >= 0");
    return render_frame(*ctx, *scene, *camera, *p, *img);
}

solrt_status solrt_batch_create(solrt_context* ctx, const solrt_job* jobs, uint32_t n, uint32_t flags,
                                solrt_batch** out) {
    CHECK_ARG(ctx && jobs && out, "null argument");
    *out = nullptr;
    CHECK_ARG((flags & ~(uint32_t)(SOLRT_BATCH_GRAPH | SOLRT_BATCH_PERSISTENT | SOLRT_BATCH_COOPERATIVE)) == 0u,
              "unknown batch flags");
    CHECK_ARG((flags & (SOLRT_BATCH_PERSISTENT | SOLRT_BATCH_COOPERATIVE)) !=
                  (uint32_t)(SOLRT_BATCH_PERSISTENT | SOLRT_BATCH_COOPERATIVE),
              "SOLRT_BATCH_PERSISTENT and SOLRT_BATCH_COOPERATIVE exclude each other");
    solrt_batch* b = new (std::nothrow) solrt_batch();
    if (!b) return SOLRT_ERR_OOM;
    const solrt_status s = batch_plan(*ctx, jobs, n, flags, *b);
    if (s != SOLRT_OK) {
        delete b;
        return s;
    }
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        set_error("batch upload failed");
        delete b;
        return SOLRT_ERR_DEVICE;
    }
    context_retain(ctx);
    *out = b;
    return SOLRT_OK;
}

solrt_status solrt_batch_update(solrt_batch* batch, const solrt_job* jobs) {
    CHECK_ARG(batch && jobs, "null argument");
    return batch_set_jobs(*batch, jobs);
}

solrt_status solrt_batch_launch(solrt_batch* batch) {
    CHECK_ARG(batch, "null batch");
    return batch_launch(*batch);
}

solrt_status solrt_batch_destroy(solrt_batch* batch) {
    if (!batch) return SOLRT_OK;
    solrt_context* c = static_cast<solrt_context*>(batch->ctx);
    cudaStreamSynchronize(c->stream);
    delete batch;
    context_release(c);
    return SOLRT_OK;
}

solrt_status solrt_context_get_tune(solrt_context* ctx, solrt_tune_config* out) {
    CHECK_ARG(ctx && out, "null argument");
    out->block_size = ctx->tune.block;
    out->smem_stack = ctx->tune.smem;
    out->pass_paths = ctx->tune.pass_paths;
    out->reserved = 0;
    return SOLRT_OK;
}

solrt_status solrt_context_set_tune(solrt_context* ctx, const solrt_tune_config* cfg) {
    CHECK_ARG(ctx && cfg, "null argument");
    CHECK_ARG(extend_variant_ok(cfg->block_size, cfg->smem_stack),
              "block_size must be 64, 128 or 256 and smem_stack 16 or 32");
    CHECK_ARG(cfg->pass_paths <= ctx->capacity, "pass_paths exceeds the path capacity");
    ctx->tune.block = cfg->block_size;
    ctx->tune.smem = cfg->smem_stack;
    ctx->tune.pass_paths = cfg->pass_paths;
    return SOLRT_OK;
}

solrt_status solrt_batch_autotune(solrt_batch* batch, solrt_tune_result* out) {
    CHECK_ARG(batch, "null batch");
    SOLRT_CUDA(cudaSetDevice(batch->ctx->device));
    return batch_autotune(*batch, out);
}

solrt_status solrt_batch_info(solrt_batch* batch, uint32_t* passes, uint32_t* items, uint64_t* paths) {
    CHECK_ARG(batch, "null batch");
    if (passes) *passes = (uint32_t)batch->passes.size();
    if (items) *items = (uint32_t)batch->items.size();
    if (paths) *paths = batch->total_paths;
    return SOLRT_OK;
}

solrt_status solrt_trace_rays(solrt_context* ctx, solrt_scene* scene, const solrt_ray* rays, uint32_t n,
                              solrt_hit* hits) {
    CHECK_ARG(ctx && scene, "null argument");
    CHECK_ARG(n == 0 || (rays && hits), "null ray or hit array");
    CHECK_ARG(n < (1u << 31), "more than 2^31 - 1 rays in one call");
    if (n == 0) return SOLRT_OK;
    DeviceBuffer dr, dh;
    SOLRT_TRY(dr.alloc(sizeof(solrt_ray) * (size_t)n));
    SOLRT_TRY(dh.alloc(sizeof(solrt_hit) * (size_t)n));
    SOLRT_CUDA(cudaMemcpyAsync(dr.ptr, rays, sizeof(solrt_ray) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    SOLRT_TRY(launch_trace_rays(*ctx, *scene, dr.as<solrt_ray>(), n, dh.as<solrt_hit>()));
    SOLRT_CUDA(cudaMemcpyAsync(hits, dh.ptr, sizeof(solrt_hit) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    SOLRT_CUDA(cudaStreamSynchronize(ctx->stream));
    return check_device_flags(*ctx);
}

solrt_status solrt_trace_rays_device(solrt_context* ctx, solrt_scene* scene, const solrt_ray* rays_dev, uint32_t n,
                                     solrt_hit* hits_dev) {
    CHECK_ARG(ctx && scene, "null argument");
    CHECK_ARG(n == 0 || (rays_dev && hits_dev), "null ray or hit array");
    CHECK_ARG(n < (1u << 31), "more than 2^31 - 1 rays in one call");
    return launch_trace_rays(*ctx, *scene, rays_dev, n, hits_dev);
}

solrt_status solrt_debug_unit(solrt_context* ctx, uint32_t op, uint32_t n, const uint32_t* a, const uint32_t* b,
                              const float* in_f32, uint32_t* out_u32, float* out_f32) {
    CHECK_ARG(ctx, "null context");
    return debug_unit(*ctx, op, n, a, b, in_f32, out_u32, out_f32);
}

}  // extern "C"
