// glsl_shim.h — the GLSL types and built-ins that the reference's
// assets/glsl/sampling.glsl, postprocess.glsl and the path's shaders
// (pathtrace.rgen / .rchit / .rmiss) use, so that those files compile as C++
// (TEST INFRASTRUCTURE: builds oracle/_ref).
//
// Semantics follow the GLSL 4.60 specification: component-wise vector
// arithmetic in single precision, mix(x,y,a) = x*(1-a) + y*a,
// clamp(x,lo,hi) = min(max(x,lo),hi), pow / sqrt / cos / sin on floats.
// Constructors are spelled vecN{...} by the rewrite in build_ref.py so that
// their arguments are evaluated left to right, as GLSL requires.
#pragma once
#include <cmath>
#include <cstdint>

#undef M_PI

namespace glsl {

typedef uint32_t uint;

struct uvec2 {
    uint x, y;
};
struct uvec3 {
    uint x, y, z;
    uvec2 xy() const { return uvec2{x, y}; }
};
struct vec2;
struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    ivec2(uvec2 v) : x((int)v.x), y((int)v.y) {}
    explicit ivec2(const vec2& v);
    ivec2 xy() const { return *this; }
};
struct ivec3 {
    int x, y, z;
    template <class A, class B, class C>
    ivec3(A a, B b, C c) : x((int)a), y((int)b), z((int)c) {}
};

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(uvec2 v) : x((float)v.x), y((float)v.y) {}
    vec2(ivec2 v) : x((float)v.x), y((float)v.y) {}
};
inline ivec2::ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}

struct vec4;
struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(const vec4& v);
    vec3 xyz() const { return *this; }
    vec3& operator+=(vec3 o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator*=(vec3 o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
};

struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(vec3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec3 xyz() const { return vec3{x, y, z}; }
    float operator[](uint i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

// column-major: four columns; m * v sums the columns in order, per row
// ((c0 x + c1 y) + c2 z) + c3 w
struct mat4 {
    vec4 c[4];
};
inline vec4 operator*(const mat4& m, vec4 v) {
    return vec4{((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z) + m.c[3].x * v.w,
                ((m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z) + m.c[3].y * v.w,
                ((m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z) + m.c[3].z * v.w,
                ((m.c[0].w * v.x + m.c[1].w * v.y) + m.c[2].w * v.z) + m.c[3].w * v.w};
}

inline vec2 operator+(vec2 a, vec2 b) { return vec2{a.x + b.x, a.y + b.y}; }
inline vec2 operator/(vec2 a, vec2 b) { return vec2{a.x / b.x, a.y / b.y}; }
inline vec2 operator*(vec2 a, float s) { return vec2{a.x * s, a.y * s}; }
inline vec2 operator-(vec2 a, float s) { return vec2{a.x - s, a.y - s}; }
inline vec2 operator-(vec2 a, vec2 b) { return vec2{a.x - b.x, a.y - b.y}; }
inline vec2 operator*(vec2 a, vec2 b) { return vec2{a.x * b.x, a.y * b.y}; }
// mixed integer / float operands convert to float, as GLSL does implicitly
inline vec2 operator*(vec2 a, ivec2 b) { return a * vec2{b}; }
inline vec2 operator+(uvec2 a, vec2 b) { return vec2{a} + b; }
// GLSL mod(x, y) = x - y * floor(x / y)
inline vec2 mod(vec2 x, vec2 y) {
    return vec2{x.x - y.x * std::floor(x.x / y.x), x.y - y.y * std::floor(x.y / y.y)};
}

inline vec3 operator+(vec3 a, vec3 b) { return vec3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(vec3 a, vec3 b) { return vec3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(vec3 a, vec3 b) { return vec3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator/(vec3 a, vec3 b) { return vec3{a.x / b.x, a.y / b.y, a.z / b.z}; }
inline vec3 operator+(vec3 a, float s) { return vec3{a.x + s, a.y + s, a.z + s}; }
inline vec3 operator-(vec3 a, float s) { return vec3{a.x - s, a.y - s, a.z - s}; }
inline vec3 operator*(vec3 a, float s) { return vec3{a.x * s, a.y * s, a.z * s}; }
inline vec3 operator/(vec3 a, float s) { return vec3{a.x / s, a.y / s, a.z / s}; }
inline vec3 operator+(float s, vec3 a) { return vec3{s + a.x, s + a.y, s + a.z}; }
inline vec3 operator-(float s, vec3 a) { return vec3{s - a.x, s - a.y, s - a.z}; }
inline vec3 operator*(float s, vec3 a) { return vec3{s * a.x, s * a.y, s * a.z}; }
inline vec3 operator/(float s, vec3 a) { return vec3{s / a.x, s / a.y, s / a.z}; }
inline vec3 operator-(vec3 a) { return vec3{-a.x, -a.y, -a.z}; }

inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(vec3 a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(vec3 a) {
    const float l = length(a);
    return vec3{a.x / l, a.y / l, a.z / l};
}
// I - 2 dot(N, I) N
inline vec3 reflect(vec3 i, vec3 n) { return i - (2.0f * dot(n, i)) * n; }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }
struct bvec3 {
    bool x, y, z;
};
inline bvec3 isnan(vec3 v) { return bvec3{std::isnan(v.x), std::isnan(v.y), std::isnan(v.z)}; }
inline bvec3 isinf(vec3 v) { return bvec3{std::isinf(v.x), std::isinf(v.y), std::isinf(v.z)}; }
inline bool any(bvec3 b) { return b.x || b.y || b.z; }
inline float abs(float x) { return std::fabs(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }

// GLSL leaves the precision of sin / cos to the implementation. The
// pipeline namespaces of ref_glsl.cpp use this one, the evaluation the
// oracle and the device kernels share (Cody-Waite reduction by pi/2 with a
// three-part split, 8 + 12 + 24 bits; Taylor series of sin to x^9 and cos to
// x^10 on |r| <= pi/4, Horner order); the golden-vector functions keep the C
// library's (an independent accuracy check of that evaluation).
inline void sincos_poly(float x, float& s_out, float& c_out) {
    const float k = std::rint(x * 0x1.45f306p-1f);
    float r = x - k * 0x1.92p+0f;
    r = r - k * 0x1.fb4p-12f;
    r = r - k * 0x1.4442d2p-24f;
    const float r2 = r * r;
    float ps = 0x1.71de3ap-19f;
    ps = ps * r2 + -0x1.a01a02p-13f;
    ps = ps * r2 + 0x1.111112p-7f;
    ps = ps * r2 + -0x1.555556p-3f;
    const float sv = r + (r * r2) * ps;
    float pc = -0x1.27e4fcp-22f;
    pc = pc * r2 + 0x1.a01a02p-16f;
    pc = pc * r2 + -0x1.6c16c2p-10f;
    pc = pc * r2 + 0x1.555556p-5f;
    pc = pc * r2 + -0.5f;
    const float cv = 1.0f + r2 * pc;
    switch (((int)k) & 3) {
        case 0: s_out = sv; c_out = cv; break;
        case 1: s_out = cv; c_out = -sv; break;
        case 2: s_out = -sv; c_out = -cv; break;
        default: s_out = -cv; c_out = sv; break;
    }
}
inline float poly_cos(float x) {
    float s, c;
    sincos_poly(x, s, c);
    return c;
}
inline float poly_sin(float x) {
    float s, c;
    sincos_poly(x, s, c);
    return s;
}
inline float pow(float x, float y) { return std::pow(x, y); }
inline vec3 pow(vec3 a, vec3 b) { return vec3{std::pow(a.x, b.x), std::pow(a.y, b.y), std::pow(a.z, b.z)}; }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec3 clamp(vec3 x, vec3 lo, vec3 hi) {
    return vec3{clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y), clamp(x.z, lo.z, hi.z)};
}
inline float smoothstep(float e0, float e1, float x) {
    const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return (t * t) * (3.0f - 2.0f * t);
}

// --- ray-tracing pipeline built-ins (GL_EXT_ray_tracing), per CPU thread ---
typedef int accelerationStructureEXT;
constexpr uint gl_RayFlagsOpaqueEXT = 1u;
extern thread_local uvec3 gl_LaunchIDEXT;
extern thread_local uvec3 gl_LaunchSizeEXT;
extern thread_local int gl_InstanceID;
extern thread_local int gl_PrimitiveID;
extern thread_local vec3 gl_WorldRayOriginEXT;
extern thread_local vec3 gl_WorldRayDirectionEXT;
extern thread_local vec3 attribs;  // the closest-hit shader's hitAttributeEXT

// traceRayEXT: the pipeline's closest-hit or miss shader runs on the payload
// (the acceleration structure, flags, masks and SBT offsets are not used:
// one opaque geometry, one hit group, one miss shader)
typedef void (*TraceFn)(vec3 origin, float tmin, vec3 direction, float tmax);
extern TraceFn g_trace;
inline void traceRayEXT(accelerationStructureEXT, uint, uint, uint, uint, uint, vec3 origin, float tmin,
                        vec3 direction, float tmax, int) {
    g_trace(origin, tmin, direction, tmax);
}

// image2D of the ray-generation shader: RGBA32F (float data) or RGBA8 UNORM
// (byte data, stored as clamp(c, 0, 1) * 255 rounded half up)
struct image2D {
    float* f32 = nullptr;
    unsigned char* u8 = nullptr;
    int width = 0;
};
inline vec4 imageLoad(const image2D& im, ivec2 p) {
    const size_t i = 4 * ((size_t)p.y * im.width + p.x);
    if (im.f32) return vec4{im.f32[i], im.f32[i + 1], im.f32[i + 2], im.f32[i + 3]};
    return vec4{im.u8[i] / 255.0f, im.u8[i + 1] / 255.0f, im.u8[i + 2] / 255.0f, im.u8[i + 3] / 255.0f};
}

// sampler2D of an RGBA8 UNORM texture: texelFetch returns c / 255
struct sampler2D {
    const unsigned char* texels = nullptr;
    int width = 0, height = 0;
};
inline ivec2 textureSize(const sampler2D& s, int) { return ivec2{s.width, s.height}; }
inline vec4 texelFetch(const sampler2D& s, ivec2 p, int) {
    const unsigned char* t = s.texels + 4 * ((size_t)p.y * s.width + p.x);
    return vec4{t[0] / 255.0f, t[1] / 255.0f, t[2] / 255.0f, t[3] / 255.0f};
}
inline void imageStore(image2D& im, ivec2 p, vec4 v) {
    const size_t i = 4 * ((size_t)p.y * im.width + p.x);
    if (im.f32) {
        im.f32[i] = v.x; im.f32[i + 1] = v.y; im.f32[i + 2] = v.z; im.f32[i + 3] = v.w;
    } else {
        const float c[4] = {v.x, v.y, v.z, v.w};
        for (int k = 0; k < 4; ++k) im.u8[i + k] = (unsigned char)(clamp(c[k], 0.0f, 1.0f) * 255.0f + 0.5f);
    }
}

}  // namespace glsl

// GLSL parameter qualifier `in` has no C++ meaning.
#define in
