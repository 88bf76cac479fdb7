// glsl_shim.h — the few GLSL types and built-ins that the reference's
// assets/glsl/sampling.glsl and assets/glsl/postprocess.glsl use, so that
// those two files compile as C++ (TEST INFRASTRUCTURE: builds oracle/_ref).
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

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};

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
inline float abs(float x) { return std::fabs(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline vec3 pow(vec3 a, vec3 b) { return vec3{std::pow(a.x, b.x), std::pow(a.y, b.y), std::pow(a.z, b.z)}; }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec3 clamp(vec3 x, vec3 lo, vec3 hi) {
    return vec3{clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y), clamp(x.z, lo.z, hi.z)};
}

}  // namespace glsl

// GLSL parameter qualifier `in` has no C++ meaning.
#define in
