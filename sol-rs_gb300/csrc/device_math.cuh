// device_math.cuh — shader arithmetic of the 5-pathtrace path on sm_103a.
//
// Restates assets/glsl/sampling.glsl:18-96, pathtrace.rmiss:8-21 and the
// vector built-ins they use. The library is compiled with -fmad=false, so
// each a*b+c below is a rounded multiply then a rounded add, in the order the
// GLSL source writes it; division and sqrt are IEEE round-to-nearest
// (-prec-div=true -prec-sqrt=true). With the same evaluation order on the
// host, primary and secondary rays agree bit for bit with a CPU evaluation.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/solrt.h"

#define SOLRT_HD __host__ __device__ __forceinline__
#define SOLRT_D __device__ __forceinline__

namespace solrt {

struct f3 {
    float x, y, z;
};

SOLRT_HD f3 mk(float x, float y, float z) { return f3{x, y, z}; }
SOLRT_HD f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
SOLRT_HD f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
SOLRT_HD f3 operator*(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
SOLRT_HD f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
SOLRT_HD f3 operator*(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
SOLRT_HD f3 operator-(f3 a) { return f3{-a.x, -a.y, -a.z}; }
SOLRT_HD float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
SOLRT_D float length(f3 a) { return sqrtf(dot(a, a)); }
SOLRT_D f3 normalize(f3 a) {
    const float l = length(a);
    return f3{a.x / l, a.y / l, a.z / l};
}
// GLSL min/max: min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x (a NaN
// first operand propagates, as in the C++ standard library's std::min/max).
SOLRT_HD float glsl_min(float x, float y) { return y < x ? y : x; }
SOLRT_HD float glsl_max(float x, float y) { return x < y ? y : x; }
SOLRT_D float saturate(float x) { return glsl_min(glsl_max(x, 0.0f), 1.0f); }
SOLRT_D float glsl_sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
// reflect(I, N) = I - 2 * dot(N, I) * N
SOLRT_D f3 reflect(f3 i, f3 n) {
    const float k = 2.0f * dot(n, i);
    return i - k * n;
}
// mix(x, y, a) = x * (1 - a) + y * a
SOLRT_D f3 mix(f3 x, f3 y, float a) { return x * (1.0f - a) + y * a; }
SOLRT_D float smoothstep(float e0, float e1, float x) {
    float t = (x - e0) / (e1 - e0);
    t = glsl_min(glsl_max(t, 0.0f), 1.0f);
    return (t * t) * (3.0f - 2.0f * t);
}

// column-major mat4 times (x, y, z, w), summed column by column.
SOLRT_HD void mat4_mul(const float* m, float x, float y, float z, float w, float out[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) out[r] = ((m[0 + r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] * w;
}

// ---------------------------------------------------------------------------
// RNG: TEA seeding (sampling.glsl:18-32) and the PCG RXS-M-XS step
// (sampling.glsl:35-42). Integer arithmetic, identical everywhere.
// ---------------------------------------------------------------------------

SOLRT_HD uint32_t tea(uint32_t val0, uint32_t val1) {
    uint32_t v0 = val0, v1 = val1, s0 = 0;
#pragma unroll
    for (int n = 0; n < 16; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

SOLRT_D float next_rand(uint32_t& rng) {
    rng = rng * 747796405u + 1u;
    uint32_t word = ((rng >> ((rng >> 28) + 4u)) ^ rng) * 277803737u;
    word = (word >> 22) ^ word;
    return __fdiv_rn(__uint2float_rn(word), 4294967295.0f);
}

// ---------------------------------------------------------------------------
// sin/cos of the sampling angle. One fixed evaluation written from the
// mathematics: Cody-Waite reduction by pi/2 with a three-part split of pi/2
// (8 + 12 + 24 significant bits; k * part is exact for |k| < 2^12), then the
// Taylor series of sin to x^9 and of cos to x^10 on |r| <= pi/4 (truncation
// below 2e-9), Horner order. Used instead of the CUDA math library so that
// the device and a CPU evaluation give the same bits.
// ---------------------------------------------------------------------------

SOLRT_D void sincos_poly(float x, float& s_out, float& c_out) {
    const float k = rintf(x * 0x1.45f306p-1f);
    float r = x - k * 0x1.92p+0f;
    r = r - k * 0x1.fb4p-12f;
    r = r - k * 0x1.4442d2p-24f;
    const float r2 = r * r;
    float ps = 0x1.71de3ap-19f;
    ps = ps * r2 + -0x1.a01a02p-13f;
    ps = ps * r2 + 0x1.111112p-7f;
    ps = ps * r2 + -0x1.555556p-3f;
    const float s = r + (r * r2) * ps;
    float pc = -0x1.27e4fcp-22f;
    pc = pc * r2 + 0x1.a01a02p-16f;
    pc = pc * r2 + -0x1.6c16c2p-10f;
    pc = pc * r2 + 0x1.555556p-5f;
    pc = pc * r2 + -0.5f;
    const float c = 1.0f + r2 * pc;
    const int q = ((int)k) & 3;
    if (q == 0) { s_out = s; c_out = c; }
    else if (q == 1) { s_out = c; c_out = -s; }
    else if (q == 2) { s_out = -s; c_out = -c; }
    else { s_out = -c; c_out = s; }
}

// ---------------------------------------------------------------------------
// Sampling (sampling.glsl:52-96)
// ---------------------------------------------------------------------------

#define SOLRT_TWO_PI 6.28318530718f

SOLRT_D float fresnel_dielectric(f3 i, f3 m, float eta) {
    float result = 1.0f;
    const float cos_i = fabsf(dot(i, m));
    const float sin_o2 = (eta * eta) * (1.0f - cos_i * cos_i);
    if (sin_o2 <= 1.0f) {
        const float cos_o = sqrtf(saturate(1.0f - sin_o2));
        const float rs = (cos_i - eta * cos_o) / (cos_i + eta * cos_o);
        const float rp = (eta * cos_i - cos_o) / (eta * cos_i + cos_o);
        result = 0.5f * (rs * rs + rp * rp);
    }
    return result;
}

SOLRT_D void onb(f3 n, f3& u, f3& v) {
    const float s = n.z < 0.0f ? -1.0f : 1.0f;
    const float a = -1.0f / (s + n.z);
    const float b = n.x * n.y * a;
    u = f3{1.0f + s * n.x * n.x * a, s * b, -s * n.x};
    v = f3{b, s + n.y * n.y * a, -n.y};
}

SOLRT_D f3 align_to_direction(f3 n, float cos_t, float phi) {
    const float sin_t = sqrtf(saturate(1.0f - cos_t * cos_t));
    f3 u, v;
    onb(n, u, v);
    float sp, cp;
    sincos_poly(phi, sp, cp);
    return (u * cp + v * sp) * sin_t + n * cos_t;
}

SOLRT_D f3 sample_ggx(f3 n, float xi0, float xi1, float alpha2) {
    const float cos_t = sqrtf(saturate((1.0f - xi0) / (xi0 * (alpha2 - 1.0f) + 1.0f)));
    return align_to_direction(n, cos_t, xi1 * SOLRT_TWO_PI);
}

SOLRT_D f3 sample_cosine(f3 n, float xi0, float xi1) {
    const float cos_t = sqrtf(xi0);
    return align_to_direction(n, cos_t, xi1 * SOLRT_TWO_PI);
}

// pathtrace.rmiss:8-21 (REF_SKY = ENABLE_SKYLIGHT) and the gradient sky.
SOLRT_D f3 miss_color(f3 dir, uint32_t mode) {
    if (mode == SOLRT_MISS_REF_SKY) {
        const f3 wi = normalize(dir);
        const float t = smoothstep(0.35f, 0.65f, 0.5f * (wi.y + 1.0f));
        const f3 sky = mix(f3{0.58f, 0.45f, 0.25f}, f3{0.3f, 0.4f, 0.5f}, t);
        const f3 sun_dir = normalize(f3{0.0f, 1.0f, -0.25f});
        const bool is_sun = dot(wi, sun_dir) > 0.99f;
        return mix(sky, f3{120.0f, 100.0f, 50.0f}, is_sun ? 1.0f : 0.0f);
    }
    if (mode == SOLRT_MISS_GRADIENT) {
        const f3 wi = normalize(dir);
        const float t = 0.5f * (wi.y + 1.0f);
        return mix(f3{1.0f, 1.0f, 1.0f}, f3{0.5f, 0.7f, 1.0f}, t);
    }
    return f3{0.0f, 0.0f, 0.0f};
}

}  // namespace solrt
