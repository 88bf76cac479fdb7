// ref_glsl.cpp — exports the reference's own sampling.glsl / postprocess.glsl
// functions (mechanically rewritten to C++ by build_ref.py into oracle/_ref)
// through a C ABI, to produce golden vectors. TEST INFRASTRUCTURE ONLY.
#include "glsl_shim.h"

namespace glsl {
#include "sampling.glsl.inc"
#include "postprocess.glsl.inc"
}  // namespace glsl

#undef in

extern "C" {

uint32_t ref_tea(uint32_t a, uint32_t b) { return glsl::tea(a, b); }

float ref_next_rand(uint32_t* state) {
    glsl::uint s = *state;
    const float r = glsl::nextRand(s);
    *state = s;
    return r;
}

void ref_next_rand2(uint32_t* state, float out[2]) {
    glsl::uint s = *state;
    const glsl::vec2 r = glsl::nextRand2(s);
    *state = s;
    out[0] = r.x;
    out[1] = r.y;
}

void ref_sample_ggx(const float n[3], float xi0, float xi1, float alpha2, float out[3]) {
    const glsl::vec3 r = glsl::sampleGGXDistribution(glsl::vec3{n[0], n[1], n[2]}, glsl::vec2{xi0, xi1}, alpha2);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void ref_sample_cosine(const float n[3], float xi0, float xi1, float out[3]) {
    const glsl::vec3 r = glsl::sampleCosineWeightedHemisphere(glsl::vec3{n[0], n[1], n[2]}, glsl::vec2{xi0, xi1});
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

float ref_fresnel(const float i[3], const float m[3], float eta) {
    return glsl::fresnelDielectric(glsl::vec3{i[0], i[1], i[2]}, glsl::vec3{m[0], m[1], m[2]}, eta);
}

void ref_onb(const float n[3], float u[3], float v[3]) {
    glsl::vec3 a, b;
    glsl::buildOrthonormalBasis(glsl::vec3{n[0], n[1], n[2]}, a, b);
    u[0] = a.x; u[1] = a.y; u[2] = a.z;
    v[0] = b.x; v[1] = b.y; v[2] = b.z;
}

void ref_gamma(const float c[3], float power, float out[3]) {
    const glsl::vec3 r = glsl::gammaCorrect(glsl::vec3{c[0], c[1], c[2]}, power);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

}  // extern "C"
