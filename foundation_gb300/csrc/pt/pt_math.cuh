// pt_math.cuh — device-side sampling and shading math of the path tracer
// (FP32): PCG32, orthonormal bases, Lambert and GGX BSDFs, MIS.
//
// Methods:
//  * PCG32 (PCG-XSH-RR 64/32), O'Neill 2014;
//  * orthonormal basis from one vector, Duff et al., "Building an Orthonormal
//    Basis, Revisited", JCGT 6(1) 2017;
//  * GGX / Trowbridge-Reitz microfacet reflection (Walter et al. 2007) with
//    height-correlated Smith masking-shadowing and Schlick's Fresnel, alpha
//    taken directly from the material roughness, sampled through the
//    distribution of visible normals (Heitz, "Sampling the GGX Distribution
//    of Visible Normals", JCGT 7(4) 2018);
//  * power-heuristic MIS (Veach 1997, beta = 2).
// The FP64 CPU oracle (oracle/pt_oracle.cpp) implements the same
// definitions in double precision.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace Foundation {
namespace PT {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;

struct Pcg32 {
    uint64_t state;
    uint64_t inc;
    __device__ __forceinline__ void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    __device__ __forceinline__ uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return __funnelshift_r(xorshifted, xorshifted, rot);
    }
    // uniform in [0, 1)
    __device__ __forceinline__ float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};

// The generator streams of the path tracer. Every path owns one stream,
// chosen by its frame seed, pixel and sample, so a path's samples do not
// depend on which kernel (wavefront stage, tail or training megakernel)
// draws them.
//  * camera path (pixel, sample) of a frame seeded frame_seed:
//    initstate = frame_seed * 0x9E3779B97F4A7C15 + pixel, sequence = sample;
//  * training path i of a round seeded round_seed (its pixel drawn by the
//    round's hash): initstate = frame_seed * 0x9E3779B97F4A7C15 + pixel +
//    0x5851F42D4C957F2D * (i + 1), sequence = 2^30 + (round_seed mod 2^30),
//    so training streams never share a sequence with camera samples below
//    2^30.
__device__ __forceinline__ Pcg32 camera_path_rng(uint64_t frame_seed, uint32_t pixel, uint32_t sample) {
    Pcg32 g;
    g.seed(frame_seed * 0x9E3779B97F4A7C15ull + pixel, sample);
    return g;
}
__device__ __forceinline__ Pcg32 training_path_rng(uint64_t frame_seed, uint32_t pixel, uint32_t i,
                                                   uint32_t round_seed) {
    Pcg32 g;
    g.seed(frame_seed * 0x9E3779B97F4A7C15ull + pixel + 0x5851F42D4C957F2Dull * (i + 1ull),
           0x40000000u + (round_seed & 0x3FFFFFFFu));
    return g;
}
// A camera path's generator in its 16-byte path record: (state low, state
// high, sequence, w). The increment is rebuilt from the sequence (the
// sample index), so the record holds the stream exactly.
__device__ __forceinline__ uint4 pack_rng(const Pcg32& g, uint32_t sequence, uint32_t w) {
    return make_uint4((uint32_t)g.state, (uint32_t)(g.state >> 32), sequence, w);
}
__device__ __forceinline__ Pcg32 unpack_rng(uint4 rec) {
    Pcg32 g;
    g.state = (uint64_t)rec.x | ((uint64_t)rec.y << 32);
    g.inc = ((uint64_t)rec.z << 1) | 1u;
    return g;
}

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return a * s; }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize(float3 a) { return a * rsqrtf(dot(a, a)); }
__device__ __forceinline__ float max3(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }

// Orthonormal basis (t, b, n) around unit n (Duff et al. 2017).
__device__ __forceinline__ void onb(float3 n, float3& t, float3& b) {
    const float sign = copysignf(1.0f, n.z);
    const float a = -1.0f / (sign + n.z);
    const float c = n.x * n.y * a;
    t = f3(1.0f + sign * n.x * n.x * a, sign * c, -sign * n.x);
    b = f3(c, sign + n.y * n.y * a, -n.y);
}

// ---- GGX, local frame (z = normal) ----------------------------------------
__device__ __forceinline__ float ggx_D(float cos_h, float a2) {
    const float d = cos_h * cos_h * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * d * d);
}
__device__ __forceinline__ float ggx_Lambda(float3 w, float a2) {
    const float z2 = w.z * w.z;
    const float tan2 = fmaxf(0.0f, 1.0f - z2) / z2;
    return 0.5f * (-1.0f + sqrtf(1.0f + a2 * tan2));
}
__device__ __forceinline__ float3 schlick(float3 f0, float c) {
    const float m = fminf(fmaxf(1.0f - c, 0.0f), 1.0f);
    const float m5 = (m * m) * (m * m) * m;
    return f0 + (f3(1.0f, 1.0f, 1.0f) - f0) * m5;
}

// BSDF value f (without the cosine) and solid-angle pdf of sampling wi.
struct BsdfEval {
    float3 f;
    float pdf;
};

__device__ __forceinline__ BsdfEval eval_bsdf(uint32_t type, float3 albedo, float alpha, float3 wo, float3 wi) {
    BsdfEval r{f3(0.f, 0.f, 0.f), 0.0f};
    if (wo.z <= 0.0f || wi.z <= 0.0f) return r;
    if (type == 0u) {
        r.f = albedo * kInvPi;
        r.pdf = wi.z * kInvPi;
        return r;
    }
    const float a2 = alpha * alpha;
    const float3 h = normalize(wo + wi);
    const float D = ggx_D(h.z, a2);
    const float lo = ggx_Lambda(wo, a2), li = ggx_Lambda(wi, a2);
    const float G2 = 1.0f / (1.0f + lo + li);
    const float G1o = 1.0f / (1.0f + lo);
    const float3 F = schlick(albedo, dot(wi, h));
    r.f = F * (D * G2 / (4.0f * wo.z * wi.z));
    r.pdf = G1o * D / (4.0f * wo.z);
    return r;
}

struct BsdfSample {
    float3 wi;
    float3 weight;  // f * cos / pdf
    float pdf;
    bool ok;
};

__device__ __forceinline__ BsdfSample sample_bsdf(uint32_t type, float3 albedo, float alpha, float3 wo, float u1,
                                                  float u2) {
    BsdfSample s;
    s.ok = false;
    s.pdf = 0.0f;
    s.weight = f3(0.f, 0.f, 0.f);
    s.wi = f3(0.f, 0.f, 1.f);
    if (wo.z <= 0.0f) return s;
    if (type == 0u) {
        const float r = sqrtf(u1);
        float sp, cp;
        sincosf(2.0f * kPi * u2, &sp, &cp);
        const float z = sqrtf(fmaxf(0.0f, 1.0f - u1));
        s.wi = f3(r * cp, r * sp, z);
        s.pdf = z * kInvPi;
        s.weight = albedo;
        s.ok = z > 0.0f;
        return s;
    }
    const float a2 = alpha * alpha;
    // visible-normal sampling (Heitz 2018)
    const float3 vh = normalize(f3(alpha * wo.x, alpha * wo.y, wo.z));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    const float3 T1 = lensq > 0.0f ? f3(-vh.y, vh.x, 0.0f) * rsqrtf(lensq) : f3(1.0f, 0.0f, 0.0f);
    const float3 T2 = cross(vh, T1);
    const float r = sqrtf(u1);
    float sp, cp;
    sincosf(2.0f * kPi * u2, &sp, &cp);
    const float t1 = r * cp;
    float t2 = r * sp;
    const float sh = 0.5f * (1.0f + vh.z);
    t2 = (1.0f - sh) * sqrtf(fmaxf(0.0f, 1.0f - t1 * t1)) + sh * t2;
    const float3 nh = T1 * t1 + T2 * t2 + vh * sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2));
    const float3 h = normalize(f3(alpha * nh.x, alpha * nh.y, fmaxf(0.0f, nh.z)));
    const float woh = dot(wo, h);
    s.wi = h * (2.0f * woh) - wo;
    if (s.wi.z <= 0.0f || woh <= 0.0f) return s;
    const float D = ggx_D(h.z, a2);
    const float lo = ggx_Lambda(wo, a2), li = ggx_Lambda(s.wi, a2);
    const float G1o = 1.0f / (1.0f + lo);
    const float G2 = 1.0f / (1.0f + lo + li);
    s.pdf = G1o * D / (4.0f * wo.z);
    s.weight = schlick(albedo, dot(s.wi, h)) * (G2 / G1o);
    s.ok = s.pdf > 0.0f;
    return s;
}

__device__ __forceinline__ float power_heuristic(float a, float b) {
    const float a2 = a * a, b2 = b * b;
    return a2 + b2 > 0.0f ? a2 / (a2 + b2) : 0.0f;
}

}  // namespace PT
}  // namespace Foundation
