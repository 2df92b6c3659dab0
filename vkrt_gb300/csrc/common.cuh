// common.cuh — device-side vector math, constants and random streams shared by the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vkrt_cuda.h"

#define VKRT_DEV __device__ __forceinline__
#define VKRT_HD __host__ __device__ __forceinline__

namespace vkrt {

// ---- constants (src/shaders/scene/constants.slang:6-15, bsdf/base/math.slang:6-7) --------------------------
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kTMin = 0.001f;
constexpr float kTMax = 10000.0f;
constexpr float kShadowOriginOffset = 0.001f;
constexpr float kShadowDistanceOffset = 0.002f;
constexpr float kRRMin = 0.05f;
constexpr float kRRMax = 0.95f;
constexpr float kSafeNormalizeEps = 1e-12f;
constexpr float kTangentParallel = 0.999f;
constexpr float kGgxMinAlpha = 1e-3f;
constexpr float kGgxEps = 1e-6f;
constexpr float kLambdaMin = 360.0f;
constexpr float kLambdaRange = 470.0f;
constexpr float kCieYIntegral = 106.9461715f;

// ---- float3 / float4 helpers ----------------------------------------------------------------------------------
VKRT_HD float3 f3(float a) { return make_float3(a, a, a); }
VKRT_HD float3 f3(float a, float b, float c) { return make_float3(a, b, c); }
VKRT_HD float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
VKRT_HD float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
VKRT_HD float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
VKRT_HD float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
VKRT_HD float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
VKRT_HD float3 operator*(float s, float3 a) { return make_float3(a.x * s, a.y * s, a.z * s); }
VKRT_HD float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
VKRT_HD float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
VKRT_HD float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
VKRT_HD float3& operator*=(float3& a, float s) { a = a * s; return a; }
VKRT_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
VKRT_HD float3 cross(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
VKRT_HD float maxc(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
VKRT_HD float3 fmax3(float3 a, float3 b) { return make_float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
VKRT_HD float sat(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }
VKRT_HD float3 sat(float3 v) { return make_float3(sat(v.x), sat(v.y), sat(v.z)); }
VKRT_HD bool anyPos(float3 v) { return v.x > 0.0f || v.y > 0.0f || v.z > 0.0f; }
VKRT_HD float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }
VKRT_DEV float3 normalize(float3 v) { return v * rsqrtf(dot(v, v)); }
VKRT_DEV float3 safeNormalize(float3 v) {  // camera/ray.slang:32-39
    float l2 = dot(v, v);
    if (l2 <= kSafeNormalizeEps) return make_float3(0.0f, 0.0f, 1.0f);
    return v * rsqrtf(l2);
}
VKRT_HD float fracf(float v) { return v - floorf(v); }

VKRT_HD float4 f4(float a) { return make_float4(a, a, a, a); }
VKRT_HD float4 operator+(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
VKRT_HD float4 operator*(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
VKRT_HD float4 operator*(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
VKRT_HD float4 operator/(float4 a, float s) { return make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
VKRT_HD float4& operator+=(float4& a, float4 b) { a = a + b; return a; }
VKRT_HD float4& operator*=(float4& a, float4 b) { a = a * b; return a; }
VKRT_HD float sum4(float4 a) { return a.x + a.y + a.z + a.w; }
VKRT_HD float max4(float4 a) { return fmaxf(fmaxf(a.x, a.y), fmaxf(a.z, a.w)); }
VKRT_HD bool anyPos(float4 v) { return v.x > 0.0f || v.y > 0.0f || v.z > 0.0f || v.w > 0.0f; }

// ---- random streams -----------------------------------------------------------------------------------------
// Wellons integer hash and vkrt's per-sample seed (sampling/random.slang:7-27)
VKRT_HD uint32_t wellonsHash(uint32_t v) {
    v ^= v >> 16;
    v *= 0x7feb352du;
    v ^= v >> 15;
    v *= 0x846ca68bu;
    v ^= v >> 16;
    return v;
}

VKRT_HD uint32_t pixelSeed(int32_t x, int32_t y, uint32_t frame, uint32_t sampleIndex) {
    uint32_t s = uint32_t(x) * 73856093u;
    s ^= uint32_t(y) * 19349663u;
    s ^= frame * 83492791u;
    s ^= sampleIndex * 2654435761u;
    return wellonsHash(s);
}

// PCG32 XSH-RR (O'Neill 2014)
VKRT_HD uint32_t pcg32Next(uint64_t& state, uint64_t inc) {
    uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    uint32_t xs = uint32_t(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = uint32_t(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}

// One path's stream. In reference mode only `h` is live; PCG32 keeps a 64-bit state and increment.
struct Rng {
    uint64_t state;
    uint64_t inc;  // 0 selects the reference (hash) stream
    VKRT_DEV float next() {
        if (inc == 0u) {
            uint32_t h = wellonsHash(uint32_t(state) + 0x9e3779b9u);
            state = h;
            return float(h & 0x00ffffffu) * (1.0f / 16777216.0f);
        }
        return float(pcg32Next(state, inc) >> 8) * (1.0f / 16777216.0f);
    }
};

// Alpha-tested hits (rt/alpha_test.slang). vkrt draws a stochastic alpha decision from the path's random stream in
// any-hit order, which the driver leaves unspecified; here the decision for a triangle is a hash of a per-ray seed
// (the path stream's state when the ray starts, salted per shadow request) and the triangle's id, so the closest
// accepted hit does not depend on traversal order and the path stream is not advanced.
VKRT_DEV uint32_t alphaSeedOf(const Rng& r) { return uint32_t(r.state) ^ uint32_t(r.state >> 32); }
VKRT_HD uint32_t alphaShadowSeed(uint32_t seed, uint32_t request) { return seed ^ (0x68bc21ebu * (request + 1u)); }
VKRT_HD float alphaRandom(uint32_t seed, uint32_t gid) {
    return float(wellonsHash(seed ^ wellonsHash(gid + 0x632be5abu)) & 0x00ffffffu) * (1.0f / 16777216.0f);
}

VKRT_DEV Rng makeRng(uint32_t mode, uint64_t seed, int32_t x, int32_t y, uint32_t frame, uint32_t sampleIndex) {
    Rng r;
    if (mode == VKRT_CUDA_RNG_REFERENCE) {
        r.state = pixelSeed(x, y, frame, sampleIndex);
        r.inc = 0u;
        return r;
    }
    uint64_t initstate = seed + uint64_t(frame) * 0x9E3779B97F4A7C15ull;
    uint64_t initseq = (uint64_t(uint32_t(y)) << 48) ^ (uint64_t(uint32_t(x)) << 32) ^ uint64_t(sampleIndex);
    r.inc = (initseq << 1u) | 1u;
    r.state = 0u;
    pcg32Next(r.state, r.inc);
    r.state += initstate;
    pcg32Next(r.state, r.inc);
    return r;
}

VKRT_HD uint32_t reverseBits32(uint32_t v) {
#ifdef __CUDA_ARCH__
    return __brev(v);
#else
    v = ((v & 0x55555555u) << 1u) | ((v >> 1u) & 0x55555555u);
    v = ((v & 0x33333333u) << 2u) | ((v >> 2u) & 0x33333333u);
    v = ((v & 0x0f0f0f0fu) << 4u) | ((v >> 4u) & 0x0f0f0f0fu);
    v = ((v & 0x00ff00ffu) << 8u) | ((v >> 8u) & 0x00ff00ffu);
    return (v << 16u) | (v >> 16u);
#endif
}

}  // namespace vkrt
