// integrator.cuh — helpers shared by the megakernel, wavefront and adjoint integrators: traversal wrappers,
// the camera ray (camera/ray.slang:15-30), MIS helpers (light/direct/mis_weights.slang) and the display encode
// (film/tonemap.slang:9-32).
#pragma once

#include "shading.cuh"
#include "traverse.cuh"

namespace vkrt {

constexpr uint32_t kDefaultThreads = 128;

struct PathCounts {
    uint32_t primary, extension, shadow, samples;
};

VKRT_DEV float powerHeuristic(float a, float b) {
    float a2 = a * a;
    return a2 / (a2 + b * b);
}

struct KernelCtx {
    const DeviceScene& sc;
    const VKRT_CudaSceneData& sd;
    uint2* stackColumn;
    uint32_t stackStride;
    RenderCounters* counters;
};

template <bool kCountBytes>
VKRT_DEV TraceHit closest(const KernelCtx& k, float3 o, float3 d) {
    TraceRay r{o, d, kTMin, kTMax};
    return traceBvh<false, kCountBytes>(k.sc, r, k.stackColumn, k.stackStride, k.counters);
}

template <bool kCountBytes>
VKRT_DEV bool visible(const KernelCtx& k, float3 p, float3 gn, float3 wi, float tmax) {
    // light/direct/common.slang:37-44
    float3 off = dot(wi, gn) >= 0.0f ? gn : -gn;
    TraceRay r{p + off * kShadowOriginOffset, wi, kTMin, tmax};
    return traceBvh<true, kCountBytes>(k.sc, r, k.stackColumn, k.stackStride, k.counters).mesh ==
           VKRT_CUDA_INVALID_INDEX;
}

VKRT_DEV float3 primaryRay(const VKRT_CudaSceneData& sd, int px, int py, float jx, float jy, float3& origin) {
    // camera/ray.slang:15-30
    float vx = float(px - int(sd.viewportRect[0])) + 0.5f + jx;
    float vy = float(py - int(sd.viewportRect[1])) + 0.5f + jy;
    float ndcx = vx / float(sd.viewportRect[2]) * 2.0f - 1.0f;
    float ndcy = vy / float(sd.viewportRect[3]) * 2.0f - 1.0f;
    float vd[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        vd[r] = sd.projInverse[0][r] * ndcx + sd.projInverse[1][r] * ndcy + sd.projInverse[2][r] + sd.projInverse[3][r];
    origin = make_float3(sd.viewInverse[3][0], sd.viewInverse[3][1], sd.viewInverse[3][2]);
    float3 d = make_float3(sd.viewInverse[0][0] * vd[0] + sd.viewInverse[1][0] * vd[1] + sd.viewInverse[2][0] * vd[2],
                           sd.viewInverse[0][1] * vd[0] + sd.viewInverse[1][1] * vd[1] + sd.viewInverse[2][1] * vd[2],
                           sd.viewInverse[0][2] * vd[0] + sd.viewInverse[1][2] * vd[1] + sd.viewInverse[2][2] * vd[2]);
    return normalize(d);
}

// emitter-hit MIS against emissive-triangle NEE (integrator/path/loop.slang:62-80, light/direct/mis_weights.slang)
VKRT_DEV float emitterLightPdfSA(const DeviceScene& sc, uint32_t mesh, float t, float3 d, float3 gn) {
    float lpa = sc.meshes[mesh].lightPdfArea;
    if (lpa <= 0.0f) return 0.0f;
    float d2 = t * t;
    float cl = fabsf(dot(d, gn));
    if (d2 <= 0.0f || cl <= 0.0f) return 0.0f;
    return lpa * d2 / cl;
}

VKRT_DEV float srgbEncode(float v) {
    return v <= 0.0031308f ? 12.92f * v : 1.055f * powf(v, 1.0f / 2.4f) - 0.055f;
}

VKRT_DEV ushort4 encodeOutput(const VKRT_CudaSceneData& sd, float3 acc, bool spectral) {
    float3 c = spectral ? xyzToLinearSrgb(acc) : acc;
    c = fmax3(c * sd.exposure, f3(0.0f));
    if (VKRT_CUDA_TONE_MAPPING_OF(sd.packedRenderSettings) == VKRT_CUDA_TONE_MAPPING_ACES) {
        float3 n = c * (c * 2.51f + f3(0.03f));
        float3 dd = c * (c * 2.43f + f3(0.59f)) + f3(0.14f);
        c = make_float3(n.x / dd.x, n.y / dd.y, n.z / dd.z);
    }
    c = sat(c);
    return make_ushort4((unsigned short)lrintf(sat(srgbEncode(c.x)) * 65535.0f),
                        (unsigned short)lrintf(sat(srgbEncode(c.y)) * 65535.0f),
                        (unsigned short)lrintf(sat(srgbEncode(c.z)) * 65535.0f), 65535);
}


}  // namespace vkrt
