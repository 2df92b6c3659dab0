// render.h — host-side launchers of the render, trace, film, environment and rgb2spec kernels.
#pragma once

#include <cuda_runtime.h>

#include "scene.cuh"

namespace vkrt {

struct RenderParams {
    uint32_t rngMode;
    uint64_t rngSeed;
    uint32_t envNee;     // environment importance sampling active for this frame
    uint32_t width;      // film size (the viewport rectangle lives in SceneData)
    uint32_t height;
    uint32_t countBytes; // accumulate node / triangle fetch bytes
    uint32_t extended;   // some material uses vkrt's stack beyond the glTF subset, alpha tests included
    uint32_t alpha;      // some material or mesh is alpha-tested (rt/alpha_test.slang)
};

struct FilmBuffers {
    float4* accumRead;
    float4* accumWrite;
    ushort4* output;
    // denoiser feature films (albedo, shading normal; .w = resolved samples), ping-ponged like the accumulation;
    // null when the context does not render features
    float4* albedoRead = nullptr;
    float4* albedoWrite = nullptr;
    float4* normalRead = nullptr;
    float4* normalWrite = nullptr;
};

// writeback.slang:72-114 for a feature film: the frame mean (sum / weight) blended into the running mean by weight
VKRT_DEV void blendFeature(const float4* read, float4* write, size_t pix, float3 sum, float weight) {
    const float4 prev = read[pix];
    const float tw = prev.w + weight;
    float3 v = f3(0.0f);
    if (tw > 0.0f) v = (xyz(prev) * prev.w + sum) / tw;
    write[pix] = make_float4(v.x, v.y, v.z, tw);
}

// One frame of vkrt's ray-generation pass (entry/path/raygen_rgb.slang / raygen_spectral_hero.slang).
cudaError_t launchRender(const DeviceScene& sc, const VKRT_CudaSceneData& sd, const RenderParams& rp,
                         const FilmBuffers& film, RenderCounters* counters, uint32_t threadsPerBlock,
                         cudaStream_t stream);

cudaError_t launchTraceRays(const DeviceScene& sc, const VKRT_CudaRay* rays, uint32_t count, uint32_t anyHit,
                            VKRT_CudaHit* hits, RenderCounters* counters, cudaStream_t stream);

cudaError_t launchClearFilm(float4* a, float4* b, ushort4* out, size_t pixels, cudaStream_t stream);

// Environment importance distribution from an RGBA32F lat-long map; buffers sized by the caller:
// marginal H+1, conditional H*(W+1), texelPdf W*H floats; scratch (W*H + H) doubles + 2 doubles.
cudaError_t launchBuildEnvDistribution(const float4* texels, uint32_t width, uint32_t height, float* marginal,
                                       float* conditional, float* texelPdf, double* scratch, cudaStream_t stream);

// Guide tables of the environment CDFs (kEnvGuide + 1 entries per CDF; marginal guide, then one per row).
cudaError_t launchBuildEnvGuides(const float* marginal, const float* conditional, uint32_t width, uint32_t height,
                                 uint32_t* marginalGuide, uint32_t* conditionalGuide, cudaStream_t stream);

// rgb2spec coefficients starting at dataOffset repacked to 3*res^3 float4 cells.
cudaError_t launchRepackRgb2Spec(const float* table, uint32_t res, uint32_t dataOffset, float4* cells,
                                 cudaStream_t stream);

// Brightness guide of an rgb2spec table: kRgb2SpecGuide + 1 interval indices (see DeviceScene::rgb2specGuide).
cudaError_t launchRgb2SpecGuide(const float* table, uint32_t res, uint32_t scaleOffset, uint16_t* guide,
                                cudaStream_t stream);

// rgb2spec table fit on the device; `table` holds res + 3*res^3*3 floats.
cudaError_t launchGenerateRgb2Spec(uint32_t res, float* table, cudaStream_t stream);

}  // namespace vkrt
