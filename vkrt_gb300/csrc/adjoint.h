// adjoint.h — host interface of the path-replay adjoint integrator (adjoint.cu).
#pragma once

#include <cuda_runtime.h>

#include "render.h"

namespace vkrt {

// Gradient of the loss with respect to one material's parameters (layout of VKRT_CudaMaterialGradient).
struct MaterialGradient {
    float4 base;      // xyz: baseColor, w: roughness
    float4 emission;  // xyz: emission radiance (emissionColor x emissionLuminance), w: unused
};

struct AdjointParams {
    uint32_t rngMode;
    uint64_t rngSeed;
    uint32_t envNee;
    uint32_t width, height;       // film size; dImage holds width * height RGBA32F values
    uint32_t sampleBase;          // sample index of the differentiated frame's first sample
    uint32_t wantBase, wantRoughness, wantEmission;
    const float4* dImage;         // dLoss / d(accumulated film), alpha ignored
    float4* const* textureGrad;   // VKRT_CUDA_MAX_TEXTURES entries, null where no gradient is kept
    MaterialGradient* materialGrad;          // materialCount entries
    const uint32_t* emissiveMeshMaterial;    // emissiveMeshCount entries (material of each emissive mesh)
};

// Gradients of sum(dImage * film) for the frame rendered by the same seeds and sample indices, added to the
// gradient buffers.
cudaError_t launchAdjoint(const DeviceScene& sc, const VKRT_CudaSceneData& sd, const AdjointParams& ap,
                          RenderCounters* counters, cudaStream_t stream);

}  // namespace vkrt
