// overlay.h — host-side launchers of the selection passes (overlay.cu).
#pragma once

#include <cuda_runtime.h>

#include "scene.cuh"

namespace vkrt {

// width x height mask: 1 where the pixel-centre camera ray hits sd.selectedMeshIndex (0 everywhere when
// sd.selectionEnabled is 0 or no mesh is selected, and outside the viewport)
cudaError_t launchSelectionMask(const DeviceScene& sc, const VKRT_CudaSceneData& sd, uint32_t width, uint32_t height,
                                uint32_t* mask, cudaStream_t stream);

// draws the outline of `mask` into the RGBA16 display image
cudaError_t launchOutline(const uint32_t* mask, uint32_t width, uint32_t height, ushort4* output,
                          cudaStream_t stream);

// mesh index of the closest hit of pixel (x, y)'s centre ray (VKRT_CUDA_INVALID_INDEX on a miss) into *out (device)
cudaError_t launchPick(const DeviceScene& sc, const VKRT_CudaSceneData& sd, uint32_t x, uint32_t y, uint32_t* out,
                       cudaStream_t stream);

}  // namespace vkrt
