// overlay.cu — vkrt's selection passes on sm_103a: the selection mask of the selected mesh, the outline post-pass
// that draws its silhouette into the display image, and the pick query that names the mesh under a pixel.
//
//   selection mask  src/shaders/entry/select/raygen.slang:5-14 (+ rt/queries/selection_query.slang:7-11): per
//                   pixel, a pixel-centre camera ray traced with first-hit termination against a TLAS that holds
//                   the selected mesh alone; mask = hit. Here: the scene BVH with hits restricted to that mesh.
//                   Mask cut-outs do not count (selectionAlphaHitAccepted, rt/alpha_test.slang:68-76).
//   outline         src/shaders/entry/post/outline.slang:9-60: 16 x 16 tiles, the mask tile plus a 5-pixel apron
//                   in shared memory; a pixel outside the mask with a masked pixel within the square of radius
//                   clamp(round(min(W, H) * 2 / 1080), 1, 5) takes the outline colour (1, 0.55, 0.1)
//                   (scene/constants.slang:17-18), its alpha kept.
//   pick            src/shaders/integrator/path/debug.slang:21-29: the closest hit of the pixel-centre camera ray,
//                   mask cut-outs dropped as for the selection rays (the deterministic part of the path any-hit).
#include <cuda_runtime.h>

#include "integrator.cuh"
#include "overlay.h"
#include "traverse.cuh"

namespace vkrt {

namespace {

constexpr int kOutlineGroup = 16;
constexpr int kOutlineMaxRadius = 5;
constexpr int kOutlineSpan = kOutlineGroup + 2 * kOutlineMaxRadius;
constexpr uint32_t kMaskThreads = 128;

VKRT_DEV bool insideViewport(const VKRT_CudaSceneData& sd, int px, int py) {
    const int vx0 = int(sd.viewportRect[0]), vy0 = int(sd.viewportRect[1]);
    const int vw = int(sd.viewportRect[2]), vh = int(sd.viewportRect[3]);
    return vw > 0 && vh > 0 && px >= vx0 && py >= vy0 && px < vx0 + vw && py < vy0 + vh;
}

__global__ void __launch_bounds__(kMaskThreads) kSelectionMask(DeviceScene sc, VKRT_CudaSceneData sd, uint32_t width,
                                                                uint32_t height, uint32_t* __restrict__ mask) {
    extern __shared__ uint2 smemStack[];
    const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= width * height) return;
    const int px = int(pixel % width), py = int(pixel / width);
    uint32_t m = 0u;
    if (sd.selectionEnabled != 0u && sd.selectedMeshIndex != VKRT_CUDA_INVALID_INDEX && insideViewport(sd, px, py)) {
        float3 org;
        const float3 dir = primaryRay(sd, px, py, 0.0f, 0.0f, org);
        const TraceRay r{org, dir, kTMin, kTMax};
        const TraceHit h = traceBvh<true, false, true, false, 2>(sc, r, smemStack + threadIdx.x, blockDim.x, nullptr,
                                                       sd.selectedMeshIndex);
        m = h.mesh != VKRT_CUDA_INVALID_INDEX ? 1u : 0u;
    }
    mask[pixel] = m;
}

__global__ void __launch_bounds__(kOutlineGroup* kOutlineGroup)
    kOutline(const uint32_t* __restrict__ mask, uint32_t width, uint32_t height, ushort4* __restrict__ output) {
    __shared__ uint8_t tile[kOutlineSpan * kOutlineSpan];
    const int baseX = int(blockIdx.x) * kOutlineGroup - kOutlineMaxRadius;
    const int baseY = int(blockIdx.y) * kOutlineGroup - kOutlineMaxRadius;
    for (int ty = int(threadIdx.y); ty < kOutlineSpan; ty += kOutlineGroup)
        for (int tx = int(threadIdx.x); tx < kOutlineSpan; tx += kOutlineGroup) {
            const int sx = baseX + tx, sy = baseY + ty;
            uint8_t v = 0;
            if (sx >= 0 && sy >= 0 && sx < int(width) && sy < int(height))
                v = mask[size_t(sy) * width + size_t(sx)] != 0u ? 1 : 0;
            tile[ty * kOutlineSpan + tx] = v;
        }
    __syncthreads();
    const int px = int(blockIdx.x) * kOutlineGroup + int(threadIdx.x);
    const int py = int(blockIdx.y) * kOutlineGroup + int(threadIdx.y);
    if (px >= int(width) || py >= int(height)) return;
    // halfway cases of the rounding (min dimension 1350 or 2430) go to the even radius
    const int radius = min(max(int(rintf(float(min(width, height)) * (2.0f / 1080.0f))), 1), kOutlineMaxRadius);
    const int cx = int(threadIdx.x) + kOutlineMaxRadius, cy = int(threadIdx.y) + kOutlineMaxRadius;
    if (tile[cy * kOutlineSpan + cx] != 0) return;
    for (int dy = -radius; dy <= radius; ++dy)
        for (int dx = -radius; dx <= radius; ++dx) {
            if ((dx == 0 && dy == 0) || tile[(cy + dy) * kOutlineSpan + cx + dx] == 0) continue;
            ushort4& o = output[size_t(py) * width + size_t(px)];
            // (1, 0.55, 0.1) stored to RGBA16 UNORM: round(c * 65535)
            o = make_ushort4(65535u, 36044u, 6554u, o.w);
            return;
        }
}

__global__ void kPick(DeviceScene sc, VKRT_CudaSceneData sd, uint32_t x, uint32_t y, uint32_t* __restrict__ out) {
    extern __shared__ uint2 smemStack[];
    if (threadIdx.x != 0u) return;
    uint32_t mesh = VKRT_CUDA_INVALID_INDEX;
    if (insideViewport(sd, int(x), int(y))) {
        float3 org;
        const float3 dir = primaryRay(sd, int(x), int(y), 0.0f, 0.0f, org);
        const TraceRay r{org, dir, kTMin, kTMax};
        mesh = traceBvh<false, false, false, false, 2>(sc, r, smemStack, 1u, nullptr).mesh;
    }
    *out = mesh;
}

}  // namespace

cudaError_t launchSelectionMask(const DeviceScene& sc, const VKRT_CudaSceneData& sd, uint32_t width, uint32_t height,
                                uint32_t* mask, cudaStream_t stream) {
    const size_t pixels = size_t(width) * height;
    if (pixels == 0) return cudaSuccess;
    const size_t smem = size_t(kMaskThreads) * VKRT_SMEM_STACK * sizeof(uint2);
    kSelectionMask<<<uint32_t((pixels + kMaskThreads - 1) / kMaskThreads), kMaskThreads, smem, stream>>>(
        sc, sd, width, height, mask);
    return cudaGetLastError();
}

cudaError_t launchOutline(const uint32_t* mask, uint32_t width, uint32_t height, ushort4* output,
                          cudaStream_t stream) {
    if (width == 0 || height == 0) return cudaSuccess;
    const dim3 grid((width + kOutlineGroup - 1) / kOutlineGroup, (height + kOutlineGroup - 1) / kOutlineGroup);
    kOutline<<<grid, dim3(kOutlineGroup, kOutlineGroup), 0, stream>>>(mask, width, height, output);
    return cudaGetLastError();
}

cudaError_t launchPick(const DeviceScene& sc, const VKRT_CudaSceneData& sd, uint32_t x, uint32_t y, uint32_t* out,
                       cudaStream_t stream) {
    kPick<<<1, 32, VKRT_SMEM_STACK * sizeof(uint2), stream>>>(sc, sd, x, y, out);
    return cudaGetLastError();
}

}  // namespace vkrt
