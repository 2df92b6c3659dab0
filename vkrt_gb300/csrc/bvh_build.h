// bvh_build.h — host interface of the device BVH builder (bvh_build.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "scene.cuh"

namespace vkrt {

struct BvhBuildInput {
    const VKRT_CudaShaderVertex* vertices;  // device
    const uint32_t* indices;                // device
    const VKRT_CudaMeshInfo* meshes;        // device
    const VKRT_CudaMeshInfo* hostMeshes;    // host copy (triangle counts)
    const float* hostWorld;                 // host, 16 floats (column-major TRS) per mesh
    const uint32_t* hostIdentity;           // host, 1 when the mesh transform is the identity
    uint32_t meshCount;
    uint32_t triCount;
    uint32_t treeletPasses;  // bottom-up treelet restructuring passes after the LBVH (0: none)
};

struct BvhBuffers {
    WideNode* nodes = nullptr;
    TriRecord* tris = nullptr;
    uint32_t nodeCount = 0;
    uint32_t triCount = 0;
    void release();
};

struct BvhBuildStats {
    float buildMs;
    uint32_t nodeCount;
    uint32_t triCount;
    float sahLbvh;      // SAH cost of the binary tree / root area, before treelet restructuring
    float sahTreelets;  // after
};

// Builds the 8-wide BVH on `stream` (synchronises it). Scratch buffers are allocated and freed inside.
cudaError_t buildBvh(const BvhBuildInput& in, BvhBuffers& out, BvhBuildStats* stats, cudaStream_t stream);

}  // namespace vkrt
