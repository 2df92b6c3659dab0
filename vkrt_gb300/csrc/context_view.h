// context_view.h — what entry points living outside capi.cu may read from a context.
#pragma once

#include <cuda_runtime.h>

#include "scene.cuh"

namespace vkrt {

struct ContextView {
    int device;
    cudaStream_t stream;
    RenderCounters* counters;
    const WideNode* nodes;
    const TriRecord* tris;
    uint32_t nodeCount;
    uint32_t triCount;
};

ContextView contextView(VKRT_CudaContext* c);
void contextSetError(VKRT_CudaContext* c, const char* message);
void contextMarkCountersPending(VKRT_CudaContext* c);

}  // namespace vkrt
