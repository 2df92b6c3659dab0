// noalloc.cu — ray tracing through the C ABI for callers that must not allocate device memory.
//
// vkrt_cuda_trace_rays stages the caller's rays and the hit records in buffers it allocates with cudaMalloc and
// frees with cudaFree on every call. Some callers cannot allow that: a frame loop on a real-time thread (cudaFree
// synchronises the whole device and stalls every stream, including the presentation work of that frame), a
// host that runs under a fixed device-memory budget handed out up front, or code that must not fail with
// out-of-memory halfway through a frame. vkrt_cuda_trace_rays_noalloc gives them the same trace with its staging
// in two file-scope device arrays of a fixed size instead: no cudaMalloc, cudaFree or allocating library call.
//
// Limits and sharing rules:
//  * at most kNoAllocMaxRays (65,536) rays per call; larger counts are rejected with VKRT_CUDA_ERROR_INVALID_ARGUMENT;
//  * the arrays (2 MiB of rays + 2 MiB of hits) exist once per device that loads the library and stay until the
//    process exits;
//  * every call on a device uses the same arrays and they keep the previous call's contents; each call overwrites
//    the rays and hits it uses, so nothing needs clearing, but two calls whose work overlaps on the GPU (different
//    streams or contexts on one device) race on the arrays and must be serialised by the caller;
//  * the first call on a device resolves the arrays' device addresses (cudaGetSymbolAddress with that device
//    current) and caches them; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "context_view.h"
#include "render.h"
#include "vkrt_cuda.h"

namespace {

constexpr uint32_t kNoAllocMaxRays = 65536;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) VKRT_CudaRay gNoAllocRays[kNoAllocMaxRays];
static __device__ __align__(256) VKRT_CudaHit gNoAllocHits[kNoAllocMaxRays];

struct ScratchAddresses {
    VKRT_CudaRay* rays;
    VKRT_CudaHit* hits;
    bool ready;
};

std::mutex gScratchMutex;
ScratchAddresses gScratch[kMaxDevices];

// Device addresses of the scratch arrays on `device` (which must be current). In host code the symbols name
// host-side stand-ins, never device memory, so only these resolved addresses are handed to kernels and copies.
cudaError_t scratchFor(int device, ScratchAddresses& out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(gScratchMutex);
    ScratchAddresses& s = gScratch[device];
    if (!s.ready) {
        void* rays = nullptr;
        void* hits = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&rays, gNoAllocRays);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress(&hits, gNoAllocHits);
        if (e != cudaSuccess) return e;
        s.rays = static_cast<VKRT_CudaRay*>(rays);
        s.hits = static_cast<VKRT_CudaHit*>(hits);
        s.ready = true;
    }
    out = s;
    return cudaSuccess;
}

}  // namespace

extern "C" int32_t vkrt_cuda_trace_rays_noalloc(VKRT_CudaContext* c, const VKRT_CudaRay* rays, uint32_t count,
                                                uint32_t anyHit, VKRT_CudaHit* hits) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (count && (!rays || !hits)) {
        vkrt::contextSetError(c, "invalid argument: null ray or hit array");
        return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    }
    if (count > kNoAllocMaxRays) {
        vkrt::contextSetError(c, "invalid argument: vkrt_cuda_trace_rays_noalloc takes at most 65536 rays per call");
        return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    }
    if (count == 0) return VKRT_CUDA_SUCCESS;
    vkrt::ContextView v = vkrt::contextView(c);
    cudaError_t e = cudaSetDevice(v.device);
    ScratchAddresses s{};
    if (e == cudaSuccess) e = scratchFor(v.device, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.rays, rays, sizeof(VKRT_CudaRay) * count, cudaMemcpyHostToDevice, v.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(v.counters, 0, sizeof(vkrt::RenderCounters), v.stream);
    if (e == cudaSuccess) {
        // traversal reads only the BVH; textures and shading records are not touched
        vkrt::DeviceScene scene{};
        scene.nodes = v.nodes;
        scene.tris = v.tris;
        scene.nodeCount = v.nodeCount;
        scene.triCount = v.triCount;
        e = vkrt::launchTraceRays(scene, s.rays, count, anyHit, s.hits, v.counters, v.stream);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hits, s.hits, sizeof(VKRT_CudaHit) * count, cudaMemcpyDeviceToHost, v.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
    if (e != cudaSuccess) {
        vkrt::contextSetError(c, cudaGetErrorString(e));
        return e == cudaErrorInvalidDevice ? VKRT_CUDA_ERROR_INVALID_ARGUMENT : VKRT_CUDA_ERROR_OPERATION_FAILED;
    }
    vkrt::contextMarkCountersPending(c);
    return VKRT_CUDA_SUCCESS;
}
