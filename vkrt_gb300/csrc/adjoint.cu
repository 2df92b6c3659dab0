// adjoint.cu — path-replay backpropagation (Vicini, Speierer, Jakob 2021) for vkrt's RGB integrator on sm_103a.
//
// Differentiates the frame that render_frame produced with the same seeds, sample indices and scene: given
// dLoss/d(film), it adds dLoss/d(parameter) to per-texel and per-material gradient buffers for
//   base colour       Material.baseColor and the texels of the baseColor texture (material/textures.slang:123-141)
//   roughness         Material.roughness and the G texels of the metallic-roughness texture
//   emitter radiance  emissionColor x emissionLuminance of each material, through both emitter hits and NEE.
//
// Two implementations share the per-vertex arithmetic of adjoint.cuh:
//   * this file: one thread per (pixel, sample). Pass 0 runs the forward path (path.cuh, the megakernel's
//     arithmetic) and keeps its total radiance L; pass 1 replays it with the same random numbers and scatters each
//     vertex's gradient to the bilinear texel footprint of its hit with atomics, reusing pass 0's closest hits and
//     shadow visibility for the first kReplayCache vertices.
//   * wavefront.cu: a primal wavefront pass stores L per (pixel, sample) and an adjoint wavefront pass replays the
//     paths through the stage kernels, finishing each vertex once its shadow rays have been traced.
// Sampling decisions, MIS weights and Russian roulette are held fixed (detached), which is unbiased for the gradient
// of the expected image; when no sampling density depends on the differentiated parameters and Russian roulette is
// off, the result is the exact derivative of the fixed-seed estimator, so it matches central differences with common
// random numbers.
#include <cuda_runtime.h>

#include <algorithm>

#include "adjoint.cuh"

namespace vkrt {

namespace {

constexpr uint32_t kAdjThreads = 128;
constexpr uint32_t kReplayCache = 8;

// ---------------------------------------------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kAdjThreads) kAdjoint(DeviceScene sc, VKRT_CudaSceneData sd, AdjointParams ap,
                                                        RenderCounters* counters) {
    extern __shared__ uint2 smemStack[];
    __shared__ MaterialGradient smemMatStorage[kSmemMaterials];
    MaterialGradient* smemMat = sc.materialCount <= kSmemMaterials ? smemMatStorage : nullptr;
    clearMaterialSmem(smemMat, sc.materialCount);
    __syncthreads();
    const uint32_t vx0 = sd.viewportRect[0], vy0 = sd.viewportRect[1];
    const uint32_t vw = sd.viewportRect[2], vh = sd.viewportRect[3];
    const uint32_t spp = max(sd.samplesPerPixel, 1u);
    const uint32_t pixels = vw * vh;
    const uint32_t items = pixels * spp;
    const float invTw = 1.0f / float(ap.sampleBase + spp);
    KernelCtx k{sc, sd, smemStack + threadIdx.x, blockDim.x, counters};
    const StepConfig cfg{false, sd.misNeeEnabled != 0u && sd.emissiveMeshCount > 0u, ap.envNee != 0u, ap.rngMode,
                         ap.rngSeed};
    const SpecTable tab = makeSpecTable(sc, sd);
    PathCounts pc{0u, 0u, 0u, 0u};
    for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item < items; item += gridDim.x * blockDim.x) {
        // sample-major order: a warp holds neighbouring pixels of one sample, so its texel atomics spread out
        const uint32_t sample = item / pixels, local = item % pixels;
        const int px = int(vx0 + local % vw), py = int(vy0 + local / vw);
        const uint32_t pix = uint32_t(py) * ap.width + uint32_t(px);
        const float3 delta = xyz(ap.dImage[pix]) * invTw;
        if (delta.x == 0.0f && delta.y == 0.0f && delta.z == 0.0f) continue;
        TraceHit cache[kReplayCache];
        uint32_t visBits = 0u;
        float3 total = f3(0.0f);
        // pass 0 runs the forward path and keeps its radiance; pass 1 replays it with the same random numbers and
        // accumulates gradients vertex by vertex. One loop body serves both passes, so the path step, the
        // traversal and the gradient code each exist once in the kernel.
        for (uint32_t pass = 0; pass < 2u; ++pass) {
            const bool grad = pass == 1u;
            PathState p = beginPath<false>(cfg, sd, px, py, ap.sampleBase + sample);
            for (uint32_t v = 0;; ++v) {
                const bool cached = grad && v < kReplayCache;
                TraceHit h;
                if (cached) {
                    h = cache[v];
                } else {
                    h = closest<false>(k, p.o, p.d);
                    if (v == 0u) pc.primary++;
                    else pc.extension++;
                    if (v < kReplayCache) cache[v] = h;
                }
                AdjVertex av;
                av.hasSurface = av.emitted = av.sampled = false;
                av.reqValid[0] = av.reqValid[1] = false;
                ShadowRequest sh[2];
                uint32_t ns;
                bool cont = shadePathVertex<false, AdjointHook>(sc, sd, cfg, tab, p, h, sh, ns,
                                                                AdjointHook{grad ? &av : nullptr, delta});
                bool vis[2] = {false, false};
                for (uint32_t i = 0; i < ns; ++i) {
                    if (cached) {
                        vis[i] = ((visBits >> (2u * v + i)) & 1u) != 0u;
                    } else {
                        pc.shadow++;
                        TraceRay r{sh[i].origin, sh[i].dir, kTMin, sh[i].tmax};
                        vis[i] = traceBvh<true, false>(sc, r, k.stackColumn, k.stackStride, counters).mesh ==
                                 VKRT_CUDA_INVALID_INDEX;
                        if (vis[i] && v < kReplayCache) visBits |= 1u << (2u * v + i);
                    }
                    if (vis[i]) p.radiance += sh[i].contribution;
                }
                if (grad && av.hasSurface) {
                    if (ap.wantEmission && av.emitted) scatterHitEmission(sc, ap, smemMat, av);
                    finishVertex(sc, ap, smemMat, av, vis, cont, delta, total, xyz(p.radiance));
                }
                if (!cont) break;
            }
            if (!grad) total = xyz(p.radiance);
        }
        pc.samples++;
    }
    __syncthreads();
    flushMaterialSmem(ap, smemMat, sc.materialCount);
    if (blockIdx.x == 0 && threadIdx.x == 0 && counters) atomicAdd(&counters->kernelLaunches, 1ull);
    for (int off = 16; off > 0; off >>= 1) {
        pc.primary += __shfl_xor_sync(0xFFFFFFFFu, pc.primary, off);
        pc.extension += __shfl_xor_sync(0xFFFFFFFFu, pc.extension, off);
        pc.shadow += __shfl_xor_sync(0xFFFFFFFFu, pc.shadow, off);
        pc.samples += __shfl_xor_sync(0xFFFFFFFFu, pc.samples, off);
    }
    if ((threadIdx.x & 31u) == 0u && counters) {
        atomicAdd(&counters->primaryRays, (unsigned long long)pc.primary);
        atomicAdd(&counters->extensionRays, (unsigned long long)pc.extension);
        atomicAdd(&counters->shadowRays, (unsigned long long)pc.shadow);
        atomicAdd(&counters->pathSamples, (unsigned long long)pc.samples);
    }
}

}  // namespace

cudaError_t launchAdjoint(const DeviceScene& sc, const VKRT_CudaSceneData& sd, const AdjointParams& ap,
                          RenderCounters* counters, cudaStream_t stream) {
    const uint64_t items = uint64_t(sd.viewportRect[2]) * sd.viewportRect[3] * std::max(sd.samplesPerPixel, 1u);
    if (items == 0) return cudaSuccess;
    if (items > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    int device = 0, sms = 0, perSM = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const size_t smem = size_t(kAdjThreads) * VKRT_SMEM_STACK * sizeof(uint2);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kAdjoint, kAdjThreads, smem);
    // a resident grid that loops over the items: blocks flush their material gradients once, at the end
    const uint64_t needed = (items + kAdjThreads - 1) / kAdjThreads;
    const uint32_t blocks = uint32_t(std::min<uint64_t>(needed, uint64_t(std::max(sms, 1)) * std::max(perSM, 1)));
    kAdjoint<<<blocks, kAdjThreads, smem, stream>>>(sc, sd, ap, counters);
    return cudaGetLastError();
}

}  // namespace vkrt
