// wavefront.h — host interface of the batched wavefront integrator (wavefront.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "adjoint.h"
#include "nrc.h"
#include "render.h"
#include "scene.cuh"

namespace vkrt {

// one scene of a batch as the stage kernels read it
struct WfScene {
    DeviceScene sc;
    VKRT_CudaSceneData sd;
    FilmBuffers film;
    uint32_t filmWidth, filmHeight;
    uint32_t vx0, vy0, vw, vh;  // viewport rectangle
    uint32_t spp;
    uint32_t spectral;
    uint32_t neeEnabled;
    uint32_t envNee;
    uint32_t extended;      // some material uses vkrt's stack beyond the glTF subset (the full instantiations)
    uint32_t transmissive;  // some material has transmission (media, per-lane hero pdfs, transmissive shadows)
    uint32_t alpha;         // some material or mesh is alpha-tested (alpha-aware intersect and shadow kernels)
    // filled by the engine
    uint32_t tileW, tileH, tilesX;
    uint32_t workBase, workCount;  // padded pixel work items (tile order)
    uint32_t itemBase;             // first (pixel, sample) item of the scene; items of a pixel are consecutive
    uint32_t materialKeyBase;      // first shade-order key of the scene's materials (material-ordered shading)
};

// forward: a frame blended into each scene's film; primal: the same paths, each (pixel, sample) radiance kept in the
// engine's sample buffer and the film untouched; adjoint: the primal paths replayed with gradients (one scene)
// train: the radiance cache's training paths of a cache frame (items are training paths at hashed pixels of the
// scene; their surface vertices become training records)
enum WavefrontMode : uint32_t { kWavefrontForward = 0, kWavefrontPrimal = 1, kWavefrontAdjoint = 2, kWavefrontTrain = 3 };

struct WavefrontConfig {
    uint32_t queueCapacity;  // path slots; 0 = one per (pixel, sample) item, capped at 64M
    uint32_t tileWidth;
    uint32_t tileHeight;
    uint32_t sortByMaterial;
    uint32_t intersectBlocksPerSM;
    uint32_t shadeBlocksPerSM;
    uint32_t useGraph;
    uint32_t profileStages;  // 1: no graph; traversal kernels count fetch bytes; per-stage device times recorded
    uint32_t refillLanes;    // persistent traversal refill threshold (lanes still traversing), 1..32
    uint32_t rayOrder;       // 1: traversal queues binned by ray-direction octant
};

// stages of the per-stage device times
enum WavefrontStage : uint32_t {
    kStagePrologue = 0, kStageBegin, kStageIntersect, kStageSort, kStageShade, kStageShadow, kStageFinalize,
    kStageResolve, kStageCount
};

// Radiance cache of a forward frame (one scene): trained on `trainingPaths` paths first, then queried by render paths
// at surface depth `cacheDepth`.
struct WfCacheFrame {
    NrcEngine* engine;
    uint32_t cacheDepth;
    uint32_t trainingPaths;
    uint32_t trainingSteps;
    uint32_t seed;
    uint32_t frame;
    float cacheSpread;  // area-spread constant c (0: paths end at cacheDepth only)
    uint32_t trainingTracer;  // 0: one thread per training path; 1: the training paths run as a wavefront pass
};

class WavefrontEngine {
public:
    WavefrontEngine();
    ~WavefrontEngine();
    WavefrontEngine(const WavefrontEngine&) = delete;
    WavefrontEngine& operator=(const WavefrontEngine&) = delete;

    // Renders one frame of every scene (all spectral or all RGB) on `stream`, asynchronously.
    // `adjoint` is read in adjoint mode, which must follow a primal pass over the same scene, configuration and
    // sampleBase.
    cudaError_t render(const std::vector<WfScene>& scenes, bool spectral, const WavefrontConfig& cfg,
                       uint32_t rngMode, uint64_t rngSeed, RenderCounters* counters, cudaStream_t stream,
                       WavefrontMode mode = kWavefrontForward, const AdjointParams* adjoint = nullptr,
                       const WfCacheFrame* cache = nullptr);
    // records and steps of the last cache training
    uint32_t lastCacheRecords() const;
    // the last cache frame's training records (NrcInput and float4 target each), up to `capacity`; *count = records
    cudaError_t readTrainingRecords(void* inputs, void* targets, uint32_t capacity, uint32_t* count,
                                    cudaStream_t stream) const;
    void release();
    // per-stage device milliseconds of the last render call made with profileStages (zeros otherwise)
    const float* lastStageMs() const;

private:
    cudaError_t trainOnRecords(const WfCacheFrame& cache, cudaStream_t stream);
    struct Buffers;
    Buffers* b_;
};

}  // namespace vkrt
