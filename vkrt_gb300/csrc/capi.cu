// capi.cu — the extern "C" boundary declared in include/vkrt_cuda.h.
//
// A context owns one CUDA stream and every device buffer of one scene; uploads copy caller arrays (vkrt copies at
// upload too, src/core/scene/geometry.c:411-429) and kernels read only context memory. Errors follow VKRT_Result:
// invalid arguments -1, other failures -2, allocation failures -3, CUDA faults that poison the context -4.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "adjoint.h"
#include "bvh_build.h"
#include "nrc.h"
#include "overlay.h"
#include "context_view.h"
#include "render.h"
#include "wavefront.h"
#include "scene.cuh"
#include "vkrt_cuda.h"
#include "vkrt_cuda_host.h"

using namespace vkrt;

namespace {

template <class T>
struct DeviceArray {
    T* ptr = nullptr;
    size_t count = 0;
    cudaError_t assign(const T* host, size_t n, cudaStream_t s) {
        cudaError_t e = reserve(n);
        if (e != cudaSuccess || n == 0) return e;
        return cudaMemcpyAsync(ptr, host, sizeof(T) * n, cudaMemcpyHostToDevice, s);
    }
    cudaError_t reserve(size_t n) {
        if (n <= count && ptr) return cudaSuccess;
        release();
        if (n == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&ptr, sizeof(T) * n);
        if (e != cudaSuccess) {
            ptr = nullptr;
            return e;
        }
        count = n;
        return cudaSuccess;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
};

}  // namespace

struct VKRT_CudaContext {
    VKRT_CudaConfig cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string lastError = "";

    // geometry
    DeviceArray<VKRT_CudaShaderVertex> vertices;
    DeviceArray<uint32_t> indices;
    DeviceArray<VKRT_CudaMeshInfo> meshes;
    std::vector<VKRT_CudaMeshInfo> hostMeshes;
    uint32_t vertexCount = 0, indexCount = 0, triCount = 0;
    BvhBuffers bvh;
    BvhBuildStats bvhStats{};

    // materials, lights
    DeviceArray<VKRT_CudaMaterial> materials;
    std::vector<VKRT_CudaMaterial> hostMaterials;
    uint32_t materialCount = 0;
    bool extendedMaterials = false;     // some material has clearcoat, subsurface, diffuseRoughness or transmission
    bool transmissiveMaterials = false;  // some material has transmission above 0
    DeviceArray<VKRT_CudaEmissiveMesh> emissiveMeshes;
    DeviceArray<VKRT_CudaEmissiveTriangle> emissiveTriangles;
    DeviceArray<float> meshAliasQ, triAliasQ;
    DeviceArray<uint32_t> meshAliasIdx, triAliasIdx;
    uint32_t emissiveMeshCount = 0, emissiveTriangleCount = 0;

    // textures: one RGBA32F buffer per bound slot and the descriptor table the kernels index
    std::vector<DeviceArray<float4>> textureData;
    std::vector<TextureDesc> textureDescs;
    DeviceArray<TextureDesc> textureTable;
    bool textureTableDirty = true;

    // spectral table
    DeviceArray<float> rgb2spec;
    uint32_t rgb2specFloats = 0;
    DeviceArray<float> sheenTable;  // the sheen LTC table once uploaded (VKRT_CUDA_SHEEN_TABLE_FLOATS)
    bool sheenMaterials = false;    // some material has a sheen colour
    bool alphaTested = false;       // some mesh's material (or the mesh) is alpha-tested
    VKRT_CudaRGB2SpecTableInfo rgb2specInfo{};
    DeviceArray<float4> rgb2specCells;  // the table of rgb2specInfo repacked one float4 per cell
    DeviceArray<uint16_t> rgb2specGuide;  // its brightness guide

    // environment distribution
    DeviceArray<float> envMarginal, envConditional, envTexelPdf;
    DeviceArray<uint32_t> envMarginalGuide, envConditionalGuide;
    DeviceArray<double> envScratch;
    uint32_t envWidth = 0, envHeight = 0, envTexture = VKRT_CUDA_INVALID_INDEX;

    // film
    DeviceArray<float4> accum[2];
    DeviceArray<ushort4> output;
    // denoiser feature films (albedo, shading normal; .w = resolved samples), ping-ponged with the accumulation
    bool features = false;
    DeviceArray<float4> albedo[2], normal[2];
    uint32_t width = 0, height = 0;
    int readIndex = 0;
    // pipelined readback (vkrt_cuda_read_accumulation_async): copies of accum[b] on copyStream end at copyDone[b]
    cudaStream_t copyStream = nullptr;
    cudaEvent_t filmReady = nullptr, copyDone[2] = {nullptr, nullptr};
    bool copyPending[2] = {false, false};

    // counters
    RenderCounters* counters = nullptr;
    RenderCounters lastCounters{};
    bool countersPending = false;

    // wavefront integrator (owned by the context that leads a batch)
    VKRT_CudaWavefrontConfig wfCfg{};
    std::unique_ptr<WavefrontEngine> wavefront;
    cudaEvent_t order = nullptr;  // orders this context's stream against a batch leader's stream

    // path-replay adjoint: gradient buffers (per texture slot, per material) and its input
    std::vector<DeviceArray<float4>> textureGrad;
    DeviceArray<float4*> textureGradTable;
    DeviceArray<MaterialGradient> materialGrad;
    DeviceArray<uint32_t> emissiveMeshMaterial;
    uint32_t emissiveMeshMaterialCount = 0;
    DeviceArray<float4> dImage;

    // scene bounds of the uploaded geometry (world space)
    float3 boundsLo = make_float3(0.0f, 0.0f, 0.0f), boundsHi = make_float3(0.0f, 0.0f, 0.0f);
    // neural radiance cache
    VKRT_CudaNrcConfig nrcCfg{};
    std::unique_ptr<NrcEngine> nrc;
    DeviceArray<NrcInput> nrcIn;
    DeviceArray<float4> nrcTarget, nrcOut;
    DeviceArray<float> nrcLoss;

    // selection passes: mask of the selected mesh, pick result
    DeviceArray<uint32_t> selectionMask;
    DeviceArray<uint32_t> pickResult;
    // device time of the last render call (events on the context's stream around it)
    cudaEvent_t frameStart = nullptr, frameEnd = nullptr;
    bool frameTimed = false;
};

namespace {

int32_t fail(VKRT_CudaContext* c, cudaError_t e, const char* what) {
    if (c) c->lastError = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return VKRT_CUDA_ERROR_OUT_OF_MEMORY;
    // errors that leave the context unusable
    if (e == cudaErrorIllegalAddress || e == cudaErrorLaunchFailure || e == cudaErrorIllegalInstruction ||
        e == cudaErrorMisalignedAddress || e == cudaErrorHardwareStackError || e == cudaErrorAssert ||
        e == cudaErrorLaunchTimeout || e == cudaErrorECCUncorrectable)
        return VKRT_CUDA_ERROR_DEVICE_LOST;
    return VKRT_CUDA_ERROR_OPERATION_FAILED;
}

int32_t invalid(VKRT_CudaContext* c, const char* what) {
    if (c) c->lastError = std::string("invalid argument: ") + what;
    return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
}

#define VKRT_TRY(ctx, expr, what)                      \
    do {                                               \
        cudaError_t _e = (expr);                       \
        if (_e != cudaSuccess) return fail(ctx, _e, what); \
    } while (0)

bool isIdentityTRS(const VKRT_CudaMeshInfo& m) {
    return m.position[0] == 0.0f && m.position[1] == 0.0f && m.position[2] == 0.0f && m.rotation[0] == 0.0f &&
           m.rotation[1] == 0.0f && m.rotation[2] == 0.0f && m.scale[0] == 1.0f && m.scale[1] == 1.0f &&
           m.scale[2] == 1.0f;
}

// afterEdit: the rebuild follows a mesh-transform edit (treelets only when the config asks for them there)
cudaError_t rebuildBvh(VKRT_CudaContext* c, bool afterEdit) {
    std::vector<float> world(size_t(c->hostMeshes.size()) * 16);
    std::vector<uint32_t> ident(c->hostMeshes.size());
    for (size_t i = 0; i < c->hostMeshes.size(); ++i) {
        const VKRT_CudaMeshInfo& m = c->hostMeshes[i];
        vkrt_host_mesh_transform(m.position, m.rotation, m.scale, &world[i * 16]);
        ident[i] = isIdentityTRS(m) ? 1u : 0u;
    }
    BvhBuildInput in;
    in.vertices = c->vertices.ptr;
    in.indices = c->indices.ptr;
    in.meshes = c->meshes.ptr;
    in.hostMeshes = c->hostMeshes.data();
    in.hostWorld = world.data();
    in.hostIdentity = ident.data();
    in.meshCount = uint32_t(c->hostMeshes.size());
    in.triCount = c->triCount;
    const uint32_t minTris = c->cfg.treeletMinTriangles ? c->cfg.treeletMinTriangles : 65536u;
    const bool treelets = c->triCount >= minTris && (!afterEdit || c->cfg.treeletsOnUpdate != 0u);
    in.treeletPasses = treelets ? (c->cfg.treeletPasses ? c->cfg.treeletPasses : 2u) : 0u;
    return buildBvh(in, c->bvh, &c->bvhStats, c->stream);
}

// Work on `stream` that writes accum[b] first waits for a pipelined readback of that buffer still in flight.
cudaError_t awaitFilmCopy(VKRT_CudaContext* c, int b, cudaStream_t stream) {
    if (!c->copyPending[b]) return cudaSuccess;
    c->copyPending[b] = false;
    return cudaStreamWaitEvent(stream, c->copyDone[b], 0);
}
cudaError_t awaitFilmCopies(VKRT_CudaContext* c, cudaStream_t stream) {
    cudaError_t e = awaitFilmCopy(c, 0, stream);
    return e != cudaSuccess ? e : awaitFilmCopy(c, 1, stream);
}
// before the film buffers are reallocated or freed: no copy may still read them
cudaError_t drainFilmCopies(VKRT_CudaContext* c) {
    c->copyPending[0] = c->copyPending[1] = false;
    return c->copyStream ? cudaStreamSynchronize(c->copyStream) : cudaSuccess;
}

FilmBuffers filmOf(VKRT_CudaContext* c) {
    FilmBuffers f{c->accum[c->readIndex].ptr, c->accum[c->readIndex ^ 1].ptr, c->output.ptr};
    if (c->features) {
        f.albedoRead = c->albedo[c->readIndex].ptr;
        f.albedoWrite = c->albedo[c->readIndex ^ 1].ptr;
        f.normalRead = c->normal[c->readIndex].ptr;
        f.normalWrite = c->normal[c->readIndex ^ 1].ptr;
    }
    return f;
}

cudaError_t clearFeatureFilms(VKRT_CudaContext* c) {
    if (!c->features || !c->width) return cudaSuccess;
    const size_t bytes = size_t(c->width) * c->height * sizeof(float4);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = c->albedo[i].reserve(size_t(c->width) * c->height);
        if (e == cudaSuccess) e = c->normal[i].reserve(size_t(c->width) * c->height);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->albedo[i].ptr, 0, bytes, c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->normal[i].ptr, 0, bytes, c->stream);
    }
    return e;
}

DeviceScene makeDeviceScene(VKRT_CudaContext* c) {
    if (c->textureTableDirty) {
        c->textureTable.assign(c->textureDescs.data(), c->textureDescs.size(), c->stream);
        c->textureTableDirty = false;
    }
    DeviceScene s{};
    s.nodes = c->bvh.nodes;
    s.tris = c->bvh.tris;
    s.nodeCount = c->bvh.nodeCount;
    s.triCount = c->bvh.triCount;
    s.vertices = c->vertices.ptr;
    s.indices = c->indices.ptr;
    s.meshes = c->meshes.ptr;
    s.meshCount = uint32_t(c->hostMeshes.size());
    s.materials = c->materials.ptr;
    s.materialCount = c->materialCount;
    s.emissiveMeshes = c->emissiveMeshes.ptr;
    s.emissiveTriangles = c->emissiveTriangles.ptr;
    s.meshAliasQ = c->meshAliasQ.ptr;
    s.meshAliasIdx = c->meshAliasIdx.ptr;
    s.triAliasQ = c->triAliasQ.ptr;
    s.triAliasIdx = c->triAliasIdx.ptr;
    s.emissiveMeshCount = c->emissiveMeshCount;
    s.emissiveTriangleCount = c->emissiveTriangleCount;
    s.textures = c->textureTable.ptr;
    s.rgb2spec = c->rgb2spec.ptr;
    s.rgb2specFloatCount = c->rgb2specFloats;
    s.sheenLtc = c->sheenTable.ptr;
    s.rgb2specCells = c->rgb2specCells.ptr;
    s.rgb2specCellsInfo = c->rgb2specInfo;
    s.rgb2specGuide = c->rgb2specGuide.ptr;
    s.env.marginal = c->envMarginal.ptr;
    s.env.conditional = c->envConditional.ptr;
    s.env.texelPdf = c->envTexelPdf.ptr;
    s.env.marginalGuide = c->envMarginalGuide.ptr;
    s.env.conditionalGuide = c->envConditionalGuide.ptr;
    s.env.width = c->envWidth;
    s.env.height = c->envHeight;
    s.env.textureIndex = c->envTexture;
    return s;
}

uint16_t halfToFloatBits(uint16_t h, float& out) {
    uint32_t sign = (h >> 15) & 1u, exp = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
    float v;
    if (exp == 0) v = std::ldexp(float(man), -24);
    else if (exp == 31) v = man ? NAN : INFINITY;
    else v = std::ldexp(float(man | 0x400u), int(exp) - 25);
    out = sign ? -v : v;
    return 0;
}

float srgbToLinear(float c) { return c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f); }

int32_t validateFrame(VKRT_CudaContext* c, const VKRT_CudaSceneData* sd) {
    if (!sd) return invalid(c, "null SceneData");
    if (!c->width) return invalid(c, "no film: call vkrt_cuda_resize first");
    if (uint64_t(sd->viewportRect[0]) + sd->viewportRect[2] > c->width ||
        uint64_t(sd->viewportRect[1]) + sd->viewportRect[3] > c->height)
        return invalid(c, "viewport outside the film");
    if (sd->rrMaxDepth > 1024u) return invalid(c, "rrMaxDepth above 1024");
    // vkrt's debug views (constants.h:35-52, integrator/path/debug.slang) are not built: refuse rather than render
    // a normal frame in their place
    if (sd->debugMode != VKRT_CUDA_DEBUG_MODE_NONE) return invalid(c, "debug render modes are not built");
    if (sd->emissiveMeshCount > c->emissiveMeshCount) return invalid(c, "SceneData.emissiveMeshCount exceeds the uploaded lights");
    for (const VKRT_CudaMeshInfo& m : c->hostMeshes)
        if (m.materialIndex >= c->materialCount) return invalid(c, "mesh material index out of range");
    if (c->sheenMaterials && !c->sheenTable.ptr)
        return invalid(c, "a material has sheen: install vkrt's sheen LTC table (vkrt_cuda_upload_sheen_table)");
    const bool spectral = VKRT_CUDA_RENDER_MODE_OF(sd->packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL;
    if (spectral) {
        const VKRT_CudaRGB2SpecTableInfo& ti = sd->rgb2specSRGB;
        if (!c->rgb2spec.ptr || ti.res < 2 ||
            uint64_t(ti.scaleOffset) + ti.res > c->rgb2specFloats ||
            uint64_t(ti.dataOffset) + 9ull * ti.res * ti.res * ti.res > c->rgb2specFloats)
            return invalid(c, "spectral mode needs an rgb2spec table matching SceneData.rgb2specSRGB");
        const uint32_t sm = VKRT_CUDA_SPECTRAL_MODE_OF(sd->packedRenderSettings);
        if (sm != VKRT_CUDA_SPECTRAL_HERO && sm != VKRT_CUDA_SPECTRAL_SINGLE)
            return invalid(c, "unknown spectral sampling mode");
    }
    return VKRT_CUDA_SUCCESS;
}

// Environment NEE (this backend's addition) is off in scenes with transmissive materials, where vkrt's estimator
// (NEE unsupported through transmissive surfaces, no environment light inside media) has no environment technique.
// Which instantiations and kernels the scene's materials and meshes need (refreshed on every material or mesh upload)
void refreshMaterialFlags(VKRT_CudaContext* c) {
    c->extendedMaterials = c->transmissiveMaterials = c->sheenMaterials = c->alphaTested = false;
    for (const VKRT_CudaMaterial& m : c->hostMaterials) {
        // bsdfSheenColor (material.slang:63-73) is saturate(tint) * saturate(weight)
        const float w = std::min(std::max(m.sheenTintWeight[3], 0.0f), 1.0f);
        const float tint = std::max({m.sheenTintWeight[0], m.sheenTintWeight[1], m.sheenTintWeight[2]});
        if (w > 0.0f && tint > 0.0f) c->sheenMaterials = true;
        if (m.transmission > 0.0f) c->transmissiveMaterials = true;
        if (m.clearcoat > 0.0f || m.subsurface > 0.0f || m.diffuseRoughness > 0.0f || m.transmission > 0.0f)
            c->extendedMaterials = true;
    }
    for (const VKRT_CudaMeshInfo& mesh : c->hostMeshes) {  // alphaMayRejectHit (rt/alpha_test.slang:8-10)
        if (mesh.materialIndex >= c->hostMaterials.size()) continue;
        const VKRT_CudaMaterial& m = c->hostMaterials[mesh.materialIndex];
        if (m.alphaMode != VKRT_CUDA_ALPHA_MODE_OPAQUE || m.opacity < 0.999f || mesh.opacity < 0.999f)
            c->alphaTested = true;
    }
    if (c->sheenMaterials || c->alphaTested) c->extendedMaterials = true;
}

// Single-wavelength spectral mode (raygen_spectral_single.slang): paths carry one wavelength from the start and run
// the full-stack kernels, whose collapsed-path branch is that integrator.
bool singleWavelengthMode(const VKRT_CudaSceneData* sd) {
    return VKRT_CUDA_RENDER_MODE_OF(sd->packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL &&
           VKRT_CUDA_SPECTRAL_MODE_OF(sd->packedRenderSettings) == VKRT_CUDA_SPECTRAL_SINGLE;
}

bool envNeeActive(const VKRT_CudaContext* c, const VKRT_CudaSceneData* sd) {
    return c->cfg.environmentSampling == VKRT_CUDA_ENV_IMPORTANCE && c->envTexture != VKRT_CUDA_INVALID_INDEX &&
           sd->environmentTextureIndex == c->envTexture && sd->misNeeEnabled != 0u && !c->transmissiveMaterials &&
           !singleWavelengthMode(sd);
}

WfScene makeWfScene(VKRT_CudaContext* c, const VKRT_CudaSceneData& sd, bool spectral) {
    WfScene S;
    std::memset(&S, 0, sizeof(S));
    S.sc = makeDeviceScene(c);
    S.sd = sd;
    S.film = filmOf(c);
    S.filmWidth = c->width;
    S.filmHeight = c->height;
    S.vx0 = sd.viewportRect[0];
    S.vy0 = sd.viewportRect[1];
    S.vw = sd.viewportRect[2];
    S.vh = sd.viewportRect[3];
    S.spp = std::max(sd.samplesPerPixel, 1u);
    S.spectral = spectral ? 1u : 0u;
    S.neeEnabled = (sd.misNeeEnabled != 0u && sd.emissiveMeshCount > 0u) ? 1u : 0u;
    S.envNee = envNeeActive(c, &sd) ? 1u : 0u;
    S.extended = c->extendedMaterials || singleWavelengthMode(&sd) ? 1u : 0u;
    S.transmissive = c->transmissiveMaterials ? 1u : 0u;
    S.alpha = c->alphaTested ? 1u : 0u;
    return S;
}

WavefrontConfig engineConfig(const VKRT_CudaContext* c) {
    return WavefrontConfig{c->wfCfg.queueCapacity,  c->wfCfg.tileWidth,           c->wfCfg.tileHeight,
                           c->wfCfg.sortByMaterial, c->wfCfg.intersectBlocksPerSM, c->wfCfg.shadeBlocksPerSM,
                           c->wfCfg.useGraph,       c->wfCfg.profileStages,
                           c->wfCfg.refillLanes ? c->wfCfg.refillLanes : uint32_t(kVoteRefillLanes),
                           c->wfCfg.rayOrder};
}

}  // namespace

extern "C" {

void vkrt_cuda_default_config(VKRT_CudaConfig* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->deviceIndex = 0;
    cfg->rngMode = VKRT_CUDA_RNG_REFERENCE;
    cfg->rngSeed = 1u;
    cfg->environmentSampling = VKRT_CUDA_ENV_BSDF_ONLY;
    cfg->countRays = 0u;
    cfg->threadsPerBlock = 0u;
    cfg->blocksPerSM = 0u;
    cfg->integrator = VKRT_CUDA_INTEGRATOR_MEGAKERNEL;
}

int32_t vkrt_cuda_create(const VKRT_CudaConfig* config, VKRT_CudaContext** out) {
    if (!out) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    VKRT_CudaConfig cfg;
    if (config) cfg = *config;
    else vkrt_cuda_default_config(&cfg);
    if (cfg.rngMode > VKRT_CUDA_RNG_PCG32 || cfg.environmentSampling > VKRT_CUDA_ENV_IMPORTANCE ||
        cfg.treeletsOnUpdate > 1u || cfg.treeletPasses > 8u)
        return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0 || cfg.deviceIndex < 0 || cfg.deviceIndex >= count)
        return VKRT_CUDA_ERROR_INITIALIZATION_FAILED;
    if (cudaSetDevice(cfg.deviceIndex) != cudaSuccess) return VKRT_CUDA_ERROR_INITIALIZATION_FAILED;
    VKRT_CudaContext* c = new VKRT_CudaContext();
    c->cfg = cfg;
    c->device = cfg.deviceIndex;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->order, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&c->frameStart) != cudaSuccess || cudaEventCreate(&c->frameEnd) != cudaSuccess ||
        cudaMalloc(&c->counters, sizeof(RenderCounters)) != cudaSuccess) {
        if (c->order) cudaEventDestroy(c->order);
        if (c->frameStart) cudaEventDestroy(c->frameStart);
        if (c->frameEnd) cudaEventDestroy(c->frameEnd);
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return VKRT_CUDA_ERROR_INITIALIZATION_FAILED;
    }
    cudaMemsetAsync(c->counters, 0, sizeof(RenderCounters), c->stream);
    c->textureData.resize(VKRT_CUDA_MAX_TEXTURES);
    vkrt_cuda_default_wavefront_config(&c->wfCfg);
    if (cfg.integrator > VKRT_CUDA_INTEGRATOR_WAVEFRONT) {
        vkrt_cuda_destroy(c);
        return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    }
    c->textureDescs.assign(VKRT_CUDA_MAX_TEXTURES, TextureDesc{nullptr, 0u, 0u});
    *out = c;
    return VKRT_CUDA_SUCCESS;
}

void vkrt_cuda_destroy(VKRT_CudaContext* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drainFilmCopies(c);
    if (c->copyStream) cudaStreamDestroy(c->copyStream);
    if (c->filmReady) cudaEventDestroy(c->filmReady);
    for (cudaEvent_t e : c->copyDone)
        if (e) cudaEventDestroy(e);
    c->vertices.release();
    c->indices.release();
    c->meshes.release();
    c->bvh.release();
    c->materials.release();
    c->emissiveMeshes.release();
    c->emissiveTriangles.release();
    c->meshAliasQ.release();
    c->meshAliasIdx.release();
    c->triAliasQ.release();
    c->triAliasIdx.release();
    for (auto& t : c->textureData) t.release();
    c->textureTable.release();
    c->rgb2spec.release();
    c->rgb2specCells.release();
    c->rgb2specGuide.release();
    c->envMarginalGuide.release();
    c->envConditionalGuide.release();
    c->envMarginal.release();
    c->envConditional.release();
    c->envTexelPdf.release();
    c->envScratch.release();
    c->accum[0].release();
    c->accum[1].release();
    c->output.release();
    for (auto& t : c->textureGrad) t.release();
    c->textureGradTable.release();
    c->materialGrad.release();
    c->emissiveMeshMaterial.release();
    c->dImage.release();
    c->selectionMask.release();
    c->pickResult.release();
    for (int i = 0; i < 2; ++i) {
        c->albedo[i].release();
        c->normal[i].release();
    }
    if (c->counters) cudaFree(c->counters);
    c->wavefront.reset();
    if (c->order) cudaEventDestroy(c->order);
    if (c->frameStart) cudaEventDestroy(c->frameStart);
    if (c->frameEnd) cudaEventDestroy(c->frameEnd);
    cudaStreamDestroy(c->stream);
    delete c;
}

int32_t vkrt_cuda_upload_geometry(VKRT_CudaContext* c, const VKRT_CudaShaderVertex* vertices, uint32_t vertexCount,
                                  const uint32_t* indices, uint32_t indexCount, const VKRT_CudaMeshInfo* meshes,
                                  uint32_t meshCount) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if ((vertexCount && !vertices) || (indexCount && !indices) || (meshCount && !meshes))
        return invalid(c, "null array with a non-zero count");
    if (indexCount % 3u) return invalid(c, "indexCount is not a multiple of 3");
    // every mesh's triangles must address valid indices and vertices (vkrt validates the same ranges)
    uint64_t tris = 0;
    for (uint32_t i = 0; i < meshCount; ++i) {
        const VKRT_CudaMeshInfo& m = meshes[i];
        if (m.indexCount % 3u) return invalid(c, "MeshInfo.indexCount is not a multiple of 3");
        if (uint64_t(m.indexBase) + m.indexCount > indexCount) return invalid(c, "MeshInfo index range out of bounds");
        if (uint64_t(m.vertexBase) + m.vertexCount > vertexCount) return invalid(c, "MeshInfo vertex range out of bounds");
        for (uint32_t k = 0; k < m.indexCount; ++k)
            if (indices[m.indexBase + k] >= m.vertexCount) return invalid(c, "index outside its mesh's vertex range");
        tris += m.indexCount / 3u;
    }
    if (tris >= 0xFFFFFFF0ull) return invalid(c, "too many triangles");
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->vertices.assign(vertices, vertexCount, c->stream), "upload vertices");
    VKRT_TRY(c, c->indices.assign(indices, indexCount, c->stream), "upload indices");
    VKRT_TRY(c, c->meshes.assign(meshes, meshCount, c->stream), "upload meshes");
    c->hostMeshes.assign(meshes, meshes + meshCount);
    refreshMaterialFlags(c);
    c->vertexCount = vertexCount;
    c->indexCount = indexCount;
    c->triCount = uint32_t(tris);
    // world-space bounds (the radiance cache's hash grid spans them)
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < meshCount; ++i) {
        const VKRT_CudaMeshInfo& m = meshes[i];
        float w[16];
        vkrt_host_mesh_transform(m.position, m.rotation, m.scale, w);
        for (uint32_t v = 0; v < m.vertexCount; ++v) {
            const float* p = vertices[m.vertexBase + v].position;
            for (int r = 0; r < 3; ++r) {
                float q = w[0 * 4 + r] * p[0] + w[1 * 4 + r] * p[1] + w[2 * 4 + r] * p[2] + w[3 * 4 + r];
                lo[r] = std::min(lo[r], q);
                hi[r] = std::max(hi[r], q);
            }
        }
    }
    if (!(lo[0] <= hi[0])) lo[0] = lo[1] = lo[2] = hi[0] = hi[1] = hi[2] = 0.0f;
    c->boundsLo = make_float3(lo[0], lo[1], lo[2]);
    c->boundsHi = make_float3(hi[0], hi[1], hi[2]);
    VKRT_TRY(c, rebuildBvh(c, false), "BVH build");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_update_meshes(VKRT_CudaContext* c, const VKRT_CudaMeshInfo* meshes, uint32_t meshCount) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (meshCount != c->hostMeshes.size() || (meshCount && !meshes)) return invalid(c, "mesh count mismatch");
    bool geometryChanged = false;
    for (uint32_t i = 0; i < meshCount; ++i) {
        const VKRT_CudaMeshInfo &a = c->hostMeshes[i], &b = meshes[i];
        if (std::memcmp(a.position, b.position, sizeof(a.position)) || std::memcmp(a.rotation, b.rotation, sizeof(a.rotation)) ||
            std::memcmp(a.scale, b.scale, sizeof(a.scale)) || a.vertexBase != b.vertexBase || a.indexBase != b.indexBase ||
            a.indexCount != b.indexCount || a.vertexCount != b.vertexCount)
            geometryChanged = true;
    }
    if (geometryChanged) {
        for (uint32_t i = 0; i < meshCount; ++i) {
            const VKRT_CudaMeshInfo& m = meshes[i];
            if (m.indexCount % 3u || uint64_t(m.indexBase) + m.indexCount > c->indexCount ||
                uint64_t(m.vertexBase) + m.vertexCount > c->vertexCount)
                return invalid(c, "MeshInfo range out of bounds");
        }
    }
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->meshes.assign(meshes, meshCount, c->stream), "upload meshes");
    c->hostMeshes.assign(meshes, meshes + meshCount);
    refreshMaterialFlags(c);
    if (geometryChanged) {
        uint64_t tris = 0;
        for (auto& m : c->hostMeshes) tris += m.indexCount / 3u;
        c->triCount = uint32_t(tris);
        VKRT_TRY(c, rebuildBvh(c, true), "BVH build");
    }
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_upload_materials(VKRT_CudaContext* c, const VKRT_CudaMaterial* materials, uint32_t count) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (count && !materials) return invalid(c, "null materials");
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->materials.assign(materials, count, c->stream), "upload materials");
    c->hostMaterials.assign(materials, materials + count);
    c->materialCount = count;
    refreshMaterialFlags(c);
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_upload_lights(VKRT_CudaContext* c, const VKRT_CudaEmissiveMesh* meshes, uint32_t meshCount,
                                const VKRT_CudaEmissiveTriangle* triangles, uint32_t triangleCount,
                                const float* meshAliasQ, const uint32_t* meshAliasIdx, const float* triAliasQ,
                                const uint32_t* triAliasIdx) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (meshCount && (!meshes || !meshAliasQ || !meshAliasIdx)) return invalid(c, "null emissive mesh arrays");
    if (triangleCount && (!triangles || !triAliasQ || !triAliasIdx)) return invalid(c, "null emissive triangle arrays");
    for (uint32_t i = 0; i < meshCount; ++i) {
        if (uint64_t(meshes[i].triOffset) + meshes[i].triCount > triangleCount)
            return invalid(c, "EmissiveMesh triangle range out of bounds");
        if (meshAliasIdx[i] >= meshCount) return invalid(c, "mesh alias index out of range");
    }
    for (uint32_t i = 0; i < meshCount; ++i)
        for (uint32_t t = 0; t < meshes[i].triCount; ++t)
            if (triAliasIdx[meshes[i].triOffset + t] >= meshes[i].triCount)
                return invalid(c, "triangle alias index out of range");
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->emissiveMeshes.assign(meshes, meshCount, c->stream), "upload emissive meshes");
    VKRT_TRY(c, c->emissiveTriangles.assign(triangles, triangleCount, c->stream), "upload emissive triangles");
    VKRT_TRY(c, c->meshAliasQ.assign(meshAliasQ, meshCount, c->stream), "upload alias");
    VKRT_TRY(c, c->meshAliasIdx.assign(meshAliasIdx, meshCount, c->stream), "upload alias");
    VKRT_TRY(c, c->triAliasQ.assign(triAliasQ, triangleCount, c->stream), "upload alias");
    VKRT_TRY(c, c->triAliasIdx.assign(triAliasIdx, triangleCount, c->stream), "upload alias");
    if (meshCount != c->emissiveMeshCount) c->emissiveMeshMaterialCount = 0;  // the mapping no longer applies
    c->emissiveMeshCount = meshCount;
    c->emissiveTriangleCount = triangleCount;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_upload_texture(VKRT_CudaContext* c, uint32_t index, const void* pixels, uint32_t w, uint32_t h,
                                 uint32_t format, uint32_t colorSpace) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (index >= VKRT_CUDA_MAX_TEXTURES) return invalid(c, "texture index out of range");
    if (!pixels || w == 0 || h == 0) return invalid(c, "empty texture");
    if (format > VKRT_CUDA_TEXTURE_FORMAT_RGBA32_SFLOAT || colorSpace > VKRT_CUDA_COLOR_SPACE_LINEAR)
        return invalid(c, "unknown texture format or colour space");
    size_t n = size_t(w) * h;
    // texels are stored linear RGBA32F: 8/16-bit UNORM sRGB data is decoded here, as the sampler would before
    // filtering; alpha is always linear
    std::vector<float4> texels(n);
    for (size_t i = 0; i < n; ++i) {
        float v[4];
        for (int k = 0; k < 4; ++k) {
            switch (format) {
                case VKRT_CUDA_TEXTURE_FORMAT_RGBA8_UNORM:
                    v[k] = float(static_cast<const uint8_t*>(pixels)[i * 4 + k]) / 255.0f;
                    break;
                case VKRT_CUDA_TEXTURE_FORMAT_RGBA16_UNORM:
                    v[k] = float(static_cast<const uint16_t*>(pixels)[i * 4 + k]) / 65535.0f;
                    break;
                case VKRT_CUDA_TEXTURE_FORMAT_RGBA16_SFLOAT:
                    halfToFloatBits(static_cast<const uint16_t*>(pixels)[i * 4 + k], v[k]);
                    break;
                default:
                    v[k] = static_cast<const float*>(pixels)[i * 4 + k];
            }
            if (k < 3 && colorSpace == VKRT_CUDA_COLOR_SPACE_SRGB &&
                (format == VKRT_CUDA_TEXTURE_FORMAT_RGBA8_UNORM || format == VKRT_CUDA_TEXTURE_FORMAT_RGBA16_UNORM))
                v[k] = srgbToLinear(v[k]);
        }
        texels[i] = make_float4(v[0], v[1], v[2], v[3]);
    }
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->textureData[index].assign(texels.data(), n, c->stream), "upload texture");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "upload texture");
    c->textureDescs[index] = TextureDesc{c->textureData[index].ptr, w, h};
    c->textureTableDirty = true;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_set_environment(VKRT_CudaContext* c, uint32_t textureIndex) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (textureIndex == VKRT_CUDA_INVALID_INDEX) {
        c->envTexture = VKRT_CUDA_INVALID_INDEX;
        c->envWidth = c->envHeight = 0;
        return VKRT_CUDA_SUCCESS;
    }
    if (textureIndex >= VKRT_CUDA_MAX_TEXTURES || !c->textureDescs[textureIndex].texels)
        return invalid(c, "environment texture slot is not bound");
    const TextureDesc& t = c->textureDescs[textureIndex];
    uint32_t W = t.width, H = t.height;
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->envMarginal.reserve(H + 1), "environment CDF");
    VKRT_TRY(c, c->envConditional.reserve(size_t(H) * (W + 1)), "environment CDF");
    VKRT_TRY(c, c->envTexelPdf.reserve(size_t(W) * H), "environment CDF");
    VKRT_TRY(c, c->envScratch.reserve(size_t(W) * H + H + 2), "environment CDF");
    VKRT_TRY(c, launchBuildEnvDistribution(t.texels, W, H, c->envMarginal.ptr, c->envConditional.ptr, c->envTexelPdf.ptr,
                                           c->envScratch.ptr, c->stream),
             "environment CDF");
    VKRT_TRY(c, c->envMarginalGuide.reserve(kEnvGuide + 1u), "environment guide");
    VKRT_TRY(c, c->envConditionalGuide.reserve(size_t(H) * (kEnvGuide + 1u)), "environment guide");
    VKRT_TRY(c, launchBuildEnvGuides(c->envMarginal.ptr, c->envConditional.ptr, W, H, c->envMarginalGuide.ptr,
                                     c->envConditionalGuide.ptr, c->stream),
             "environment guide");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "environment CDF");
    c->envWidth = W;
    c->envHeight = H;
    c->envTexture = textureIndex;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_read_environment_distribution(VKRT_CudaContext* c, uint32_t width, uint32_t height, float* marginal,
                                                float* conditional, float* texelPdf) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (c->envTexture == VKRT_CUDA_INVALID_INDEX) return invalid(c, "no environment distribution is built");
    if (width != c->envWidth || height != c->envHeight) return invalid(c, "environment distribution size mismatch");
    cudaSetDevice(c->device);
    const size_t W = width, H = height;
    if (marginal)
        VKRT_TRY(c, cudaMemcpyAsync(marginal, c->envMarginal.ptr, sizeof(float) * (H + 1), cudaMemcpyDeviceToHost,
                                    c->stream),
                 "read environment distribution");
    if (conditional)
        VKRT_TRY(c, cudaMemcpyAsync(conditional, c->envConditional.ptr, sizeof(float) * H * (W + 1),
                                    cudaMemcpyDeviceToHost, c->stream),
                 "read environment distribution");
    if (texelPdf)
        VKRT_TRY(c, cudaMemcpyAsync(texelPdf, c->envTexelPdf.ptr, sizeof(float) * W * H, cudaMemcpyDeviceToHost,
                                    c->stream),
                 "read environment distribution");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "read environment distribution");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_upload_sheen_table(VKRT_CudaContext* c, const float* table, uint32_t floatCount) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!table || floatCount != VKRT_CUDA_SHEEN_TABLE_FLOATS) return invalid(c, "sheen table: 3072 floats");
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->sheenTable.assign(table, floatCount, c->stream), "upload sheen table");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "upload sheen table");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_upload_rgb2spec(VKRT_CudaContext* c, const float* table, uint32_t floatCount,
                                  const VKRT_CudaRGB2SpecTableInfo* info) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!table || !info || info->res < 2) return invalid(c, "rgb2spec table");
    uint64_t need = std::max<uint64_t>(uint64_t(info->scaleOffset) + info->res,
                                       uint64_t(info->dataOffset) + 9ull * info->res * info->res * info->res);
    if (floatCount < need) return invalid(c, "rgb2spec table smaller than its layout");
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->rgb2spec.assign(table, floatCount, c->stream), "upload rgb2spec");
    c->rgb2specFloats = floatCount;
    c->rgb2specInfo = *info;
    VKRT_TRY(c, c->rgb2specCells.reserve(size_t(3) * info->res * info->res * info->res), "rgb2spec cells");
    VKRT_TRY(c, launchRepackRgb2Spec(c->rgb2spec.ptr, info->res, info->dataOffset, c->rgb2specCells.ptr, c->stream),
             "rgb2spec cells");
    VKRT_TRY(c, c->rgb2specGuide.reserve(kRgb2SpecGuide + 1u), "rgb2spec guide");
    VKRT_TRY(c, launchRgb2SpecGuide(c->rgb2spec.ptr, info->res, info->scaleOffset, c->rgb2specGuide.ptr, c->stream),
             "rgb2spec guide");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_generate_rgb2spec(VKRT_CudaContext* c, uint32_t res, VKRT_CudaRGB2SpecTableInfo* outInfo) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (res < 3 || res > 256) return invalid(c, "rgb2spec resolution must be in [3, 256]");
    uint32_t floats = res + 9u * res * res * res;
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->rgb2spec.reserve(floats), "rgb2spec");
    VKRT_TRY(c, launchGenerateRgb2Spec(res, c->rgb2spec.ptr, c->stream), "rgb2spec fit");
    c->rgb2specFloats = floats;
    c->rgb2specInfo = VKRT_CudaRGB2SpecTableInfo{res, 0u, res};
    VKRT_TRY(c, c->rgb2specCells.reserve(size_t(3) * res * res * res), "rgb2spec cells");
    VKRT_TRY(c, launchRepackRgb2Spec(c->rgb2spec.ptr, res, res, c->rgb2specCells.ptr, c->stream), "rgb2spec cells");
    VKRT_TRY(c, c->rgb2specGuide.reserve(kRgb2SpecGuide + 1u), "rgb2spec guide");
    VKRT_TRY(c, launchRgb2SpecGuide(c->rgb2spec.ptr, res, 0u, c->rgb2specGuide.ptr, c->stream), "rgb2spec guide");
    if (outInfo) *outInfo = c->rgb2specInfo;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_download_rgb2spec(VKRT_CudaContext* c, float* table, uint32_t floatCount) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!table || floatCount < c->rgb2specFloats || !c->rgb2spec.ptr) return invalid(c, "rgb2spec download buffer");
    cudaSetDevice(c->device);
    VKRT_TRY(c, cudaMemcpyAsync(table, c->rgb2spec.ptr, sizeof(float) * c->rgb2specFloats, cudaMemcpyDeviceToHost, c->stream),
             "download rgb2spec");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "download rgb2spec");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_resize(VKRT_CudaContext* c, uint32_t w, uint32_t h) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (w == 0 || h == 0 || uint64_t(w) * h > (1ull << 31)) return invalid(c, "film size");
    cudaSetDevice(c->device);
    size_t n = size_t(w) * h;
    VKRT_TRY(c, drainFilmCopies(c), "film readback");
    VKRT_TRY(c, c->accum[0].reserve(n), "film");
    VKRT_TRY(c, c->accum[1].reserve(n), "film");
    VKRT_TRY(c, c->output.reserve(n), "film");
    c->width = w;
    c->height = h;
    c->readIndex = 0;
    VKRT_TRY(c, launchClearFilm(c->accum[0].ptr, c->accum[1].ptr, c->output.ptr, n, c->stream), "film clear");
    VKRT_TRY(c, clearFeatureFilms(c), "feature films");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_reset_accumulation(VKRT_CudaContext* c) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!c->width) return invalid(c, "no film");
    cudaSetDevice(c->device);
    VKRT_TRY(c, awaitFilmCopies(c, c->stream), "film readback");
    VKRT_TRY(c, launchClearFilm(c->accum[0].ptr, c->accum[1].ptr, c->output.ptr, size_t(c->width) * c->height, c->stream),
             "film clear");
    VKRT_TRY(c, clearFeatureFilms(c), "feature films");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_set_denoiser_features(VKRT_CudaContext* c, uint32_t enabled) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (enabled > 1u) return invalid(c, "denoiser features: 0 or 1");
    cudaSetDevice(c->device);
    if ((enabled != 0u) == c->features) return VKRT_CUDA_SUCCESS;
    c->features = enabled != 0u;
    if (!c->features) {
        for (int i = 0; i < 2; ++i) {
            c->albedo[i].release();
            c->normal[i].release();
        }
        return VKRT_CUDA_SUCCESS;
    }
    VKRT_TRY(c, clearFeatureFilms(c), "feature films");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_read_denoiser_features(VKRT_CudaContext* c, float* albedo, float* normal, size_t bytes) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!c->features) return invalid(c, "denoiser features are off");
    const size_t need = size_t(c->width) * c->height * sizeof(float4);
    if (!need || bytes < need || (!albedo && !normal)) return invalid(c, "feature buffers too small");
    cudaSetDevice(c->device);
    if (albedo)
        VKRT_TRY(c, cudaMemcpyAsync(albedo, c->albedo[c->readIndex].ptr, need, cudaMemcpyDeviceToHost, c->stream),
                 "read features");
    if (normal)
        VKRT_TRY(c, cudaMemcpyAsync(normal, c->normal[c->readIndex].ptr, need, cudaMemcpyDeviceToHost, c->stream),
                 "read features");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "read features");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_render_frame(VKRT_CudaContext* c, const VKRT_CudaSceneData* sd) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    int32_t v = validateFrame(c, sd);
    if (v != VKRT_CUDA_SUCCESS) return v;
    cudaSetDevice(c->device);
    if (c->cfg.integrator != VKRT_CUDA_INTEGRATOR_WAVEFRONT)  // the batch path waits for its own contexts
        VKRT_TRY(c, awaitFilmCopy(c, c->readIndex ^ 1, c->stream), "film readback");
    VKRT_TRY(c, cudaEventRecord(c->frameStart, c->stream), "frame timing");
    if (c->cfg.integrator == VKRT_CUDA_INTEGRATOR_WAVEFRONT) {
        VKRT_CudaContext* one[1] = {c};
        int32_t r = vkrt_cuda_render_batch(one, sd, 1);
        if (r == VKRT_CUDA_SUCCESS) {
            VKRT_TRY(c, cudaEventRecord(c->frameEnd, c->stream), "frame timing");
            c->frameTimed = true;
        }
        return r;
    }
    const bool spectral = VKRT_CUDA_RENDER_MODE_OF(sd->packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL;
    (void)spectral;
    DeviceScene scene = makeDeviceScene(c);
    RenderParams rp{};
    rp.rngMode = c->cfg.rngMode;
    rp.rngSeed = c->cfg.rngSeed;
    rp.envNee = envNeeActive(c, sd) ? 1u : 0u;
    rp.width = c->width;
    rp.height = c->height;
    rp.countBytes = c->cfg.countRays;
    rp.extended = c->extendedMaterials || singleWavelengthMode(sd) ? 1u : 0u;
    rp.alpha = c->alphaTested ? 1u : 0u;
    FilmBuffers film = filmOf(c);
    VKRT_TRY(c, cudaMemsetAsync(c->counters, 0, sizeof(RenderCounters), c->stream), "render");
    VKRT_TRY(c, launchRender(scene, *sd, rp, film, c->counters, c->cfg.threadsPerBlock, c->stream), "render launch");
    VKRT_TRY(c, cudaEventRecord(c->frameEnd, c->stream), "frame timing");
    c->frameTimed = true;
    c->readIndex ^= 1;  // VKRT_endFrame's ping-pong swap (frame.c:386-389)
    c->countersPending = true;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_last_frame_ms(VKRT_CudaContext* c, float* ms) {
    if (!c || !ms) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!c->frameTimed) return invalid(c, "no frame rendered yet");
    cudaSetDevice(c->device);
    VKRT_TRY(c, cudaEventSynchronize(c->frameEnd), "frame timing");
    VKRT_TRY(c, cudaEventElapsedTime(ms, c->frameStart, c->frameEnd), "frame timing");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_render_selection_overlay(VKRT_CudaContext* c, const VKRT_CudaSceneData* sd) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    int32_t v = validateFrame(c, sd);
    if (v != VKRT_CUDA_SUCCESS) return v;
    if (sd->selectionEnabled != 0u && sd->selectedMeshIndex != VKRT_CUDA_INVALID_INDEX &&
        sd->selectedMeshIndex >= uint32_t(c->hostMeshes.size()))
        return invalid(c, "selected mesh index out of range");
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->selectionMask.reserve(size_t(c->width) * c->height), "selection mask");
    DeviceScene scene = makeDeviceScene(c);
    VKRT_TRY(c, launchSelectionMask(scene, *sd, c->width, c->height, c->selectionMask.ptr, c->stream), "selection mask");
    if (sd->selectionEnabled != 0u)
        VKRT_TRY(c, launchOutline(c->selectionMask.ptr, c->width, c->height, c->output.ptr, c->stream), "outline");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_read_selection_mask(VKRT_CudaContext* c, uint32_t* mask, size_t bytes) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    const size_t need = size_t(c->width) * c->height * sizeof(uint32_t);
    if (!mask || bytes < need || !need) return invalid(c, "selection mask buffer too small");
    if (c->selectionMask.count * sizeof(uint32_t) < need) return invalid(c, "no selection mask rendered yet");
    cudaSetDevice(c->device);
    VKRT_TRY(c, cudaMemcpyAsync(mask, c->selectionMask.ptr, need, cudaMemcpyDeviceToHost, c->stream), "read mask");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "read mask");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_pick_mesh(VKRT_CudaContext* c, const VKRT_CudaSceneData* sd, uint32_t x, uint32_t y,
                            uint32_t* meshIndex) {
    if (!c || !meshIndex) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    int32_t v = validateFrame(c, sd);
    if (v != VKRT_CUDA_SUCCESS) return v;
    if (x >= c->width || y >= c->height) return invalid(c, "pick pixel outside the film");
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->pickResult.reserve(1), "pick");
    DeviceScene scene = makeDeviceScene(c);
    VKRT_TRY(c, launchPick(scene, *sd, x, y, c->pickResult.ptr, c->stream), "pick");
    VKRT_TRY(c, cudaMemcpyAsync(meshIndex, c->pickResult.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream),
             "pick");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "pick");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_set_integrator(VKRT_CudaContext* c, uint32_t integrator) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (integrator > VKRT_CUDA_INTEGRATOR_WAVEFRONT) return invalid(c, "unknown integrator");
    c->cfg.integrator = integrator;
    return VKRT_CUDA_SUCCESS;
}

void vkrt_cuda_default_wavefront_config(VKRT_CudaWavefrontConfig* w) {
    if (!w) return;
    std::memset(w, 0, sizeof(*w));
    w->queueCapacity = 0u;
    w->tileWidth = 16u;
    w->tileHeight = 8u;
    w->sortByMaterial = 2u;
    w->intersectBlocksPerSM = 8u;
    w->shadeBlocksPerSM = 4u;  // 128-register shading kernels: on the 1080p spectral frame shade 11.3 ms against
                               // 12.4 ms for the spill-free 168-register build at 3 blocks
    w->useGraph = 1u;
}

int32_t vkrt_cuda_set_wavefront_config(VKRT_CudaContext* c, const VKRT_CudaWavefrontConfig* w) {
    if (!c || !w) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (w->tileWidth == 0 || w->tileHeight == 0 || w->tileWidth * w->tileHeight > 4096u)
        return invalid(c, "tile must be between 1 and 4096 pixels");
    if (w->intersectBlocksPerSM == 0 || w->intersectBlocksPerSM > 16u || w->shadeBlocksPerSM == 0 ||
        w->shadeBlocksPerSM > 16u)
        return invalid(c, "blocks per SM must be in [1, 16]");
    if (w->queueCapacity > (1u << 28)) return invalid(c, "queue capacity above 256M path slots");  // ~70 GB
    if (w->profileStages > 1u) return invalid(c, "profileStages is 0 or 1");
    if (w->sortByMaterial > 3u) return invalid(c, "sortByMaterial is 0, 1, 2 or 3");
    if (w->refillLanes > 32u) return invalid(c, "refillLanes is 0 (default) or 1..32");
    if (w->rayOrder > 1u) return invalid(c, "rayOrder is 0 or 1");
    c->wfCfg = *w;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_get_wavefront_config(VKRT_CudaContext* c, VKRT_CudaWavefrontConfig* w) {
    if (!c || !w) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    *w = c->wfCfg;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_render_batch(VKRT_CudaContext* const* contexts, const VKRT_CudaSceneData* sds, uint32_t count) {
    if (!contexts || !sds || count == 0) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    VKRT_CudaContext* c0 = contexts[0];
    if (!c0) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    bool spectral = VKRT_CUDA_RENDER_MODE_OF(sds[0].packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL;
    std::vector<WfScene> scenes(count);
    for (uint32_t i = 0; i < count; ++i) {
        VKRT_CudaContext* c = contexts[i];
        if (!c) return invalid(c0, "null context in batch");
        if (c->device != c0->device) return invalid(c0, "all contexts of a batch must be on one device");
        if ((VKRT_CUDA_RENDER_MODE_OF(sds[i].packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL) != spectral)
            return invalid(c0, "all scenes of a batch must share the render mode");
        if (c->cfg.rngMode != c0->cfg.rngMode || c->cfg.rngSeed != c0->cfg.rngSeed)
            return invalid(c0, "all contexts of a batch must share the random stream configuration");
        for (uint32_t j = 0; j < i; ++j)
            if (contexts[j] == c) return invalid(c0, "a context appears twice in the batch");
        int32_t v = validateFrame(c, &sds[i]);
        if (v != VKRT_CUDA_SUCCESS) {
            c0->lastError = c->lastError;
            return v;
        }
    }
    cudaSetDevice(c0->device);
    for (uint32_t i = 0; i < count; ++i) {
        VKRT_CudaContext* c = contexts[i];
        scenes[i] = makeWfScene(c, sds[i], spectral);
        VKRT_TRY(c0, awaitFilmCopy(c, c->readIndex ^ 1, c0->stream), "film readback");
        // c0's stream reads this context's buffers: order it after the work already queued on its own stream
        if (c != c0) {
            VKRT_TRY(c0, cudaEventRecord(c->order, c->stream), "batch ordering");
            VKRT_TRY(c0, cudaStreamWaitEvent(c0->stream, c->order, 0), "batch ordering");
        }
    }
    if (!c0->wavefront) c0->wavefront.reset(new WavefrontEngine());
    WavefrontConfig wc = engineConfig(c0);
    VKRT_TRY(c0, cudaMemsetAsync(c0->counters, 0, sizeof(RenderCounters), c0->stream), "batch render");
    // a single context with an enabled radiance cache trains it and renders cache-terminated paths
    WfCacheFrame cache{};
    const bool useCache = count == 1 && c0->nrc && c0->nrc->ready() && c0->nrcCfg.enabled;
    if (useCache && (c0->transmissiveMaterials || c0->alphaTested))
        return invalid(c0, "the radiance cache covers opaque reflection-only materials (transmission or alpha)");
    if (useCache && singleWavelengthMode(&sds[0]))
        return invalid(c0, "the radiance cache covers RGB and hero-wavelength frames");
    if (useCache)
        cache = WfCacheFrame{c0->nrc.get(), c0->nrcCfg.terminationDepth, c0->nrcCfg.trainingPaths,
                             c0->nrcCfg.trainingSteps, c0->nrcCfg.seed, sds[0].frameNumber,
                             c0->nrcCfg.terminationSpread, c0->nrcCfg.trainingTracer};
    VKRT_TRY(c0, c0->wavefront->render(scenes, spectral, wc, c0->cfg.rngMode, c0->cfg.rngSeed, c0->counters, c0->stream,
                                       kWavefrontForward, nullptr, useCache ? &cache : nullptr),
             "batch render");
    for (uint32_t i = 0; i < count; ++i) {
        VKRT_CudaContext* c = contexts[i];
        c->readIndex ^= 1;
        if (c != c0) {
            // later work on this context's own stream (reads, next frames) waits for the batch
            VKRT_TRY(c0, cudaEventRecord(c->order, c0->stream), "batch ordering");
            VKRT_TRY(c0, cudaStreamWaitEvent(c->stream, c->order, 0), "batch ordering");
        }
    }
    c0->countersPending = true;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_autotune_batch(VKRT_CudaContext* const* contexts, const VKRT_CudaSceneData* sds, uint32_t count,
                                 uint32_t framesPerTrial, VKRT_CudaWavefrontConfig* best, float* bestFrameMs) {
    if (!contexts || !sds || count == 0 || !contexts[0]) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    VKRT_CudaContext* c0 = contexts[0];
    cudaSetDevice(c0->device);
    framesPerTrial = std::max(1u, std::min(framesPerTrial, 8u));
    std::vector<VKRT_CudaSceneData> trial(sds, sds + count);
    uint64_t pixels = 0;
    for (auto& sd : trial) {
        sd.samplesPerPixel = 2u;
        pixels += uint64_t(sd.viewportRect[2]) * sd.viewportRect[3];
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto timeConfig = [&](const VKRT_CudaWavefrontConfig& w, float& ms) -> int32_t {
        int32_t r = vkrt_cuda_set_wavefront_config(c0, &w);
        if (r != VKRT_CUDA_SUCCESS) return r;
        r = vkrt_cuda_render_batch(contexts, trial.data(), count);  // warm-up (graph build)
        if (r != VKRT_CUDA_SUCCESS) return r;
        cudaEventRecord(e0, c0->stream);
        for (uint32_t f = 0; f < framesPerTrial; ++f) {
            r = vkrt_cuda_render_batch(contexts, trial.data(), count);
            if (r != VKRT_CUDA_SUCCESS) return r;
        }
        cudaEventRecord(e1, c0->stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) return fail(c0, e, "autotune");
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= float(framesPerTrial);
        return VKRT_CUDA_SUCCESS;
    };
    VKRT_CudaWavefrontConfig cur;
    vkrt_cuda_default_wavefront_config(&cur);
    cur.queueCapacity = 0u;  // one slot per item, up to 64M
    float curMs = 0.0f;
    int32_t r = timeConfig(cur, curMs);
    if (r != VKRT_CUDA_SUCCESS) return r;
    // coordinate descent over the knobs, each axis scanned with the others fixed at the best so far
    // slot counts: 0 (one per item of the trial, up to 64M) and 2M, 8M, 32M below that
    std::vector<uint32_t> qs{0u};
    for (uint64_t q = 1u << 21; q < std::min<uint64_t>(pixels * 2u, 1u << 26); q <<= 2) qs.push_back(uint32_t(q));
    const uint32_t tiles[][2] = {{8, 8}, {16, 8}, {32, 4}, {16, 16}, {32, 8}};
    for (int axis = 0; axis < 6; ++axis) {
        std::vector<VKRT_CudaWavefrontConfig> cands;
        if (axis == 0)
            for (uint32_t q : qs) {
                VKRT_CudaWavefrontConfig w = cur;
                w.queueCapacity = q;
                cands.push_back(w);
            }
        if (axis == 1)
            for (auto& t : tiles) {
                VKRT_CudaWavefrontConfig w = cur;
                w.tileWidth = t[0];
                w.tileHeight = t[1];
                cands.push_back(w);
            }
        if (axis == 2)
            for (uint32_t s = 0; s < 4; ++s) {
                VKRT_CudaWavefrontConfig w = cur;
                w.sortByMaterial = s;
                cands.push_back(w);
            }
        if (axis == 3)
            for (uint32_t b : {4u, 6u, 8u}) {
                VKRT_CudaWavefrontConfig w = cur;
                w.intersectBlocksPerSM = b;
                cands.push_back(w);
            }
        if (axis == 5)
            for (uint32_t l : {12u, 16u, 20u, 24u}) {
                VKRT_CudaWavefrontConfig w = cur;
                w.refillLanes = l;
                cands.push_back(w);
            }
        if (axis == 4)
            for (uint32_t b : {3u, 4u, 6u, 8u}) {  // 168-, 128-, 80- and 64-register shading kernels
                VKRT_CudaWavefrontConfig w = cur;
                w.shadeBlocksPerSM = b;
                cands.push_back(w);
            }
        for (const auto& w : cands) {
            if (std::memcmp(&w, &cur, sizeof(w)) == 0) continue;
            float ms = 0.0f;
            r = timeConfig(w, ms);
            if (r != VKRT_CUDA_SUCCESS) return r;
            if (ms < curMs) {
                curMs = ms;
                cur = w;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    r = vkrt_cuda_set_wavefront_config(c0, &cur);
    if (r != VKRT_CUDA_SUCCESS) return r;
    for (uint32_t i = 0; i < count; ++i) {
        r = vkrt_cuda_reset_accumulation(contexts[i]);
        if (r != VKRT_CUDA_SUCCESS) return r;
    }
    if (best) *best = cur;
    if (bestFrameMs) *bestFrameMs = curMs;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_sync(VKRT_CudaContext* c, uint32_t timeoutMs) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (timeoutMs == 0) {
        VKRT_TRY(c, cudaStreamSynchronize(c->stream), "sync");
        return VKRT_CUDA_SUCCESS;
    }
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(c->stream);
        if (e == cudaSuccess) return VKRT_CUDA_SUCCESS;
        if (e != cudaErrorNotReady) return fail(c, e, "sync");
        if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeoutMs)) {
            c->lastError = "sync: timed out";
            return VKRT_CUDA_ERROR_OPERATION_FAILED;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

int32_t vkrt_cuda_read_accumulation(VKRT_CudaContext* c, float* rgba, size_t bytes) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    size_t need = size_t(c->width) * c->height * sizeof(float4);
    if (!rgba || bytes < need || !need) return invalid(c, "accumulation buffer too small");
    cudaSetDevice(c->device);
    VKRT_TRY(c, cudaMemcpyAsync(rgba, c->accum[c->readIndex].ptr, need, cudaMemcpyDeviceToHost, c->stream), "read accumulation");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "read accumulation");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_read_accumulation_async(VKRT_CudaContext* c, float* rgba, size_t bytes) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    size_t need = size_t(c->width) * c->height * sizeof(float4);
    if (!rgba || bytes < need || !need) return invalid(c, "accumulation buffer too small");
    cudaSetDevice(c->device);
    if (!c->copyStream) {
        VKRT_TRY(c, cudaStreamCreateWithFlags(&c->copyStream, cudaStreamNonBlocking), "readback stream");
        VKRT_TRY(c, cudaEventCreateWithFlags(&c->filmReady, cudaEventDisableTiming), "readback stream");
        for (cudaEvent_t& e : c->copyDone) VKRT_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "readback stream");
    }
    const int b = c->readIndex;
    VKRT_TRY(c, cudaEventRecord(c->filmReady, c->stream), "read accumulation async");
    VKRT_TRY(c, cudaStreamWaitEvent(c->copyStream, c->filmReady, 0), "read accumulation async");
    VKRT_TRY(c, cudaMemcpyAsync(rgba, c->accum[b].ptr, need, cudaMemcpyDeviceToHost, c->copyStream),
             "read accumulation async");
    VKRT_TRY(c, cudaEventRecord(c->copyDone[b], c->copyStream), "read accumulation async");
    c->copyPending[b] = true;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_wait_readback(VKRT_CudaContext* c, uint32_t timeoutMs) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!c->copyStream) return VKRT_CUDA_SUCCESS;
    cudaSetDevice(c->device);
    if (timeoutMs == 0) {
        VKRT_TRY(c, cudaStreamSynchronize(c->copyStream), "wait readback");
        return VKRT_CUDA_SUCCESS;
    }
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(c->copyStream);
        if (e == cudaSuccess) return VKRT_CUDA_SUCCESS;
        if (e != cudaErrorNotReady) return fail(c, e, "wait readback");
        if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeoutMs)) {
            c->lastError = "wait readback: timed out";
            return VKRT_CUDA_ERROR_OPERATION_FAILED;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

void vkrt_cuda_default_nrc_config(VKRT_CudaNrcConfig* n) {
    if (!n) return;
    std::memset(n, 0, sizeof(*n));
    n->enabled = 1u;
    n->terminationDepth = 2u;
    n->trainingPaths = 65536u;
    n->trainingSteps = 4u;
    n->learningRate = 1e-2f;
    n->seed = 1u;
}

int32_t vkrt_cuda_nrc_configure(VKRT_CudaContext* c, const VKRT_CudaNrcConfig* n) {
    if (!c || !n) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!(n->learningRate >= 0.0f) || n->trainingPaths > (1u << 22) || n->trainingSteps > 64u ||
        n->inferenceTensorPath > VKRT_CUDA_NRC_MMA_SYNC || !(n->inferenceAverage >= 0.0f && n->inferenceAverage < 1.0f) ||
        !(n->terminationSpread >= 0.0f && n->terminationSpread <= 3.0e38f) || n->trainingTracer > 1u)
        return invalid(c, "radiance cache configuration out of range");
    cudaSetDevice(c->device);
    if (!c->nrc) c->nrc.reset(new NrcEngine());
    NrcSettings s{n->learningRate, 0.9f, 0.99f, 1e-8f, n->seed};
    // pad the bounds a little so surface points never sit on the grid's outer faces
    float3 ext = make_float3(c->boundsHi.x - c->boundsLo.x, c->boundsHi.y - c->boundsLo.y, c->boundsHi.z - c->boundsLo.z);
    float pad = 1e-3f * std::max(std::max(ext.x, ext.y), std::max(ext.z, 1e-3f));
    float3 lo = make_float3(c->boundsLo.x - pad, c->boundsLo.y - pad, c->boundsLo.z - pad);
    float3 hi = make_float3(c->boundsHi.x + pad, c->boundsHi.y + pad, c->boundsHi.z + pad);
    VKRT_TRY(c, c->nrc->reset(s, lo, hi, c->stream), "radiance cache init");
    c->nrc->setTensorPath(n->inferenceTensorPath);
    VKRT_TRY(c, c->nrc->setAverageDecay(n->inferenceAverage, c->stream), "radiance cache init");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "radiance cache init");
    c->nrcCfg = *n;
    return VKRT_CUDA_SUCCESS;
}

namespace {
int32_t nrcReady(VKRT_CudaContext* c) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!c->nrc || !c->nrc->ready()) return invalid(c, "radiance cache not configured");
    return VKRT_CUDA_SUCCESS;
}
}  // namespace

int32_t vkrt_cuda_nrc_read_training_records(VKRT_CudaContext* c, float* inputs, float* targets, uint32_t capacity,
                                            uint32_t* count) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (capacity && (!inputs || !targets)) return invalid(c, "null training-record buffer");
    if (count) *count = 0;
    if (!c->wavefront) return VKRT_CUDA_SUCCESS;
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->wavefront->readTrainingRecords(inputs, targets, capacity, count, c->stream), "read training records");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_nrc_infer(VKRT_CudaContext* c, const float* inputs, uint32_t n, float* outputs) {
    int32_t r = nrcReady(c);
    if (r != VKRT_CUDA_SUCCESS) return r;
    if (n && (!inputs || !outputs)) return invalid(c, "null cache input or output");
    if (!n) return VKRT_CUDA_SUCCESS;
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->nrcIn.assign(reinterpret_cast<const NrcInput*>(inputs), n, c->stream), "cache inputs");
    VKRT_TRY(c, c->nrcOut.reserve(n), "cache outputs");
    VKRT_TRY(c, c->nrc->infer(c->nrcIn.ptr, n, c->nrcOut.ptr, c->stream), "cache inference");
    VKRT_TRY(c, cudaMemcpyAsync(outputs, c->nrcOut.ptr, sizeof(float4) * n, cudaMemcpyDeviceToHost, c->stream),
             "cache outputs");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "cache inference");
    unsigned int err = 0u;
    VKRT_TRY(c, c->nrc->errorWord(&err, c->stream), "cache inference");
    if (err) {
        c->lastError = "cache inference: a tensor-core completion wait ran out";
        return VKRT_CUDA_ERROR_OPERATION_FAILED;
    }
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_nrc_train(VKRT_CudaContext* c, const float* inputs, const float* targets, uint32_t n, uint32_t apply,
                            float* loss) {
    int32_t r = nrcReady(c);
    if (r != VKRT_CUDA_SUCCESS) return r;
    if (n && (!inputs || !targets)) return invalid(c, "null training records");
    if (!n) return VKRT_CUDA_SUCCESS;
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->nrcIn.assign(reinterpret_cast<const NrcInput*>(inputs), n, c->stream), "training inputs");
    VKRT_TRY(c, c->nrcTarget.assign(reinterpret_cast<const float4*>(targets), n, c->stream), "training targets");
    VKRT_TRY(c, c->nrcLoss.reserve(1), "training loss");
    VKRT_TRY(c, cudaMemsetAsync(c->nrcLoss.ptr, 0, sizeof(float), c->stream), "training loss");
    VKRT_TRY(c, c->nrc->train(c->nrcIn.ptr, c->nrcTarget.ptr, n, c->nrcLoss.ptr, apply != 0u, c->stream),
             "cache training");
    float l = 0.0f;
    VKRT_TRY(c, cudaMemcpyAsync(&l, c->nrcLoss.ptr, sizeof(float), cudaMemcpyDeviceToHost, c->stream), "training loss");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "cache training");
    if (loss) *loss = l;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_nrc_parameters(VKRT_CudaContext* c, uint16_t* weights, uint16_t* table, uint32_t write) {
    int32_t r = nrcReady(c);
    if (r != VKRT_CUDA_SUCCESS) return r;
    cudaSetDevice(c->device);
    const cudaMemcpyKind kind = write ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    if (weights) {
        void* dst = write ? static_cast<void*>(c->nrc->weights()) : static_cast<void*>(weights);
        const void* src = write ? static_cast<const void*>(weights) : static_cast<const void*>(c->nrc->weights());
        VKRT_TRY(c, cudaMemcpyAsync(dst, src, sizeof(uint16_t) * kNrcWeightCount, kind, c->stream), "cache weights");
    }
    if (table) {
        void* dst = write ? static_cast<void*>(c->nrc->table()) : static_cast<void*>(table);
        const void* src = write ? static_cast<const void*>(table) : static_cast<const void*>(c->nrc->table());
        VKRT_TRY(c, cudaMemcpyAsync(dst, src, sizeof(uint16_t) * size_t(kNrcTableParams), kind, c->stream),
                 "cache table");
    }
    if (write) VKRT_TRY(c, c->nrc->syncMasters(c->stream), "cache parameters");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "cache parameters");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_nrc_gradients(VKRT_CudaContext* c, float* weights, float* table) {
    int32_t r = nrcReady(c);
    if (r != VKRT_CUDA_SUCCESS) return r;
    cudaSetDevice(c->device);
    if (weights)
        VKRT_TRY(c, cudaMemcpyAsync(weights, c->nrc->weightGrad(), sizeof(float) * kNrcWeightCount,
                                    cudaMemcpyDeviceToHost, c->stream),
                 "cache gradients");
    if (table)
        VKRT_TRY(c, cudaMemcpyAsync(table, c->nrc->tableGrad(), sizeof(float) * size_t(kNrcTableParams),
                                    cudaMemcpyDeviceToHost, c->stream),
                 "cache gradients");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "cache gradients");
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_nrc_grid(VKRT_CudaContext* c, float* lo, float* hi, uint32_t* res, uint32_t* dense) {
    int32_t r = nrcReady(c);
    if (r != VKRT_CUDA_SUCCESS) return r;
    const NrcGridInfo& g = c->nrc->grid();
    if (lo) {
        lo[0] = g.lo.x;
        lo[1] = g.lo.y;
        lo[2] = g.lo.z;
    }
    if (hi) {
        hi[0] = g.lo.x + 1.0f / g.invExtent.x;
        hi[1] = g.lo.y + 1.0f / g.invExtent.y;
        hi[2] = g.lo.z + 1.0f / g.invExtent.z;
    }
    for (int l = 0; l < kNrcLevels; ++l) {
        if (res) res[l] = g.res[l];
        if (dense) dense[l] = g.dense[l];
    }
    return VKRT_CUDA_SUCCESS;
}

void vkrt_cuda_default_adjoint_config(VKRT_CudaAdjointConfig* a) {
    if (!a) return;
    std::memset(a, 0, sizeof(*a));
}

int32_t vkrt_cuda_set_emissive_mesh_materials(VKRT_CudaContext* c, const uint32_t* materials, uint32_t count) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (count != c->emissiveMeshCount) return invalid(c, "one material per uploaded emissive mesh");
    if (count && !materials) return invalid(c, "null material array");
    for (uint32_t i = 0; i < count; ++i)
        if (materials[i] >= c->materialCount) return invalid(c, "emissive mesh material out of range");
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->emissiveMeshMaterial.assign(materials, count, c->stream), "emissive mesh materials");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "emissive mesh materials");
    c->emissiveMeshMaterialCount = count;
    return VKRT_CUDA_SUCCESS;
}

namespace {

int32_t renderAdjoint(VKRT_CudaContext* c, const VKRT_CudaSceneData* sd, const float4* dImageDevice,
                      const VKRT_CudaAdjointConfig* cfg) {
    int32_t v = validateFrame(c, sd);
    if (v != VKRT_CUDA_SUCCESS) return v;
    if (VKRT_CUDA_RENDER_MODE_OF(sd->packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL)
        return invalid(c, "the adjoint differentiates the RGB render mode only");
    for (const VKRT_CudaMaterial& m : c->hostMaterials) {
        if (m.specularTint != 0.0f) return invalid(c, "the adjoint needs specularTint 0 on every material");
        if (m.clearcoat > 0.0f || m.subsurface > 0.0f || m.diffuseRoughness > 0.0f || m.transmission > 0.0f)
            return invalid(c, "the adjoint covers the metal / dielectric / Lambert stack only");
    if (c->sheenMaterials || c->alphaTested)
        return invalid(c, "the adjoint covers the opaque metal / dielectric / Lambert stack only");
    }
    VKRT_CudaAdjointConfig a{};
    if (cfg) a = *cfg;
    const uint32_t want = a.gradients ? a.gradients
                                      : (VKRT_CUDA_GRADIENT_BASE_COLOR | VKRT_CUDA_GRADIENT_ROUGHNESS |
                                         VKRT_CUDA_GRADIENT_EMISSION);
    const bool neeActive = sd->misNeeEnabled != 0u && sd->emissiveMeshCount > 0u;
    if ((want & VKRT_CUDA_GRADIENT_EMISSION) && neeActive && c->emissiveMeshMaterialCount != c->emissiveMeshCount)
        return invalid(c, "emission gradients need vkrt_cuda_set_emissive_mesh_materials after uploading lights");
    cudaSetDevice(c->device);
    // gradient buffers: one per texture slot that a material samples as base colour or metallic-roughness
    if (c->textureGrad.size() != c->textureDescs.size()) c->textureGrad.resize(c->textureDescs.size());
    std::vector<float4*> table(c->textureDescs.size(), nullptr);
    std::vector<uint8_t> used(c->textureDescs.size(), 0);
    for (const VKRT_CudaMaterial& m : c->hostMaterials) {
        if (m.baseColorTextureIndex < used.size()) used[m.baseColorTextureIndex] = 1;
        if (m.metallicRoughnessTextureIndex < used.size()) used[m.metallicRoughnessTextureIndex] = 1;
    }
    for (size_t i = 0; i < used.size(); ++i) {
        const TextureDesc& t = c->textureDescs[i];
        if (!used[i] || !t.texels) continue;
        size_t n = size_t(t.width) * t.height;
        bool fresh = c->textureGrad[i].count != n;
        if (fresh) c->textureGrad[i].release();
        VKRT_TRY(c, c->textureGrad[i].reserve(n), "texture gradient");
        if (fresh || !a.accumulate)
            VKRT_TRY(c, cudaMemsetAsync(c->textureGrad[i].ptr, 0, n * sizeof(float4), c->stream), "texture gradient");
        table[i] = c->textureGrad[i].ptr;
    }
    VKRT_TRY(c, c->textureGradTable.assign(table.data(), table.size(), c->stream), "texture gradient table");
    bool freshMat = c->materialGrad.count != c->materialCount;
    if (freshMat) c->materialGrad.release();
    VKRT_TRY(c, c->materialGrad.reserve(std::max(c->materialCount, 1u)), "material gradient");
    if (freshMat || !a.accumulate)
        VKRT_TRY(c, cudaMemsetAsync(c->materialGrad.ptr, 0, sizeof(MaterialGradient) * std::max(c->materialCount, 1u),
                                    c->stream),
                 "material gradient");

    DeviceScene scene = makeDeviceScene(c);
    AdjointParams ap{};
    ap.rngMode = c->cfg.rngMode;
    ap.rngSeed = c->cfg.rngSeed;
    ap.envNee = envNeeActive(c, sd) ? 1u : 0u;
    ap.width = c->width;
    ap.height = c->height;
    ap.sampleBase = a.sampleBase;
    ap.wantBase = (want & VKRT_CUDA_GRADIENT_BASE_COLOR) ? 1u : 0u;
    ap.wantRoughness = (want & VKRT_CUDA_GRADIENT_ROUGHNESS) ? 1u : 0u;
    ap.wantEmission = (want & VKRT_CUDA_GRADIENT_EMISSION) ? 1u : 0u;
    ap.dImage = dImageDevice;
    ap.textureGrad = c->textureGradTable.ptr;
    ap.materialGrad = c->materialGrad.ptr;
    ap.emissiveMeshMaterial = c->emissiveMeshMaterial.ptr;
    VKRT_TRY(c, cudaMemsetAsync(c->counters, 0, sizeof(RenderCounters), c->stream), "adjoint");
    VKRT_TRY(c, awaitFilmCopies(c, c->stream), "film readback");
    if (c->cfg.integrator == VKRT_CUDA_INTEGRATOR_WAVEFRONT) {
        // a primal wavefront pass keeps each (pixel, sample) radiance, the adjoint pass replays those paths
        std::vector<WfScene> scenes(1, makeWfScene(c, *sd, false));
        if (!c->wavefront) c->wavefront.reset(new WavefrontEngine());
        WavefrontConfig wc = engineConfig(c);
        VKRT_TRY(c, c->wavefront->render(scenes, false, wc, c->cfg.rngMode, c->cfg.rngSeed, c->counters, c->stream,
                                         kWavefrontPrimal, &ap),
                 "adjoint primal pass");
        VKRT_TRY(c, c->wavefront->render(scenes, false, wc, c->cfg.rngMode, c->cfg.rngSeed, c->counters, c->stream,
                                         kWavefrontAdjoint, &ap),
                 "adjoint pass");
    } else {
        VKRT_TRY(c, launchAdjoint(scene, *sd, ap, c->counters, c->stream), "adjoint launch");
    }
    c->countersPending = true;
    return VKRT_CUDA_SUCCESS;
}

}  // namespace

int32_t vkrt_cuda_render_adjoint(VKRT_CudaContext* c, const VKRT_CudaSceneData* sd, const float* dImage,
                                 const VKRT_CudaAdjointConfig* cfg) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!dImage) return invalid(c, "null dImage");
    if (!c->width) return invalid(c, "no film: call vkrt_cuda_resize first");
    size_t n = size_t(c->width) * c->height;
    cudaSetDevice(c->device);
    VKRT_TRY(c, c->dImage.reserve(n), "adjoint input");
    VKRT_TRY(c, cudaMemcpyAsync(c->dImage.ptr, dImage, n * sizeof(float4), cudaMemcpyHostToDevice, c->stream),
             "adjoint input");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "adjoint input");
    return renderAdjoint(c, sd, c->dImage.ptr, cfg);
}

int32_t vkrt_cuda_render_adjoint_device(VKRT_CudaContext* c, const VKRT_CudaSceneData* sd, const float* dImage,
                                        const VKRT_CudaAdjointConfig* cfg) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (!dImage) return invalid(c, "null dImage");
    if ((reinterpret_cast<uintptr_t>(dImage) & 15u) != 0u) return invalid(c, "dImage must be 16-byte aligned");
    return renderAdjoint(c, sd, reinterpret_cast<const float4*>(dImage), cfg);
}

int32_t vkrt_cuda_read_texture_gradient(VKRT_CudaContext* c, uint32_t index, float* rgba, size_t bytes) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (index >= c->textureDescs.size() || !c->textureDescs[index].texels)
        return invalid(c, "texture slot is not bound");
    const TextureDesc& t = c->textureDescs[index];
    size_t n = size_t(t.width) * t.height;
    if (!rgba || bytes < n * sizeof(float4)) return invalid(c, "gradient buffer too small");
    cudaSetDevice(c->device);
    if (index < c->textureGrad.size() && c->textureGrad[index].count == n) {
        VKRT_TRY(c, cudaMemcpyAsync(rgba, c->textureGrad[index].ptr, n * sizeof(float4), cudaMemcpyDeviceToHost,
                                    c->stream),
                 "read texture gradient");
        VKRT_TRY(c, cudaStreamSynchronize(c->stream), "read texture gradient");
    } else {
        std::memset(rgba, 0, n * sizeof(float4));
    }
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_read_material_gradients(VKRT_CudaContext* c, VKRT_CudaMaterialGradient* out, uint32_t count) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (count > c->materialCount) return invalid(c, "more materials than uploaded");
    if (count && !out) return invalid(c, "null gradient array");
    if (!count) return VKRT_CUDA_SUCCESS;
    cudaSetDevice(c->device);
    if (c->materialGrad.count == c->materialCount) {
        static_assert(sizeof(MaterialGradient) == sizeof(VKRT_CudaMaterialGradient), "material gradient layout");
        VKRT_TRY(c, cudaMemcpyAsync(out, c->materialGrad.ptr, count * sizeof(VKRT_CudaMaterialGradient),
                                    cudaMemcpyDeviceToHost, c->stream),
                 "read material gradients");
        VKRT_TRY(c, cudaStreamSynchronize(c->stream), "read material gradients");
    } else {
        std::memset(out, 0, count * sizeof(VKRT_CudaMaterialGradient));
    }
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_read_output(VKRT_CudaContext* c, uint16_t* rgba, size_t bytes) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    size_t need = size_t(c->width) * c->height * sizeof(ushort4);
    if (!rgba || bytes < need || !need) return invalid(c, "output buffer too small");
    cudaSetDevice(c->device);
    VKRT_TRY(c, cudaMemcpyAsync(rgba, c->output.ptr, need, cudaMemcpyDeviceToHost, c->stream), "read output");
    VKRT_TRY(c, cudaStreamSynchronize(c->stream), "read output");
    return VKRT_CUDA_SUCCESS;
}

static_assert(sizeof(VKRT_CudaStats) == 144, "VKRT_CudaStats layout");
static_assert(sizeof(VKRT_CudaWavefrontConfig) == 64, "VKRT_CudaWavefrontConfig layout");

int32_t vkrt_cuda_get_stats(VKRT_CudaContext* c, VKRT_CudaStats* st) {
    if (!c || !st) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (c->countersPending) {
        VKRT_TRY(c, cudaMemcpyAsync(&c->lastCounters, c->counters, sizeof(RenderCounters), cudaMemcpyDeviceToHost, c->stream),
                 "stats");
        VKRT_TRY(c, cudaStreamSynchronize(c->stream), "stats");
        c->countersPending = false;
    }
    std::memset(st, 0, sizeof(*st));
    st->primaryRays = c->lastCounters.primaryRays;
    st->extensionRays = c->lastCounters.extensionRays;
    st->shadowRays = c->lastCounters.shadowRays;
    st->pathSamples = c->lastCounters.pathSamples;
    st->nodeFetchBytes = c->lastCounters.nodeBytes;
    st->triFetchBytes = c->lastCounters.triBytes;
    st->errorFlags = c->lastCounters.errorFlags;
    st->wavefrontBodies = c->lastCounters.wfBodies;
    st->shadowNodeFetchBytes = c->lastCounters.shadowNodeBytes;
    st->shadowTriFetchBytes = c->lastCounters.shadowTriBytes;
    st->kernelLaunches = c->lastCounters.kernelLaunches;
    if (c->wavefront) {
        const float* ms = c->wavefront->lastStageMs();
        for (int i = 0; i < 8; ++i) st->stageMs[i] = ms[i];
        st->cacheTrainingRecords = c->wavefront->lastCacheRecords();
    }
    st->bvhNodeCount = c->bvh.nodeCount;
    st->bvhTriangleCount = c->bvh.triCount;
    st->bvhBytes = uint64_t(c->bvh.nodeCount) * sizeof(WideNode) + uint64_t(c->bvh.triCount) * sizeof(TriRecord);
    st->bvhBuildMs = c->bvhStats.buildMs;
    st->bvhSahLbvh = c->bvhStats.sahLbvh;
    st->bvhSahTreelets = c->bvhStats.sahTreelets;
    return VKRT_CUDA_SUCCESS;
}

void* vkrt_cuda_stream(VKRT_CudaContext* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

int32_t vkrt_cuda_trace_rays_device(VKRT_CudaContext* c, const VKRT_CudaRay* rays, uint32_t count, uint32_t anyHit,
                                    VKRT_CudaHit* hits) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (count && (!rays || !hits)) return invalid(c, "null ray or hit array");
    if ((reinterpret_cast<uintptr_t>(rays) | reinterpret_cast<uintptr_t>(hits)) & 15u)
        return invalid(c, "ray and hit arrays must be 16-byte aligned");
    cudaSetDevice(c->device);
    DeviceScene scene = makeDeviceScene(c);
    VKRT_TRY(c, cudaMemsetAsync(c->counters, 0, sizeof(RenderCounters), c->stream), "trace");
    VKRT_TRY(c, launchTraceRays(scene, rays, count, anyHit, hits, c->counters, c->stream), "trace launch");
    c->countersPending = true;
    return VKRT_CUDA_SUCCESS;
}

int32_t vkrt_cuda_trace_rays(VKRT_CudaContext* c, const VKRT_CudaRay* rays, uint32_t count, uint32_t anyHit,
                             VKRT_CudaHit* hits) {
    if (!c) return VKRT_CUDA_ERROR_INVALID_ARGUMENT;
    if (count && (!rays || !hits)) return invalid(c, "null ray or hit array");
    if (count == 0) return VKRT_CUDA_SUCCESS;
    cudaSetDevice(c->device);
    VKRT_CudaRay* dRays = nullptr;
    VKRT_CudaHit* dHits = nullptr;
    cudaError_t e = cudaMalloc(&dRays, sizeof(VKRT_CudaRay) * count);
    if (e == cudaSuccess) e = cudaMalloc(&dHits, sizeof(VKRT_CudaHit) * count);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dRays, rays, sizeof(VKRT_CudaRay) * count, cudaMemcpyHostToDevice, c->stream);
    int32_t r = VKRT_CUDA_SUCCESS;
    if (e == cudaSuccess) r = vkrt_cuda_trace_rays_device(c, dRays, count, anyHit, dHits);
    if (e == cudaSuccess && r == VKRT_CUDA_SUCCESS)
        e = cudaMemcpyAsync(hits, dHits, sizeof(VKRT_CudaHit) * count, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && r == VKRT_CUDA_SUCCESS) e = cudaStreamSynchronize(c->stream);
    cudaFree(dRays);
    cudaFree(dHits);
    if (e != cudaSuccess) return fail(c, e, "trace rays");
    return r;
}

const char* vkrt_cuda_last_error(VKRT_CudaContext* c) { return c ? c->lastError.c_str() : "null context"; }

}  // extern "C"

// Read-only view of a context for entry points implemented in other translation units (context_view.h).
namespace vkrt {
ContextView contextView(VKRT_CudaContext* c) {
    ContextView v{};
    if (!c) return v;
    v.device = c->device;
    v.stream = c->stream;
    v.counters = c->counters;
    v.nodes = c->bvh.nodes;
    v.tris = c->bvh.tris;
    v.nodeCount = c->bvh.nodeCount;
    v.triCount = c->bvh.triCount;
    return v;
}

void contextSetError(VKRT_CudaContext* c, const char* message) {
    if (c) c->lastError = message;
}

void contextMarkCountersPending(VKRT_CudaContext* c) {
    if (c) c->countersPending = true;
}
}  // namespace vkrt

extern "C" {

}  // extern "C"
