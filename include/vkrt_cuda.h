/*
 * vkrt_cuda.h — C ABI of the GB300 (sm_103a) path-tracing backend for vkrt.
 *
 * The backend replaces vkrt's Vulkan ray-tracing dispatch: the body of recordMainTracePass
 * (src/core/runtime/command/record.c:448-486, vkCmdTraceRaysKHR(W,H,1)), the per-mesh BLAS / TLAS builds it
 * traverses (src/core/render/accel/blas.c:14-262, tlas.c:291-346) and the descriptor bindings the ray-generation
 * shader reads (src/shaders/scene/resources.slang:7-59). Everything here takes plain host pointers and counts;
 * records use the vkrt layouts from vkrt_cuda_types.h. One context = one device, one CUDA stream, one film.
 * Like vkrt's API (src/core/api/vkrt.h), calls on a context are not thread-safe: the caller serialises them.
 *
 * Results are vkrt's VKRT_Result codes (src/core/api/vkrt_types.h:16-26).
 */
#ifndef VKRT_CUDA_H
#define VKRT_CUDA_H

#include "vkrt_cuda_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* VKRT_Result values (vkrt_types.h:16-26) */
#define VKRT_CUDA_SUCCESS 0
#define VKRT_CUDA_ERROR_INVALID_ARGUMENT (-1)
#define VKRT_CUDA_ERROR_OPERATION_FAILED (-2)
#define VKRT_CUDA_ERROR_OUT_OF_MEMORY (-3)
#define VKRT_CUDA_ERROR_DEVICE_LOST (-4)
#define VKRT_CUDA_ERROR_INITIALIZATION_FAILED (-5)

/* random-number stream of the path sampler */
#define VKRT_CUDA_RNG_REFERENCE 0u /* vkrt's Wellons-hash stream, seed = f(pixel, frame, sample): random.slang:7-27 */
#define VKRT_CUDA_RNG_PCG32 1u     /* PCG32 (O'Neill 2014), one stream per (pixel, sample), state from rngSeed */

/* environment-light estimator */
#define VKRT_CUDA_ENV_BSDF_ONLY 0u   /* vkrt: environment only on BSDF-sampled misses (environment.slang:16-27) */
#define VKRT_CUDA_ENV_IMPORTANCE 1u  /* equirect luminance*sin(theta) importance sampling + MIS with the BSDF */

/* integrator selected by VKRT_CudaConfig.integrator */
#define VKRT_CUDA_INTEGRATOR_MEGAKERNEL 0u /* one thread per pixel runs whole paths (vkrt's raygen structure) */
#define VKRT_CUDA_INTEGRATOR_WAVEFRONT 1u  /* persistent stage kernels over compacted path queues, one graph launch */

typedef struct VKRT_CudaContext VKRT_CudaContext;

typedef struct VKRT_CudaConfig {
    int32_t deviceIndex;          /* CUDA device ordinal */
    uint32_t rngMode;             /* VKRT_CUDA_RNG_* */
    uint64_t rngSeed;             /* PCG32 seed (ignored by the reference stream) */
    uint32_t environmentSampling; /* VKRT_CUDA_ENV_* */
    uint32_t countRays;           /* 1: also count BVH node / triangle fetch bytes per frame */
    uint32_t threadsPerBlock;     /* megakernel block size, 0 = default (128) */
    uint32_t blocksPerSM;         /* reserved for the megakernel, 0 = default */
    uint32_t integrator;          /* VKRT_CUDA_INTEGRATOR_* */
    uint32_t treeletMinTriangles; /* BVH builds of scenes with at least this many triangles run treelet
                                     restructuring (Karras & Aila 2013: about 5% fewer node bytes per ray for
                                     2.4 ms per pass on 1M triangles, against 3.0 ms for the whole plain build);
                                     0 = the default (65,536), 0xFFFFFFFF = never */
    uint32_t treeletsOnUpdate;    /* 1: rebuilds after mesh-transform edits (vkrt_cuda_update_meshes) restructure too;
                                     0 (default): they build the plain LBVH, so interactive edits stay fast */
    uint32_t treeletPasses;       /* bottom-up treelet restructuring passes when treelets run, at most 8; 0 = the
                                     default (2: the second pass gives 2% fewer node visits per ray than one
                                     alone) */
    uint32_t reserved[4];
} VKRT_CudaConfig;

/* Wavefront integrator parameters (autotuned by vkrt_cuda_autotune_batch). 64 bytes. */
typedef struct VKRT_CudaWavefrontConfig {
    uint32_t queueCapacity;        /* path slots, at most 256M (about 70 GB of slot state); 0 = one per (pixel,
                                      sample) item of the batch, capped at 64M */
    uint32_t tileWidth;            /* pixels are handed to path slots in tiles of tileWidth x tileHeight */
    uint32_t tileHeight;
    uint32_t sortByMaterial;       /* shade-queue order: 0 as traced; 1 counting-sorted by (scene, hit class);
                                      2 partitioned into misses, dielectric and metal hits by the intersect kernel;
                                      3 counting-sorted by material (each warp shades one material's lobes) */
    uint32_t intersectBlocksPerSM; /* persistent grid of the traversal kernels, per SM */
    uint32_t shadeBlocksPerSM;     /* persistent grid of the shading kernels, per SM; also their register budget:
                                      3: 168 registers, 4 (default): 128, 6: 80, 8: 64 (the full-material-stack,
                                      feature and adjoint kernels keep one budget: 168, 168 and 128) */
    uint32_t useGraph;             /* 1: the frame is one CUDA-graph launch (conditional while node) */
    uint32_t profileStages;        /* 1: stage-by-stage launches with device timers and fetch-byte counting (slower;
                                      for profiling), reported in VKRT_CudaStats.stageMs / *FetchBytes */
    uint32_t refillLanes;          /* persistent traversal: a warp fetches new rays once fewer than this many of its
                                      32 lanes are still traversing; 0 = the default (20), else 1..32 */
    uint32_t rayOrder;             /* 1: paths are queued for traversal in 8 bins by the octant of their ray direction,
                                      so a traversal warp draws rays of one octant; 0: in the order the previous stage
                                      produced them (camera rays in tile order) */
    uint32_t reserved[6];
} VKRT_CudaWavefrontConfig;

typedef struct VKRT_CudaStats {
    uint64_t primaryRays;    /* camera rays traced by the last render call */
    uint64_t extensionRays;  /* closest-hit rays after the first bounce */
    uint64_t shadowRays;     /* any-hit (occlusion) rays */
    uint64_t pathSamples;    /* pixel samples started */
    uint64_t nodeFetchBytes; /* closest-hit BVH node bytes fetched (countRays, or wavefront profileStages) */
    uint64_t triFetchBytes;  /* closest-hit triangle bytes fetched (same) */
    uint32_t bvhNodeCount;   /* 8-wide nodes */
    uint32_t bvhTriangleCount;
    uint64_t bvhBytes;       /* nodes + triangle records resident in HBM */
    float bvhBuildMs;        /* device time of the last BVH build */
    uint32_t errorFlags;     /* device-side error word (bit 0: traversal stack overflow guard hit) */
    uint32_t wavefrontBodies;      /* wavefront loop bodies (two bounces each) of the last call */
    uint32_t cacheTrainingRecords; /* radiance-cache training records gathered by the last call (cache enabled) */
    uint64_t shadowNodeFetchBytes; /* any-hit traversal node / triangle bytes (same conditions as nodeFetchBytes) */
    uint64_t shadowTriFetchBytes;
    uint64_t kernelLaunches;       /* this backend's kernel launches made by the last call */
    float stageMs[8];              /* wavefront profileStages device ms: prologue, begin, intersect, sort, shade,
                                      shadow, finalize, resolve */
    float bvhSahLbvh;              /* SAH cost / root area of the binary tree before treelet restructuring */
    float bvhSahTreelets;          /* the same after */
} VKRT_CudaStats;

/* ray record for the trace entry points: origin/tMin, direction/tMax (32 bytes, 16-byte aligned) */
typedef struct VKRT_CudaRay {
    float origin[3];
    float tMin;
    float direction[3];
    float tMax;
} VKRT_CudaRay;

/* closest-hit record: the payload vkrt's closest-hit shader stores (entry/path/closest_hit.slang:3-5,
 * rt/payloads/scene_payload.slang:6-43). Misses report instanceIndex = primitiveIndex = VKRT_CUDA_INVALID_INDEX. */
typedef struct VKRT_CudaHit {
    uint32_t instanceIndex;  /* mesh index (TLAS instance) */
    uint32_t primitiveIndex; /* triangle index within the mesh */
    float t;
    float u; /* barycentric weight of vertex 1 */
    float v; /* barycentric weight of vertex 2 */
    uint32_t reserved[3];
} VKRT_CudaHit;

void vkrt_cuda_default_config(VKRT_CudaConfig* config);

/* Creates a context on config->deviceIndex (NULL config = defaults). Replaces VKRT_initWithCreateInfo's device and
 * pipeline setup (src/core/api/lifecycle.c:586-610) for the tracing path. */
int32_t vkrt_cuda_create(const VKRT_CudaConfig* config, VKRT_CudaContext** outContext);
void vkrt_cuda_destroy(VKRT_CudaContext* context);

/* Uploads the global vertex/index buffers and mesh records and builds the BVH on the device (Morton codes, radix
 * sort, LBVH, treelet refinement, 8-wide compressed collapse). Indices are mesh-relative, addressed through
 * MeshInfo.indexBase and offset by MeshInfo.vertexBase, exactly as loadTriangleVertices reads them
 * (geometry/surface/interpolation.slang:8-25). Replaces the BLAS/TLAS builds (record.c:124-168). */
int32_t vkrt_cuda_upload_geometry(VKRT_CudaContext* context, const VKRT_CudaShaderVertex* vertices,
                                  uint32_t vertexCount, const uint32_t* indices, uint32_t indexCount,
                                  const VKRT_CudaMeshInfo* meshes, uint32_t meshCount);

/* Replaces the mesh records only (transform / material / lightPdfArea edits); rebuilds the BVH when a transform
 * changed. Counts must match the last upload. */
int32_t vkrt_cuda_update_meshes(VKRT_CudaContext* context, const VKRT_CudaMeshInfo* meshes, uint32_t meshCount);

int32_t vkrt_cuda_upload_materials(VKRT_CudaContext* context, const VKRT_CudaMaterial* materials, uint32_t count);

/* Emissive-light tables for NEE (lighting.c:496-544 builds them; light_sampling.slang:9-37 reads them). */
int32_t vkrt_cuda_upload_lights(VKRT_CudaContext* context, const VKRT_CudaEmissiveMesh* meshes, uint32_t meshCount,
                                const VKRT_CudaEmissiveTriangle* triangles, uint32_t triangleCount,
                                const float* meshAliasQ, const uint32_t* meshAliasIdx, const float* triAliasQ,
                                const uint32_t* triAliasIdx);

/* Bindless texture slot `textureIndex` (< VKRT_CUDA_MAX_TEXTURES), sampled bilinearly without mips as vkrt's
 * samplers do (src/core/scene/textures.c:141-164). format: VKRT_CUDA_TEXTURE_FORMAT_*; colorSpace SRGB decodes
 * 8/16-bit UNORM texels to linear. */
int32_t vkrt_cuda_upload_texture(VKRT_CudaContext* context, uint32_t textureIndex, const void* pixels,
                                 uint32_t width, uint32_t height, uint32_t format, uint32_t colorSpace);

/* Selects the environment texture used for importance sampling and builds its 2D CDF (FP64 prefix sums) on the
 * device; VKRT_CUDA_INVALID_INDEX = constant environment colour. The texture index and rotation that shading
 * uses still come from SceneData.environmentTextureIndex / environmentRotation each frame. */
int32_t vkrt_cuda_set_environment(VKRT_CudaContext* context, uint32_t textureIndex);

/* Copies the environment importance distribution that vkrt_cuda_set_environment built to host memory: the marginal
 * CDF over rows (height + 1 floats), the conditional CDFs of the rows (height x (width + 1) floats) and the per-texel
 * sampling weights (width x height floats, pdf over the unit square). width and height must be the environment
 * texture's; any output pointer may be NULL. No counterpart in vkrt, which samples the environment only through the
 * BSDF: it lets a host check the distribution. */
int32_t vkrt_cuda_read_environment_distribution(VKRT_CudaContext* context, uint32_t width, uint32_t height,
                                                float* marginal, float* conditional, float* texelPdf);

/* rgb2spec coefficient table in vkrt's buffer layout: `res` z-scale floats followed by 3*res^3*3 coefficients
 * (src/core/scene/rgb2spec.c:17-89). */
int32_t vkrt_cuda_upload_rgb2spec(VKRT_CudaContext* context, const float* table, uint32_t floatCount,
                                  const VKRT_CudaRGB2SpecTableInfo* info);

/* The sheen lobe's LTC fit table, SHEEN_LTC_TABLE of vkrt (src/shaders/bsdf/data/sheen_ltc.slang:6-8): three
 * 32 x 32 layers (transform a, transform b, directional albedo) over (cos theta_o, sheen roughness), row-major by
 * roughness; floatCount must be 3072. Materials with a sheen colour (sheenTintWeight) render only once it is
 * installed (a frame without it returns VKRT_CUDA_ERROR_INVALID_ARGUMENT). */
#define VKRT_CUDA_SHEEN_TABLE_FLOATS 3072u
int32_t vkrt_cuda_upload_sheen_table(VKRT_CudaContext* context, const float* table, uint32_t floatCount);

/* Generates the sRGB rgb2spec table on the device (Jakob & Hanika 2019 Gauss-Newton fit against the CIE 1931
 * analytic fits under illuminant E, the colour space of vkrt's spectral output transform) and installs it.
 * Returns the table layout in outInfo; the table stays resident. */
int32_t vkrt_cuda_generate_rgb2spec(VKRT_CudaContext* context, uint32_t res, VKRT_CudaRGB2SpecTableInfo* outInfo);
int32_t vkrt_cuda_download_rgb2spec(VKRT_CudaContext* context, float* table, uint32_t floatCount);

/* (Re)allocates the film: accumulation RGBA32F ping-pong (.w = sample count) and the RGBA16 UNORM output; clears. */
int32_t vkrt_cuda_resize(VKRT_CudaContext* context, uint32_t width, uint32_t height);

/* Clears the accumulation film (the accumulationNeedsReset clear, record.c:300-446). */
int32_t vkrt_cuda_reset_accumulation(VKRT_CudaContext* context);

/* Renders one frame: SceneData.samplesPerPixel samples per pixel blended into the running mean, then swaps the
 * ping-pong accumulation images (VKRT_trace -> recordMainTracePass plus the swap in VKRT_endFrame,
 * src/core/api/frame.c:267-337,380-390). Asynchronous on the context stream; SceneData is copied at call time. */
int32_t vkrt_cuda_render_frame(VKRT_CudaContext* context, const VKRT_CudaSceneData* sceneData);

/* Selects the integrator of later render calls (VKRT_CUDA_INTEGRATOR_*); images are the same either way. */
int32_t vkrt_cuda_set_integrator(VKRT_CudaContext* context, uint32_t integrator);

void vkrt_cuda_default_wavefront_config(VKRT_CudaWavefrontConfig* config);
int32_t vkrt_cuda_set_wavefront_config(VKRT_CudaContext* context, const VKRT_CudaWavefrontConfig* config);
int32_t vkrt_cuda_get_wavefront_config(VKRT_CudaContext* context, VKRT_CudaWavefrontConfig* config);

/* Renders one frame of every context in one batched wavefront pass: all contexts on one device and in one render
 * mode (all RGB or all hero spectral), each with its own scene, BVH, camera (sceneDatas[i]) and film; scenes and
 * resolutions may differ. The work runs on contexts[0]'s stream as a single CUDA-graph launch with contexts[0]'s
 * wavefront configuration; every context's accumulation images are swapped as by vkrt_cuda_render_frame. Ray
 * counters of the whole batch are reported by contexts[0]. This has no single counterpart in vkrt, which renders
 * one scene per VKRT_draw; per scene it computes what vkrt_cuda_render_frame computes. */
int32_t vkrt_cuda_render_batch(VKRT_CudaContext* const* contexts, const VKRT_CudaSceneData* sceneDatas,
                               uint32_t count);

/* Picks queue capacity, tile shape, material sorting and per-SM residency of the wavefront integrator for this
 * batch by timing candidate configurations (coordinate descent, `framesPerTrial` frames each at two samples per
 * pixel), stores the best in contexts[0] and returns it with its frame time. Clears the accumulation of every
 * context in the batch. */
int32_t vkrt_cuda_autotune_batch(VKRT_CudaContext* const* contexts, const VKRT_CudaSceneData* sceneDatas,
                                 uint32_t count, uint32_t framesPerTrial, VKRT_CudaWavefrontConfig* best,
                                 float* bestFrameMs);

/* Waits for all work on the context stream, polling up to timeoutMs (0 = wait without limit). Returns
 * VKRT_CUDA_ERROR_OPERATION_FAILED on timeout, VKRT_CUDA_ERROR_DEVICE_LOST on a CUDA error. */
int32_t vkrt_cuda_sync(VKRT_CudaContext* context, uint32_t timeoutMs);

/* Copies the latest accumulation (RGBA32F, .w = samples; linear sRGB in RGB mode, CIE XYZ in spectral mode) or
 * the tone-mapped RGBA16 UNORM output to host memory; `bytes` must be >= width*height*16 (resp. *8). */
int32_t vkrt_cuda_read_accumulation(VKRT_CudaContext* context, float* rgba, size_t bytes);
int32_t vkrt_cuda_read_output(VKRT_CudaContext* context, uint16_t* rgba, size_t bytes);

/* Pipelined readback of the latest accumulation (same contents and size rule as vkrt_cuda_read_accumulation), an
 * addition of this backend for frame loops that hand every frame to the host: the copy runs on the context's own
 * copy stream once the frames queued so far are done, while the next frame renders (a frame only reads the
 * accumulation it blends into; the frame after it, which overwrites that buffer, first waits for the copy).
 * Returns without waiting; `rgba` must stay valid and untouched until vkrt_cuda_wait_readback returns. With pageable
 * host memory the copy is correct but does not overlap; pinned memory (cudaHostAlloc) lets it run on a copy engine.
 * vkrt_cuda_wait_readback waits for every readback started on the context (timeoutMs as for vkrt_cuda_sync). */
int32_t vkrt_cuda_read_accumulation_async(VKRT_CudaContext* context, float* rgba, size_t bytes);
int32_t vkrt_cuda_wait_readback(VKRT_CudaContext* context, uint32_t timeoutMs);

int32_t vkrt_cuda_get_stats(VKRT_CudaContext* context, VKRT_CudaStats* stats);

/* Denoiser features (integrator/path/loop.slang:83-111, writeback.slang:87-114): with enabled = 1, forward frames of
 * either integrator also accumulate, per pixel, the albedo and shading normal of each sample's first vertex that is
 * not followed through a sharp specular lobe (bsdf/principled/denoiser.slang), as running means weighted by the
 * number of samples whose feature resolved (.w). The feature films are cleared with the accumulation.
 * vkrt_cuda_read_denoiser_features copies the latest albedo and normal films (RGBA32F, width*height*16 bytes each;
 * either pointer may be NULL). */
int32_t vkrt_cuda_set_denoiser_features(VKRT_CudaContext* context, uint32_t enabled);
int32_t vkrt_cuda_read_denoiser_features(VKRT_CudaContext* context, float* albedo, float* normal, size_t bytes);

/* CUDA stream (cudaStream_t) the context launches on, for callers that time or order work around it. */
void* vkrt_cuda_stream(VKRT_CudaContext* context);

/* Flags of the trace calls' `anyHit` word. VKRT_CUDA_TRACE_ANY_HIT (1) stops at the first accepted hit (shadow
 * query, rt/queries/shadow_query.slang:8-28; the record then carries that hit); without it the call returns the closest
 * hit (scene query, rt/queries/scene_query.slang:10-42). VKRT_CUDA_TRACE_PERSISTENT (2) runs the rays through the
 * wavefront integrator's persistent traversal (dynamic ray fetch, a warp vote per step between node visits and
 * triangle tests) instead of one ray per thread; both give identical records. */
#define VKRT_CUDA_TRACE_ANY_HIT 1u
#define VKRT_CUDA_TRACE_PERSISTENT 2u

/* Traces `count` rays against the current BVH; `anyHit` holds VKRT_CUDA_TRACE_* flags (0 = closest hit by one ray
 * per thread). Host arrays; synchronous. */
int32_t vkrt_cuda_trace_rays(VKRT_CudaContext* context, const VKRT_CudaRay* rays, uint32_t count, uint32_t anyHit,
                             VKRT_CudaHit* hits);
/* Same on device arrays, asynchronous on the context stream. */
int32_t vkrt_cuda_trace_rays_device(VKRT_CudaContext* context, const VKRT_CudaRay* deviceRays, uint32_t count,
                                    uint32_t anyHit, VKRT_CudaHit* deviceHits);

/* Same trace as vkrt_cuda_trace_rays, for callers that must not allocate device memory (a real-time frame thread
 * that cannot absorb the device-wide synchronisation of cudaFree, or a host with a fixed device-memory budget).
 * No counterpart in vkrt: it is an addition of this backend. Rays and hits are staged in two fixed file-scope
 * device arrays instead of per-call cudaMalloc buffers, so the call performs no allocation. At most 65,536 rays per
 * call (larger counts return VKRT_CUDA_ERROR_INVALID_ARGUMENT). The arrays (4 MiB) exist once per device and are
 * shared by every call on that device: calls that overlap on the GPU race and must be serialised by the caller.
 * The first call on a device resolves the arrays' addresses; make it before any stream capture. The resolved
 * addresses are kept for the life of the process: after a cudaDeviceReset (or anything else that destroys and
 * re-creates the device's primary context) this entry point must not be called again. Host arrays; synchronous. */
int32_t vkrt_cuda_trace_rays_noalloc(VKRT_CudaContext* context, const VKRT_CudaRay* rays, uint32_t count,
                                     uint32_t anyHit, VKRT_CudaHit* hits);

/* ---------------------------------------------------------------------------------------------------------------
 * Differentiable rendering (path-replay backpropagation). No counterpart in vkrt, whose renderer has no adjoint:
 * these calls are an addition of this backend, built on the same RGB integrator as vkrt_cuda_render_frame.
 * ------------------------------------------------------------------------------------------------------------- */
#define VKRT_CUDA_GRADIENT_BASE_COLOR 1u /* Material.baseColor and baseColor-texture texels (RGB) */
#define VKRT_CUDA_GRADIENT_ROUGHNESS 2u  /* Material.roughness and metallic-roughness-texture texels (G) */
#define VKRT_CUDA_GRADIENT_EMISSION 4u   /* emission radiance (emissionColor x emissionLuminance) per material */

typedef struct VKRT_CudaAdjointConfig {
    uint32_t sampleBase; /* accumulated sample count before the differentiated frame (0 after a reset) */
    uint32_t gradients;  /* VKRT_CUDA_GRADIENT_* mask; 0 = all */
    uint32_t accumulate; /* nonzero: add to the gradient buffers; zero: clear them first */
    uint32_t reserved[5];
} VKRT_CudaAdjointConfig;

/* Per-material gradient record, 32 bytes. */
typedef struct VKRT_CudaMaterialGradient {
    float baseColor[3];
    float roughness;
    float emission[3];
    float reserved;
} VKRT_CudaMaterialGradient;

void vkrt_cuda_default_adjoint_config(VKRT_CudaAdjointConfig* config);

/* Material of each emissive-mesh entry uploaded with vkrt_cuda_upload_lights (the mesh whose emission the entry
 * copies), needed to route light-sampling terms to emission gradients. */
int32_t vkrt_cuda_set_emissive_mesh_materials(VKRT_CudaContext* context, const uint32_t* materials, uint32_t count);

/* Adds to the gradient buffers d(loss)/d(parameters) for the frame vkrt_cuda_render_frame renders from
 * `sceneData` (same frame number, seeds and scene), given dImage = d(loss)/d(accumulation) as width*height RGBA32F
 * values (alpha ignored). RGB render mode only; materials must have specularTint 0 (its F0 tint couples the colour
 * channels and is not differentiated). Gradients are unbiased for the expected image; with Russian roulette off
 * (rrMinDepth > rrMaxDepth) and sampling densities independent of the parameters they are the exact derivative of
 * the fixed-seed estimator. Host dImage: synchronous upload, asynchronous kernel on the context stream. */
int32_t vkrt_cuda_render_adjoint(VKRT_CudaContext* context, const VKRT_CudaSceneData* sceneData, const float* dImage,
                                 const VKRT_CudaAdjointConfig* config);
/* Same with dImage in device memory (asynchronous on the context stream). */
int32_t vkrt_cuda_render_adjoint_device(VKRT_CudaContext* context, const VKRT_CudaSceneData* sceneData,
                                        const float* deviceDImage, const VKRT_CudaAdjointConfig* config);

/* Gradient of the texels of texture slot `textureIndex` (width*height RGBA32F, same layout as the upload; zeros
 * for slots no material samples as baseColor or metallic-roughness). Synchronous. */
int32_t vkrt_cuda_read_texture_gradient(VKRT_CudaContext* context, uint32_t textureIndex, float* rgba, size_t bytes);
/* Per-material gradients, `count` <= material count. Synchronous. */
int32_t vkrt_cuda_read_material_gradients(VKRT_CudaContext* context, VKRT_CudaMaterialGradient* gradients,
                                          uint32_t count);

/* ---------------------------------------------------------------------------------------------------------------
 * Neural radiance cache. No counterpart in vkrt: an addition of this backend (wavefront integrator). A multiresolution
 * hash grid (16 levels x 2 FP16 features, 2^19 entries per level, base resolution 16, growth 1.5) and an MLP of five
 * hidden ReLU layers of width 64 (FP16 weights, FP32 accumulation on the tensor cores) predict the radiance a surface
 * vertex scatters toward the previous vertex. With the cache enabled, every wavefront frame first traces
 * `trainingPaths` full-length paths from random pixels, trains the cache on their per-vertex radiance (relative L2
 * loss, Adam), then renders with paths that stop at bounce `terminationDepth` and add the cache's prediction.
 * ------------------------------------------------------------------------------------------------------------- */
typedef struct VKRT_CudaNrcConfig {
    uint32_t enabled;          /* 1: cache-terminated render paths and per-frame training (wavefront frames) */
    uint32_t terminationDepth; /* bounce at which render paths query the cache and stop (default 2) */
    uint32_t trainingPaths;    /* training paths traced per frame (default 65536) */
    uint32_t trainingSteps;    /* optimiser steps per frame over the frame's training records (default 4) */
    float learningRate;        /* Adam step size (default 1e-2; beta1 0.9, beta2 0.99, epsilon 1e-8) */
    uint32_t seed;             /* parameter initialisation and training-pixel selection */
    uint32_t inferenceTensorPath; /* cache inference on VKRT_CUDA_NRC_TCGEN05 (0, default: tcgen05 MMAs with
                                     tensor-memory accumulators) or VKRT_CUDA_NRC_MMA_SYNC (1: warp-level mma.sync,
                                     the path training uses); same network, FP16 operands, FP32 accumulation */
    float inferenceAverage;    /* 0 (default): inference reads the optimiser's current parameters; in (0, 1): it reads
                                  their exponential moving average, updated after every optimiser step with this
                                  decay (less frame-to-frame noise in the cache's predictions) */
    float terminationSpread;   /* 0 (default): render paths query the cache at bounce `terminationDepth`; c > 0: they
                                  also query it at the first vertex where the area spread of the path after its
                                  primary vertex exceeds c times the primary vertex's footprint seen from the camera
                                  (Mueller et al. 2021, "Real-time Neural Radiance Caching for Path Tracing", 3.3;
                                  the paper uses c = 0.01), and at `terminationDepth` at the latest */
    uint32_t trainingTracer;   /* 0 (default): one thread traces each training path; 1: the training paths run
                                  through the wavefront stages as a pass of their own before the frame (the same
                                  paths and records; slower at the default 65,536 paths, which fill a dozen
                                  bounces of stage launches poorly) */
    uint32_t reserved[6];
} VKRT_CudaNrcConfig;
#define VKRT_CUDA_NRC_TCGEN05 0u
#define VKRT_CUDA_NRC_MMA_SYNC 1u

/* cache input record: 16 floats (position xyz + roughness, outgoing direction xyz + metallic, shading normal xyz + 0,
 * base colour rgb + 0); outputs are 4 floats per input (linear sRGB radiance, unused) */
#define VKRT_CUDA_NRC_INPUT_FLOATS 16u
#define VKRT_CUDA_NRC_WEIGHTS 21504u           /* FP16 weights: 5 x (64 x 64) then 16 x 64, [out][in] row-major */
#define VKRT_CUDA_NRC_TABLE_HALVES 16777216u   /* FP16 hash table: 16 levels x 2^19 entries x 2 features */

void vkrt_cuda_default_nrc_config(VKRT_CudaNrcConfig* config);
/* (Re)initialises the cache over the bounds of the uploaded geometry and stores the configuration. */
int32_t vkrt_cuda_nrc_configure(VKRT_CudaContext* context, const VKRT_CudaNrcConfig* config);
/* Predictions for n host input records. Synchronous. */
int32_t vkrt_cuda_nrc_infer(VKRT_CudaContext* context, const float* inputs, uint32_t n, float* outputs);
/* The last cache frame's training records, in the order they were written: up to `capacity` inputs (16 floats each)
 * and targets (4 floats each, linear sRGB in rgb); *count (may be NULL) receives how many the frame wrote.
 * Synchronous. */
int32_t vkrt_cuda_nrc_read_training_records(VKRT_CudaContext* context, float* inputs, float* targets,
                                            uint32_t capacity, uint32_t* count);
/* One optimiser step on n host records (targets: 4 floats each, rgb used); apply = 0 computes the gradients only.
 * *loss (may be NULL) receives the step's loss. Synchronous. */
int32_t vkrt_cuda_nrc_train(VKRT_CudaContext* context, const float* inputs, const float* targets, uint32_t n,
                            uint32_t apply, float* loss);
/* Reads (write = 0) or writes (write = 1) the FP16 parameters; table may be NULL. */
int32_t vkrt_cuda_nrc_parameters(VKRT_CudaContext* context, uint16_t* weights, uint16_t* table, uint32_t write);
/* FP32 gradients of the last training step (weights: VKRT_CUDA_NRC_WEIGHTS floats; table: NULL or
 * VKRT_CUDA_NRC_TABLE_HALVES floats). */
int32_t vkrt_cuda_nrc_gradients(VKRT_CudaContext* context, float* weights, float* table);
/* Hash-grid placement: scene bounds (3 + 3 floats), per-level resolution and dense flag (16 each). */
int32_t vkrt_cuda_nrc_grid(VKRT_CudaContext* context, float* lo, float* hi, uint32_t* resolution, uint32_t* dense);

/* Selection overlay, replacing vkrt's selection trace and outline post-pass (entry/select/raygen.slang:5-14,
 * entry/post/outline.slang:19-60, recorded by runtime/command/record.c when selection is enabled): when
 * sceneData->selectionEnabled is set, traces the selection mask of sceneData->selectedMeshIndex (a pixel-centre
 * camera ray per pixel, first hit on that mesh only) and draws its outline (colour (1, 0.55, 0.1), radius
 * clamp(round(min(W, H) * 2 / 1080), 1, 5)) into the current output image; otherwise the mask is cleared.
 * Call after the frame's render. Asynchronous on the context stream. */
int32_t vkrt_cuda_render_selection_overlay(VKRT_CudaContext* context, const VKRT_CudaSceneData* sceneData);
/* Copies the last selection mask (width*height uint32, 1 = selected mesh) to host memory. Synchronous. */
int32_t vkrt_cuda_read_selection_mask(VKRT_CudaContext* context, uint32_t* mask, size_t bytes);
/* Pick query (VKRT_requestSelectionAtPixel, api/settings.c:236-245, answered in integrator/path/debug.slang:21-29):
 * mesh index of the closest hit of pixel (x, y)'s centre ray, VKRT_CUDA_INVALID_INDEX on a miss. Synchronous. */
int32_t vkrt_cuda_pick_mesh(VKRT_CudaContext* context, const VKRT_CudaSceneData* sceneData, uint32_t x, uint32_t y,
                            uint32_t* meshIndex);
/* Device milliseconds of the last vkrt_cuda_render_frame call (CUDA events on the context stream); waits for that
 * frame to finish. The render time vkrt's auto-SPP controller reads (scene/timing.c:54-59). */
int32_t vkrt_cuda_last_frame_ms(VKRT_CudaContext* context, float* milliseconds);

/* Last error message of this context (never NULL). */
const char* vkrt_cuda_last_error(VKRT_CudaContext* context);

#ifdef __cplusplus
}
#endif

#endif /* VKRT_CUDA_H */
