// oracle.h — TEST INFRASTRUCTURE ONLY. C interface of the CPU oracle for the vkrt CUDA backend:
//   * a restatement of vkrt's Slang path tracer (RGB and hero-spectral integrators, glTF metallic-roughness
//     Principled subset, alias-table NEE, environment lookup, Russian roulette, film blend), templated so it runs
//     in FP32 (the reference's own arithmetic width) or FP64;
//   * a binned-SAH BVH2 with the watertight ray/triangle test in FP32 (same operation order as the CUDA kernels);
//   * a brute-force FP64 all-triangle intersector with a near-tie / near-edge ambiguity classifier;
//   * a CPU rgb2spec table fit and an FP64 environment CDF, to validate the device generators.
// Only tests, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load this library.
#pragma once

#include <stdint.h>

#include "vkrt_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleTexture {
    const float* rgba; /* linear RGBA32F, width*height*4 */
    uint32_t width;
    uint32_t height;
} OracleTexture;

typedef struct OracleSceneDesc {
    const VKRT_CudaShaderVertex* vertices;
    uint32_t vertexCount;
    const uint32_t* indices;
    uint32_t indexCount;
    const VKRT_CudaMeshInfo* meshes;
    uint32_t meshCount;
    const VKRT_CudaMaterial* materials;
    uint32_t materialCount;
    const VKRT_CudaEmissiveMesh* emissiveMeshes;
    uint32_t emissiveMeshCount;
    const VKRT_CudaEmissiveTriangle* emissiveTriangles;
    uint32_t emissiveTriangleCount;
    const float* meshAliasQ;
    const uint32_t* meshAliasIdx;
    const float* triAliasQ;
    const uint32_t* triAliasIdx;
    const OracleTexture* textures; /* indexed by texture slot; entries with rgba == NULL are unbound */
    uint32_t textureCount;
    const float* rgb2spec; /* vkrt table layout, may be NULL for RGB-only scenes */
    uint32_t rgb2specFloatCount;
    uint32_t environmentSampling; /* VKRT_CUDA_ENV_*: 1 builds the importance distribution of envTextureIndex */
    uint32_t envTextureIndex;
    const float* sheenLtc; /* 3 x 32 x 32 sheen LTC table (bsdf/data/sheen_ltc.slang layout), NULL: no sheen lobe */
    uint32_t sheenLtcFloatCount;
} OracleSceneDesc;

typedef struct OracleRenderParams {
    uint32_t rngMode;   /* VKRT_CUDA_RNG_* */
    uint64_t rngSeed;
    uint32_t precision; /* 32 or 64 */
    uint32_t threads;   /* 0 = hardware concurrency */
    uint32_t rowBegin;  /* render rows [rowBegin, rowEnd) only; other pixels of accumOut are left untouched */
    uint32_t rowEnd;    /* 0 = full height */
    uint32_t useBruteForce; /* 1: FP64 brute-force closest hit instead of the BVH (tiny scenes only) */
    uint32_t rowStep;   /* render every rowStep-th row of [rowBegin, rowEnd) (0 or 1 = every row): a sample of the
                           frame spread over its whole height */
} OracleRenderParams;

typedef struct OracleRenderStats {
    uint64_t primaryRays;
    uint64_t extensionRays;
    uint64_t shadowRays;
    uint64_t pathSamples;
} OracleRenderStats;

void* oracle_scene_create(const OracleSceneDesc* desc);
void oracle_scene_destroy(void* scene);

/* FP32 watertight traversal of the oracle BVH2; hits use the same record as VKRT_CudaHit. `anyHit` bit 0: first
 * accepted hit; bit 1: mask cut-outs are dropped as selection rays drop them (rt/alpha_test.slang:68-76). */
int32_t oracle_trace_fp32(void* scene, const VKRT_CudaRay* rays, uint32_t count, uint32_t anyHit,
                          VKRT_CudaHit* hits, uint32_t threads);
/* FP64 brute force over all world-space triangles (vertices transformed in FP64 from the FP32 mesh TRS);
 * ambiguous[i] = 1 when a near-tie or near-edge candidate could change the answer under FP32 rounding. */
int32_t oracle_trace_fp64_bruteforce(void* scene, const VKRT_CudaRay* rays, uint32_t count, VKRT_CudaHit* hits,
                                     uint8_t* ambiguous, double eps, uint32_t threads);

/* One frame of the restated integrator: reads accumIn (RGBA32F, .w = count; may equal accumOut), writes accumOut
 * and, when outputRGBA16 != NULL, the tone-mapped output. */
int32_t oracle_render(void* scene, const VKRT_CudaSceneData* sceneData, const OracleRenderParams* params,
                      const float* accumIn, float* accumOut, uint16_t* outputRGBA16, OracleRenderStats* stats);

/* Same frame with the accumulation written in double precision (the image before its FP32 store), for
 * finite-difference checks of gradients. */
/* oracle_render with the denoiser features: albedoOut / normalOut receive the frame's per-pixel feature means
 * (RGBA32F, .w = number of samples whose feature resolved). */
int32_t oracle_render_features(void* scene, const VKRT_CudaSceneData* sceneData, const OracleRenderParams* params,
                               const float* accIn, float* accOut, float* albedoOut, float* normalOut);
int32_t oracle_render_f64(void* scene, const VKRT_CudaSceneData* sceneData, const OracleRenderParams* params,
                          const float* accumIn, double* accumOut);

/* RNG known answers */
uint32_t oracle_hash(uint32_t v);
uint32_t oracle_init_pixel_seed(int32_t x, int32_t y, uint32_t frame, uint32_t sampleIndex);
float oracle_rand(uint32_t* state);
uint32_t oracle_pcg32(uint64_t* state, uint64_t inc);

/* world-space triangle soup (v0,v1,v2 as 9 floats per triangle, FP32 exactly as the device flattens it) */
uint32_t oracle_world_triangles(void* scene, float* out, uint32_t capacity);

/* environment importance distribution: marginal (H+1) and conditional (H*(W+1)) CDFs in FP64 -> FP32, and the
 * solid-angle pdf of directions */
int32_t oracle_env_cdf(const float* rgba, uint32_t width, uint32_t height, float* marginal, float* conditional,
                       double* totalOut, float* texelPdf);
float oracle_env_pdf(void* scene, const float dir[3], float rotationDegrees);
int32_t oracle_env_sample(void* scene, float u1, float u2, float rotationDegrees, float dirOut[3], float* pdfOut);

/* rgb2spec table fit on the CPU (Gauss-Newton per cell), same layout as vkrt's table */
int32_t oracle_rgb2spec_generate(uint32_t res, float* out, uint32_t floatCount, uint32_t threads);
/* eval helpers for tests */
void oracle_rgb2spec_fetch(const float* table, uint32_t res, const float rgb[3], float coeff[3]);
float oracle_rgb2spec_eval(const float coeff[3], float lambdaNm);
void oracle_spectral_to_xyz(float lambdaNm, float xyz[3]);
void oracle_xyz_to_linear_srgb(const float xyz[3], float rgb[3]);

/* BSDF probes for unit tests: evaluates/samples the restated RGB Principled subset in the local frame */
int32_t oracle_bsdf_eval_rgb(const VKRT_CudaMaterial* material, const float wo[3], const float wi[3],
                             uint32_t frontFace, float value[3], float* pdf);
int32_t oracle_bsdf_sample_rgb(const VKRT_CudaMaterial* material, const float wo[3], uint32_t frontFace,
                               uint32_t rngState, float wi[3], float weight[3], float* pdf);

#ifdef __cplusplus
}
#endif
