/*
 * vkrt_cuda_host.h — host-side scene preparation in C, the part of vkrt's scene layer that feeds the CUDA backend.
 *
 * vkrt prepares these records on the host before each upload; this library restates that preparation so a host
 * without vkrt (tests, benchmarks, other front ends) produces byte-identical inputs:
 *   vkrt_host_pack_shader_vertices  <- packShaderVertex          (src/core/utility/packing.c:145-156)
 *   vkrt_host_mesh_transform        <- VKRT_buildMeshTransformMatrix (src/core/scene/transform.c:26-35)
 *   vkrt_host_camera_matrices       <- syncCameraMatrices         (src/core/scene/camera.c:128-143)
 *   vkrt_host_default_scene_data    <- initializeDefaultSceneSettings + writeSceneStateUniform
 *                                                                (src/core/scene/uniform.c:93-174)
 *   vkrt_host_build_light_tables    <- populateEmissiveLightScratch / finalizeMeshSelectionWeights / buildAliasTable
 *                                                                (src/core/scene/lighting.c:55-164,267-433)
 * All functions are pure host code, thread-safe, and never touch the GPU.
 */
#ifndef VKRT_CUDA_HOST_H
#define VKRT_CUDA_HOST_H

#include "vkrt_cuda_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Packs `count` authoring vertices into the 48-byte GPU layout (octahedral normal, snorm15 tangent, RGBA8 colour). */
void vkrt_host_pack_shader_vertices(const VKRT_CudaVertex* vertices, uint32_t count, VKRT_CudaShaderVertex* out);

/* Column-major 4x4 world matrix T * Rz * Ry * Rx * S with rotation in degrees. */
void vkrt_host_mesh_transform(const float position[3], const float rotationDegrees[3], const float scale[3],
                              float outColumnMajor[16]);

/* Fills sceneData->viewInverse / projInverse from a look-at camera: right-handed view, OpenGL-style [-1,1] depth
 * perspective with the Y axis flipped for Vulkan, both inverted. */
void vkrt_host_camera_matrices(const float position[3], const float target[3], const float up[3], float vfovDegrees,
                               float nearZ, float farZ, uint32_t viewportWidth, uint32_t viewportHeight,
                               VKRT_CudaSceneData* sceneData);

/* vkrt's default per-frame uniform for a width x height render: spp 8, rrMax 8, rrMin 4, ACES, RGB, hero spectral
 * sampling selected, exposure 1, environment (0.25)^3 x 1, MIS/NEE on, default camera. */
void vkrt_host_default_scene_data(uint32_t width, uint32_t height, VKRT_CudaSceneData* sceneData);

/* Emissive-light tables for NEE. Writes at most `meshCapacity` EmissiveMesh records, at most `triangleCapacity`
 * EmissiveTriangle records and their alias tables, and sets meshInfos[i].lightPdfArea = pmfMesh / area for every
 * emissive mesh (0 elsewhere). `vertices` are the unpacked authoring vertices addressed by MeshInfo.vertexBase and
 * `indices` by MeshInfo.indexBase (mesh-relative indices, as vkrt stores them).
 * Returns 0 on success, -1 on invalid arguments, -2 when a capacity is exceeded. */
int32_t vkrt_host_build_light_tables(VKRT_CudaMeshInfo* meshInfos, uint32_t meshCount,
                                     const VKRT_CudaMaterial* materials, uint32_t materialCount,
                                     const VKRT_CudaVertex* vertices, const uint32_t* indices,
                                     VKRT_CudaEmissiveMesh* outMeshes, uint32_t meshCapacity,
                                     VKRT_CudaEmissiveTriangle* outTriangles, uint32_t triangleCapacity,
                                     float* outMeshAliasQ, uint32_t* outMeshAliasIdx,
                                     float* outTriAliasQ, uint32_t* outTriAliasIdx,
                                     uint32_t* outEmissiveMeshCount, uint32_t* outEmissiveTriangleCount);

/* Vose/Walker alias table over a probability mass function of `count` entries (count >= 1). */
void vkrt_host_build_alias_table(const float* pmf, uint32_t count, float* outQ, uint32_t* outIdx);

/* vkrt's default Material (src/core/api/vkrt_types.h:79-121). */
void vkrt_host_default_material(VKRT_CudaMaterial* material);

/* Auto-SPP controller state (VKRT renderControl.autoSPP, src/core/scene/timing.c). */
typedef struct VKRT_CudaAutoSpp {
    float targetFrameMs; /* frame budget: 1000 / target FPS */
    float controlMs;     /* smoothed milliseconds per sample per pixel; 0 = no measurement yet */
} VKRT_CudaAutoSpp;

/* VKRT_setAutoSPPTargetFPS (src/core/api/settings.c:68-79): 0 selects 60 (no display refresh here), then clamps to
 * [30, 360]; resets the smoothed measurement. */
void vkrt_host_auto_spp_init(VKRT_CudaAutoSpp* state, uint32_t targetFPS);

/* updateAutoSPP (src/core/scene/timing.c:121-178): given the last frame's render milliseconds at *samplesPerPixel,
 * updates the smoothed cost per sample and moves *samplesPerPixel toward 90% of the budget, within deadbands and
 * step limits, in [1, 2048]. Returns 1 when *samplesPerPixel changed, 0 when not, -1 on invalid arguments. */
int32_t vkrt_host_auto_spp_update(VKRT_CudaAutoSpp* state, float renderMs, uint32_t* samplesPerPixel);

/* Reverses the scanline filters of a PNG image (PNG specification, 2nd ed., section 9: filter method 0, types 0 None,
 * 1 Sub, 2 Up, 3 Average, 4 Paeth), the step of image decoding that vkrt's texture import leaves to libspng
 * (src/core/utility/image.c:122-192, decodePNGImage). `src` holds `height` filtered scanlines of 1 + rowBytes bytes,
 * the filter-type byte first, as inflated from the IDAT stream (one Adam7 pass for interlaced images); `dst`
 * receives height x rowBytes reconstructed bytes. bytesPerPixel is the byte distance the Sub, Average and Paeth
 * predictors look back (at least 1). Returns 0, or -1 on an unknown filter type or invalid arguments. */
int32_t vkrt_host_png_unfilter(const uint8_t* src, uint32_t height, uint64_t rowBytes, uint32_t bytesPerPixel,
                               uint8_t* dst);

#ifdef __cplusplus
}
#endif

#endif /* VKRT_CUDA_HOST_H */
