/*
 * vkrt_cuda_types.h — GPU/host records shared between a vkrt host and the CUDA path-tracing backend.
 *
 * These are byte-for-byte layout twins of vkrt's shared records (src/shared/types.h:25-159), written as plain C
 * so that a vkrt host can pass its own arrays (Material[], MeshInfo[], ShaderVertex[], SceneData) through the
 * C ABI in vkrt_cuda.h without repacking. vkrt declares vec2/vec3 as float[N] (no padding) and vec4/mat4 with
 * 16-byte alignment (cglm without AVX), so float3 members are followed by a 4-byte scalar and every float4/float4x4
 * member starts on a 16-byte boundary. The static asserts at the end pin the sizes (80/48/80/272/32/48/240 bytes)
 * and the offsets that the CUDA kernels read.
 *
 * Constants mirror src/shared/constants.h:1-78 and src/shared/formats.h:1-16.
 */
#ifndef VKRT_CUDA_TYPES_H
#define VKRT_CUDA_TYPES_H

#include <stddef.h>
#include <stdint.h>

#if defined(__cplusplus)
#define VKRT_CUDA_ALIGN16 alignas(16)
#define VKRT_CUDA_STATIC_ASSERT(c, m) static_assert(c, m)
#else
#define VKRT_CUDA_ALIGN16 _Alignas(16)
#define VKRT_CUDA_STATIC_ASSERT(c, m) _Static_assert(c, m)
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- constants (src/shared/constants.h) ---------------------------------------------------------------- */
#define VKRT_CUDA_INVALID_INDEX 0xFFFFFFFFu

#define VKRT_CUDA_TONE_MAPPING_NONE 0u
#define VKRT_CUDA_TONE_MAPPING_ACES 1u
#define VKRT_CUDA_RENDER_MODE_RGB 0u
#define VKRT_CUDA_RENDER_MODE_SPECTRAL 1u
#define VKRT_CUDA_SPECTRAL_SINGLE 0u
#define VKRT_CUDA_SPECTRAL_HERO 1u

/* packedRenderSettings: tone mapping in bits 0-15, render mode in 16-23, spectral sampling mode in 24-31
 * (src/shared/constants.h:18-33). */
#define VKRT_CUDA_PACK_RENDER_SETTINGS(tone, mode, spectral) \
    (((tone) & 0xFFFFu) | (((mode) & 0xFFu) << 16u) | (((spectral) & 0xFFu) << 24u))
#define VKRT_CUDA_TONE_MAPPING_OF(p) ((p) & 0xFFFFu)
#define VKRT_CUDA_RENDER_MODE_OF(p) (((p) >> 16u) & 0xFFu)
#define VKRT_CUDA_SPECTRAL_MODE_OF(p) (((p) >> 24u) & 0xFFu)

#define VKRT_CUDA_DEBUG_MODE_NONE 0u

#define VKRT_CUDA_ALPHA_MODE_OPAQUE 0u
#define VKRT_CUDA_COLOR_SPACE_SRGB 0u
#define VKRT_CUDA_COLOR_SPACE_LINEAR 1u
#define VKRT_CUDA_MAX_TEXTURES 1024u

#define VKRT_CUDA_TEXTURE_WRAP_REPEAT 10497u
#define VKRT_CUDA_TEXTURE_WRAP_CLAMP_TO_EDGE 33071u
#define VKRT_CUDA_TEXTURE_WRAP_MIRRORED_REPEAT 33648u

/* texture formats (src/shared/formats.h:8-14) */
#define VKRT_CUDA_TEXTURE_FORMAT_RGBA8_UNORM 0u
#define VKRT_CUDA_TEXTURE_FORMAT_RGBA16_UNORM 1u
#define VKRT_CUDA_TEXTURE_FORMAT_RGBA16_SFLOAT 2u
#define VKRT_CUDA_TEXTURE_FORMAT_RGBA32_SFLOAT 3u

/* ---- records (src/shared/types.h) ---------------------------------------------------------------------- */

/* unpacked authoring vertex (types.h:25-32), 80 bytes */
typedef struct VKRT_CudaVertex {
    VKRT_CUDA_ALIGN16 float position[4];
    VKRT_CUDA_ALIGN16 float normal[4];
    VKRT_CUDA_ALIGN16 float tangent[4];
    VKRT_CUDA_ALIGN16 float color[4];
    float texcoord0[2];
    float texcoord1[2];
} VKRT_CudaVertex;

/* GPU vertex (types.h:34-41), 48 bytes: octahedral snorm16 normal, snorm15x2+sign tangent, RGBA8 colour */
typedef struct VKRT_CudaShaderVertex {
    VKRT_CUDA_ALIGN16 float position[4];
    float texcoord0[2];
    float texcoord1[2];
    uint32_t packedNormal;
    uint32_t packedTangent;
    uint32_t packedColor;
} VKRT_CudaShaderVertex;

/* per-mesh instance record (types.h:43-58), 80 bytes; TRS = T * Rz * Ry * Rx * S, rotation in degrees */
typedef struct VKRT_CudaMeshInfo {
    float position[3];
    uint32_t vertexBase;
    float rotation[3];
    uint32_t vertexCount;
    float scale[3];
    uint32_t indexBase;
    uint32_t indexCount;
    uint32_t materialIndex;
    uint32_t renderBackfaces;
    float lightPdfArea;
    float opacity;
    uint32_t reserved0;
    uint32_t reserved1;
    uint32_t reserved2;
} VKRT_CudaMeshInfo;

/* Principled material (types.h:60-101), 272 bytes */
typedef struct VKRT_CudaMaterial {
    float baseColor[3];
    float roughness;
    float emissionColor[3];
    float emissionLuminance;
    float eta[3];
    float metallic;
    float k[3];
    float anisotropic;
    float specular;
    float specularTint;
    float abbeNumber;
    float reserved0;
    VKRT_CUDA_ALIGN16 float sheenTintWeight[4];
    float clearcoat;
    float clearcoatGloss;
    float ior;
    float diffuseRoughness;
    float transmission;
    float subsurface;
    float sheenRoughness;
    float absorptionCoefficient;
    float attenuationColor[3];
    float normalTextureScale;
    uint32_t baseColorTextureIndex;
    uint32_t metallicRoughnessTextureIndex;
    uint32_t normalTextureIndex;
    uint32_t emissiveTextureIndex;
    uint32_t baseColorTextureWrap;
    uint32_t metallicRoughnessTextureWrap;
    uint32_t normalTextureWrap;
    uint32_t emissiveTextureWrap;
    float opacity;
    float alphaCutoff;
    uint32_t alphaMode;
    uint32_t textureTexcoordSets;
    VKRT_CUDA_ALIGN16 float baseColorTextureTransform[4];
    VKRT_CUDA_ALIGN16 float metallicRoughnessTextureTransform[4];
    VKRT_CUDA_ALIGN16 float normalTextureTransform[4];
    VKRT_CUDA_ALIGN16 float emissiveTextureTransform[4];
    VKRT_CUDA_ALIGN16 float textureRotations[4];
} VKRT_CudaMaterial;

/* emissive mesh for alias-table NEE (types.h:103-110), 32 bytes */
typedef struct VKRT_CudaEmissiveMesh {
    uint32_t triOffset;
    uint32_t triCount;
    float pmfMesh;
    float invTotalArea;
    float emission[3];
    float reserved0;
} VKRT_CudaEmissiveMesh;

/* world-space emissive triangle: v0 + area, edge1, edge2 (types.h:112-116), 48 bytes */
typedef struct VKRT_CudaEmissiveTriangle {
    VKRT_CUDA_ALIGN16 float v0Area[4];
    VKRT_CUDA_ALIGN16 float e1Pad[4];
    VKRT_CUDA_ALIGN16 float e2Pad[4];
} VKRT_CudaEmissiveTriangle;

/* rgb2spec table addressing (types.h:118-122) */
typedef struct VKRT_CudaRGB2SpecTableInfo {
    uint32_t res;
    uint32_t scaleOffset;
    uint32_t dataOffset;
} VKRT_CudaRGB2SpecTableInfo;

/* per-frame uniform (types.h:128-150), 240 bytes; matrices are column-major (cglm mat4[col][row]) */
typedef struct VKRT_CudaSceneData {
    VKRT_CUDA_ALIGN16 float viewInverse[4][4];
    VKRT_CUDA_ALIGN16 float projInverse[4][4];
    uint32_t frameNumber;
    uint32_t samplesPerPixel;
    uint32_t rrMaxDepth;
    uint32_t rrMinDepth;
    VKRT_CUDA_ALIGN16 uint32_t viewportRect[4];
    uint32_t packedRenderSettings;
    float exposure;
    float timeBase;
    float timeStep;
    VKRT_CUDA_ALIGN16 float environmentLight[4];
    uint32_t environmentTextureIndex;
    float environmentRotation;
    uint32_t debugMode;
    uint32_t misNeeEnabled;
    uint32_t emissiveMeshCount;
    uint32_t emissiveTriangleCount;
    uint32_t selectionEnabled;
    uint32_t selectedMeshIndex;
    VKRT_CudaRGB2SpecTableInfo rgb2specSRGB;
} VKRT_CudaSceneData;

VKRT_CUDA_STATIC_ASSERT(sizeof(VKRT_CudaVertex) == 80, "Vertex layout");
VKRT_CUDA_STATIC_ASSERT(sizeof(VKRT_CudaShaderVertex) == 48, "ShaderVertex layout");
VKRT_CUDA_STATIC_ASSERT(sizeof(VKRT_CudaMeshInfo) == 80, "MeshInfo layout");
VKRT_CUDA_STATIC_ASSERT(sizeof(VKRT_CudaMaterial) == 272, "Material layout");
VKRT_CUDA_STATIC_ASSERT(sizeof(VKRT_CudaEmissiveMesh) == 32, "EmissiveMesh layout");
VKRT_CUDA_STATIC_ASSERT(sizeof(VKRT_CudaEmissiveTriangle) == 48, "EmissiveTriangle layout");
VKRT_CUDA_STATIC_ASSERT(sizeof(VKRT_CudaRGB2SpecTableInfo) == 12, "RGB2SpecTableInfo layout");
VKRT_CUDA_STATIC_ASSERT(sizeof(VKRT_CudaSceneData) == 240, "SceneData layout");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaMaterial, sheenTintWeight) == 80, "Material.sheenTintWeight");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaMaterial, attenuationColor) == 128, "Material.attenuationColor");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaMaterial, baseColorTextureIndex) == 144, "Material.baseColorTextureIndex");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaMaterial, baseColorTextureTransform) == 192, "Material.textureTransform");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaSceneData, frameNumber) == 128, "SceneData.frameNumber");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaSceneData, viewportRect) == 144, "SceneData.viewportRect");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaSceneData, environmentLight) == 176, "SceneData.environmentLight");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaSceneData, rgb2specSRGB) == 224, "SceneData.rgb2specSRGB");
VKRT_CUDA_STATIC_ASSERT(offsetof(VKRT_CudaMeshInfo, lightPdfArea) == 60, "MeshInfo.lightPdfArea");

#ifdef __cplusplus
}
#endif

#endif /* VKRT_CUDA_TYPES_H */
