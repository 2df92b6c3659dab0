// scene.cuh — HBM layout of one scene as the kernels see it, and the host-side context that owns it.
//
// BVH layout (all 16-byte aligned, fetched with 128-bit read-only loads):
//   nodes : 8-wide compressed nodes, 80 bytes = 5 x uint4 (Ylitie, Karras, Laine 2017 layout):
//           [0] origin.xyz (f32), exponents x/y/z (u8 each) | internal-child mask (u8)
//           [1] first child node, first triangle, meta[0..3], meta[4..7]
//           [2] qlo.x[0..7], qlo.y[0..7]   [3] qlo.z[0..7], qhi.x[0..7]   [4] qhi.y[0..7], qhi.z[0..7]
//           meta: 0 = empty slot; internal child = 0b001_xxxxx with xxxxx = 24 + slot; leaf = unary triangle count
//           in bits 5-7 and the triangle offset (< 24) relative to the node's first triangle in bits 0-4.
//   tris  : 48 bytes = 3 x float4 per triangle in BVH order: v0.xyz | global id, v1.xyz | mesh, v2.xyz | primitive.
//           Vertices are world space, transformed once at build time (flattened instancing).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace vkrt {

struct __align__(16) WideNode {
    uint4 w[5];
};
static_assert(sizeof(WideNode) == 80, "wide node is 80 bytes");

struct __align__(16) TriRecord {
    float4 v0;  // .w = global triangle id (bits)
    float4 v1;  // .w = mesh index (bits)
    float4 v2;  // .w = primitive index within the mesh (bits)
};
static_assert(sizeof(TriRecord) == 48, "triangle record is 48 bytes");

struct TextureDesc {
    const float4* texels;  // linear RGBA32F
    uint32_t width;
    uint32_t height;
};

struct EnvDistribution {
    const float* marginal;     // H + 1
    const float* conditional;  // H * (W + 1)
    const float* texelPdf;     // W * H, pdf over the unit square
    // guide tables (cutpoint method): entry k of a CDF's guide is the search result for u = k / kEnvGuide, so a
    // search for u in [k, k + 1) / kEnvGuide only scans between two neighbouring entries
    const uint32_t* marginalGuide;     // kEnvGuide + 1
    const uint32_t* conditionalGuide;  // H * (kEnvGuide + 1)
    uint32_t width, height;
    uint32_t textureIndex;     // texture the distribution was built from (VKRT_CUDA_INVALID_INDEX = none)
};

// Everything a render / trace kernel reads, passed by value as a kernel parameter.
struct DeviceScene {
    const WideNode* nodes;
    const TriRecord* tris;
    uint32_t nodeCount;
    uint32_t triCount;
    const VKRT_CudaShaderVertex* vertices;
    const uint32_t* indices;
    const VKRT_CudaMeshInfo* meshes;
    uint32_t meshCount;
    const VKRT_CudaMaterial* materials;
    uint32_t materialCount;
    const VKRT_CudaEmissiveMesh* emissiveMeshes;
    const VKRT_CudaEmissiveTriangle* emissiveTriangles;
    const float* meshAliasQ;
    const uint32_t* meshAliasIdx;
    const float* triAliasQ;
    const uint32_t* triAliasIdx;
    uint32_t emissiveMeshCount;
    uint32_t emissiveTriangleCount;
    const TextureDesc* textures;  // VKRT_CUDA_MAX_TEXTURES entries
    const float* rgb2spec;
    uint32_t rgb2specFloatCount;
    // the table selected by rgb2specCellsInfo repacked one float4 (3 coefficients) per cell: [3][res][res][res]
    const float4* rgb2specCells;
    // for the same table: the brightness interval of z = b / kRgb2SpecGuide for b = 0..kRgb2SpecGuide (0xFFFF in every
    // entry when the table's scale is not non-decreasing)
    const uint16_t* rgb2specGuide;
    VKRT_CudaRGB2SpecTableInfo rgb2specCellsInfo;
    EnvDistribution env;
    const float* sheenLtc;  // sheen LTC table (3 x 32 x 32), null until uploaded
};

struct RenderCounters {
    unsigned long long primaryRays;
    unsigned long long extensionRays;
    unsigned long long shadowRays;
    unsigned long long pathSamples;
    unsigned long long nodeBytes;        // closest-hit traversal: node / triangle bytes fetched (counting kernels)
    unsigned long long triBytes;
    unsigned long long shadowNodeBytes;  // any-hit traversal
    unsigned long long shadowTriBytes;
    unsigned long long kernelLaunches;   // launches of this backend's kernels since the counters were cleared
    unsigned int wfBodies;               // wavefront loop bodies executed (two iterations each)
    unsigned int errorFlags;
    unsigned int workCursor;  // persistent-kernel pixel cursor
};

constexpr uint32_t kErrorStackOverflow = 1u;
constexpr uint32_t kEnvGuide = 256u;
// buckets of the rgb2spec brightness guide; a power of two, so b = floor(z * kRgb2SpecGuide) is exact and b / kRgb2SpecGuide
// never exceeds z
constexpr uint32_t kRgb2SpecGuide = 1024u;
// persistent vote-scheduled traversal: by default a warp fetches new rays once fewer than this many of its lanes are
// still traversing
constexpr int kVoteRefillLanes = 20;

}  // namespace vkrt
