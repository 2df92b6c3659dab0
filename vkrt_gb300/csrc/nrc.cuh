// nrc.cuh — neural radiance cache: input encoding and the tensor-core MLP building blocks (device code shared by
// nrc.cu and the wavefront integrator).
//
// The cache maps a surface vertex to the radiance it scatters toward the previous vertex (its own emission
// excluded), in linear sRGB. Inputs per vertex (NrcInput, 64 bytes): world position, outgoing direction, shading
// normal, roughness, base colour, metallic. Encoding into 64 FP16 network inputs:
//   [ 0, 32)  multiresolution hash grid (Mueller et al. 2022): 16 levels x 2 FP16 features, 2^19 entries per level,
//             level resolution floor(16 * 1.5^l), trilinear interpolation; levels whose (res+1)^3 grid fits the
//             table are indexed densely, the others by the spatial hash (x * 1) ^ (y * 2654435761) ^ (z * 805459861)
//   [32, 48)  real spherical harmonics of the outgoing direction, degrees 0-3
//   [48, 51)  shading normal, [51] roughness, [52, 55) base colour, [55] metallic, [56] constant 1 (bias), zeros
// MLP: 64 -> 64 -> 64 -> 64 -> 64 -> 64 (five hidden ReLU layers of width 64) -> 16 (3 used), no biases, FP16
// weights and activations, FP32 accumulation on the tensor cores (mma.sync m16n8k16).
#pragma once

#include <cuda_fp16.h>

#include "common.cuh"

namespace vkrt {

constexpr int kNrcLevels = 16;
constexpr int kNrcFeatures = 2;
constexpr uint32_t kNrcLog2Table = 19;
constexpr uint32_t kNrcTable = 1u << kNrcLog2Table;
constexpr int kNrcWidth = 64;       // network input and hidden width
constexpr int kNrcHidden = 5;       // hidden layers
constexpr int kNrcLayers = 6;       // weight matrices: 5 of 64x64, then 16x64
constexpr int kNrcOut = 16;         // padded output width (3 used)
constexpr int kNrcBaseRes = 16;
constexpr float kNrcGrowth = 1.5f;
constexpr uint32_t kNrcWeightCount = 5u * 64u * 64u + 16u * 64u;  // 21,504
constexpr uint32_t kNrcTableParams = uint32_t(kNrcLevels) * kNrcTable * kNrcFeatures;

struct NrcInput {
    float4 posRough;     // world position, roughness
    float4 dirMetal;     // outgoing direction (unit, toward the previous vertex), metallic
    float4 normal;       // shading normal, unused
    float4 albedo;       // base colour, unused
};

struct NrcGridInfo {
    float3 lo, invExtent;             // scene bounds -> unit cube
    uint32_t res[kNrcLevels];         // per-level resolution
    uint32_t dense[kNrcLevels];       // 1 when (res + 1)^3 <= table size
};

VKRT_DEV uint32_t nrcIndex(const NrcGridInfo& gi, int level, uint32_t x, uint32_t y, uint32_t z) {
    if (gi.dense[level]) {
        uint32_t r1 = gi.res[level] + 1u;
        return x + r1 * (y + r1 * z);
    }
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (kNrcTable - 1u);
}

// Cell corner and trilinear weights of a unit-cube point on one level.
VKRT_DEV void nrcCell(const NrcGridInfo& gi, int level, float3 u, uint32_t c[3], float f[3]) {
    const float res = float(gi.res[level]);
    const float p[3] = {u.x * res, u.y * res, u.z * res};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float fl = floorf(p[a]);
        fl = fminf(fmaxf(fl, 0.0f), res - 1.0f);
        c[a] = uint32_t(fl);
        f[a] = fminf(fmaxf(p[a] - fl, 0.0f), 1.0f);
    }
}

VKRT_DEV float3 nrcUnit(const NrcGridInfo& gi, float3 p) {
    return make_float3(sat((p.x - gi.lo.x) * gi.invExtent.x), sat((p.y - gi.lo.y) * gi.invExtent.y),
                       sat((p.z - gi.lo.z) * gi.invExtent.z));
}

// real spherical harmonics, degrees 0..3, of a unit direction
VKRT_DEV void nrcSH16(float3 d, float* o) {
    const float x = d.x, y = d.y, z = d.z;
    const float xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = -1.0925484305920792f * y * z;
    o[6] = 0.94617469575755997f * zz - 0.31539156525251999f;
    o[7] = -1.0925484305920792f * x * z;
    o[8] = 0.54627421529603959f * (xx - yy);
    o[9] = 0.59004358992664352f * y * (-3.0f * xx + yy);
    o[10] = 2.8906114426405538f * x * y * z;
    o[11] = 0.45704579946446572f * y * (1.0f - 5.0f * zz);
    o[12] = 0.3731763325901154f * z * (5.0f * zz - 3.0f);
    o[13] = 0.45704579946446572f * x * (1.0f - 5.0f * zz);
    o[14] = 1.4453057213202769f * z * (xx - yy);
    o[15] = 0.59004358992664352f * x * (-xx + 3.0f * yy);
}

// The two interpolated hash features of one level (network inputs 2l, 2l+1), read from `table` (levels x entries x
// 2 halves), as an FP16 pair.
VKRT_DEV __half2 nrcEncodeLevel(const NrcGridInfo& gi, const __half2* __restrict__ table, float3 u, int l) {
    uint32_t c[3];
    float f[3];
    nrcCell(gi, l, u, c, f);
    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t dx = k & 1u, dy = (k >> 1) & 1u, dz = (k >> 2) & 1u;
        const float w = (dx ? f[0] : 1.0f - f[0]) * (dy ? f[1] : 1.0f - f[1]) * (dz ? f[2] : 1.0f - f[2]);
        const float2 v = __half22float2(table[size_t(l) * kNrcTable + nrcIndex(gi, l, c[0] + dx, c[1] + dy, c[2] + dz)]);
        a0 += w * v.x;
        a1 += w * v.y;
    }
    return __floats2half2_rn(a0, a1);
}

// Network inputs 32 + 2q and 33 + 2q (q = 0..15) of one vertex: spherical harmonics, then the material inputs.
VKRT_DEV __half2 nrcEncodeTail(const NrcInput& in, int q) {
    if (q < 8) {
        float sh[16];
        nrcSH16(xyz(in.dirMetal), sh);
        float lo = sh[0], hi = sh[1];
#pragma unroll
        for (int i = 1; i < 8; ++i)
            if (q == i) {
                lo = sh[2 * i];
                hi = sh[2 * i + 1];
            }
        return __floats2half2_rn(lo, hi);
    }
    switch (q) {
        case 8: return __floats2half2_rn(in.normal.x, in.normal.y);
        case 9: return __floats2half2_rn(in.normal.z, in.posRough.w);
        case 10: return __floats2half2_rn(in.albedo.x, in.albedo.y);
        case 11: return __floats2half2_rn(in.albedo.z, in.dirMetal.w);
        case 12: return __floats2half2_rn(1.0f, 0.0f);
        default: return __floats2half2_rn(0.0f, 0.0f);
    }
}

// ---------------------------------------------------------------------------------------------------------------
// tensor-core fragments: mma.sync.m16n8k16, A row-major 16x16 FP16, B column-major 16x8 FP16, C/D 16x8 FP32.
// Lane (g = lane / 4, t = lane % 4) holds A rows g and g+8, columns 2t..2t+1 and 2t+8..2t+9; B column g, rows
// 2t..2t+1 and 2t+8..2t+9; C rows g and g+8, columns 2t..2t+1. The C fragments of two adjacent 8-column tiles are
// the A fragment of the next layer's 16-column slice, so activations stay in registers from layer to layer.
// Weight matrices sit in shared memory as rows of 64 halves at a stride of 72 halves (144 bytes): the eight row
// addresses of an ldmatrix phase then fall on eight distinct groups of four banks.
// ---------------------------------------------------------------------------------------------------------------
VKRT_DEV void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ldmatrix.x4: four 8x8 FP16 matrices from shared memory; lane L gives the address of row L % 8 of matrix L / 8
// (16 bytes, 16-byte aligned). Lane (g, t) receives of matrix q, in r[q], row g columns 2t..2t+1 (plain) or column g
// rows 2t..2t+1 (transposed).
VKRT_DEV void ldsm4(uint32_t* r, const __half* p) {
    const uint32_t a = uint32_t(__cvta_generic_to_shared(p));
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

VKRT_DEV void ldsm4t(uint32_t* r, const __half* p) {
    const uint32_t a = uint32_t(__cvta_generic_to_shared(p));
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

VKRT_DEV uint32_t packHalf2(float lo, float hi) {
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}

VKRT_DEV float2 unpackHalf2(uint32_t v) {
    __half2 h = *reinterpret_cast<__half2*>(&v);
    return __half22float2(h);
}

}  // namespace vkrt
