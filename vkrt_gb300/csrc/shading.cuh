// shading.cuh — device shading for the sm_103a megakernels: surface reconstruction, textures, the glTF
// metallic-roughness subset of vkrt's layered Principled BSDF, emissive-triangle NEE, the environment light and its
// importance distribution, and rgb2spec hero-wavelength spectral upsampling. Each function names the vkrt shader it
// computes the same quantity as (paths relative to src/shaders/).
//
// Material coverage here: the glTF metallic-roughness subset (metal, dielectric specular and Lambert lobes), which the
// reflection-only instantiations use. The rest of vkrt's stack (clearcoat, Oren-Nayar, fake subsurface, the
// transmissive interface with dispersion and media) is in bsdf_full.cuh for the full instantiations. Sheen (its LTC
// fit table) is in bsdf_full.cuh too.
#pragma once

#include "scene.cuh"

namespace vkrt {

// ---------------------------------------------------------------------------------------------------------------
// geometry/packing.slang
// ---------------------------------------------------------------------------------------------------------------
VKRT_DEV float3 decodeOct(float px, float py) {
    float z = 1.0f - fabsf(px) - fabsf(py);
    if (z < 0.0f) {
        float ox = px;
        px = (1.0f - fabsf(py)) * (ox >= 0.0f ? 1.0f : -1.0f);
        py = (1.0f - fabsf(ox)) * (py >= 0.0f ? 1.0f : -1.0f);
    }
    return normalize(make_float3(px, py, z));
}
VKRT_DEV float3 unpackNormal(uint32_t p) {
    return decodeOct(float(int32_t(p << 16) >> 16) / 32767.0f, float(int32_t(p) >> 16) / 32767.0f);
}
VKRT_DEV float unpackSnorm15(uint32_t v) {
    int32_t s = int32_t(v & 0x7fffu);
    if (s & 0x4000) s |= ~int32_t(0x7fffu);
    return fminf(fmaxf(float(s) / 16383.0f, -1.0f), 1.0f);
}
VKRT_DEV float4 unpackTangent(uint32_t p) {
    float3 d = decodeOct(unpackSnorm15(p), unpackSnorm15(p >> 15u));
    return make_float4(d.x, d.y, d.z, (p & 0x80000000u) ? -1.0f : 1.0f);
}
VKRT_DEV float4 unpackColor(uint32_t p) {
    const float s = 1.0f / 255.0f;
    return make_float4(float(p & 0xffu) * s, float((p >> 8) & 0xffu) * s, float((p >> 16) & 0xffu) * s,
                       float((p >> 24) & 0xffu) * s);
}

// ---------------------------------------------------------------------------------------------------------------
// geometry/surface/transform.slang
// ---------------------------------------------------------------------------------------------------------------
VKRT_DEV float3 rotateMesh(float3 v, const float* deg) {
    const float k = 0.01745329251994329577f;
    float s, c;
    sincosf(deg[0] * k, &s, &c);
    v = make_float3(v.x, c * v.y - s * v.z, s * v.y + c * v.z);
    sincosf(deg[1] * k, &s, &c);
    v = make_float3(c * v.x + s * v.z, v.y, -s * v.x + c * v.z);
    sincosf(deg[2] * k, &s, &c);
    return make_float3(c * v.x - s * v.y, s * v.x + c * v.y, v.z);
}
VKRT_DEV float safeRcp(float v) {
    if (fabsf(v) > 1e-6f) return 1.0f / v;
    return v < 0.0f ? -1.0f / 1e-6f : 1.0f / 1e-6f;
}
VKRT_DEV bool meshHasRotationOrScale(const VKRT_CudaMeshInfo& m) {
    return m.rotation[0] != 0.0f || m.rotation[1] != 0.0f || m.rotation[2] != 0.0f || m.scale[0] != 1.0f ||
           m.scale[1] != 1.0f || m.scale[2] != 1.0f;
}
VKRT_DEV float3 meshVector(const VKRT_CudaMeshInfo& m, float3 v) {
    return rotateMesh(v * make_float3(m.scale[0], m.scale[1], m.scale[2]), m.rotation);
}
VKRT_DEV float3 meshNormal(const VKRT_CudaMeshInfo& m, float3 n) {
    float3 inv = make_float3(safeRcp(m.scale[0]), safeRcp(m.scale[1]), safeRcp(m.scale[2]));
    return safeNormalize(rotateMesh(n * inv, m.rotation));
}

// ---------------------------------------------------------------------------------------------------------------
// surface reconstruction (geometry/surface/reconstruct.slang:8-49, interpolation.slang:8-60)
// ---------------------------------------------------------------------------------------------------------------
struct TexCoords {
    float4 color;
    float2 uv0, uv1;
};

struct Surface {
    float3 hitPoint;
    float3 shadingNormal;
    float3 geometricNormal;  // oriented against the incoming ray
    float4 tangent;
    uint32_t frontFace;
    uint32_t materialIndex;
    TexCoords tex;
};

VKRT_DEV float4 lerpTri(float4 a, float4 b, float4 c, float u, float v) {
    float w = 1.0f - u - v;
    return a * w + b * u + c * v;
}

VKRT_DEV Surface reconstructSurface(const DeviceScene& sc, uint32_t meshIndex, uint32_t prim, float u, float v,
                                    float3 org, float3 dir, float t) {
    Surface s;
    s.hitPoint = org + dir * t;
    const VKRT_CudaMeshInfo& m = sc.meshes[meshIndex];
    uint32_t base = m.indexBase + prim * 3u;
    uint32_t i0 = __ldg(sc.indices + base) + m.vertexBase;
    uint32_t i1 = __ldg(sc.indices + base + 1) + m.vertexBase;
    uint32_t i2 = __ldg(sc.indices + base + 2) + m.vertexBase;
    // 48-byte vertices: position (16 B) + texcoords (16 B) + packed normal/tangent/colour (12 B + 4 pad)
    const float4* va = reinterpret_cast<const float4*>(sc.vertices + i0);
    const float4* vb = reinterpret_cast<const float4*>(sc.vertices + i1);
    const float4* vc = reinterpret_cast<const float4*>(sc.vertices + i2);
    float4 pa = __ldg(va), ta = __ldg(va + 1), qa = __ldg(va + 2);
    float4 pb = __ldg(vb), tb = __ldg(vb + 1), qb = __ldg(vb + 2);
    float4 pc = __ldg(vc), tc = __ldg(vc + 1), qc = __ldg(vc + 2);
    float w = 1.0f - u - v;
    float3 on = unpackNormal(__float_as_uint(qa.x)) * w + unpackNormal(__float_as_uint(qb.x)) * u +
                unpackNormal(__float_as_uint(qc.x)) * v;
    on = safeNormalize(on);
    float4 ot = lerpTri(unpackTangent(__float_as_uint(qa.y)), unpackTangent(__float_as_uint(qb.y)),
                        unpackTangent(__float_as_uint(qc.y)), u, v);
    float hand = ot.w < 0.0f ? -1.0f : 1.0f;
    bool xform = meshHasRotationOrScale(m);
    float3 sn = xform ? meshNormal(m, on) : safeNormalize(on);
    float facing = dot(sn, dir) > 0.0f ? -1.0f : 1.0f;
    float3 e1 = xyz(pb) - xyz(pa), e2 = xyz(pc) - xyz(pa);
    if (xform) {
        e1 = meshVector(m, e1);
        e2 = meshVector(m, e2);
    }
    float3 gn = safeNormalize(cross(e1, e2));
    if (m.scale[0] * m.scale[1] * m.scale[2] < 0.0f) gn = -gn;
    s.materialIndex = m.materialIndex;
    s.frontFace = dot(gn, dir) < 0.0f ? 1u : 0u;
    s.shadingNormal = sn * facing;
    s.geometricNormal = s.frontFace ? gn : -gn;
    float3 tw = xyz(ot);
    tw = safeNormalize(xform ? meshVector(m, tw) : tw) * facing;
    s.tangent = make_float4(tw.x, tw.y, tw.z, hand);
    s.tex.color = lerpTri(unpackColor(__float_as_uint(qa.z)), unpackColor(__float_as_uint(qb.z)),
                          unpackColor(__float_as_uint(qc.z)), u, v);
    s.tex.uv0 = make_float2(ta.x * w + tb.x * u + tc.x * v, ta.y * w + tb.y * u + tc.y * v);
    s.tex.uv1 = make_float2(ta.z * w + tb.z * u + tc.z * v, ta.w * w + tb.w * u + tc.w * v);
    return s;
}

// ---------------------------------------------------------------------------------------------------------------
// textures: bilinear, no mips (src/core/scene/textures.c:141-164), material/textures.slang
// ---------------------------------------------------------------------------------------------------------------
VKRT_DEV int wrapIndex(int i, int n, uint32_t mode) {
    if (mode == VKRT_CUDA_TEXTURE_WRAP_CLAMP_TO_EDGE) return min(max(i, 0), n - 1);
    if (mode == VKRT_CUDA_TEXTURE_WRAP_MIRRORED_REPEAT) {
        int p = ((i % (2 * n)) + 2 * n) % (2 * n);
        return p < n ? p : 2 * n - 1 - p;
    }
    return ((i % n) + n) % n;
}
VKRT_DEV uint32_t wrapMode(uint32_t m) {
    return (m == VKRT_CUDA_TEXTURE_WRAP_CLAMP_TO_EDGE || m == VKRT_CUDA_TEXTURE_WRAP_MIRRORED_REPEAT)
               ? m
               : VKRT_CUDA_TEXTURE_WRAP_REPEAT;
}

VKRT_DEV float4 sampleBilinear(const TextureDesc& t, float u, float v, uint32_t wrapU, uint32_t wrapV) {
    float x = u * float(t.width) - 0.5f, y = v * float(t.height) - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    int x0 = int(fx), y0 = int(fy);
    float ax = x - fx, ay = y - fy;
    int xa = wrapIndex(x0, int(t.width), wrapU), xb = wrapIndex(x0 + 1, int(t.width), wrapU);
    int ya = wrapIndex(y0, int(t.height), wrapV), yb = wrapIndex(y0 + 1, int(t.height), wrapV);
    float4 c00 = __ldg(t.texels + size_t(ya) * t.width + xa), c10 = __ldg(t.texels + size_t(ya) * t.width + xb);
    float4 c01 = __ldg(t.texels + size_t(yb) * t.width + xa), c11 = __ldg(t.texels + size_t(yb) * t.width + xb);
    return c00 * ((1.0f - ax) * (1.0f - ay)) + c10 * (ax * (1.0f - ay)) + c01 * ((1.0f - ax) * ay) + c11 * (ax * ay);
}

VKRT_DEV float4 sampleMaterialTexture(const DeviceScene& sc, uint32_t idx, uint32_t wrap, const float* xf, float rot,
                                      uint32_t set, const TexCoords& tc, float4 fallback) {
    if (idx >= VKRT_CUDA_MAX_TEXTURES) return fallback;
    TextureDesc t = sc.textures[idx];
    if (!t.texels) return fallback;
    float2 uv = set == 1u ? tc.uv1 : tc.uv0;
    float sx = uv.x * xf[0], sy = uv.y * xf[1];
    float sn, cs;
    sincosf(rot, &sn, &cs);
    return sampleBilinear(t, cs * sx - sn * sy + xf[2], sn * sx + cs * sy + xf[3], wrapMode(wrap & 0xffffu),
                          wrapMode((wrap >> 16) & 0xffffu));
}

// ---------------------------------------------------------------------------------------------------------------
// alpha test (rt/alpha_test.slang:8-68): mask (cut-out against alphaCutoff, then mesh x material x vertex opacity)
// and blend (mesh x material x texture opacity) decided with alphaRandom
// ---------------------------------------------------------------------------------------------------------------
constexpr uint32_t kAlphaModeMask = 1u, kAlphaModeBlend = 2u;  // VKRT_MATERIAL_ALPHA_MODE_* (shared/constants.h)

VKRT_DEV bool alphaMayReject(const VKRT_CudaMaterial& mat, float meshOpacity) {  // alphaMayRejectHit (:8-10)
    return mat.alphaMode == kAlphaModeMask || mat.alphaMode == kAlphaModeBlend || mat.opacity < 0.999f ||
           meshOpacity < 0.999f;
}

// The texture alpha of a candidate hit (evaluateMaterialTextureAlpha, :19-25) and its vertex alpha in `vertexAlpha`
VKRT_DEV float hitTextureAlpha(const DeviceScene& sc, const VKRT_CudaMeshInfo& m, const VKRT_CudaMaterial& mat,
                               uint32_t prim, float u, float v, float& vertexAlpha) {
    // evaluateSurfaceTextureData (geometry/surface/interpolation.slang:46-60)
    const uint32_t base = m.indexBase + prim * 3u;
    const float4* va = reinterpret_cast<const float4*>(sc.vertices + __ldg(sc.indices + base) + m.vertexBase);
    const float4* vb = reinterpret_cast<const float4*>(sc.vertices + __ldg(sc.indices + base + 1) + m.vertexBase);
    const float4* vc = reinterpret_cast<const float4*>(sc.vertices + __ldg(sc.indices + base + 2) + m.vertexBase);
    const float4 ta = __ldg(va + 1), tb = __ldg(vb + 1), tc = __ldg(vc + 1);
    const float w = 1.0f - u - v;
    TexCoords tex;
    tex.color = lerpTri(unpackColor(__float_as_uint(__ldg(va + 2).z)), unpackColor(__float_as_uint(__ldg(vb + 2).z)),
                        unpackColor(__float_as_uint(__ldg(vc + 2).z)), u, v);
    tex.uv0 = make_float2(ta.x * w + tb.x * u + tc.x * v, ta.y * w + tb.y * u + tc.y * v);
    tex.uv1 = make_float2(ta.z * w + tb.z * u + tc.z * v, ta.w * w + tb.w * u + tc.w * v);
    vertexAlpha = tex.color.w;
    float texAlpha = tex.color.w;
    if (mat.alphaMode != VKRT_CUDA_ALPHA_MODE_OPAQUE)
        texAlpha *= sampleMaterialTexture(sc, mat.baseColorTextureIndex, mat.baseColorTextureWrap,
                                          mat.baseColorTextureTransform, mat.textureRotations[0],
                                          mat.textureTexcoordSets & 0xffu, tex, f4(1.0f)).w;
    return texAlpha;
}

VKRT_DEV bool alphaAccepts(const DeviceScene& sc, uint32_t mesh, uint32_t prim, float u, float v, uint32_t seed,
                           uint32_t gid) {
    const VKRT_CudaMeshInfo& m = sc.meshes[mesh];
    const VKRT_CudaMaterial& mat = sc.materials[m.materialIndex];
    if (!alphaMayReject(mat, m.opacity)) return true;
    float vertexAlpha;
    const float texAlpha = hitTextureAlpha(sc, m, mat, prim, u, v, vertexAlpha);
    if (mat.alphaMode == kAlphaModeMask) {  // alphaPass (:31-47)
        if (texAlpha < mat.alphaCutoff) return false;
        const float o = sat(m.opacity * mat.opacity * vertexAlpha);
        if (o >= 1.0f) return true;
        if (o <= 0.0f) return false;
        return alphaRandom(seed, gid) <= o;
    }
    const float o = sat(m.opacity * mat.opacity * texAlpha);
    if (o <= 0.0f) return false;
    if (o >= 1.0f) return true;
    return alphaRandom(seed, gid) <= o;
}

// selectionAlphaHitAccepted (:68-76): the selection and pick rays drop mask cut-outs only
VKRT_DEV bool selectionAlphaAccepts(const DeviceScene& sc, uint32_t mesh, uint32_t prim, float u, float v) {
    const VKRT_CudaMeshInfo& m = sc.meshes[mesh];
    const VKRT_CudaMaterial& mat = sc.materials[m.materialIndex];
    if (mat.alphaMode != kAlphaModeMask) return true;
    float vertexAlpha;
    return hitTextureAlpha(sc, m, mat, prim, u, v, vertexAlpha) >= mat.alphaCutoff;
}

// ---------------------------------------------------------------------------------------------------------------
// spectral utilities (utility/rgb2spec.slang, utility/spectral.slang)
// ---------------------------------------------------------------------------------------------------------------
struct SpecTable {
    const float* t;
    uint32_t res, scaleOffset, dataOffset;
    const float4* cells;    // the same coefficients one float4 per cell, or null
    const uint16_t* guide;  // brightness guide of the same table (DeviceScene::rgb2specGuide), or null
};

// the frame's table (SceneData.rgb2specSRGB) with its repacked cells when the context holds them for that layout
VKRT_DEV SpecTable makeSpecTable(const DeviceScene& sc, const VKRT_CudaSceneData& sd) {
    const VKRT_CudaRGB2SpecTableInfo& i = sd.rgb2specSRGB;
    bool packed = sc.rgb2specCells && sc.rgb2specCellsInfo.res == i.res &&
                  sc.rgb2specCellsInfo.scaleOffset == i.scaleOffset && sc.rgb2specCellsInfo.dataOffset == i.dataOffset;
    return SpecTable{sc.rgb2spec, i.res, i.scaleOffset, i.dataOffset, packed ? sc.rgb2specCells : nullptr,
                     packed ? sc.rgb2specGuide : nullptr};
}

// Largest i in [0, res - 2] with scale[i] <= x (utility/rgb2spec.slang:14-32), by binary search.
VKRT_DEV uint32_t rgb2specIntervalSearch(const SpecTable& tab, float x) {
    int left = 0, size = int(tab.res) - 2;
    while (size > 0) {
        int half = size >> 1, middle = left + half + 1;
        if (__ldg(tab.t + tab.scaleOffset + uint32_t(middle)) <= x) {
            left = middle;
            size -= half + 1;
        } else {
            size = half;
        }
    }
    return min(uint32_t(left), tab.res - 2u);
}

// The same interval from the brightness guide: the guide holds the interval of b / kRgb2SpecGuide <= x, and on a
// non-decreasing scale the interval of x is reached by stepping forward from it (usually zero or one step).
VKRT_DEV uint32_t rgb2specInterval(const SpecTable& tab, float x) {
    if (tab.guide && x >= 0.0f && x <= 1.0f) {
        const uint32_t g = __ldg(tab.guide + uint32_t(x * float(kRgb2SpecGuide)));
        if (g != 0xFFFFu) {
            uint32_t i = g;
            while (i + 2u < tab.res && __ldg(tab.t + tab.scaleOffset + i + 1u) <= x) ++i;
            return i;
        }
    }
    return rgb2specIntervalSearch(tab, x);
}

VKRT_DEV float3 rgb2specFetch(const SpecTable& tab, float3 rgb) {
    float z = fmaxf(rgb.x, fmaxf(rgb.y, rgb.z));
    if (z <= 1e-8f || !tab.t) return f3(0.0f);
    uint32_t dom = 0;
    if (rgb.y >= rgb.x) dom = 1;
    if (rgb.z >= (dom == 0 ? rgb.x : rgb.y)) dom = 2;
    float c[3] = {rgb.x, rgb.y, rgb.z};
    float xyScale = float(tab.res - 1u) / z;
    float x = c[dom == 2 ? 0 : dom + 1] * xyScale;
    float y = c[dom == 0 ? 2 : dom - 1] * xyScale;
    uint32_t xi = min(uint32_t(x), tab.res - 2u), yi = min(uint32_t(y), tab.res - 2u);
    uint32_t zi = rgb2specInterval(tab, z);
    uint32_t off = ((((dom * tab.res + zi) * tab.res + yi) * tab.res + xi) * 3u);
    uint32_t dx = 3u, dy = dx * tab.res, dz = dy * tab.res;
    float x1 = x - float(xi), y1 = y - float(yi), x0 = 1.0f - x1, y0 = 1.0f - y1;
    float s0 = __ldg(tab.t + tab.scaleOffset + zi), s1 = __ldg(tab.t + tab.scaleOffset + zi + 1u);
    float z1 = (z - s0) / fmaxf(s1 - s0, 1e-8f), z0 = 1.0f - z1;
    if (tab.cells) {  // eight 16-byte cell loads, the same arithmetic as the scalar path below
        const float4* d = tab.cells + (((dom * tab.res + zi) * tab.res + yi) * tab.res + xi);
        const uint32_t ry = tab.res, rz = tab.res * tab.res;
        float4 c000 = __ldg(d), c100 = __ldg(d + 1), c010 = __ldg(d + ry), c110 = __ldg(d + ry + 1);
        float4 c001 = __ldg(d + rz), c101 = __ldg(d + rz + 1), c011 = __ldg(d + rz + ry), c111 = __ldg(d + rz + ry + 1);
        float a[3] = {c000.x, c000.y, c000.z}, b[3] = {c100.x, c100.y, c100.z}, c[3] = {c010.x, c010.y, c010.z},
              e[3] = {c110.x, c110.y, c110.z}, f[3] = {c001.x, c001.y, c001.z}, g[3] = {c101.x, c101.y, c101.z},
              h[3] = {c011.x, c011.y, c011.z}, k[3] = {c111.x, c111.y, c111.z}, o[3];
#pragma unroll
        for (uint32_t j = 0; j < 3; ++j)
            o[j] = ((a[j] * x0 + b[j] * x1) * y0 + (c[j] * x0 + e[j] * x1) * y1) * z0 +
                   ((f[j] * x0 + g[j] * x1) * y0 + (h[j] * x0 + k[j] * x1) * y1) * z1;
        return make_float3(o[0], o[1], o[2]);
    }
    float out[3];
#pragma unroll
    for (uint32_t j = 0; j < 3; ++j) {
        const float* d = tab.t + tab.dataOffset + off + j;
        out[j] = ((__ldg(d) * x0 + __ldg(d + dx) * x1) * y0 + (__ldg(d + dy) * x0 + __ldg(d + dy + dx) * x1) * y1) * z0 +
                 ((__ldg(d + dz) * x0 + __ldg(d + dz + dx) * x1) * y0 +
                  (__ldg(d + dz + dy) * x0 + __ldg(d + dz + dy + dx) * x1) * y1) * z1;
    }
    return make_float3(out[0], out[1], out[2]);
}

VKRT_DEV float rgb2specEval(float3 c, float l) {
    float x = (c.x * l + c.y) * l + c.z;
    return 0.5f * x * rsqrtf(x * x + 1.0f) + 0.5f;
}

// spectralScalarFromLinearSrgb (spectral.slang:37-48)
VKRT_DEV float spectral1(const SpecTable& tab, float3 rgb, float l) {
    float m = maxc(rgb);
    if (m <= 0.0f) return 0.0f;
    float scale = m <= 1.0f ? 1.0f : m;
    return rgb2specEval(rgb2specFetch(tab, rgb / scale), l) * scale;
}

// spectralScalarFromLinearSrgb4 (spectral.slang:50-64)
VKRT_DEV float4 spectral4(const SpecTable& tab, float3 rgb, float4 l) {
    float m = maxc(rgb);
    if (m <= 0.0f) return f4(0.0f);
    float scale = m <= 1.0f ? 1.0f : m;
    float3 c = rgb2specFetch(tab, rgb / scale);
    return make_float4(rgb2specEval(c, l.x), rgb2specEval(c, l.y), rgb2specEval(c, l.z), rgb2specEval(c, l.w)) * scale;
}

// spectral4 as a called function rather than inlined at every use: the full-material-stack kernels, which are bound by
// instruction fetch, call it from a dozen places (the full-material frame ran 91.2 -> 87.2 ms with it)
static __device__ __noinline__ float4 spectral4Call(const SpecTable& tab, float3 rgb, float4 l) {
    return spectral4(tab, rgb, l);
}

// CIE 1931 analytic fits (spectral.slang:66-87)
VKRT_DEV float3 cieXYZ(float l) {
    float t1 = (l - 442.0f) * (l < 442.0f ? 0.0624f : 0.0374f);
    float t2 = (l - 599.8f) * (l < 599.8f ? 0.0264f : 0.0323f);
    float t3 = (l - 501.1f) * (l < 501.1f ? 0.0490f : 0.0382f);
    float X = 0.362f * __expf(-0.5f * t1 * t1) + 1.056f * __expf(-0.5f * t2 * t2) - 0.065f * __expf(-0.5f * t3 * t3);
    float u1 = (l - 568.8f) * (l < 568.8f ? 0.0213f : 0.0247f);
    float u2 = (l - 530.9f) * (l < 530.9f ? 0.0613f : 0.0322f);
    float Y = 0.821f * __expf(-0.5f * u1 * u1) + 0.286f * __expf(-0.5f * u2 * u2);
    float v1 = (l - 437.0f) * (l < 437.0f ? 0.0845f : 0.0278f);
    float v2 = (l - 459.0f) * (l < 459.0f ? 0.0385f : 0.0725f);
    float Z = 1.217f * __expf(-0.5f * v1 * v1) + 0.681f * __expf(-0.5f * v2 * v2);
    return make_float3(fmaxf(X, 0.0f), fmaxf(Y, 0.0f), fmaxf(Z, 0.0f));
}

VKRT_DEV float3 spectral4ToXYZ(float4 s, float4 l, float invPdf) {  // spectral.slang:104-113
    const float k = invPdf / kCieYIntegral;
    return cieXYZ(l.x) * (s.x * k) + cieXYZ(l.y) * (s.y * k) + cieXYZ(l.z) * (s.z * k) + cieXYZ(l.w) * (s.w * k);
}

// Bradford E->D65 then XYZ->linear sRGB (spectral.slang:14-20,89-97)
VKRT_DEV float3 xyzToLinearSrgb(float3 c) {
    float3 lms = make_float3(0.8951f * c.x + 0.2664f * c.y - 0.1614f * c.z, -0.7502f * c.x + 1.7135f * c.y + 0.0367f * c.z,
                             0.0389f * c.x - 0.0685f * c.y + 1.0296f * c.z);
    lms = lms * make_float3(0.9413344f, 1.0404175f, 1.0895327f);
    float3 d = make_float3(0.9869929f * lms.x - 0.1470543f * lms.y + 0.1599627f * lms.z,
                           0.4323053f * lms.x + 0.5183603f * lms.y + 0.0492912f * lms.z,
                           -0.0085287f * lms.x + 0.0400428f * lms.y + 0.9684867f * lms.z);
    return make_float3(3.2404542f * d.x - 1.5371385f * d.y - 0.4985314f * d.z,
                       -0.9692660f * d.x + 1.8760108f * d.y + 0.0415560f * d.z,
                       0.0556434f * d.x - 0.2040259f * d.y + 1.0572252f * d.z);
}

// ---------------------------------------------------------------------------------------------------------------
// shading basis (bsdf/base/basis.slang)
// ---------------------------------------------------------------------------------------------------------------
struct Basis {
    float3 t, b, n;
};

VKRT_DEV Basis makeBasis(float3 normal, float4 td) {
    Basis B;
    B.n = safeNormalize(normal);
    float3 tv = xyz(td);
    float3 t = tv - B.n * dot(tv, B.n);
    if (dot(t, t) <= kSafeNormalizeEps) {
        float3 up = fabsf(B.n.z) < kTangentParallel ? make_float3(0.0f, 0.0f, 1.0f) : make_float3(1.0f, 0.0f, 0.0f);
        t = safeNormalize(cross(up, B.n));
    } else {
        t = safeNormalize(t);
    }
    B.t = t;
    B.b = cross(B.n, B.t) * (td.w < 0.0f ? -1.0f : 1.0f);
    return B;
}
VKRT_DEV float3 toWorld(float3 l, const Basis& B) { return B.t * l.x + B.b * l.y + B.n * l.z; }
VKRT_DEV float3 toLocal(float3 w, const Basis& B) { return make_float3(dot(w, B.t), dot(w, B.b), dot(w, B.n)); }
VKRT_DEV float3 sanitizeNormal(float3 sn, float3 gn, float3 out) {
    float3 n = safeNormalize(sn), g = safeNormalize(gn), o = safeNormalize(out);
    if (dot(n, g) <= 1e-4f || dot(n, o) <= 1e-4f) return g;
    return n;
}

// ---------------------------------------------------------------------------------------------------------------
// material after texturing (material/textures.slang:123-155)
// ---------------------------------------------------------------------------------------------------------------
struct ShadeMaterial {
    float3 baseColor;
    float roughness, metallic, anisotropic, specular, specularTint, ior;
    float3 eta, k;
    float3 emission;  // emissionColor * emissionLuminance after the emissive texture
    bool conductor;
    float clearcoat, clearcoatGloss, subsurface, diffuseRoughness;  // the extended reflection stack's inputs
    float transmission, abbe, absorption;                            // the transmissive interface and its medium
    float3 attenuationColor;
    float3 sheenColor;  // bsdfSheenColor: saturate(tint) * saturate(weight) (material.slang:63-73)
    float sheenRoughness;
};

VKRT_DEV void shadeVertex(const DeviceScene& sc, Surface& s, float3 dir, ShadeMaterial& mat, Basis& basis) {
    const VKRT_CudaMaterial& m = sc.materials[s.materialIndex];
    Basis b0 = makeBasis(s.shadingNormal, s.tangent);
    float3 n = b0.n;
    if (m.normalTextureIndex != VKRT_CUDA_INVALID_INDEX) {
        float4 smp = sampleMaterialTexture(sc, m.normalTextureIndex, m.normalTextureWrap, m.normalTextureTransform,
                                           m.textureRotations[2], (m.textureTexcoordSets >> 16) & 0xffu, s.tex,
                                           make_float4(0.5f, 0.5f, 1.0f, 1.0f));
        float3 tn = make_float3(smp.x * 2.0f - 1.0f, smp.y * 2.0f - 1.0f, smp.z * 2.0f - 1.0f);
        tn.x *= m.normalTextureScale;
        tn.y *= m.normalTextureScale;
        tn = safeNormalize(tn);
        n = safeNormalize(b0.t * tn.x + b0.b * tn.y + b0.n * tn.z);
    }
    s.shadingNormal = sanitizeNormal(n, s.geometricNormal, -dir);
    basis = makeBasis(s.shadingNormal, s.tangent);

    mat.baseColor = make_float3(m.baseColor[0], m.baseColor[1], m.baseColor[2]);
    mat.roughness = m.roughness;
    mat.metallic = m.metallic;
    mat.anisotropic = m.anisotropic;
    mat.specular = m.specular;
    mat.specularTint = m.specularTint;
    mat.ior = m.ior;
    mat.eta = make_float3(m.eta[0], m.eta[1], m.eta[2]);
    mat.k = make_float3(m.k[0], m.k[1], m.k[2]);
    mat.conductor = m.k[0] > 0.0f || m.k[1] > 0.0f || m.k[2] > 0.0f;
    mat.clearcoat = m.clearcoat;
    mat.clearcoatGloss = m.clearcoatGloss;
    mat.subsurface = m.subsurface;
    mat.diffuseRoughness = m.diffuseRoughness;
    mat.transmission = m.transmission;
    mat.abbe = m.abbeNumber;
    mat.absorption = m.absorptionCoefficient;
    mat.attenuationColor = make_float3(m.attenuationColor[0], m.attenuationColor[1], m.attenuationColor[2]);
    mat.sheenColor = sat(make_float3(m.sheenTintWeight[0], m.sheenTintWeight[1], m.sheenTintWeight[2])) *
                     sat(m.sheenTintWeight[3]);
    mat.sheenRoughness = m.sheenRoughness;
    float4 bc = sampleMaterialTexture(sc, m.baseColorTextureIndex, m.baseColorTextureWrap, m.baseColorTextureTransform,
                                      m.textureRotations[0], m.textureTexcoordSets & 0xffu, s.tex, f4(1.0f));
    mat.baseColor = mat.baseColor * xyz(bc) * xyz(s.tex.color);
    if (m.metallicRoughnessTextureIndex != VKRT_CUDA_INVALID_INDEX) {
        float4 mr = sampleMaterialTexture(sc, m.metallicRoughnessTextureIndex, m.metallicRoughnessTextureWrap,
                                          m.metallicRoughnessTextureTransform, m.textureRotations[1],
                                          (m.textureTexcoordSets >> 8) & 0xffu, s.tex, f4(1.0f));
        mat.roughness = sat(mat.roughness * mr.y);
        mat.metallic = sat(mat.metallic * mr.z);
    } else {
        mat.roughness = sat(mat.roughness);
        mat.metallic = sat(mat.metallic);
    }
    float3 e = make_float3(m.emissionColor[0], m.emissionColor[1], m.emissionColor[2]) * m.emissionLuminance;
    if (m.emissiveTextureIndex != VKRT_CUDA_INVALID_INDEX) {
        float4 em = sampleMaterialTexture(sc, m.emissiveTextureIndex, m.emissiveTextureWrap, m.emissiveTextureTransform,
                                          m.textureRotations[3], (m.textureTexcoordSets >> 24) & 0xffu, s.tex, f4(1.0f));
        e = e * xyz(em);
    }
    mat.emission = maxc(e) > 0.0f ? e : f3(0.0f);
}

// ---------------------------------------------------------------------------------------------------------------
// Principled subset (bsdf/**)
// ---------------------------------------------------------------------------------------------------------------
VKRT_DEV float lum(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
VKRT_DEV float pow5(float v) { float v2 = v * v; return v2 * v2 * v; }
VKRT_DEV float3 schlick(float c, float3 f0) { return f0 + (f3(1.0f) - f0) * pow5(1.0f - sat(c)); }

VKRT_DEV float3 dielSpecF0(const ShadeMaterial& m) {  // fresnel.slang:15-20
    float num = m.ior - 1.0f, den = m.ior + 1.0f;
    float f = num / fmaxf(den, 1e-6f);
    float d = f * f;
    float l = lum(m.baseColor);
    float3 tint = l <= 0.0f ? f3(1.0f) : m.baseColor / l;
    float3 tt = f3(1.0f) + (tint - f3(1.0f)) * sat(m.specularTint);
    return sat(tt * (d * (m.specular / 0.5f)));
}

VKRT_DEV float3 fresnelConductor(float cosT, float3 eta, float3 k);

// Denoiser features (bsdf/principled/denoiser.slang:7-46): a vertex whose only visible response is a sharp specular
// lobe (or an identity transmissive interface) is followed through; the first other vertex gives the feature albedo
// (a weighted mix of the diffuse, dielectric, transmission, metallic and sheen colours) and its shading normal.
VKRT_DEV bool denoiserFollowsSpecular(const ShadeMaterial& m, uint32_t frontFace) {
    const float diffuseW = maxc(m.baseColor * (1.0f - m.metallic)) * (1.0f - m.transmission);
    const float subsurfaceW = diffuseW * m.subsurface;
    const float sheenW = maxc(m.sheenColor) * (1.0f - m.transmission);
    const float coatW = frontFace != 0u ? m.clearcoat : 0.0f;
    if (diffuseW > 1e-3f || subsurfaceW > 1e-3f || sheenW > 1e-3f || coatW > 1e-3f) return false;
    if (m.transmission > 1e-3f && fmaxf(m.ior, 1.0f) <= 1.0f + 1e-4f) return true;
    if (m.roughness > 0.02f) return false;
    return m.transmission > 1e-3f || m.metallic >= 1.0f - 1e-3f || maxc(dielSpecF0(m)) > 1e-3f;
}

VKRT_DEV float3 denoiserAlbedo(const ShadeMaterial& m) {
    const float nonMetal = 1.0f - m.metallic;
    const float3 diffuse = m.baseColor * nonMetal;
    const float3 f0 = dielSpecF0(m);
    const float3 metalF0 =
        m.conductor ? fresnelConductor(1.0f, fmax3(m.eta, f3(1e-3f)), fmax3(m.k, f3(0.0f))) : sat(m.baseColor);
    const float base = nonMetal * (1.0f - m.transmission);
    const float wd = base * (1.0f - m.subsurface), wss = base * m.subsurface, ws = base * sat(lum(f0));
    const float wt = nonMetal * m.transmission, wm = m.metallic, wsh = maxc(m.sheenColor) * base;
    const float total = wd + wss + ws + wt + wm + wsh;
    if (total <= 0.0f) return sat(diffuse);
    return sat((diffuse * wd + diffuse * wss + f0 * ws + f3(1.0f) * wt + metalF0 * wm + m.sheenColor * wsh) / total);
}

VKRT_DEV float fresnelDielectric(float cosT, float eta) {  // fresnel.slang:31-48
    float ci = fminf(fmaxf(cosT, -1.0f), 1.0f);
    if (ci < 0.0f) {
        eta = 1.0f / fmaxf(eta, 1e-6f);
        ci = -ci;
    }
    float s2t = fmaxf(1.0f - ci * ci, 0.0f) / fmaxf(eta * eta, 1e-6f);
    if (s2t >= 1.0f) return 1.0f;
    float ct = sqrtf(fmaxf(1.0f - s2t, 0.0f));
    float rpa = (eta * ci - ct) / fmaxf(eta * ci + ct, 1e-6f);
    float rpe = (ci - eta * ct) / fmaxf(ci + eta * ct, 1e-6f);
    return 0.5f * (rpa * rpa + rpe * rpe);
}

VKRT_DEV float3 fresnelConductor(float cosT, float3 eta, float3 k) {  // fresnel.slang:50-68
    float ci = sat(cosT), c2 = ci * ci, s2 = fmaxf(1.0f - c2, 0.0f);
    float e[3] = {eta.x, eta.y, eta.z}, kk[3] = {k.x, k.y, k.z}, r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float e2 = e[i] * e[i], k2 = kk[i] * kk[i];
        float t0 = e2 - k2 - s2;
        float ab = sqrtf(fmaxf(t0 * t0 + 4.0f * e2 * k2, 0.0f));
        float t1 = ab + c2;
        float a = sqrtf(fmaxf(0.5f * (ab + t0), 0.0f));
        float t2 = 2.0f * ci * a;
        float rs = (t1 - t2) / fmaxf(t1 + t2, 1e-6f);
        float t3 = c2 * ab + s2 * s2, t4 = t2 * s2;
        float rp = rs * ((t3 - t4) / fmaxf(t3 + t4, 1e-6f));
        r[i] = 0.5f * (rp + rs);
    }
    return make_float3(r[0], r[1], r[2]);
}

struct Ggx {
    float ax, ay, vndfK, projLen;
};

VKRT_DEV Ggx makeGgx(const ShadeMaterial& m, float3 wo) {  // ggx.slang:25-72
    Ggx g;
    float r = fmaxf(m.roughness, kGgxMinAlpha);
    float aspect = sqrtf(fmaxf(1.0f - 0.9f * m.anisotropic, kGgxMinAlpha));
    float a = r * r;
    g.ax = fmaxf(a / aspect, kGgxMinAlpha);
    g.ay = fmaxf(a * aspect, kGgxMinAlpha);
    float am = sat(fminf(g.ax, g.ay));
    float s = 1.0f + sqrtf(wo.x * wo.x + wo.y * wo.y);
    float a2 = am * am, s2 = s * s;
    g.vndfK = (1.0f - a2) * s2 / fmaxf(s2 + a2 * wo.z * wo.z, kGgxEps);
    float sx = g.ax * wo.x, sy = g.ay * wo.y;
    g.projLen = sqrtf(sx * sx + sy * sy + wo.z * wo.z);
    return g;
}
VKRT_DEV float ggxLambda(float3 w, const Ggx& g) {
    float z2 = fmaxf(w.z * w.z, kGgxEps);
    float slope2 = (g.ax * g.ax * w.x * w.x + g.ay * g.ay * w.y * w.y) / z2;
    return 0.5f * (sqrtf(1.0f + slope2) - 1.0f);
}
VKRT_DEV float ggxD(float3 m, const Ggx& g) {
    if (m.z <= 0.0f) return 0.0f;
    float c = (m.x * m.x) / (g.ax * g.ax) + (m.y * m.y) / (g.ay * g.ay) + m.z * m.z;
    return 1.0f / (kPi * g.ax * g.ay * c * c);
}
VKRT_DEV float ggxReflPdf(float3 wo, float3 m, float wom, const Ggx& g) {  // ggx.slang:88-102
    if (wo.z <= 0.0f || m.z <= 0.0f || wom <= 0.0f) return 0.0f;
    float vis = ggxD(m, g) * (1.0f / (1.0f + ggxLambda(wo, g))) * wom / fmaxf(wo.z, kGgxEps);
    return vis / fmaxf(4.0f * fabsf(wom), kGgxEps);
}
VKRT_DEV bool sampleVndf(float3 wo, const Ggx& g, float u1, float u2, float3& m) {  // ggx.slang:180-209
    if (g.projLen <= kGgxEps) return false;
    float3 ws = make_float3(wo.x * g.ax / g.projLen, wo.y * g.ay / g.projLen, wo.z / g.projLen);
    float sp, cp;
    sincosf(2.0f * kPi * u1, &sp, &cp);
    float b = g.vndfK * ws.z;
    float z = (1.0f - u2) * (1.0f + b) - b;
    float st = sqrtf(sat(1.0f - z * z));
    float3 ms = ws + make_float3(st * cp, st * sp, z);
    if (dot(ms, ms) <= kGgxEps) return false;
    float3 um = make_float3(ms.x * g.ax, ms.y * g.ay, ms.z);
    float um2 = dot(um, um);
    if (um2 <= kGgxEps) return false;
    m = um * rsqrtf(um2);
    return m.z > 0.0f;
}

// Extended reflection stack (principled/eval_rgb.slang:4-105 beyond the glTF subset): Disney clearcoat
// (lobes/clearcoat.slang: GTR1 distribution, gloss-remapped alpha, fixed 0.25 masking roughness, Schlick F0 0.04, its
// directional attenuation on everything below it), Oren-Nayar diffuse for diffuseRoughness > 0 and the Disney fake
// subsurface lobe (lobes/diffuse.slang, lobes/subsurface.slang). Used by bsdf_full.cuh.
VKRT_DEV float coatAlpha(const ShadeMaterial& m) {  // clearcoat.slang:20-28
    return fmaxf(0.1f + (0.001f - 0.1f) * sat(m.clearcoatGloss), 1e-3f);
}
VKRT_DEV float coatG1(float c, float a) {  // clearcoat.slang:30-35
    float a2 = a * a, c2 = fmaxf(c * c, 1e-6f);
    float t2 = fmaxf(1.0f - c2, 0.0f) / c2;
    return 2.0f / (1.0f + sqrtf(1.0f + a2 * t2));
}
VKRT_DEV float coatD(float cm, float a) {  // clearcoat.slang:37-45
    float a2 = a * a;
    if (a2 >= 1.0f - 1e-6f) return kInvPi;
    float den = kPi * logf(a2) * (1.0f + (a2 - 1.0f) * cm * cm);
    return (a2 - 1.0f) / fminf(den, -1e-6f);
}
VKRT_DEV float coatEval(float weight, float a, float3 wo, float3 wi, float& pdf) {  // clearcoat.slang:47-71
    pdf = 0.0f;
    if (weight <= 0.0f || wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
    float3 h = safeNormalize(wo + wi);
    float woh = sat(dot(wo, h));
    if (woh <= 0.0f) return 0.0f;
    float D = coatD(sat(h.z), a);
    float F = 0.04f + (1.0f - 0.04f) * pow5(1.0f - woh);
    float G = coatG1(wo.z, 0.25f) * coatG1(wi.z, 0.25f);
    pdf = D * sat(h.z) / fmaxf(4.0f * woh, 1e-6f);
    return 0.25f * weight * D * F * G / fmaxf(4.0f * wo.z * wi.z, 1e-6f);
}
VKRT_DEV bool coatSample(float3 wo, float a, float u1, float u2, float3& wi) {  // clearcoat.slang:73-97
    float a2 = a * a, cm;
    if (a2 >= 1.0f - 1e-6f) cm = sqrtf(fmaxf(0.0f, 1.0f - u1));
    else cm = sqrtf(sat((1.0f - powf(a2, 1.0f - u1)) / fmaxf(1.0f - a2, 1e-6f)));
    float sm = sqrtf(sat(1.0f - cm * cm)), sp, cp;
    sincosf(2.0f * kPi * u2, &sp, &cp);
    float3 m = make_float3(sm * cp, sm * sp, cm);
    float wom = dot(wo, m);
    if (wom <= 0.0f) return false;
    wi = m * (2.0f * wom) - wo;
    return wi.z > 0.0f;
}
VKRT_DEV float coatAtten(const ShadeMaterial& m, float3 w) {  // attenuation.slang:13-24
    if (m.clearcoat <= 0.0f) return 1.0f;
    float c = fabsf(w.z);
    if (c <= 0.0f) return 0.0f;
    float f = 0.04f + (1.0f - 0.04f) * pow5(1.0f - sat(c));
    return 1.0f - sat(0.25f * m.clearcoat * f);
}
VKRT_DEV float sin2Th(float3 w) { return sat(1.0f - w.z * w.z); }
VKRT_DEV float orenNayar(float rough, float3 wo, float3 wi) {  // diffuse.slang:20-53, for a unit colour
    if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
    float sg = sat(rough) * (0.5f * kPi), sg2 = sg * sg;
    float A = 1.0f - sg2 / (2.0f * (sg2 + 0.33f));
    float B = 0.45f * sg2 / (sg2 + 0.09f);
    float s2i = sin2Th(wi), s2o = sin2Th(wo);
    float si = sqrtf(s2i), so = sqrtf(s2o);
    float cphi = 0.0f;
    if (s2i > 0.0f && s2o > 0.0f) cphi = fminf(fmaxf((wi.x * wo.x + wi.y * wo.y) * rsqrtf(s2i * s2o), -1.0f), 1.0f);
    float maxCos = fmaxf(0.0f, cphi), sinA, tanB;
    if (fabsf(wi.z) > fabsf(wo.z)) {
        sinA = so;
        tanB = si / fmaxf(fabsf(wi.z), 1e-6f);
    } else {
        sinA = si;
        tanB = so / fmaxf(fabsf(wo.z), 1e-6f);
    }
    return kInvPi * (A + B * maxCos * sinA * tanB);
}
VKRT_DEV float fakeSss(float rough, float3 wo, float3 wi) {  // subsurface.slang:12-31, for a unit colour
    if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
    float3 h = safeNormalize(wo + wi);
    float wih = sat(dot(wi, h));
    float f90 = wih * wih * rough;
    float fin = 1.0f + (f90 - 1.0f) * pow5(1.0f - sat(wi.z));
    float fout = 1.0f + (f90 - 1.0f) * pow5(1.0f - sat(wo.z));
    float ss = 1.25f * (fin * fout * (1.0f / fmaxf(wi.z + wo.z, 1e-6f) - 0.5f) + 0.5f);
    return kInvPi * ss;
}

struct Bsdf {
    ShadeMaterial mat;
    float3 wo;
    Ggx ggx;
    uint32_t frontFace;
    float wMetal, wDiel, wDiff;  // normalised branch weights (principled/weights.slang:27-62)
    float wCoat, wSub;           // extended stack only (0 otherwise)
    float coatA, viewCoat;       // clearcoat alpha, coat attenuation toward wo (extended stack)
    float3 f0Diel;               // dielectric specular F0
    float3 viewAtten;            // dielectric directional attenuation at wo
};

VKRT_DEV float3 dielDirAtten(float roughness, float3 f0, float cosT) {  // attenuation.slang:30-51
    if (fabsf(cosT) <= 0.0f) return f3(0.0f);
    float rr = sat(roughness), ct = sat(fabsf(cosT));
    float r0 = rr * -1.0f + 1.0f, r1 = rr * -0.0275f + 0.0425f, r2 = rr * -0.572f + 1.04f, r3 = rr * 0.022f - 0.04f;
    float a004 = fminf(r0 * r0, exp2f(-9.28f * ct)) * r0 + r1;
    float A = sat(-1.04f * a004 + r2), B = sat(1.04f * a004 + r3);
    return sat(f3(1.0f) - sat(f0 * A + f3(B)));
}

// Branch weights of the glTF subset (principled/weights.slang:27-62 with no coat, subsurface or transmission)
VKRT_DEV Bsdf makeBsdf(const ShadeMaterial& m, float3 wo, uint32_t frontFace) {
    Bsdf s;
    s.mat = m;
    s.wo = wo;
    s.frontFace = frontFace;
    s.ggx = makeGgx(m, wo);
    s.f0Diel = dielSpecF0(m);
    s.viewAtten = dielDirAtten(m.roughness, s.f0Diel, wo.z);
    s.wCoat = s.wSub = 0.0f;
    s.coatA = 0.1f;
    s.viewCoat = 1.0f;
    float3 diff = m.baseColor * (1.0f - m.metallic);
    float nonMetal = 1.0f - m.metallic;
    float wm = m.metallic * fmaxf(lum(m.baseColor), 1e-3f);
    float wd = nonMetal * fmaxf(sat(lum(s.f0Diel)), 0.0f);
    float wf = lum(s.viewAtten) * nonMetal * fmaxf(lum(diff), 1e-3f);
    float tot = wm + wd + wf;
    if (tot <= 0.0f) {
        s.wMetal = s.wDiel = 0.0f;
        s.wDiff = 1.0f;
    } else {
        s.wMetal = wm / tot;
        s.wDiel = wd / tot;
        s.wDiff = wf / tot;
    }
    return s;
}

VKRT_DEV bool dielIdentity(const ShadeMaterial& m) { return fmaxf(m.ior, 1.0f) <= 1.0f + 1e-4f; }

VKRT_DEV float3 metalFresnel(const Bsdf& s, float c) {
    return s.mat.conductor ? fresnelConductor(c, fmax3(s.mat.eta, f3(1e-3f)), fmax3(s.mat.k, f3(0.0f)))
                           : schlick(c, s.mat.baseColor);
}

// RGB reflection stack of the subset (principled/eval_rgb.slang:4-121: metal + dielectric + Lambert)
VKRT_DEV float3 evalRgb(const Bsdf& s, float3 wi, float& pdf) {
    pdf = 0.0f;
    if (wi.z <= 0.0f) return f3(0.0f);
    float3 metal = f3(0.0f), diel = f3(0.0f);
    float3 h = s.wo + wi;
    float h2 = dot(h, h);
    float3 m = h * rsqrtf(h2);
    float wom = dot(s.wo, m);
    bool halfOk = h2 > kGgxEps && wom > 0.0f && s.wo.z > 0.0f;
    float DG = 0.0f, reflPdf = 0.0f;
    if (halfOk && (s.wMetal > 0.0f || s.wDiel > 0.0f)) {
        float G = 1.0f / (1.0f + ggxLambda(s.wo, s.ggx) + ggxLambda(wi, s.ggx));
        DG = ggxD(m, s.ggx) * G / fmaxf(4.0f * s.wo.z * wi.z, kGgxEps);
        reflPdf = ggxReflPdf(s.wo, m, wom, s.ggx);
    }
    if (s.wMetal > 0.0f && halfOk) {
        metal = metalFresnel(s, wom) * DG;
        pdf += s.wMetal * reflPdf;
    }
    if (s.wDiel > 0.0f && halfOk && !dielIdentity(s.mat)) {
        diel = schlick(wom, s.f0Diel) * DG;
        pdf += s.wDiel * reflPdf;
    }
    float3 sub = f3(0.0f);
    if (s.wDiff > 0.0f) {
        sub = s.mat.baseColor * ((1.0f - s.mat.metallic) * kInvPi);
        pdf += s.wDiff * (wi.z * kInvPi);
    }
    return metal * s.mat.metallic + (diel + s.viewAtten * sub) * (1.0f - s.mat.metallic);
}

// The direction-independent product of the spectral stack, view attenuation x diffuse (both upsampled from RGB):
// the same for every direction a vertex evaluates, so a vertex computes it once. It is multiplied by
// (1 - metallic), so a pure metal skips it (the product is finite and would contribute exactly zero).
VKRT_DEV float4 spectralDiffuseTerm(const Bsdf& s, const SpecTable& tab, float4 l) {
    if (!(1.0f - s.mat.metallic != 0.0f)) return f4(0.0f);
    float4 sub = f4(0.0f);
    if (s.wDiff > 0.0f) sub = spectral4(tab, sat(s.mat.baseColor * (1.0f - s.mat.metallic)), l) * kInvPi;
    const float4 va = spectral4(tab, sat(s.viewAtten), l);
    return va * sub;
}

// 4-lane spectral stack of the subset (principled/eval_spectral.slang:4-94); all lanes share one technique pdf.
// `vaSub` is spectralDiffuseTerm of the same Bsdf and wavelengths.
VKRT_DEV float4 evalSpectral(const Bsdf& s, const SpecTable& tab, float3 wi, float4 l, float4 vaSub, float& pdf) {
    pdf = 0.0f;
    if (wi.z <= 0.0f) return f4(0.0f);
    float4 metal = f4(0.0f), diel = f4(0.0f);
    float3 h = s.wo + wi;
    float h2 = dot(h, h);
    float3 m = h * rsqrtf(h2);
    float wom = dot(s.wo, m);
    bool halfOk = h2 > kGgxEps && wom > 0.0f && s.wo.z > 0.0f;
    float DG = 0.0f, reflPdf = 0.0f;
    if (halfOk && (s.wMetal > 0.0f || s.wDiel > 0.0f)) {
        float G = 1.0f / (1.0f + ggxLambda(s.wo, s.ggx) + ggxLambda(wi, s.ggx));
        DG = ggxD(m, s.ggx) * G / fmaxf(4.0f * s.wo.z * wi.z, kGgxEps);
        reflPdf = ggxReflPdf(s.wo, m, wom, s.ggx);
    }
    if (s.wMetal > 0.0f && halfOk) {
        metal = spectral4(tab, sat(metalFresnel(s, wom)), l) * DG;
        pdf += s.wMetal * reflPdf;
    }
    if (s.wDiel > 0.0f && halfOk && !dielIdentity(s.mat)) {
        diel = spectral4(tab, sat(schlick(wom, s.f0Diel)), l) * DG;
        pdf += s.wDiel * reflPdf;
    }
    if (s.wDiff > 0.0f) pdf += s.wDiff * (wi.z * kInvPi);
    return metal * s.mat.metallic + (diel + vaSub) * (1.0f - s.mat.metallic);
}

// sampleBSDFDirection (principled/sample.slang:4-51) of the subset: metal, dielectric reflection, diffuse
VKRT_DEV bool sampleDirection(const Bsdf& s, Rng& rng, float3& wi) {
    float sel = rng.next();
    if (sel < s.wMetal || (sel - s.wMetal) < s.wDiel) {
        bool diel = !(sel < s.wMetal);
        if (diel && (s.wo.z <= 0.0f || dielIdentity(s.mat))) return false;
        float u1 = rng.next(), u2 = rng.next();
        float3 m;
        if (!sampleVndf(s.wo, s.ggx, u1, u2, m)) return false;
        float wom = dot(s.wo, m);
        if (wom <= 0.0f) return false;
        wi = m * (2.0f * wom) - s.wo;
        return wi.z > 0.0f;
    }
    float u1 = rng.next(), u2 = rng.next();
    float r = sqrtf(u1), sp, cp;
    sincosf(2.0f * kPi * u2, &sp, &cp);
    wi = make_float3(r * cp, r * sp, sqrtf(fmaxf(0.0f, 1.0f - u1)));
    return true;
}

// ---------------------------------------------------------------------------------------------------------------
// lights
// ---------------------------------------------------------------------------------------------------------------
struct LightSample {
    float3 wi;
    float pdfSA;
    float shadowDist;
    float3 emission;
    uint32_t emissiveMesh;  // entry of the emissive-mesh table that was sampled
};

VKRT_DEV uint32_t sampleAlias(float u, uint32_t count, uint32_t off, const float* q, const uint32_t* idx) {
    float scaled = u * float(count);  // discrete.slang:13-18
    uint32_t i = min(uint32_t(scaled), count - 1u);
    return (scaled - float(i)) < __ldg(q + off + i) ? i : __ldg(idx + off + i);
}

// sampleDirectLightSurface (light/direct/light_sampling.slang:9-63); consumes 4 numbers like the reference
VKRT_DEV bool sampleEmissive(const DeviceScene& sc, float3 p, Rng& rng, LightSample& ls) {
    if (sc.emissiveMeshCount == 0u) return false;
    uint32_t mi = sampleAlias(rng.next(), sc.emissiveMeshCount, 0u, sc.meshAliasQ, sc.meshAliasIdx);
    const VKRT_CudaEmissiveMesh em = sc.emissiveMeshes[mi];
    if (em.triCount == 0u) return false;
    uint32_t lt = sampleAlias(rng.next(), em.triCount, em.triOffset, sc.triAliasQ, sc.triAliasIdx);
    const float4* tp = reinterpret_cast<const float4*>(sc.emissiveTriangles + em.triOffset + lt);
    float4 v0 = __ldg(tp), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
    float u1 = rng.next(), u2 = rng.next();
    float su = sqrtf(u1);
    float b1 = u2 * su, b2 = (1.0f - u2) * su;
    float3 pos = xyz(v0) + xyz(e1) * b1 + xyz(e2) * b2;
    float3 n = safeNormalize(cross(xyz(e1), xyz(e2)));
    float pdf = em.pmfMesh * em.invTotalArea;
    if (!(pdf > 0.0f)) return false;
    float3 tl = pos - p;
    float d2 = dot(tl, tl);
    if (d2 <= 0.0f) return false;
    float invD = rsqrtf(d2);
    ls.wi = tl * invD;
    float cosL = fabsf(dot(ls.wi, n));
    if (cosL <= 0.0f) return false;
    ls.pdfSA = pdf * d2 / cosL;
    if (ls.pdfSA <= 0.0f) return false;
    ls.shadowDist = d2 * invD - kShadowDistanceOffset;
    if (ls.shadowDist <= 0.0f) return false;
    ls.emission = make_float3(em.emission[0], em.emission[1], em.emission[2]);
    ls.emissiveMesh = mi;
    return true;
}

// environment lookup (light/environment.slang:9-27)
VKRT_DEV void envUV(float3 d, float rotDeg, float& u, float& v) {
    float3 n = normalize(d);
    float phi = atan2f(n.y, n.x) + rotDeg * (kPi / 180.0f);
    float theta = acosf(fminf(fmaxf(n.z, -1.0f), 1.0f));
    u = fracf(phi * (0.5f * kInvPi) + 0.5f);
    v = theta * kInvPi;
}

VKRT_DEV float3 envRadiance(const DeviceScene& sc, const VKRT_CudaSceneData& sd, float3 d) {
    uint32_t ti = sd.environmentTextureIndex;
    if (ti >= VKRT_CUDA_MAX_TEXTURES) return make_float3(sd.environmentLight[0], sd.environmentLight[1], sd.environmentLight[2]);
    TextureDesc t = sc.textures[ti];
    if (!t.texels) return make_float3(sd.environmentLight[0], sd.environmentLight[1], sd.environmentLight[2]);
    float u, v;
    envUV(d, sd.environmentRotation, u, v);
    return xyz(sampleBilinear(t, u, v, VKRT_CUDA_TEXTURE_WRAP_REPEAT, VKRT_CUDA_TEXTURE_WRAP_CLAMP_TO_EDGE)) *
           sd.environmentLight[3];
}

// solid-angle pdf of the environment importance distribution
VKRT_DEV float envPdf(const EnvDistribution& e, float3 d, float rotDeg) {
    float u, v;
    envUV(d, rotDeg, u, v);
    uint32_t i = min(uint32_t(u * float(e.width)), e.width - 1u);
    uint32_t j = min(uint32_t(v * float(e.height)), e.height - 1u);
    float st = sinf(v * kPi);
    if (st <= 0.0f) return 0.0f;
    return __ldg(e.texelPdf + size_t(j) * e.width + i) / (2.0f * kPi * kPi * st);
}

// Largest index in [0, n) whose CDF entry is <= u (0 when none), searched within [lo, hi)
VKRT_DEV uint32_t cdfFindRange(const float* cdf, uint32_t lo, uint32_t hi, float u) {
    while (hi - lo > 1u) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) <= u) lo = mid;
        else hi = mid;
    }
    return lo;
}

VKRT_DEV uint32_t cdfFind(const float* cdf, uint32_t n, float u) { return cdfFindRange(cdf, 0u, n, u); }

// Same answer through a guide table: the result for u lies between the guide entries of u's bucket
VKRT_DEV uint32_t cdfFindGuided(const float* cdf, uint32_t n, const uint32_t* guide, float u) {
    if (!guide || !(u >= 0.0f) || !(u < 1.0f)) return cdfFind(cdf, n, u);
    uint32_t k = min(uint32_t(u * float(kEnvGuide)), kEnvGuide - 1u);
    return cdfFindRange(cdf, __ldg(guide + k), min(__ldg(guide + k + 1u) + 1u, n), u);
}

VKRT_DEV bool envSample(const EnvDistribution& e, float u1, float u2, float rotDeg, float3& dir, float& pdf) {
    uint32_t j = cdfFindGuided(e.marginal, e.height, e.marginalGuide, u1);
    float m0 = __ldg(e.marginal + j), m1 = __ldg(e.marginal + j + 1);
    float dv = (u1 - m0) / fmaxf(m1 - m0, 1e-20f);
    const float* c = e.conditional + size_t(j) * (e.width + 1);
    uint32_t i = cdfFindGuided(c, e.width,
                               e.conditionalGuide ? e.conditionalGuide + size_t(j) * (kEnvGuide + 1u) : nullptr, u2);
    float c0 = __ldg(c + i), c1 = __ldg(c + i + 1);
    float du = (u2 - c0) / fmaxf(c1 - c0, 1e-20f);
    float u = (float(i) + sat(du)) / float(e.width);
    float v = (float(j) + sat(dv)) / float(e.height);
    float theta = v * kPi;
    float phi = (u - 0.5f) * 2.0f * kPi - rotDeg * (kPi / 180.0f);
    float st = sinf(theta);
    if (st <= 0.0f) return false;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    dir = make_float3(st * cp, st * sp, cosf(theta));
    pdf = __ldg(e.texelPdf + size_t(j) * e.width + i) / (2.0f * kPi * kPi * st);
    return pdf > 0.0f;
}

}  // namespace vkrt
