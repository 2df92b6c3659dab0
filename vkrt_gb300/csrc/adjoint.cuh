// adjoint.cuh — device pieces of the path-replay adjoint shared by the per-path kernel (adjoint.cu) and the
// wavefront adjoint pass (wavefront.cu): analytic derivatives of the RGB Principled subset, the vertex hook that
// records each radiance term's gradient factors, and the scatter of a vertex's gradient to texels and materials.
//
// Per vertex the gradient of the path contribution is
//   * emission term    d/dLe of thr * w * Le
//   * NEE terms        d/dtheta of thr * f(wl) * |cos| * Le * mis / pdf, for visible requests
//   * continuation     (L - radiance gathered through this vertex) * (df/dtheta) / f, the path-replay identity for
//                      the throughput factor f * |cos| / pdf with the sampling density held fixed.
// BSDF derivatives follow bsdf/principled/eval_rgb.slang:4-121 restricted to metal + dielectric + Lambert: GGX D and
// Smith G through alpha = max(roughness^2, 1e-3) (bsdf/lobes/ggx.slang:16-30), the dielectric directional-albedo
// attenuation of the Lambert lobe (principled/attenuation.slang:30-51), Schlick F0 of non-conducting metals, and the
// Lambert base colour.
#pragma once

#include "adjoint.h"
#include "path.cuh"

namespace vkrt {

constexpr uint32_t kSmemMaterials = 512;  // per-block material-gradient accumulators in shared memory (16 KB)

// ---------------------------------------------------------------------------------------------------------------
// analytic BSDF derivatives
// ---------------------------------------------------------------------------------------------------------------
VKRT_DEV bool interior(float x) { return x > 0.0f && x < 1.0f; }  // d sat(x) / dx = 1

// d(dielDirAtten)/d(roughness), same branches as dielDirAtten
VKRT_DEV float3 dielDirAttenDRoughness(float roughness, float3 f0, float cosT) {
    if (fabsf(cosT) <= 0.0f) return f3(0.0f);
    float rr = sat(roughness), ct = sat(fabsf(cosT));
    float drr = interior(roughness) ? 1.0f : 0.0f;
    float r0 = rr * -1.0f + 1.0f, r1 = rr * -0.0275f + 0.0425f, r2 = rr * -0.572f + 1.04f, r3 = rr * 0.022f - 0.04f;
    float e = exp2f(-9.28f * ct), r02 = r0 * r0;
    float mn = fminf(r02, e);
    float dmn = r02 < e ? -2.0f * r0 * drr : 0.0f;
    float a004 = mn * r0 + r1;
    float da = dmn * r0 - mn * drr - 0.0275f * drr;
    float Araw = -1.04f * a004 + r2, Braw = 1.04f * a004 + r3;
    float A = sat(Araw), B = sat(Braw);
    float dA = interior(Araw) ? -1.04f * da - 0.572f * drr : 0.0f;
    float dB = interior(Braw) ? 1.04f * da + 0.022f * drr : 0.0f;
    float f[3] = {f0.x, f0.y, f0.z}, out[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float inner = f[c] * A + B;
        float dInner = interior(inner) ? f[c] * dA + dB : 0.0f;
        out[c] = interior(1.0f - sat(inner)) ? -dInner : 0.0f;
    }
    return make_float3(out[0], out[1], out[2]);
}

VKRT_DEV float ggxLambdaD(float3 w, const Ggx& g, float dax, float day) {
    float z2 = fmaxf(w.z * w.z, kGgxEps);
    float slope2 = (g.ax * g.ax * w.x * w.x + g.ay * g.ay * w.y * w.y) / z2;
    float dSlope2 = (2.0f * g.ax * dax * w.x * w.x + 2.0f * g.ay * day * w.y * w.y) / z2;
    return 0.25f * dSlope2 / sqrtf(1.0f + slope2);
}

// df/d(baseColor) (diagonal) and df/d(roughness) of evalRgb at wi
VKRT_DEV void evalRgbGrad(const Bsdf& s, float3 wi, float3& dBase, float3& dRough) {
    dBase = f3(0.0f);
    dRough = f3(0.0f);
    if (wi.z <= 0.0f) return;
    const ShadeMaterial& m = s.mat;
    // alpha derivatives (makeGgx)
    float r = fmaxf(m.roughness, kGgxMinAlpha);
    float dr = m.roughness > kGgxMinAlpha ? 1.0f : 0.0f;
    float aspect = sqrtf(fmaxf(1.0f - 0.9f * m.anisotropic, kGgxMinAlpha));
    float a = r * r, da = 2.0f * r * dr;
    float dax = a / aspect > kGgxMinAlpha ? da / aspect : 0.0f;
    float day = a * aspect > kGgxMinAlpha ? da * aspect : 0.0f;

    float3 h = s.wo + wi;
    float h2 = dot(h, h);
    float3 mh = h * rsqrtf(h2);
    float wom = dot(s.wo, mh);
    bool halfOk = h2 > kGgxEps && wom > 0.0f && s.wo.z > 0.0f;
    float DG = 0.0f, dDG = 0.0f;
    if (halfOk && (s.wMetal > 0.0f || s.wDiel > 0.0f)) {
        const Ggx& g = s.ggx;
        float lo = ggxLambda(s.wo, g), li = ggxLambda(wi, g);
        float G = 1.0f / (1.0f + lo + li);
        float dG = -G * G * (ggxLambdaD(s.wo, g, dax, day) + ggxLambdaD(wi, g, dax, day));
        float D = ggxD(mh, g), dD = 0.0f;
        if (mh.z > 0.0f) {
            float c = (mh.x * mh.x) / (g.ax * g.ax) + (mh.y * mh.y) / (g.ay * g.ay) + mh.z * mh.z;
            float dcx = -2.0f * mh.x * mh.x / (g.ax * g.ax * g.ax), dcy = -2.0f * mh.y * mh.y / (g.ay * g.ay * g.ay);
            dD = (-D / g.ax - 2.0f * D / c * dcx) * dax + (-D / g.ay - 2.0f * D / c * dcy) * day;
        }
        float den = fmaxf(4.0f * s.wo.z * wi.z, kGgxEps);
        DG = D * G / den;
        dDG = (dD * G + D * dG) / den;
    }
    if (s.wMetal > 0.0f && halfOk) {
        float3 F = metalFresnel(s, wom);
        dRough += F * (dDG * m.metallic);
        if (!m.conductor) dBase += f3((1.0f - pow5(1.0f - sat(wom))) * DG * m.metallic);
    }
    if (s.wDiel > 0.0f && halfOk && !dielIdentity(m)) dRough += schlick(wom, s.f0Diel) * (dDG * (1.0f - m.metallic));
    if (s.wDiff > 0.0f) {
        float k = (1.0f - m.metallic) * kInvPi;
        float3 sub = m.baseColor * k;
        dBase += s.viewAtten * (k * (1.0f - m.metallic));
        dRough += dielDirAttenDRoughness(m.roughness, s.f0Diel, s.wo.z) * sub * (1.0f - m.metallic);
    }
}

VKRT_DEV float3 ratio(float3 a, float3 b) {
    return make_float3(b.x > 0.0f ? a.x / b.x : 0.0f, b.y > 0.0f ? a.y / b.y : 0.0f, b.z > 0.0f ? a.z / b.z : 0.0f);
}

// ---------------------------------------------------------------------------------------------------------------
// per-vertex record filled by the hook during replay 2
// ---------------------------------------------------------------------------------------------------------------
struct AdjVertex {
    uint32_t materialIndex;
    TexCoords tex;
    bool hasSurface, emitted, sampled;
    bool reqValid[2];
    float3 emitW;         // delta * thr * w
    float3 reqBase[2];    // delta * factor * Le * df/dbase
    float reqRough[2];    // sum delta * factor * Le * df/droughness
    float3 reqEmit[2];    // delta * factor * f
    uint32_t reqLight[2]; // emissive mesh, VKRT_CUDA_INVALID_INDEX for the environment
    float3 ratioBase, ratioRough;
};

struct AdjointHook {
    AdjVertex* v;  // null during the forward pass
    float3 delta;
    VKRT_DEV void surface(const Surface& s, const ShadeMaterial&, const Bsdf&) {
        if (!v) return;
        v->hasSurface = true;
        v->materialIndex = s.materialIndex;
        v->tex = s.tex;
    }
    VKRT_DEV void emission(float3 thrW) {
        if (!v) return;
        v->emitted = true;
        v->emitW = delta * thrW;
    }
    VKRT_DEV void nee(uint32_t r, const Bsdf& b, float3 wl, float3 f, float3 factor, float3 Le, uint32_t light) {
        if (!v || r > 1u) return;
        float3 dB, dR;
        evalRgbGrad(b, wl, dB, dR);
        float3 dl = delta * factor;
        v->reqValid[r] = true;
        v->reqBase[r] = dl * Le * dB;
        v->reqRough[r] = dot(dl * Le, dR);
        v->reqEmit[r] = dl * f;
        v->reqLight[r] = light;
    }
    VKRT_DEV void neeEmissive(uint32_t r, const Bsdf& b, float3 wl, float3 f, float3 factor, float3 Le, uint32_t mesh) {
        nee(r, b, wl, f, factor, Le, mesh);
    }
    VKRT_DEV void neeEnvironment(uint32_t r, const Bsdf& b, float3 wl, float3 f, float3 factor, float3 Le) {
        nee(r, b, wl, f, factor, Le, VKRT_CUDA_INVALID_INDEX);
    }
    VKRT_DEV void cacheQuery(const Surface&, const ShadeMaterial&) {}
    VKRT_DEV void bsdfSample(const Bsdf& b, float3 wl, float3 f) {
        if (!v) return;
        float3 dB, dR;
        evalRgbGrad(b, wl, dB, dR);
        v->sampled = true;
        v->ratioBase = ratio(dB, f);
        v->ratioRough = ratio(dR, f);
    }
};

// ---------------------------------------------------------------------------------------------------------------
// scatter to texels and materials
// ---------------------------------------------------------------------------------------------------------------
struct TexFootprint {
    const float4* texels;
    uint32_t index[4];
    float weight[4];
};

// Texels and weights sampleMaterialTexture blends for this lookup; false when the slot is unbound.
VKRT_DEV bool materialTextureFootprint(const DeviceScene& sc, uint32_t idx, uint32_t wrap, const float* xf, float rot,
                                       uint32_t set, const TexCoords& tc, TexFootprint& fp) {
    if (idx >= VKRT_CUDA_MAX_TEXTURES) return false;
    TextureDesc t = sc.textures[idx];
    if (!t.texels) return false;
    float2 uv = set == 1u ? tc.uv1 : tc.uv0;
    float sx = uv.x * xf[0], sy = uv.y * xf[1];
    float sn, cs;
    sincosf(rot, &sn, &cs);
    float u = cs * sx - sn * sy + xf[2], v = sn * sx + cs * sy + xf[3];
    uint32_t wu = wrapMode(wrap & 0xffffu), wv = wrapMode((wrap >> 16) & 0xffffu);
    float x = u * float(t.width) - 0.5f, y = v * float(t.height) - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    int x0 = int(fx), y0 = int(fy);
    float ax = x - fx, ay = y - fy;
    int xa = wrapIndex(x0, int(t.width), wu), xb = wrapIndex(x0 + 1, int(t.width), wu);
    int ya = wrapIndex(y0, int(t.height), wv), yb = wrapIndex(y0 + 1, int(t.height), wv);
    fp.texels = t.texels;
    fp.index[0] = uint32_t(ya) * t.width + uint32_t(xa);
    fp.index[1] = uint32_t(ya) * t.width + uint32_t(xb);
    fp.index[2] = uint32_t(yb) * t.width + uint32_t(xa);
    fp.index[3] = uint32_t(yb) * t.width + uint32_t(xb);
    fp.weight[0] = (1.0f - ax) * (1.0f - ay);
    fp.weight[1] = ax * (1.0f - ay);
    fp.weight[2] = (1.0f - ax) * ay;
    fp.weight[3] = ax * ay;
    return true;
}

VKRT_DEV float4 footprintValue(const TexFootprint& fp) {
    float4 c = f4(0.0f);
#pragma unroll
    for (int k = 0; k < 4; ++k) c += __ldg(fp.texels + fp.index[k]) * fp.weight[k];
    return c;
}

// Material gradients go to per-block shared-memory accumulators when the material table fits, else to global memory.
VKRT_DEV MaterialGradient* materialSlot(const AdjointParams& ap, MaterialGradient* smemMat, uint32_t material) {
    return smemMat ? smemMat + material : ap.materialGrad + material;
}

VKRT_DEV void addEmissionGrad(const AdjointParams& ap, MaterialGradient* smemMat, uint32_t material, float3 g) {
    MaterialGradient* mg = materialSlot(ap, smemMat, material);
    atomicAdd(&mg->emission.x, g.x);
    atomicAdd(&mg->emission.y, g.y);
    atomicAdd(&mg->emission.z, g.z);
}

// dLoss/d(shaded baseColor) = gBase and dLoss/d(shaded roughness) = gRough at one vertex, pushed back through
// shadeVertex's texturing to the material constants and the texels
VKRT_DEV void scatterSurface(const DeviceScene& sc, const AdjointParams& ap, MaterialGradient* smemMat,
                             const AdjVertex& av, float3 gBase, float gRough) {
    const VKRT_CudaMaterial& m = sc.materials[av.materialIndex];
    MaterialGradient* mg = materialSlot(ap, smemMat, av.materialIndex);
    if (ap.wantBase && (gBase.x != 0.0f || gBase.y != 0.0f || gBase.z != 0.0f)) {
        float3 vcol = xyz(av.tex.color);
        TexFootprint fp;
        bool tex = materialTextureFootprint(sc, m.baseColorTextureIndex, m.baseColorTextureWrap,
                                            m.baseColorTextureTransform, m.textureRotations[0],
                                            m.textureTexcoordSets & 0xffu, av.tex, fp);
        float3 tv = tex ? xyz(footprintValue(fp)) : f3(1.0f);
        float3 gm = gBase * tv * vcol;
        atomicAdd(&mg->base.x, gm.x);
        atomicAdd(&mg->base.y, gm.y);
        atomicAdd(&mg->base.z, gm.z);
        float4* tg = tex ? ap.textureGrad[m.baseColorTextureIndex] : nullptr;
        if (tg) {
            float3 gt = gBase * make_float3(m.baseColor[0], m.baseColor[1], m.baseColor[2]) * vcol;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float w = fp.weight[k];
                if (w == 0.0f) continue;
                float4* d = tg + fp.index[k];
                atomicAdd(&d->x, gt.x * w);
                atomicAdd(&d->y, gt.y * w);
                atomicAdd(&d->z, gt.z * w);
            }
        }
    }
    if (ap.wantRoughness && gRough != 0.0f) {
        TexFootprint fp;
        bool tex = m.metallicRoughnessTextureIndex != VKRT_CUDA_INVALID_INDEX &&
                   materialTextureFootprint(sc, m.metallicRoughnessTextureIndex, m.metallicRoughnessTextureWrap,
                                            m.metallicRoughnessTextureTransform, m.textureRotations[1],
                                            (m.textureTexcoordSets >> 8) & 0xffu, av.tex, fp);
        float mr = tex ? footprintValue(fp).y : 1.0f;
        if (interior(m.roughness * mr)) {  // shaded roughness = sat(roughness * texel.g)
            atomicAdd(&mg->base.w, gRough * mr);
            float4* tg = tex ? ap.textureGrad[m.metallicRoughnessTextureIndex] : nullptr;
            if (tg) {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (fp.weight[k] != 0.0f) atomicAdd(&tg[fp.index[k]].y, gRough * m.roughness * fp.weight[k]);
            }
        }
    }
}

VKRT_DEV void scatterHitEmission(const DeviceScene& sc, const AdjointParams& ap, MaterialGradient* smemMat,
                                  const AdjVertex& av) {
    const VKRT_CudaMaterial& m = sc.materials[av.materialIndex];
    float3 g = av.emitW;
    if (m.emissiveTextureIndex != VKRT_CUDA_INVALID_INDEX) {
        float4 em = sampleMaterialTexture(sc, m.emissiveTextureIndex, m.emissiveTextureWrap, m.emissiveTextureTransform,
                                          m.textureRotations[3], (m.textureTexcoordSets >> 24) & 0xffu, av.tex,
                                          f4(1.0f));
        g = g * xyz(em);
    }
    addEmissionGrad(ap, smemMat, av.materialIndex, g);
}


constexpr uint32_t kAdjFlagSurface = 1u, kAdjFlagContinued = 2u, kAdjFlagReq0 = 4u, kAdjFlagReq1 = 8u;

// Completes one vertex once its shadow requests' visibility is known: radiance is the path radiance through this
// vertex (its visible requests included), `continued` whether the path went on from it.
VKRT_DEV void finishVertex(const DeviceScene& sc, const AdjointParams& ap, MaterialGradient* smemMat,
                           const AdjVertex& av, const bool vis[2], bool continued, float3 delta, float3 total,
                           float3 radiance) {
    float3 gBase = f3(0.0f);
    float gRough = 0.0f;
    for (uint32_t i = 0; i < 2u; ++i) {
        if (!vis[i] || !av.reqValid[i]) continue;
        gBase += av.reqBase[i];
        gRough += av.reqRough[i];
        if (ap.wantEmission && av.reqLight[i] != VKRT_CUDA_INVALID_INDEX)
            addEmissionGrad(ap, smemMat, ap.emissiveMeshMaterial[av.reqLight[i]], av.reqEmit[i]);
    }
    if (continued && av.sampled) {
        float3 dl = delta * (total - radiance);  // radiance the continuation carries
        gBase += dl * av.ratioBase;
        gRough += dot(dl, av.ratioRough);
    }
    scatterSurface(sc, ap, smemMat, av, gBase, gRough);
}

VKRT_DEV void clearMaterialSmem(MaterialGradient* smemMat, uint32_t count) {
    if (!smemMat) return;
    for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
        smemMat[i].base = f4(0.0f);
        smemMat[i].emission = f4(0.0f);
    }
}

// adds a block's shared-memory material gradients to the global buffer (after a __syncthreads)
VKRT_DEV void flushMaterialSmem(const AdjointParams& ap, const MaterialGradient* smemMat, uint32_t count) {
    if (!smemMat) return;
    for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
        const MaterialGradient& g = smemMat[i];
        MaterialGradient* d = ap.materialGrad + i;
        if (g.base.x != 0.0f) atomicAdd(&d->base.x, g.base.x);
        if (g.base.y != 0.0f) atomicAdd(&d->base.y, g.base.y);
        if (g.base.z != 0.0f) atomicAdd(&d->base.z, g.base.z);
        if (g.base.w != 0.0f) atomicAdd(&d->base.w, g.base.w);
        if (g.emission.x != 0.0f) atomicAdd(&d->emission.x, g.emission.x);
        if (g.emission.y != 0.0f) atomicAdd(&d->emission.y, g.emission.y);
        if (g.emission.z != 0.0f) atomicAdd(&d->emission.z, g.emission.z);
    }
}

}  // namespace vkrt
