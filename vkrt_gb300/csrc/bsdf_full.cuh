// bsdf_full.cuh — vkrt's layered Principled BSDF with its transmissive interface, for the full instantiations of the
// integrators (scenes whose materials use clearcoat, Oren-Nayar, fake subsurface or transmission):
//   * branch weights of principled/weights.slang:27-62, with the transmission weight and the interior rule (a
//     transmissive material seen from the back keeps only its metal and dielectric interface lobes);
//   * the scalar stack of principled/eval_rgb.slang:4-141 in RGB and in the single-wavelength form a collapsed
//     spectral path evaluates, and the four-lane hero stack of principled/eval_spectral.slang:4-117 with one
//     technique pdf per lane (lanes differ at dispersive interfaces);
//   * the rough dielectric BTDF of lobes/dielectric/** (Walter et al. 2007) with Abbe-number dispersion
//     (utility/spectral.slang:124-136) and the Fresnel choice between reflection and refraction;
//   * sampleBSDFDirection (principled/sample.slang:4-51) reporting whether the sample refracted.
//   * the microfiber sheen lobe on top, through the LTC table the host installs.
// The reflection-only instantiations keep the smaller Bsdf of shading.cuh.
#pragma once

#include "shading.cuh"

namespace vkrt {

struct BsdfFull : Bsdf {
    bool interior;   // useInteriorDielectricInterface (attenuation.slang:4-6)
    float transAtt;  // attenuation of the layers above the interface on the transmission lobe
    // sheen: branch weight, LTC transform and albedo at wo, colour (zero without a table)
    float wSheen, sheenA, sheenB, sheenAlb;
    float3 sheenColor;
    const float* sheenLtc;
};

// Microfiber sheen through its LTC fit (lobes/sheen.slang, Zeltner, Burley and Chiang 2022): three 32 x 32 layers
// over (cos theta_o, roughness), looked up bilinearly (:23-39); the lobe is a linearly transformed cosine in the
// frame whose tangent is wo's projection (:41-85).
VKRT_DEV float sheenLookup(const float* T, float cosT, float rough, uint32_t layer) {
    const float ux = sat(cosT) * 31.0f, uy = sat(rough) * 31.0f;
    const uint32_t x0 = min(uint32_t(ux), 31u), y0 = min(uint32_t(uy), 31u);
    const uint32_t x1 = min(x0 + 1u, 31u), y1 = min(y0 + 1u, 31u);
    const float tx = ux - floorf(ux), ty = uy - floorf(uy);
    const float* L = T + layer * 1024u;
    const float e00 = __ldg(L + y0 * 32u + x0), e10 = __ldg(L + y0 * 32u + x1);
    const float e01 = __ldg(L + y1 * 32u + x0), e11 = __ldg(L + y1 * 32u + x1);
    const float a = e00 * (1.0f - tx) + e10 * tx, b = e01 * (1.0f - tx) + e11 * tx;
    return a * (1.0f - ty) + b * ty;
}
VKRT_DEV float sheenAlbedo(const float* T, float cosT, float rough) {  // sheenDirectionalAlbedo (:87-89)
    return T ? sheenLookup(T, cosT, fminf(fmaxf(rough, 1e-3f), 1.0f), 2u) : 0.0f;
}
VKRT_DEV float sheenAtten(const float* T, float weight, float cosT, float rough) {  // sheenLayerAttenuation (:91-93)
    return sat(1.0f - weight * sheenAlbedo(T, cosT, rough));
}
VKRT_DEV Basis sheenBasis(float3 wo) { return makeBasis(make_float3(0.0f, 0.0f, 1.0f), make_float4(wo.x, wo.y, wo.z, 1.0f)); }
// evalSheen (:95-111) for a unit colour: value albedo * D, pdf D
VKRT_DEV float evalSheenUnit(const BsdfFull& s, float3 wi, float& pdf) {
    pdf = 0.0f;
    if (s.wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
    const float3 lw = toLocal(wi, sheenBasis(s.wo));
    const float z = fmaxf(lw.z, 0.0f);
    if (z <= 0.0f || fabsf(s.sheenA) < 1e-5f || s.sheenAlb < 1e-5f) return 0.0f;
    const float axbz = s.sheenA * lw.x + s.sheenB * lw.z;
    const float len2 = axbz * axbz + (s.sheenA * lw.y) * (s.sheenA * lw.y) + lw.z * lw.z;
    if (len2 <= 1e-6f) return 0.0f;
    const float scale = s.sheenA / len2;
    pdf = kInvPi * z * scale * scale;
    return s.sheenAlb * pdf;
}

VKRT_DEV float dispersiveIor(float ior, float abbe, float lambdaNm) {  // utility/spectral.slang:124-136
    if (ior <= 1.0f + 1e-4f || abbe <= 0.0f) return fmaxf(ior, 1.0f);
    const float cUm = 0.6562725f, dUm = 0.5875618f, fUm = 0.4861327f;  // Fraunhofer C, D, F lines
    float lUm = fmaxf(lambdaNm * 0.001f, 1e-4f);
    float dn = (ior - 1.0f) / fmaxf(abbe, 1e-6f);
    float B = dn / (1.0f / (fUm * fUm) - 1.0f / (cUm * cUm));
    float A = ior - B / (dUm * dUm);
    return fmaxf(A + B / (lUm * lUm), 1.0f);
}
// bsdf/base/interface.slang:4-32 (dispersive in the spectral modes)
VKRT_DEV float interfaceIor(const ShadeMaterial& m, float lambdaNm, bool spectral) {
    float ior = fmaxf(m.ior, 1.0f);
    return spectral ? dispersiveIor(ior, m.abbe, lambdaNm) : ior;
}
VKRT_DEV float interfaceEta(const ShadeMaterial& m, uint32_t front, float lambdaNm, bool spectral) {
    float ior = interfaceIor(m, lambdaNm, spectral);
    return front ? ior : 1.0f / ior;
}
VKRT_DEV float refractionEta(const ShadeMaterial& m, uint32_t front, float lambdaNm, bool spectral) {
    float ior = interfaceIor(m, lambdaNm, spectral);
    return front ? 1.0f / ior : ior;
}
VKRT_DEV float3 transmissionColor(const ShadeMaterial& m) {  // material.slang:75-77
    return m.transmission > 0.0f && m.metallic <= 0.0f ? f3(1.0f) : m.baseColor;
}
VKRT_DEV float transmissionProbability(const ShadeMaterial& m, float F) {  // dielectric/interface.slang:68-72
    float tw = m.transmission * (1.0f - F), tot = F + tw;
    return tot <= 0.0f ? 0.0f : tw / tot;
}
VKRT_DEV bool mediumIsRefractive(const ShadeMaterial& m) {  // base/medium.slang:40-42
    return m.transmission > 0.0f && fmaxf(m.ior, 1.0f) > 1.0f + 1e-4f;
}
VKRT_DEV bool hasAbsorption(const ShadeMaterial& m) {  // base/medium.slang:36-38
    return m.absorption > 0.0f &&
           (m.attenuationColor.x < 0.9999f || m.attenuationColor.y < 0.9999f || m.attenuationColor.z < 0.9999f);
}
VKRT_DEV float3 refractDir(float3 i, float3 n, float eta) {  // HLSL refract: zero on total internal reflection
    float c = dot(n, i);
    float k = 1.0f - eta * eta * (1.0f - c * c);
    if (k < 0.0f) return f3(0.0f);
    return i * eta - n * (eta * c + sqrtf(k));
}

VKRT_DEV BsdfFull makeBsdfFull(const ShadeMaterial& m, float3 wo, uint32_t frontFace, const float* sheenLtc) {
    BsdfFull s;
    s.mat = m;
    s.wo = wo;
    s.frontFace = frontFace;
    s.sheenLtc = sheenLtc;
    s.sheenColor = sheenLtc ? m.sheenColor : f3(0.0f);
    s.sheenA = s.sheenB = s.sheenAlb = 0.0f;
    if (sheenLtc && wo.z > 0.0f) {  // makeSheenParams (sheen.slang:41-57)
        const float r = fminf(fmaxf(m.sheenRoughness, 1e-3f), 1.0f);
        s.sheenA = sheenLookup(sheenLtc, wo.z, r, 0u);
        s.sheenB = sheenLookup(sheenLtc, wo.z, r, 1u);
        s.sheenAlb = sheenLookup(sheenLtc, wo.z, r, 2u);
    }
    s.ggx = makeGgx(m, wo);
    s.f0Diel = dielSpecF0(m);
    s.viewAtten = dielDirAtten(m.roughness, s.f0Diel, wo.z);
    s.coatA = coatAlpha(m);
    s.interior = m.transmission > 0.0f && frontFace == 0u;
    const float nonMetal = 1.0f - m.metallic;
    const float baseW = fmaxf(lum(m.baseColor), 1e-3f);
    const float diffW = fmaxf(lum(m.baseColor * nonMetal), 1e-3f);
    const float baseScatter = nonMetal * (1.0f - m.transmission);
    const float transW = m.transmission * fmaxf(lum(transmissionColor(m)), 1e-3f);
    const float dielW = nonMetal * fmaxf(sat(lum(s.f0Diel)) + transW, 0.0f);
    float wsh = 0.0f, wc = 0.0f, wm, wd, wf = 0.0f, ws = 0.0f;
    if (s.interior) {
        s.viewCoat = 1.0f;
        s.transAtt = 1.0f;
        wm = m.metallic * baseW;
        wd = dielW;
    } else {
        s.viewCoat = coatAtten(m, wo);
        const float viewSheen = sheenAtten(sheenLtc, maxc(s.sheenColor), wo.z, m.sheenRoughness);
        s.transAtt = viewSheen * s.viewCoat;  // materialTransmissionStackAttenuation
        const float dielAtt = lum(s.viewAtten);
        wsh = lum(s.sheenColor);
        wc = viewSheen * m.clearcoat * 0.25f;
        wm = viewSheen * s.viewCoat * m.metallic * baseW;
        wd = viewSheen * s.viewCoat * dielW;
        wf = viewSheen * s.viewCoat * dielAtt * baseScatter * (1.0f - m.subsurface) * diffW;
        ws = viewSheen * s.viewCoat * dielAtt * baseScatter * m.subsurface * diffW;
    }
    const float tot = wsh + wc + wm + wd + wf + ws;
    if (tot <= 0.0f) {
        s.wSheen = s.wCoat = s.wMetal = s.wDiel = s.wSub = 0.0f;
        s.wDiff = 1.0f;
    } else {
        s.wSheen = wsh / tot;
        s.wCoat = wc / tot;
        s.wMetal = wm / tot;
        s.wDiel = wd / tot;
        s.wDiff = wf / tot;
        s.wSub = ws / tot;
    }
    return s;
}

// One transmission lane (dielectric/eval_rgb.slang:40-95, eval_spectral.slang:45-97); `color` is the lane's
// transmission colour
VKRT_DEV float transmissionLane(const BsdfFull& s, float3 wi, float color, float lambdaNm, bool spectral, float& pdf) {
    pdf = 0.0f;
    if (s.mat.transmission <= 0.0f || s.wo.z <= 0.0f || wi.z >= 0.0f) return 0.0f;
    if (dielIdentity(s.mat)) {
        if (dot(wi, -s.wo) < 0.9999f) return 0.0f;
        pdf = 1.0f;
        return s.transAtt * color / fmaxf(fabsf(wi.z), kGgxEps);
    }
    const float etap = interfaceEta(s.mat, s.frontFace, lambdaNm, spectral);
    const float3 h = s.wo + wi * etap;
    if (dot(h, h) <= kGgxEps) return 0.0f;
    float3 wm = safeNormalize(h);
    if (wm.z < 0.0f) wm = -wm;
    const float woM = dot(s.wo, wm), wiM = dot(wi, wm);
    const float denom = wiM + woM / etap;
    if (!(woM > 0.0f && wiM < 0.0f && fabsf(denom) > kGgxEps)) return 0.0f;
    const float F = fresnelDielectric(woM, etap);
    const float tprob = transmissionProbability(s.mat, F);
    if (tprob <= 0.0f) return 0.0f;
    const float D = ggxD(wm, s.ggx);
    const float G = 1.0f / (1.0f + ggxLambda(s.wo, s.ggx) + ggxLambda(wi, s.ggx));
    const float d2 = denom * denom;
    const float scale = 1.0f / fmaxf(etap * etap, kGgxEps);
    const float term = fabsf((wiM * woM) / fmaxf(fabsf(wi.z) * s.wo.z * d2, kGgxEps));
    const float dwm = fabsf(wiM) / fmaxf(d2, kGgxEps);
    const float vis = D * (1.0f / (1.0f + ggxLambda(s.wo, s.ggx))) * woM / fmaxf(s.wo.z, kGgxEps);  // ggxVisibleNormalPdf
    pdf = tprob * vis * dwm;
    return s.transAtt * color * ((1.0f - F) * D * G * term * scale);
}

// Reflection lobes shared by the scalar and hero stacks: GGX half vector terms for wi above the surface
struct ReflGeom {
    bool ok;
    float wom, DG, reflPdf;
};
VKRT_DEV ReflGeom reflGeom(const BsdfFull& s, float3 wi) {
    ReflGeom r{false, 0.0f, 0.0f, 0.0f};
    const float3 h = s.wo + wi;
    const float h2 = dot(h, h);
    if (h2 <= kGgxEps || s.wo.z <= 0.0f) return r;
    const float3 m = h * rsqrtf(h2);
    r.wom = dot(s.wo, m);
    if (r.wom <= 0.0f) return r;
    r.ok = true;
    const float G = 1.0f / (1.0f + ggxLambda(s.wo, s.ggx) + ggxLambda(wi, s.ggx));
    r.DG = ggxD(m, s.ggx) * G / fmaxf(4.0f * s.wo.z * wi.z, kGgxEps);
    r.reflPdf = ggxReflPdf(s.wo, m, r.wom, s.ggx);
    return r;
}

// The scalar stack: RGB (kSingle = false), or one wavelength of a collapsed spectral path (kSingle: colours become
// spectral scalars at `lambda`; the dielectric view attenuation stays RGB as in evalScalarReflectionStack, and the
// path reads the first component).
template <bool kSingle>
VKRT_DEV float3 evalScalarFull(const BsdfFull& s, const SpecTable& tab, float3 wi, float lambda, float& pdf) {
    pdf = 0.0f;
    auto spec = [&](float3 c) { return kSingle ? f3(spectral1(tab, sat(c), lambda)) : c; };
    if (wi.z <= 0.0f) {  // evalDielectricTransmission
        const float3 tc = spec(transmissionColor(s.mat) * ((1.0f - s.mat.metallic) * s.mat.transmission));
        float tp;
        float3 v;
        v.x = transmissionLane(s, wi, tc.x, lambda, kSingle, tp);
        v.y = transmissionLane(s, wi, tc.y, lambda, kSingle, tp);
        v.z = transmissionLane(s, wi, tc.z, lambda, kSingle, tp);
        pdf = tp * s.wDiel;
        return v;
    }
    float coat = 0.0f;
    float3 metal = f3(0.0f), diel = f3(0.0f), sub = f3(0.0f), sheenV = f3(0.0f), sc = f3(0.0f);
    if (s.wSheen > 0.0f || !s.interior) sc = spec(s.sheenColor);
    if (s.wSheen > 0.0f) {
        float sp;
        sheenV = sc * evalSheenUnit(s, wi, sp);
        pdf += s.wSheen * sp;
    }
    if (s.wCoat > 0.0f) {
        float cp;
        coat = coatEval(s.mat.clearcoat, s.coatA, s.wo, wi, cp);
        pdf += s.wCoat * cp;
    }
    const ReflGeom g = (s.wMetal > 0.0f || s.wDiel > 0.0f) ? reflGeom(s, wi) : ReflGeom{false, 0.0f, 0.0f, 0.0f};
    if (s.wMetal > 0.0f && g.ok) {
        metal = spec(metalFresnel(s, g.wom)) * g.DG;
        pdf += s.wMetal * g.reflPdf;
    }
    if (s.wDiel > 0.0f && g.ok && !dielIdentity(s.mat)) {
        const float F = fresnelDielectric(g.wom, interfaceEta(s.mat, s.frontFace, lambda, kSingle));
        const float reflP = 1.0f - transmissionProbability(s.mat, F);
        if (reflP > 0.0f) {
            const float3 color = s.mat.transmission > 0.0f && s.mat.metallic <= 0.0f ? f3(F)
                                                                                      : spec(schlick(g.wom, s.f0Diel));
            diel = color * g.DG;
            pdf += s.wDiel * (reflP * g.reflPdf);
        }
    }
    if (s.wDiff > 0.0f || s.wSub > 0.0f) {
        const float3 dc = spec(s.mat.baseColor * (1.0f - s.mat.metallic));
        if (s.wDiff > 0.0f) {
            const float unit = s.mat.diffuseRoughness <= 0.0f ? kInvPi : orenNayar(s.mat.diffuseRoughness, s.wo, wi);
            sub = sub + dc * ((1.0f - s.mat.transmission) * (1.0f - s.mat.subsurface) * unit);
            pdf += s.wDiff * (wi.z * kInvPi);
        }
        if (s.wSub > 0.0f) {
            sub = sub + dc * ((1.0f - s.mat.transmission) * s.mat.subsurface *
                              fakeSss(s.mat.diffuseRoughness, s.wo, wi));
            pdf += s.wSub * (wi.z * kInvPi);
        }
    }
    const float nonMetal = 1.0f - s.mat.metallic;
    if (s.interior) return metal * s.mat.metallic + diel * nonMetal;
    const float att = s.viewCoat * coatAtten(s.mat, wi);
    const float viewSheen = sheenAtten(s.sheenLtc, maxc(sc), s.wo.z, s.mat.sheenRoughness);
    return sheenV + (f3(coat) + (metal * s.mat.metallic + (diel + s.viewAtten * sub) * nonMetal) * att) * viewSheen;
}

// The hero stack's direction-independent upsampled colours (sheen, diffuse base, view attenuation), the same for
// every direction a vertex evaluates; each is computed under the condition evalHeroFull uses it.
struct HeroTerms {
    float4 sheen, diffuse, viewAtten;
};

VKRT_DEV HeroTerms heroTerms(const BsdfFull& s, const SpecTable& tab, float4 l) {
    HeroTerms h{f4(0.0f), f4(0.0f), f4(0.0f)};
    if (s.wSheen > 0.0f || !s.interior) h.sheen = spectral4Call(tab, sat(s.sheenColor), l);
    if (s.wDiff > 0.0f || s.wSub > 0.0f) h.diffuse = spectral4Call(tab, sat(s.mat.baseColor * (1.0f - s.mat.metallic)), l);
    if (!s.interior) h.viewAtten = spectral4Call(tab, sat(s.viewAtten), l);
    return h;
}

// Four hero lanes with one technique pdf per lane in `tp`; `ht` is heroTerms of the same BSDF and wavelengths
VKRT_DEV float4 evalHeroFull(const BsdfFull& s, const SpecTable& tab, float3 wi, float4 l, const HeroTerms& ht,
                             float4& tp) {
    tp = f4(0.0f);
    if (wi.z <= 0.0f) {  // evalSpectralDielectricTransmission
        const float4 tc = spectral4Call(tab, sat(transmissionColor(s.mat)), l) *
                          ((1.0f - s.mat.metallic) * s.mat.transmission);
        float4 v;
        v.x = transmissionLane(s, wi, tc.x, l.x, true, tp.x);
        v.y = transmissionLane(s, wi, tc.y, l.y, true, tp.y);
        v.z = transmissionLane(s, wi, tc.z, l.z, true, tp.z);
        v.w = transmissionLane(s, wi, tc.w, l.w, true, tp.w);
        tp = tp * s.wDiel;
        return v;
    }
    float coat = 0.0f;
    float4 metal = f4(0.0f), diel = f4(0.0f), sub = f4(0.0f), sheenV = f4(0.0f), sc = f4(0.0f);
    if (s.wSheen > 0.0f || !s.interior) sc = ht.sheen;
    if (s.wSheen > 0.0f) {
        float sp;
        sheenV = sc * evalSheenUnit(s, wi, sp);
        tp = tp + f4(s.wSheen * sp);
    }
    if (s.wCoat > 0.0f) {
        float cp;
        coat = coatEval(s.mat.clearcoat, s.coatA, s.wo, wi, cp);
        tp = tp + f4(s.wCoat * cp);
    }
    const ReflGeom g = (s.wMetal > 0.0f || s.wDiel > 0.0f) ? reflGeom(s, wi) : ReflGeom{false, 0.0f, 0.0f, 0.0f};
    if (s.wMetal > 0.0f && g.ok) {
        metal = spectral4Call(tab, sat(metalFresnel(s, g.wom)), l) * g.DG;
        tp = tp + f4(s.wMetal * g.reflPdf);
    }
    if (s.wDiel > 0.0f && g.ok && !dielIdentity(s.mat)) {
        float4 F, lanes;
        F.x = fresnelDielectric(g.wom, interfaceEta(s.mat, s.frontFace, l.x, true));
        F.y = fresnelDielectric(g.wom, interfaceEta(s.mat, s.frontFace, l.y, true));
        F.z = fresnelDielectric(g.wom, interfaceEta(s.mat, s.frontFace, l.z, true));
        F.w = fresnelDielectric(g.wom, interfaceEta(s.mat, s.frontFace, l.w, true));
        lanes.x = (1.0f - transmissionProbability(s.mat, F.x)) * g.reflPdf;
        lanes.y = (1.0f - transmissionProbability(s.mat, F.y)) * g.reflPdf;
        lanes.z = (1.0f - transmissionProbability(s.mat, F.z)) * g.reflPdf;
        lanes.w = (1.0f - transmissionProbability(s.mat, F.w)) * g.reflPdf;
        if (anyPos(lanes)) {
            const float4 color = s.mat.transmission > 0.0f && s.mat.metallic <= 0.0f
                                     ? F
                                     : spectral4Call(tab, sat(schlick(g.wom, s.f0Diel)), l);
            diel = color * g.DG;
            tp = tp + lanes * s.wDiel;
        }
    }
    if (s.wDiff > 0.0f || s.wSub > 0.0f) {
        const float4 dc = ht.diffuse;
        if (s.wDiff > 0.0f) {
            const float unit = s.mat.diffuseRoughness <= 0.0f ? kInvPi : orenNayar(s.mat.diffuseRoughness, s.wo, wi);
            sub = sub + dc * ((1.0f - s.mat.transmission) * (1.0f - s.mat.subsurface) * unit);
            tp = tp + f4(s.wDiff * (wi.z * kInvPi));
        }
        if (s.wSub > 0.0f) {
            sub = sub + dc * ((1.0f - s.mat.transmission) * s.mat.subsurface *
                              fakeSss(s.mat.diffuseRoughness, s.wo, wi));
            tp = tp + f4(s.wSub * (wi.z * kInvPi));
        }
    }
    const float nonMetal = 1.0f - s.mat.metallic;
    if (s.interior) return metal * s.mat.metallic + diel * nonMetal;
    const float4 va = ht.viewAtten;
    const float att = s.viewCoat * coatAtten(s.mat, wi);
    const float alb = sheenAlbedo(s.sheenLtc, s.wo.z, s.mat.sheenRoughness);
    const float4 viewSheen = make_float4(sat(1.0f - sc.x * alb), sat(1.0f - sc.y * alb), sat(1.0f - sc.z * alb),
                                         sat(1.0f - sc.w * alb));
    return sheenV + (f4(coat) + (metal * s.mat.metallic + (diel + va * sub) * nonMetal) * att) * viewSheen;
}

// sampleBSDFDirection with sampleDielectric (dielectric/sample.slang:7-53); the dielectric lobe refracts at the IOR
// of `lambda` when `spectral`
VKRT_DEV bool sampleFull(const BsdfFull& s, Rng& rng, float lambda, bool spectral, float3& wi, bool& isTrans) {
    isTrans = false;
    float sel = rng.next();
    if (sel < s.wSheen) {  // sampleSheen (sheen.slang:113-128)
        if (fabsf(s.sheenA) < 1e-5f || s.sheenAlb < 1e-5f) return false;
        const float r = sqrtf(rng.next());
        float sp, cp;
        sincosf(2.0f * kPi * rng.next(), &sp, &cp);
        const float dx = r * cp, dy = r * sp;
        const float dz = sqrtf(fmaxf(1.0f - (dx * dx + dy * dy), 0.0f));
        const float3 lw = normalize(make_float3(dx - dz * s.sheenB, dy, dz * s.sheenA));
        wi = toWorld(lw, sheenBasis(s.wo));
        return wi.z > 0.0f;
    }
    sel -= s.wSheen;
    if (sel < s.wCoat) {
        float u1 = rng.next(), u2 = rng.next();
        return coatSample(s.wo, s.coatA, u1, u2, wi);
    }
    sel -= s.wCoat;
    const bool metal = sel < s.wMetal;
    if (!metal) sel -= s.wMetal;
    if (metal || sel < s.wDiel) {
        if (!metal) {
            if (s.wo.z <= 0.0f) return false;
            if (dielIdentity(s.mat)) {
                wi = -s.wo;
                isTrans = s.mat.transmission > 0.0f;
                return isTrans;
            }
        }
        float u1 = rng.next(), u2 = rng.next();
        float3 m;
        if (!sampleVndf(s.wo, s.ggx, u1, u2, m)) return false;
        float wom = dot(s.wo, m);
        if (wom <= 0.0f) return false;
        if (!metal) {
            const float F = fresnelDielectric(wom, interfaceEta(s.mat, s.frontFace, lambda, spectral));
            const float tprob = transmissionProbability(s.mat, F);
            if (tprob > 0.0f && rng.next() < tprob) {
                const float3 t = refractDir(-s.wo, m, refractionEta(s.mat, s.frontFace, lambda, spectral));
                if (dot(t, t) > 0.0f && t.z < 0.0f) {
                    wi = t;
                    isTrans = true;
                    return true;
                }
            }
        }
        wi = m * (2.0f * wom) - s.wo;
        return wi.z > 0.0f;
    }
    float u1 = rng.next(), u2 = rng.next();
    float r = sqrtf(u1), sp, cp;
    sincosf(2.0f * kPi * u2, &sp, &cp);
    wi = make_float3(r * cp, r * sp, sqrtf(fmaxf(0.0f, 1.0f - u1)));
    return true;
}

}  // namespace vkrt
