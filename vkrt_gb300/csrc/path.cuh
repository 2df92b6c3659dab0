// path.cuh — one path vertex of vkrt's integrators as a resumable step, shared by the megakernel and the wavefront
// integrator so both compute exactly the same arithmetic.
//
// RGB:  integrator/path/rgb/integrator.slang:15-113 with rgb/transport.slang and light/direct/rgb_lighting.slang.
// Hero: integrator/path/spectral_hero/integrator.slang:16-172 with spectral_hero/transport.slang and
//       light/direct/spectral_lighting.slang. In the reflection-only material subset every hero lane shares one
//       technique pdf per vertex, so the four technique path pdfs stay equal and are tracked as one scalar.
//
// A step consumes the closest hit of the current ray and produces: radiance added to the path (emission, environment
// on a miss), up to two occlusion requests (emissive-triangle NEE, environment NEE) whose contributions already
// carry the path throughput and count once the shadow ray reports visible, and either the next ray or termination.
// Contributions are added to the path radiance in a fixed order (vertex emission, then the emissive NEE request,
// then the environment NEE request), so the result does not depend on when the shadow rays are traced.
#pragma once

#include "integrator.cuh"

namespace vkrt {

constexpr uint32_t kPathPrevNee = 1u;  // the previous vertex sampled NEE (loop.slang:69-71)
constexpr uint32_t kPathDone = 2u;
constexpr uint32_t kPathFeatureDone = 4u;  // the sample's denoiser feature was taken at an earlier vertex

struct PathState {
    Rng rng;
    float3 o, d;
    float4 thr;       // RGB throughput in xyz, or the four hero-lane throughputs
    float4 radiance;  // RGB radiance in xyz, or the four hero-lane spectral radiances
    float lamUnit;    // hero wavelength unit sample; lane i at 360 + frac(lamUnit + i/4) * 470
    float techPath, prevVertexTech, prevBsdfTech;  // hero MIS (shared by the four lanes)
    float prevBsdfPdf;                             // RGB MIS
    uint32_t depth;
    uint32_t flags;
};

struct ShadowRequest {
    float3 origin;
    float3 dir;
    float tmax;
    float4 contribution;  // to be added to the path radiance when the ray is unoccluded
};

struct StepConfig {
    bool spectral;
    bool neeEnabled;  // misNeeEnabled && emissiveMeshCount > 0 (integrator/path/state.slang:50-52)
    bool envNee;      // environment importance sampling active
    uint32_t rngMode;
    uint64_t rngSeed;
    uint32_t cacheDepth = 0xFFFFFFFFu;  // surface vertex depth at which the path queries the radiance cache and ends
};

VKRT_DEV float4 heroLambdas(float unit) {
    return make_float4(kLambdaMin + fracf(unit) * kLambdaRange, kLambdaMin + fracf(unit + 0.25f) * kLambdaRange,
                       kLambdaMin + fracf(unit + 0.5f) * kLambdaRange, kLambdaMin + fracf(unit + 0.75f) * kLambdaRange);
}

// Camera ray and per-sample state (integrator/path/state.slang:140-146,190-195).
template <bool kSpectral>
VKRT_DEV PathState beginPath(const StepConfig& cfg, const VKRT_CudaSceneData& sd, int px, int py,
                             uint32_t sampleIndex) {
    PathState p;
    p.rng = makeRng(cfg.rngMode, cfg.rngSeed, px, py, sd.frameNumber, sampleIndex);
    float jx = p.rng.next() - 0.5f;
    float jy = p.rng.next() - 0.5f;
    p.d = primaryRay(sd, px, py, jx, jy, p.o);
    p.thr = f4(1.0f);
    p.radiance = f4(0.0f);
    p.lamUnit = 0.0f;
    if (kSpectral) {  // sampleHeroWavelengths4 (sampling/wavelength.slang:29-47)
        float radInv = float(reverseBits32(sampleIndex)) * (1.0f / 4294967296.0f);
        p.lamUnit = fracf(radInv + p.rng.next());
    }
    p.techPath = 1.0f;
    p.prevVertexTech = 0.0f;
    p.prevBsdfTech = 0.0f;
    p.prevBsdfPdf = 0.0f;
    p.depth = 0;
    p.flags = 0;
    return p;
}

// Sample value of a finished path: linear sRGB, or CIE XYZ in spectral mode (spectral.slang:104-113).
template <bool kSpectral>
VKRT_DEV float3 pathResult(const StepConfig& cfg, const PathState& p) {
    if (!kSpectral) return xyz(p.radiance);
    return spectral4ToXYZ(p.radiance, heroLambdas(p.lamUnit), kLambdaRange);
}

VKRT_DEV float3 thr3(const PathState& p) { return xyz(p.thr); }

// Observer of the RGB vertex arithmetic, for the adjoint integrator. The forward integrators use NoVertexHook, whose
// empty members compile away. Arguments are the factors of each radiance term the vertex adds:
//   surface       the shaded surface, its material after texturing and the BSDF at the vertex
//   emission      radiance added = thrW * emission (thrW = throughput x MIS weight)
//   nee*          shadow request `req`: contribution = factor * f * Le, f = f(wl) the BSDF value toward the light,
//                 factor = throughput x |cos| x MIS / pdf
//   bsdfSample    the continuation: throughput *= f(wl) * |cos| / pdf
//   cacheQuery    the path ends at this vertex (depth == cacheDepth): the radiance cache's prediction for the
//                 vertex, times the throughput, completes it
struct NoVertexHook {
    VKRT_DEV void surface(const Surface&, const ShadeMaterial&, const Bsdf&) {}
    VKRT_DEV void emission(float3) {}
    VKRT_DEV void neeEmissive(uint32_t, const Bsdf&, float3, float3, float3, float3, uint32_t) {}
    VKRT_DEV void neeEnvironment(uint32_t, const Bsdf&, float3, float3, float3, float3) {}
    VKRT_DEV void bsdfSample(const Bsdf&, float3, float3) {}
    VKRT_DEV void cacheQuery(const Surface&, const ShadeMaterial&) {}
};

// A sample's denoiser feature (integrator/path/state.slang DenoiserFeatures): albedo and shading normal of the first
// vertex that is not followed through a sharp specular lobe (integrator/path/loop.slang:83-103); weight 1 once taken.
struct DenoiserFeature {
    float3 albedo;
    float3 normal;
    float weight;
};

VKRT_DEV void captureFeature(DenoiserFeature& f, const Surface& s, const ShadeMaterial& m) {
    if (f.weight > 0.0f || denoiserFollowsSpecular(m)) return;
    f.albedo = denoiserAlbedo(m);
    f.normal = s.shadingNormal;
    f.weight = 1.0f;
}

struct FeatureHook : NoVertexHook {
    DenoiserFeature* f;
    VKRT_DEV void surface(const Surface& s, const ShadeMaterial& m, const Bsdf&) { captureFeature(*f, s, m); }
};

// Processes the hit of p's current ray. Returns true when the path continues with a new ray in p.o / p.d.
// `shadows` receives up to two requests (count in `numShadows`).
template <bool kSpectral, class Hook = NoVertexHook, bool kExt = false>
VKRT_DEV bool shadePathVertex(const DeviceScene& sc, const VKRT_CudaSceneData& sd, const StepConfig& cfg,
                              const SpecTable& tab, PathState& p, const TraceHit& h, ShadowRequest* shadows,
                              uint32_t& numShadows, Hook hook = Hook()) {
    numShadows = 0;
    const uint32_t depth = p.depth;
    const float rot = sd.environmentRotation;
    const bool prevNee = (p.flags & kPathPrevNee) != 0u;
    if (h.mesh == VKRT_CUDA_INVALID_INDEX) {  // miss: environment (environment.slang:16-27)
        float3 L = envRadiance(sc, sd, p.d);
        if (kSpectral) {
            float w = p.techPath > 0.0f ? 0.25f : 0.0f;  // heroWavelengthBalanceWeight of four equal lanes
            if (cfg.envNee && prevNee && depth > 0) {
                float pe = envPdf(sc.env, p.d, rot);
                float bt = p.prevVertexTech * p.prevBsdfTech, lt = p.prevVertexTech * pe;
                float den = 4.0f * bt + 4.0f * lt;
                w = den > 0.0f ? bt / den : 0.0f;
            }
            p.radiance += p.thr * spectral4(tab, L, heroLambdas(p.lamUnit)) * w;
        } else {
            float w = 1.0f;
            if (cfg.envNee && prevNee && depth > 0 && p.prevBsdfPdf > 0.0f) {
                float pe = envPdf(sc.env, p.d, rot);
                if (pe > 0.0f) w = powerHeuristic(p.prevBsdfPdf, pe);
            }
            float3 c = thr3(p) * L * w;
            p.radiance += make_float4(c.x, c.y, c.z, 0.0f);
        }
        return false;
    }
    if (!anyPos(p.thr)) return false;
    Surface s = reconstructSurface(sc, h.mesh, h.prim, h.u, h.v, p.o, p.d, h.t);
    ShadeMaterial mat;
    Basis basis;
    shadeVertex(sc, s, p.d, mat, basis);
    Bsdf bsdf = makeBsdf<kExt>(mat, toLocal(-p.d, basis), s.frontFace);
    const float4 lam = heroLambdas(p.lamUnit);
    hook.surface(s, mat, bsdf);

    // emission at the vertex, MIS against emissive NEE at the previous vertex (loop.slang:62-80)
    if (anyPos(mat.emission)) {
        if (kSpectral) {
            float w = p.techPath > 0.0f ? 0.25f : 0.0f;
            if (cfg.neeEnabled && prevNee && depth > 0) {
                float lps = emitterLightPdfSA(sc, h.mesh, h.t, p.d, s.geometricNormal);
                float bt = p.prevVertexTech * p.prevBsdfTech, lt = p.prevVertexTech * lps;
                float den = 4.0f * bt + 4.0f * lt;
                w = den > 0.0f ? bt / den : 0.0f;
            }
            p.radiance += p.thr * spectral4(tab, mat.emission, lam) * w;
        } else {
            float w = 1.0f;
            if (cfg.neeEnabled && prevNee && depth > 0 && p.prevBsdfPdf > 0.0f) {
                float lps = emitterLightPdfSA(sc, h.mesh, h.t, p.d, s.geometricNormal);
                w = lps <= 0.0f ? 1.0f : powerHeuristic(p.prevBsdfPdf, lps);
            }
            float3 c = thr3(p) * mat.emission * w;
            p.radiance += make_float4(c.x, c.y, c.z, 0.0f);
            hook.emission(thr3(p) * w);
        }
    }

    // radiance-cache termination: the cache stands for everything the vertex scatters (NEE and continuation)
    if (depth == cfg.cacheDepth) {
        hook.cacheQuery(s, mat);
        return false;
    }

    // emissive-triangle NEE (light/direct/light_sampling.slang, rgb_lighting.slang / spectral_lighting.slang)
    if (cfg.neeEnabled && bsdf.wo.z > 0.0f) {
        LightSample ls;
        if (sampleEmissive(sc, s.hitPoint, p.rng, ls)) {
            float3 wl = toLocal(ls.wi, basis);
            float pdf;
            float4 c = f4(0.0f);
            if (kSpectral) {
                float4 fcos = evalSpectral<kExt>(bsdf, tab, wl, lam, pdf) * fabsf(wl.z);
                float lt = p.techPath * ls.pdfSA, bt = p.techPath * pdf;
                float den = 4.0f * lt + 4.0f * bt;
                float mis = den > 0.0f ? lt / den : 0.0f;
                if (mis > 0.0f) c = p.thr * (fcos * spectral4(tab, ls.emission, lam) * (mis / ls.pdfSA));
            } else {
                float3 f = evalRgb<kExt>(bsdf, wl, pdf);
                if (pdf > 0.0f) {
                    float3 v = thr3(p) * (f * fabsf(wl.z) * ls.emission * (powerHeuristic(ls.pdfSA, pdf) / ls.pdfSA));
                    c = make_float4(v.x, v.y, v.z, 0.0f);
                    hook.neeEmissive(numShadows, bsdf, wl, f,
                                     thr3(p) * (fabsf(wl.z) * (powerHeuristic(ls.pdfSA, pdf) / ls.pdfSA)), ls.emission,
                                     ls.emissiveMesh);
                }
            }
            float3 off = dot(ls.wi, s.geometricNormal) >= 0.0f ? s.geometricNormal : -s.geometricNormal;
            shadows[numShadows++] = ShadowRequest{s.hitPoint + off * kShadowOriginOffset, ls.wi, ls.shadowDist, c};
        }
    }
    // environment NEE with MIS against the BSDF (this backend's importance sampler)
    if (cfg.envNee && bsdf.wo.z > 0.0f) {
        float u1 = p.rng.next(), u2 = p.rng.next();
        float3 wi;
        float pe;
        if (envSample(sc.env, u1, u2, rot, wi, pe)) {
            float3 wl = toLocal(wi, basis);
            float pdf;
            float4 c = f4(0.0f);
            if (kSpectral) {
                float4 fcos = evalSpectral<kExt>(bsdf, tab, wl, lam, pdf) * fabsf(wl.z);
                float lt = p.techPath * pe, bt = p.techPath * pdf;
                float den = 4.0f * lt + 4.0f * bt;
                float mis = den > 0.0f ? lt / den : 0.0f;
                if (mis > 0.0f) c = p.thr * (fcos * spectral4(tab, envRadiance(sc, sd, wi), lam) * (mis / pe));
            } else {
                float3 f = evalRgb<kExt>(bsdf, wl, pdf);
                if (pdf > 0.0f) {
                    float3 Le = envRadiance(sc, sd, wi);
                    float3 v = thr3(p) * (f * fabsf(wl.z) * Le * (powerHeuristic(pe, pdf) / pe));
                    c = make_float4(v.x, v.y, v.z, 0.0f);
                    hook.neeEnvironment(numShadows, bsdf, wl, f,
                                        thr3(p) * (fabsf(wl.z) * (powerHeuristic(pe, pdf) / pe)), Le);
                }
            }
            float3 off = dot(wi, s.geometricNormal) >= 0.0f ? s.geometricNormal : -s.geometricNormal;
            shadows[numShadows++] = ShadowRequest{s.hitPoint + off * kShadowOriginOffset, wi, kTMax, c};
        }
    }

    // next direction (sample_rgb.slang:6-23 / sample_spectral.slang:6-24)
    if (bsdf.wo.z <= 0.0f) return false;
    float3 wl;
    if (!sampleDirection<kExt>(bsdf, p.rng, wl)) return false;
    float pdf;
    if (kSpectral) {
        float4 val = evalSpectral<kExt>(bsdf, tab, wl, lam, pdf);
        if (!(pdf > 0.0f)) return false;
        float4 weight = val * (fabsf(wl.z) / pdf);
        if (!anyPos(weight)) return false;
        p.prevVertexTech = p.techPath;
        p.prevBsdfTech = pdf;
        p.techPath *= pdf;
        p.thr *= weight;
    } else {
        float3 f = evalRgb<kExt>(bsdf, wl, pdf);
        if (!(pdf > 0.0f)) return false;
        float3 weight = f * (fabsf(wl.z) / pdf);
        if (!anyPos(weight)) return false;
        p.thr = make_float4(p.thr.x * weight.x, p.thr.y * weight.y, p.thr.z * weight.z, 0.0f);
        p.prevBsdfPdf = pdf;
        hook.bsdfSample(bsdf, wl, f);
    }
    if (!anyPos(p.thr)) return false;
    p.flags |= kPathPrevNee;
    // Russian roulette (rgb/integrator.slang:100-106)
    if (depth + 1u >= sd.rrMinDepth) {
        float q = kSpectral ? max4(p.thr) : maxc(thr3(p));
        float prob = fminf(fmaxf(q, kRRMin), kRRMax);
        if (p.rng.next() > prob) return false;
        if (kSpectral) p.techPath *= prob;
        p.thr = p.thr / prob;
    }
    p.o = s.hitPoint + s.geometricNormal * kShadowOriginOffset;  // loop.slang:113-120
    p.d = toWorld(wl, basis);
    p.depth = depth + 1u;
    return p.depth < sd.rrMaxDepth;
}

}  // namespace vkrt
