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

#include "bsdf_full.cuh"
#include "integrator.cuh"

namespace vkrt {

constexpr uint32_t kPathPrevNee = 1u;  // the previous vertex sampled NEE (loop.slang:69-71)
constexpr uint32_t kPathDone = 2u;
constexpr uint32_t kPathFeatureDone = 4u;  // the sample's denoiser feature was taken at an earlier vertex
constexpr uint32_t kPathRefractive = 8u;   // inside a refractive medium: no NEE (MediumState, medium.slang:7-33)
constexpr uint32_t kPathAbsorbing = 16u;   // inside an absorbing medium: Beer-Lambert along each segment
constexpr uint32_t kPathCollapsed = 32u;   // spectral path collapsed to its first hero lane by dispersion

struct PathState {
    Rng rng;
    float3 o, d;
    float4 thr;       // RGB throughput in xyz, or the four hero-lane throughputs
    float4 radiance;  // RGB radiance in xyz, or the four hero-lane spectral radiances
    float lamUnit;    // hero wavelength unit sample; lane i at 360 + frac(lamUnit + i/4) * 470
    float techPath, prevVertexTech, prevBsdfTech;  // hero MIS (shared by the four lanes)
    float prevBsdfPdf;                             // RGB MIS, and the single-wavelength MIS of a collapsed path
    uint32_t depth;
    uint32_t flags;
    // radiance-cache area-spread rule: the running sum of the footprint square roots after the primary vertex, and
    // the primary vertex's footprint a0 (set at depth 0; used only when StepConfig::cacheSpread > 0)
    float spread, spreadA0;
    // full instantiations: hero lanes 1-3 of the technique pdfs (lane 0 in the scalars above; the lanes differ after
    // dispersive interfaces) and the absorption of the medium the path is in (RGB in xyz, the four hero lanes, or the
    // collapsed lane in x). A collapsed path keeps its throughput in thr.x, the XYZ of its hero lanes in
    // radiance.xyz and its single-wavelength radiance in radiance.w.
    float3 techYZW, prevVertexYZW, prevBsdfYZW;
    float4 sigma;
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
    float cacheSpread = 0.0f;  // > 0: a path also ends in the cache once its area spread exceeds this times a0
    bool single = false;  // spectral mode with one wavelength per path (raygen_spectral_single.slang), full kernels
};

VKRT_DEV bool singleWavelength(const VKRT_CudaSceneData& sd) {
    return VKRT_CUDA_RENDER_MODE_OF(sd.packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL &&
           VKRT_CUDA_SPECTRAL_MODE_OF(sd.packedRenderSettings) == VKRT_CUDA_SPECTRAL_SINGLE;
}

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
    p.spread = 0.0f;
    p.spreadA0 = 0.0f;
    p.techYZW = f3(1.0f);
    p.prevVertexYZW = f3(0.0f);
    p.prevBsdfYZW = f3(0.0f);
    p.sigma = f4(0.0f);
    // single-wavelength mode (sampleUniformWavelength, wavelength.slang:34-42): the hero lane-0 wavelength, which is
    // the same unit sample, carried from the start as a collapsed path
    if (kSpectral && cfg.single) {
        p.flags |= kPathCollapsed;
        p.thr = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    }
    return p;
}

// Path termination by area spread (Mueller, Rousselle, Novak, Keller 2021, "Real-time Neural Radiance Caching for
// Path Tracing", section 3.3): the footprint a path's vertices x1..xn cover,
//   a(x1..xn) = (sum_{i=2..n} sqrt(|x_{i-1} - x_i|^2 / (p(w_i | x_{i-1}) |cos theta_i|)))^2,
// is compared with the primary vertex's footprint seen from the camera, a0 = |x0 - x1|^2 / (4 pi |cos theta_1|);
// the path ends in the cache at the first vertex where a > c a0. Narrow (glossy) lobes add little spread and keep a
// path going, a diffuse bounce usually ends it at the next vertex. `t` is the segment length to this vertex (unit
// direction), `cosTheta` the cosine between that segment and the geometric normal here, `pdfPrev` the solid-angle
// pdf with which the previous vertex sampled the segment. Records a0 at depth 0.
VKRT_DEV bool spreadEndsPath(const StepConfig& cfg, PathState& p, uint32_t depth, float t, float cosTheta,
                             float pdfPrev) {
    if (!(cfg.cacheSpread > 0.0f)) return false;
    if (depth == 0u) {
        p.spreadA0 = (t * t) / (4.0f * kPi * cosTheta);
        return false;
    }
    const float den = pdfPrev * cosTheta;
    p.spread += den > 0.0f ? t * rsqrtf(den) : __int_as_float(0x7F800000);
    return p.spread * p.spread > cfg.cacheSpread * p.spreadA0;
}

// Sample value of a finished path: linear sRGB, or CIE XYZ in spectral mode (spectral.slang:104-113).
template <bool kSpectral>
VKRT_DEV float3 pathResult(const StepConfig& cfg, const PathState& p) {
    if (!kSpectral) return xyz(p.radiance);
    if (p.flags & kPathCollapsed)  // spectralSampleToXYZ of the surviving lane (spectral.slang:99-102)
        return xyz(p.radiance) + cieXYZ(heroLambdas(p.lamUnit).x) * (p.radiance.w * (kLambdaRange / kCieYIntegral));
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
    if (f.weight > 0.0f || denoiserFollowsSpecular(m, s.frontFace)) return;
    f.albedo = denoiserAlbedo(m);
    f.normal = s.shadingNormal;
    f.weight = 1.0f;
}

struct FeatureHook : NoVertexHook {
    DenoiserFeature* f;
    VKRT_DEV void surface(const Surface& s, const ShadeMaterial& m, const Bsdf&) { captureFeature(*f, s, m); }
};

VKRT_DEV float sum4f(float4 a) { return a.x + a.y + a.z + a.w; }
VKRT_DEV float heroBalance(float4 t) {  // heroWavelengthBalanceWeight (spectral.slang:115-118)
    const float c = sum4f(t);
    return c > 0.0f ? t.x / c : 0.0f;
}
VKRT_DEV float4 mediumTransmittance(const PathState& p, float dist) {  // medium.slang:66-72
    if (!(p.flags & kPathAbsorbing)) return f4(1.0f);
    return make_float4(expf(-p.sigma.x * dist), expf(-p.sigma.y * dist), expf(-p.sigma.z * dist),
                       expf(-p.sigma.w * dist));
}
VKRT_DEV float absorptionSigma(float tint, float coeff) {  // materialAbsorptionSigma (medium.slang:44-64)
    return -logf(fmaxf(tint, 1e-6f)) * coeff;
}

// One vertex of the full integrators: shadePathVertex with vkrt's whole reflection stack, its transmissive
// interface and the media behind it (rgb/integrator.slang:15-113, spectral_hero/integrator.slang:16-172,
// spectral_hero/transport.slang): Beer-Lambert absorption along segments inside a medium, no NEE and no environment
// inside a refractive medium, NEE that the shadow tracer marks unsupported when its ray meets a transmissive
// surface (then p loses kPathPrevNee), refraction below the surface, and the collapse of a hero path to its first
// lane after a dispersive refraction (the path then runs as a single-wavelength path).
template <bool kSpectral, class Hook>
VKRT_DEV bool shadePathVertexFull(const DeviceScene& sc, const VKRT_CudaSceneData& sd, const StepConfig& cfg,
                                  const SpecTable& tab, PathState& p, const TraceHit& h, ShadowRequest* shadows,
                                  uint32_t& numShadows, Hook hook) {
    numShadows = 0;
    const uint32_t depth = p.depth;
    const float rot = sd.environmentRotation;
    const bool prevNee = (p.flags & kPathPrevNee) != 0u;
    bool collapsed = kSpectral && (p.flags & kPathCollapsed) != 0u;
    const float4 lam = heroLambdas(p.lamUnit);
    float4 tech = make_float4(p.techPath, p.techYZW.x, p.techYZW.y, p.techYZW.z);
    const float4 pvt = make_float4(p.prevVertexTech, p.prevVertexYZW.x, p.prevVertexYZW.y, p.prevVertexYZW.z);
    const float4 pbt = make_float4(p.prevBsdfTech, p.prevBsdfYZW.x, p.prevBsdfYZW.y, p.prevBsdfYZW.z);
    if (h.mesh == VKRT_CUDA_INVALID_INDEX) {  // environment, unless a medium boundary is active (loop.slang:4-6)
        if (p.flags & (kPathRefractive | kPathAbsorbing)) return false;
        const float3 L = envRadiance(sc, sd, p.d);
        if (kSpectral) {
            if (collapsed) {
                p.radiance.w += p.thr.x * spectral1(tab, L, lam.x);
                return false;
            }
            float w = heroBalance(tech);
            if (cfg.envNee && prevNee && depth > 0) {
                const float pe = envPdf(sc.env, p.d, rot);
                const float4 bt = pvt * pbt, lt = pvt * pe;
                const float den = sum4f(bt) + sum4f(lt);
                w = den > 0.0f ? bt.x / den : 0.0f;
            }
            p.radiance += p.thr * spectral4Call(tab, L, lam) * w;
        } else {
            float w = 1.0f;
            if (cfg.envNee && prevNee && depth > 0 && p.prevBsdfPdf > 0.0f) {
                const float pe = envPdf(sc.env, p.d, rot);
                if (pe > 0.0f) w = powerHeuristic(p.prevBsdfPdf, pe);
            }
            const float3 c = thr3(p) * L * w;
            p.radiance += make_float4(c.x, c.y, c.z, 0.0f);
        }
        return false;
    }
    if (p.flags & kPathAbsorbing) {  // apply*MediumTransmittance (rgb/transport.slang:10-17, hero :22-35)
        const float4 T = mediumTransmittance(p, h.t);
        if (collapsed) p.thr.x *= T.x;
        else p.thr = kSpectral ? p.thr * T : make_float4(p.thr.x * T.x, p.thr.y * T.y, p.thr.z * T.z, 0.0f);
    }
    if (collapsed ? !(p.thr.x > 0.0f) : !anyPos(p.thr)) return false;
    Surface s = reconstructSurface(sc, h.mesh, h.prim, h.u, h.v, p.o, p.d, h.t);
    ShadeMaterial mat;
    Basis basis;
    shadeVertex(sc, s, p.d, mat, basis);
    const BsdfFull bsdf = makeBsdfFull(mat, toLocal(-p.d, basis), s.frontFace, sc.sheenLtc);
    hook.surface(s, mat, bsdf);

    if (anyPos(mat.emission)) {  // emission, MIS against emissive NEE at the previous vertex (loop.slang:62-80)
        const bool misNee = cfg.neeEnabled && prevNee && depth > 0;
        if (kSpectral && !collapsed) {
            float w = heroBalance(tech);
            if (misNee) {
                const float lps = emitterLightPdfSA(sc, h.mesh, h.t, p.d, s.geometricNormal);
                const float4 bt = pvt * pbt, lt = pvt * lps;
                const float den = sum4f(bt) + sum4f(lt);
                w = den > 0.0f ? bt.x / den : 0.0f;
            }
            p.radiance += p.thr * spectral4Call(tab, mat.emission, lam) * w;
        } else {
            float w = 1.0f;
            if (misNee && p.prevBsdfPdf > 0.0f) {
                const float lps = emitterLightPdfSA(sc, h.mesh, h.t, p.d, s.geometricNormal);
                w = lps <= 0.0f ? 1.0f : powerHeuristic(p.prevBsdfPdf, lps);
            }
            if (collapsed) {
                p.radiance.w += p.thr.x * spectral1(tab, mat.emission, lam.x) * w;
            } else {
                const float3 c = thr3(p) * mat.emission * w;
                p.radiance += make_float4(c.x, c.y, c.z, 0.0f);
                hook.emission(thr3(p) * w);
            }
        }
    }

    if (depth == cfg.cacheDepth ||
        spreadEndsPath(cfg, p, depth, h.t, fabsf(dot(s.geometricNormal, p.d)),
                       kSpectral && !collapsed ? p.prevBsdfTech : p.prevBsdfPdf)) {
        hook.cacheQuery(s, mat);
        return false;
    }

    // the hero stack's direction-independent colours, shared by the NEE evaluations and the continuation
    const HeroTerms ht = kSpectral && !collapsed ? heroTerms(bsdf, tab, lam) : HeroTerms{f4(0.0f), f4(0.0f), f4(0.0f)};

    const bool neeHere = (p.flags & kPathRefractive) == 0u;  // currentVertexNeeAllowed
    if (cfg.neeEnabled && neeHere && bsdf.wo.z > 0.0f) {
        // sampleDirectLight{Rgb, SpectralHero, SpectralSingle} (light/direct/*.slang): the shadow ray is traced even
        // when the light lies below a refractive surface, since its answer may mark NEE unsupported
        LightSample ls;
        if (sampleEmissive(sc, s.hitPoint, p.rng, ls)) {
            const float3 wl = toLocal(ls.wi, basis);
            float4 c = f4(0.0f);
            if (!(mediumIsRefractive(mat) && wl.z <= 0.0f)) {
                const float4 T = mediumTransmittance(p, ls.shadowDist);
                float pdf;
                if (!kSpectral) {
                    const float3 f = evalScalarFull<false>(bsdf, tab, wl, 0.0f, pdf);
                    if (pdf > 0.0f) {
                        const float3 v = thr3(p) * (make_float3(T.x, T.y, T.z) * f * fabsf(wl.z) * ls.emission *
                                                    (powerHeuristic(ls.pdfSA, pdf) / ls.pdfSA));
                        c = make_float4(v.x, v.y, v.z, 0.0f);
                    }
                } else if (collapsed) {
                    const float3 f = evalScalarFull<true>(bsdf, tab, wl, lam.x, pdf);
                    if (pdf > 0.0f) {
                        const float value = f.x * fabsf(wl.z) * spectral1(tab, ls.emission, lam.x);
                        c.w = p.thr.x * (powerHeuristic(ls.pdfSA, pdf) * T.x * value / ls.pdfSA);
                    }
                } else {
                    float4 tp;
                    const float4 fcos = evalHeroFull(bsdf, tab, wl, lam, ht, tp) * fabsf(wl.z);
                    const float4 lt = tech * ls.pdfSA, bt = tech * tp;
                    const float den = sum4f(lt) + sum4f(bt);
                    const float mis = den > 0.0f ? lt.x / den : 0.0f;
                    if (mis > 0.0f) c = p.thr * (T * fcos * spectral4Call(tab, ls.emission, lam) * (mis / ls.pdfSA));
                }
            }
            const float3 off = dot(ls.wi, s.geometricNormal) >= 0.0f ? s.geometricNormal : -s.geometricNormal;
            shadows[numShadows++] = ShadowRequest{s.hitPoint + off * kShadowOriginOffset, ls.wi, ls.shadowDist, c};
        }
    }
    // environment NEE: off when any material is transmissive (vkrt has none), so never on a collapsed path
    if (cfg.envNee && bsdf.wo.z > 0.0f) {
        const float u1 = p.rng.next(), u2 = p.rng.next();
        float3 wi;
        float pe;
        if (envSample(sc.env, u1, u2, rot, wi, pe)) {
            const float3 wl = toLocal(wi, basis);
            float4 c = f4(0.0f);
            if (kSpectral) {
                float4 tp;
                const float4 fcos = evalHeroFull(bsdf, tab, wl, lam, ht, tp) * fabsf(wl.z);
                const float4 lt = tech * pe, bt = tech * tp;
                const float den = sum4f(lt) + sum4f(bt);
                const float mis = den > 0.0f ? lt.x / den : 0.0f;
                if (mis > 0.0f) c = p.thr * (fcos * spectral4Call(tab, envRadiance(sc, sd, wi), lam) * (mis / pe));
            } else {
                float pdf;
                const float3 f = evalScalarFull<false>(bsdf, tab, wl, 0.0f, pdf);
                if (pdf > 0.0f) {
                    const float3 v = thr3(p) * (f * fabsf(wl.z) * envRadiance(sc, sd, wi) * (powerHeuristic(pe, pdf) / pe));
                    c = make_float4(v.x, v.y, v.z, 0.0f);
                }
            }
            const float3 off = dot(wi, s.geometricNormal) >= 0.0f ? s.geometricNormal : -s.geometricNormal;
            shadows[numShadows++] = ShadowRequest{s.hitPoint + off * kShadowOriginOffset, wi, kTMax, c};
        }
    }

    // next direction (sample_rgb.slang:6-23, sample_spectral.slang:6-24, spectral_hero/transport.slang:49-109)
    if (bsdf.wo.z <= 0.0f) return false;
    float3 wl;
    bool isTrans;
    if (!sampleFull(bsdf, p.rng, lam.x, kSpectral, wl, isTrans)) return false;
    float pdf;
    if (!kSpectral) {
        const float3 f = evalScalarFull<false>(bsdf, tab, wl, 0.0f, pdf);
        if (!(pdf > 0.0f)) return false;
        const float3 weight = f * (fabsf(wl.z) / pdf);
        if (!anyPos(weight)) return false;
        p.thr = make_float4(p.thr.x * weight.x, p.thr.y * weight.y, p.thr.z * weight.z, 0.0f);
        if (!anyPos(p.thr)) return false;
        p.prevBsdfPdf = pdf;
    } else if (collapsed) {
        const float3 f = evalScalarFull<true>(bsdf, tab, wl, lam.x, pdf);
        if (!(pdf > 0.0f)) return false;
        const float3 weight = f * (fabsf(wl.z) / pdf);
        if (!anyPos(weight)) return false;
        p.thr.x *= weight.x;
        if (!(p.thr.x > 0.0f)) return false;
        p.prevBsdfPdf = pdf;
    } else {
        float4 tp;
        const float4 val = evalHeroFull(bsdf, tab, wl, lam, ht, tp);
        if (!(tp.x > 0.0f)) return false;
        const float4 weight = val * (fabsf(wl.z) / tp.x);
        if (!anyPos(weight)) return false;
        p.prevVertexTech = tech.x;
        p.prevVertexYZW = make_float3(tech.y, tech.z, tech.w);
        p.prevBsdfTech = tp.x;
        p.prevBsdfYZW = make_float3(tp.y, tp.z, tp.w);
        tech = tech * tp;
        p.thr *= weight;
        if (!anyPos(p.thr)) return false;
        if (isTrans && mediumIsRefractive(mat) && mat.abbe > 0.0f) {
            // dispersion: the hero lanes' radiance (and this vertex's pending NEE) moves to XYZ, lane 0 goes on
            const float3 done = spectral4ToXYZ(p.radiance, lam, kLambdaRange);
            p.radiance = make_float4(done.x, done.y, done.z, 0.0f);
            for (uint32_t r = 0; r < numShadows; ++r) {
                const float3 c = spectral4ToXYZ(shadows[r].contribution, lam, kLambdaRange);
                shadows[r].contribution = make_float4(c.x, c.y, c.z, 0.0f);
            }
            p.thr = make_float4(p.thr.x, 0.0f, 0.0f, 0.0f);
            p.prevBsdfPdf = tp.x;
            p.flags |= kPathCollapsed;
            collapsed = true;
        }
    }
    if (neeHere && !isTrans) p.flags |= kPathPrevNee;
    else p.flags &= ~kPathPrevNee;
    if (isTrans) {  // updateMediumStateFromTransmission[Spectral] (medium.slang:79-115)
        const bool entering = s.frontFace != 0u;
        const bool absorbing = entering && hasAbsorption(mat);
        p.flags &= ~(kPathRefractive | kPathAbsorbing);
        if (entering && mediumIsRefractive(mat)) p.flags |= kPathRefractive;
        p.sigma = f4(0.0f);
        if (absorbing) {
            p.flags |= kPathAbsorbing;
            const float3 tint = sat(mat.attenuationColor);
            const float k = mat.absorption;
            if (!kSpectral) {
                p.sigma = make_float4(absorptionSigma(tint.x, k), absorptionSigma(tint.y, k), absorptionSigma(tint.z, k),
                                      0.0f);
            } else if (collapsed) {
                p.sigma = f4(absorptionSigma(spectral1(tab, tint, lam.x), k));
            } else {
                const float4 s4 = spectral4Call(tab, tint, lam);
                p.sigma = make_float4(absorptionSigma(s4.x, k), absorptionSigma(s4.y, k), absorptionSigma(s4.z, k),
                                      absorptionSigma(s4.w, k));
            }
        }
    }
    if (depth + 1u >= sd.rrMinDepth) {  // Russian roulette
        const float q = !kSpectral ? maxc(thr3(p)) : (collapsed ? p.thr.x : max4(p.thr));
        const float prob = fminf(fmaxf(q, kRRMin), kRRMax);
        if (p.rng.next() > prob) return false;
        if (kSpectral && !collapsed) tech = tech * prob;
        p.thr = p.thr / prob;
    }
    p.techPath = tech.x;
    p.techYZW = make_float3(tech.y, tech.z, tech.w);
    // advancePathRay (loop.slang:113-120): a refracted ray starts below the surface
    p.o = s.hitPoint + (isTrans ? -s.geometricNormal : s.geometricNormal) * kShadowOriginOffset;
    p.d = toWorld(wl, basis);
    p.depth = depth + 1u;
    return p.depth < sd.rrMaxDepth;
}

// The vertex step of the reflection-only instantiations (the glTF subset of shading.cuh).
template <bool kSpectral, class Hook>
VKRT_DEV bool shadePathVertexSubset(const DeviceScene& sc, const VKRT_CudaSceneData& sd, const StepConfig& cfg,
                                    const SpecTable& tab, PathState& p, const TraceHit& h, ShadowRequest* shadows,
                                    uint32_t& numShadows, Hook hook) {
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
    Bsdf bsdf = makeBsdf(mat, toLocal(-p.d, basis), s.frontFace);
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
    if (depth == cfg.cacheDepth ||
        spreadEndsPath(cfg, p, depth, h.t, fabsf(dot(s.geometricNormal, p.d)),
                       kSpectral ? p.prevBsdfTech : p.prevBsdfPdf)) {
        hook.cacheQuery(s, mat);
        return false;
    }

    // the spectral stack's direction-independent term, shared by the NEE evaluations and the continuation
    const float4 vaSub = kSpectral && bsdf.wo.z > 0.0f ? spectralDiffuseTerm(bsdf, tab, lam) : f4(0.0f);

    // emissive-triangle NEE (light/direct/light_sampling.slang, rgb_lighting.slang / spectral_lighting.slang)
    if (cfg.neeEnabled && bsdf.wo.z > 0.0f) {
        LightSample ls;
        if (sampleEmissive(sc, s.hitPoint, p.rng, ls)) {
            float3 wl = toLocal(ls.wi, basis);
            float pdf;
            float4 c = f4(0.0f);
            if (kSpectral) {
                float4 fcos = evalSpectral(bsdf, tab, wl, lam, vaSub, pdf) * fabsf(wl.z);
                float lt = p.techPath * ls.pdfSA, bt = p.techPath * pdf;
                float den = 4.0f * lt + 4.0f * bt;
                float mis = den > 0.0f ? lt / den : 0.0f;
                if (mis > 0.0f) c = p.thr * (fcos * spectral4(tab, ls.emission, lam) * (mis / ls.pdfSA));
            } else {
                float3 f = evalRgb(bsdf, wl, pdf);
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
                float4 fcos = evalSpectral(bsdf, tab, wl, lam, vaSub, pdf) * fabsf(wl.z);
                float lt = p.techPath * pe, bt = p.techPath * pdf;
                float den = 4.0f * lt + 4.0f * bt;
                float mis = den > 0.0f ? lt / den : 0.0f;
                if (mis > 0.0f) c = p.thr * (fcos * spectral4(tab, envRadiance(sc, sd, wi), lam) * (mis / pe));
            } else {
                float3 f = evalRgb(bsdf, wl, pdf);
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
    if (!sampleDirection(bsdf, p.rng, wl)) return false;
    float pdf;
    if (kSpectral) {
        float4 val = evalSpectral(bsdf, tab, wl, lam, vaSub, pdf);
        if (!(pdf > 0.0f)) return false;
        float4 weight = val * (fabsf(wl.z) / pdf);
        if (!anyPos(weight)) return false;
        p.prevVertexTech = p.techPath;
        p.prevBsdfTech = pdf;
        p.techPath *= pdf;
        p.thr *= weight;
    } else {
        float3 f = evalRgb(bsdf, wl, pdf);
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

// Processes the hit of p's current ray. Returns true when the path continues with a new ray in p.o / p.d.
// `shadows` receives up to two requests (count in `numShadows`). kExt selects vkrt's whole material stack.
template <bool kSpectral, class Hook = NoVertexHook, bool kExt = false>
VKRT_DEV bool shadePathVertex(const DeviceScene& sc, const VKRT_CudaSceneData& sd, const StepConfig& cfg,
                              const SpecTable& tab, PathState& p, const TraceHit& h, ShadowRequest* shadows,
                              uint32_t& numShadows, Hook hook = Hook()) {
    if constexpr (kExt) return shadePathVertexFull<kSpectral>(sc, sd, cfg, tab, p, h, shadows, numShadows, hook);
    else return shadePathVertexSubset<kSpectral>(sc, sd, cfg, tab, p, h, shadows, numShadows, hook);
}

}  // namespace vkrt
