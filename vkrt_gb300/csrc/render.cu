// render.cu — the render-frame megakernels and their helpers on sm_103a.
//
// One launch = vkrt's main trace pass (src/core/runtime/command/record.c:448-486 dispatching
// entry/path/raygen_rgb.slang:4-35 or raygen_spectral_hero.slang:4-35 over W x H) plus the film blend
// (integrator/path/writeback.slang:9-123) and the display encode (film/tonemap.slang:9-32), fused: each thread owns
// one pixel, runs its SceneData.samplesPerPixel paths, blends them into the running mean read from the previous
// accumulation image and writes the next accumulation image and the RGBA16 output.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "path.cuh"
#include "render.h"

namespace vkrt {

namespace {

// One pixel: SceneData.samplesPerPixel paths, blended into the running mean (writeback.slang:72-114) and encoded
// for display. The loop is flat: every iteration traces exactly one ray of the thread — the next segment of its path
// or one of the shadow rays its last vertex asked for — through a single inlined copy of the traversal, and a thread
// whose path ended starts its next sample in the same iteration (path regeneration). With the sample loop nested
// around the bounce loop instead, a warp waited at the end of every sample for its longest path (3.5 of 32 lanes
// active on the 1M-triangle field) and held three copies of the traversal code. Each thread still sums its own samples
// in sample order and applies a vertex's shadow contributions in request order before its next segment, so the image
// is the nested loop's, bit for bit.
// kFull: vkrt's whole material stack, alpha tests and the denoiser features (written when the film has feature
// images)
// kFeatures alone: the denoiser features with the reflection-only materials (the plain vertex step plus the feature
// hook).
template <bool kSpectral, bool kCountBytes, bool kFull, bool kFeatures = kFull>
__global__ void __launch_bounds__(kDefaultThreads) kRenderMega(DeviceScene sc, VKRT_CudaSceneData sd, RenderParams rp,
                                                               FilmBuffers film, RenderCounters* counters) {
    extern __shared__ uint2 smemStack[];
    const uint32_t W = rp.width;
    const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
    PathCounts pc{0u, 0u, 0u, 0u};
    if (pixel < W * rp.height) {
        const int px = int(pixel % W), py = int(pixel / W);
        const int vx0 = int(sd.viewportRect[0]), vy0 = int(sd.viewportRect[1]);
        const int vw = int(sd.viewportRect[2]), vh = int(sd.viewportRect[3]);
        bool inside = vw > 0 && vh > 0 && px >= vx0 && py >= vy0 && px < vx0 + vw && py < vy0 + vh;
        if (!inside) {
            film.accumWrite[pixel] = f4(0.0f);
            film.output[pixel] = make_ushort4(0, 0, 0, 0);
            if (kFeatures && film.albedoWrite) film.albedoWrite[pixel] = film.normalWrite[pixel] = f4(0.0f);
        } else {
            uint2* const stackColumn = smemStack + threadIdx.x;
            const float4 prev = film.accumRead[pixel];
            const uint32_t prevN = uint32_t(prev.w + 0.5f);  // integrator/path/state.slang:72
            const uint32_t spp = max(sd.samplesPerPixel, 1u);
            StepConfig cfg{kSpectral, sd.misNeeEnabled != 0u && sd.emissiveMeshCount > 0u, rp.envNee != 0u, rp.rngMode,
                           rp.rngSeed};
            cfg.single = kSpectral && kFull && singleWavelength(sd);
            SpecTable tab = makeSpecTable(sc, sd);
            const bool alpha = kFull && rp.alpha != 0u;
            float3 sum = f3(0.0f);
            DenoiserFeature fsum{f3(0.0f), f3(0.0f), 0.0f};
            DenoiserFeature feat{f3(0.0f), f3(0.0f), 0.0f};
            PathState p;
            uint32_t si = 0u;  // samples started
            bool live = false;
            for (;;) {
                if (!live) {
                    if (si >= spp) break;
                    p = beginPath<kSpectral>(cfg, sd, px, py, prevN + si);
                    ++si;
                    live = true;
                    feat = DenoiserFeature{f3(0.0f), f3(0.0f), 0.0f};
                    pc.samples++;
                }
                if (p.depth == 0) pc.primary++;
                else pc.extension++;
                // alpha-tested scenes: the ray's alpha seed, which the vertex's shadow rays reuse salted
                const uint32_t alphaSeed = alphaSeedOf(p.rng);
                TraceHit h;
                if (alpha)
                    h = traceBvh<false, kCountBytes, false, false, 1>(sc, TraceRay{p.o, p.d, kTMin, kTMax},
                                                                      stackColumn, blockDim.x, counters, 0u,
                                                                      alphaSeed);
                else h = traceBvh<false, kCountBytes>(sc, TraceRay{p.o, p.d, kTMin, kTMax}, stackColumn, blockDim.x,
                                                      counters);
                ShadowRequest sh[2];
                uint32_t ns;
                bool cont;
                if (kFull)
                    cont = shadePathVertex<kSpectral, FeatureHook, true>(sc, sd, cfg, tab, p, h, sh, ns,
                                                                         FeatureHook{{}, &feat});
                else if (kFeatures)
                    cont = shadePathVertex<kSpectral, FeatureHook>(sc, sd, cfg, tab, p, h, sh, ns,
                                                                   FeatureHook{{}, &feat});
                else cont = shadePathVertex<kSpectral>(sc, sd, cfg, tab, p, h, sh, ns);
                for (uint32_t i = 0; i < ns; ++i) {
                    pc.shadow++;
                    const TraceRay r{sh[i].origin, sh[i].dir, kTMin, sh[i].tmax};
                    const TraceHit o = traceBvh<true, kCountBytes, false, false, 0, true>(
                        sc, r, stackColumn, blockDim.x, counters, 0u, alphaShadowSeed(alphaSeed, i), true, kFull,
                        alpha);
                    if (o.mesh == VKRT_CUDA_INVALID_INDEX) {
                        // a transmissive occluder makes the vertex's NEE unsupported (full stack only)
                        if (kFull && o.prim == kShadowThroughTransmission) p.flags &= ~kPathPrevNee;
                        else p.radiance += sh[i].contribution;
                    }
                }
                if (!cont) {
                    sum += pathResult<kSpectral>(cfg, p);
                    if (kFeatures) {
                        fsum.albedo += feat.albedo;
                        fsum.normal += feat.normal;
                        fsum.weight += feat.weight;
                    }
                    live = false;
                }
            }
            if (kFeatures && film.albedoWrite) {
                blendFeature(film.albedoRead, film.albedoWrite, pixel, fsum.albedo, fsum.weight);
                blendFeature(film.normalRead, film.normalWrite, pixel, fsum.normal, fsum.weight);
            }
            float3 cur = sum / float(spp);
            float pw = float(prevN), tw = pw + float(spp);
            float3 acc = tw <= 0.0f ? f3(0.0f) : (xyz(prev) * pw + cur * float(spp)) / tw;
            film.accumWrite[pixel] = make_float4(acc.x, acc.y, acc.z, tw);
            film.output[pixel] = encodeOutput(sd, acc, kSpectral);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && counters) atomicAdd(&counters->kernelLaunches, 1ull);
    // warp-aggregated ray counters
    for (int off = 16; off > 0; off >>= 1) {
        pc.primary += __shfl_xor_sync(0xFFFFFFFFu, pc.primary, off);
        pc.extension += __shfl_xor_sync(0xFFFFFFFFu, pc.extension, off);
        pc.shadow += __shfl_xor_sync(0xFFFFFFFFu, pc.shadow, off);
        pc.samples += __shfl_xor_sync(0xFFFFFFFFu, pc.samples, off);
    }
    if ((threadIdx.x & 31u) == 0u && counters) {
        atomicAdd(&counters->primaryRays, (unsigned long long)pc.primary);
        atomicAdd(&counters->extensionRays, (unsigned long long)pc.extension);
        atomicAdd(&counters->shadowRays, (unsigned long long)pc.shadow);
        atomicAdd(&counters->pathSamples, (unsigned long long)pc.samples);
    }
}

template <bool kAnyHit>
__global__ void __launch_bounds__(kDefaultThreads) kTraceRays(DeviceScene sc, const VKRT_CudaRay* __restrict__ rays,
                                                              uint32_t count, VKRT_CudaHit* __restrict__ hits,
                                                              RenderCounters* counters) {
    extern __shared__ uint2 smemStack[];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float4* rp = reinterpret_cast<const float4*>(rays + i);
    float4 a = __ldg(rp), b = __ldg(rp + 1);
    TraceRay r{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), a.w, b.w};
    TraceHit h = traceBvh<kAnyHit, false>(sc, r, smemStack + threadIdx.x, blockDim.x, counters);
    bool hit = h.mesh != VKRT_CUDA_INVALID_INDEX;
    float4* hp = reinterpret_cast<float4*>(hits + i);
    hp[0] = make_float4(__uint_as_float(h.mesh), __uint_as_float(h.prim), hit ? h.t : 0.0f, hit ? h.u : 0.0f);
    hp[1] = make_float4(hit ? h.v : 0.0f, 0.0f, 0.0f, 0.0f);
}

// The same trace through the wavefront's persistent traversal (persistentTraceVote: dynamic ray fetch and a warp vote
// per step between node visits and triangle tests), so the kernel the wavefront's intersect and shadow stages run can
// be checked ray by ray. Rays are fetched through counters->workCursor, which the launch clears.
template <bool kAnyHit>
__global__ void __launch_bounds__(kDefaultThreads) kTraceRaysPersistent(DeviceScene sc,
                                                                        const VKRT_CudaRay* __restrict__ rays,
                                                                        uint32_t count, VKRT_CudaHit* __restrict__ hits,
                                                                        RenderCounters* counters) {
    extern __shared__ uint2 smemStack[];
    uint32_t nodeVisits = 0u, triTests = 0u;
    persistentTraceVote<kAnyHit, false>(
        count, &counters->workCursor, smemStack + threadIdx.x, blockDim.x, &counters->errorFlags, kVoteRefillLanes,
        [&](uint32_t i, TraceRay& r, const WideNode*& nodes, const TriRecord*& tris, uint32_t& nodeCount) {
            const float4* rp = reinterpret_cast<const float4*>(rays + i);
            const float4 a = __ldg(rp), b = __ldg(rp + 1);
            r = TraceRay{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), a.w, b.w};
            nodes = sc.nodes;
            tris = sc.tris;
            nodeCount = sc.nodeCount;
        },
        [&](uint32_t i, const TraceHit& h) {
            const bool hit = h.mesh != VKRT_CUDA_INVALID_INDEX;
            float4* hp = reinterpret_cast<float4*>(hits + i);
            hp[0] = make_float4(__uint_as_float(h.mesh), __uint_as_float(h.prim), hit ? h.t : 0.0f, hit ? h.u : 0.0f);
            hp[1] = make_float4(hit ? h.v : 0.0f, 0.0f, 0.0f, 0.0f);
        },
        nodeVisits, triTests);
}

__global__ void kClearFilm(float4* a, float4* b, ushort4* out, size_t pixels) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= pixels) return;
    a[i] = f4(0.0f);
    b[i] = f4(0.0f);
    out[i] = make_ushort4(0, 0, 0, 0);
}

// ---- environment importance distribution (FP64 sums) ------------------------------------------------------------
__device__ __forceinline__ double texelLum(const float4* t, uint32_t W, int i, int j) {
    float4 p = __ldg(t + size_t(j) * W + size_t(i));
    double l = 0.2126 * double(p.x) + 0.7152 * double(p.y) + 0.0722 * double(p.z);
    return l > 0.0 ? l : 0.0;
}

__global__ void kEnvLumSum(const float4* t, uint32_t W, uint32_t H, double* sum) {
    double acc = 0.0;
    for (size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x; k < size_t(W) * H; k += size_t(gridDim.x) * blockDim.x)
        acc += texelLum(t, W, int(k % W), int(k / W));
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, off);
    if ((threadIdx.x & 31u) == 0u) atomicAdd(sum, acc);
}

__global__ void kEnvImportance(const float4* t, uint32_t W, uint32_t H, const double* lumSum, double* f) {
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= size_t(W) * H) return;
    int i = int(k % W), j = int(k / W);
    double mean = lumSum[0] / (double(W) * double(H));
    double m = 0.0;
    for (int dj = -1; dj <= 1; ++dj) {
        int jj = min(max(j + dj, 0), int(H) - 1);
        for (int di = -1; di <= 1; ++di) {
            int ii = ((i + di) % int(W) + int(W)) % int(W);
            m = fmax(m, texelLum(t, W, ii, jj));
        }
    }
    double sinT = sin(3.14159265358979323846 * (double(j) + 0.5) / double(H));
    f[k] = (m + 1e-3 * mean + 1e-12) * sinT;
}

// one block per row: inclusive FP64 prefix of the row -> conditional CDF, row sum -> rowSum[j]
__global__ void __launch_bounds__(1024) kEnvRows(const double* f, uint32_t W, float* conditional, double* rowSum) {
    __shared__ double warpTot[32];
    __shared__ double carry;
    const uint32_t j = blockIdx.x;
    const double* row = f + size_t(j) * W;
    if (threadIdx.x == 0) carry = 0.0;
    __syncthreads();
    // first pass: total
    double part = 0.0;
    for (uint32_t i = threadIdx.x; i < W; i += blockDim.x) part += row[i];
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, off);
    if ((threadIdx.x & 31u) == 0u) warpTot[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (uint32_t w = 0; w < (blockDim.x + 31u) / 32u; ++w) s += warpTot[w];
        rowSum[j] = s;
    }
    __syncthreads();
    const double total = rowSum[j];
    float* c = conditional + size_t(j) * (W + 1);
    if (threadIdx.x == 0) c[0] = 0.0f;
    for (uint32_t base = 0; base < W; base += blockDim.x) {
        uint32_t i = base + threadIdx.x;
        double v = i < W ? row[i] : 0.0;
        double x = v;
        for (int off = 1; off < 32; off <<= 1) {
            double y = __shfl_up_sync(0xFFFFFFFFu, x, off);
            if ((threadIdx.x & 31u) >= uint32_t(off)) x += y;
        }
        __syncthreads();
        if ((threadIdx.x & 31u) == 31u) warpTot[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32u) {
            double s = warpTot[threadIdx.x];
            for (int off = 1; off < 32; off <<= 1) {
                double y = __shfl_up_sync(0xFFFFFFFFu, s, off);
                if (threadIdx.x >= uint32_t(off)) s += y;
            }
            warpTot[threadIdx.x] = s;
        }
        __syncthreads();
        double incl = x + ((threadIdx.x >> 5) ? warpTot[(threadIdx.x >> 5) - 1u] : 0.0) + carry;
        if (i < W) c[i + 1] = float(incl / total);
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1u) carry = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) c[W] = 1.0f;
}

__global__ void kEnvMarginal(const double* rowSum, uint32_t H, float* marginal, double* totalOut) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double total = 0.0;
    for (uint32_t j = 0; j < H; ++j) total += rowSum[j];
    double acc = 0.0;
    marginal[0] = 0.0f;
    for (uint32_t j = 0; j < H; ++j) {
        acc += rowSum[j];
        marginal[j + 1] = float(acc / total);
    }
    marginal[H] = 1.0f;
    totalOut[0] = total;
}

// guide entry k of each CDF = search result for u = k / kEnvGuide (row H = the marginal)
__global__ void kEnvGuides(const float* marginal, const float* conditional, uint32_t W, uint32_t H,
                           uint32_t* marginalGuide, uint32_t* conditionalGuide) {
    const uint32_t G1 = kEnvGuide + 1u;
    const uint32_t total = (H + 1u) * G1;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        uint32_t row = t / G1, k = t % G1;
        float u = float(k) / float(kEnvGuide);
        if (row == H) marginalGuide[k] = cdfFind(marginal, H, u);
        else conditionalGuide[size_t(row) * G1 + k] = cdfFind(conditional + size_t(row) * (W + 1u), W, u);
    }
}

// the selected rgb2spec table repacked one float4 per cell
__global__ void kRepackRgb2Spec(const float* table, uint32_t res, uint32_t dataOffset, float4* cells) {
    const uint32_t n = 3u * res * res * res;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* c = table + dataOffset + size_t(i) * 3u;
        cells[i] = make_float4(c[0], c[1], c[2], 0.0f);
    }
}

// The brightness guide of a table (one block): entry b is the interval of b / kRgb2SpecGuide, found by the binary
// search itself; every entry is 0xFFFF when the scale is not non-decreasing, so lookups keep the binary search.
__global__ void __launch_bounds__(1024) kBuildRgb2SpecGuide(const float* table, uint32_t res, uint32_t scaleOffset,
                                                        uint16_t* guide) {
    __shared__ int monotone;
    if (threadIdx.x == 0) monotone = 1;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i + 1u < res; i += blockDim.x)
        if (!(table[scaleOffset + i] <= table[scaleOffset + i + 1u])) monotone = 0;
    __syncthreads();
    const SpecTable tab{table, res, scaleOffset, 0u, nullptr, nullptr};
    for (uint32_t b = threadIdx.x; b <= kRgb2SpecGuide; b += blockDim.x)
        guide[b] = monotone ? uint16_t(rgb2specIntervalSearch(tab, float(b) / float(kRgb2SpecGuide))) : 0xFFFFu;
}

__global__ void kEnvTexelPdf(const double* f, uint32_t W, uint32_t H, const double* total, float* pdf) {
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= size_t(W) * H) return;
    pdf[k] = float(f[k] / total[0] * double(W) * double(H));
}

// ---- rgb2spec fit on the device -------------------------------------------------------------------------------
// Jakob & Hanika 2019 per-cell Gauss-Newton, warm-started along the brightness axis. The device fit solves for the
// root of the linear-sRGB residual with the analytic Jacobian in FP32; quadrature weights (XYZ -> sRGB of the CIE
// fits, illuminant E, composite Simpson 3/8 over 283 samples) are prepared on the host in double.
constexpr int kFineSamples = 283;
__constant__ float4 cSpecQuad[kFineSamples];  // (t, w_r, w_g, w_b)

__device__ void reflectedRgbAndJacobian(const float c[3], float rgb[3], float J[9]) {
    for (int k = 0; k < 3; ++k) rgb[k] = 0.0f;
    for (int k = 0; k < 9; ++k) J[k] = 0.0f;
    for (int i = 0; i < kFineSamples; ++i) {
        float4 q = cSpecQuad[i];
        float t = q.x;
        float x = (c[0] * t + c[1]) * t + c[2];
        float r = rsqrtf(1.0f + x * x);
        float s = 0.5f * x * r + 0.5f;
        float ds = 0.5f * r * r * r;
        float w[3] = {q.y, q.z, q.w};
        float dx[3] = {t * t, t, 1.0f};
        for (int k = 0; k < 3; ++k) {
            rgb[k] += w[k] * s;
            for (int j = 0; j < 3; ++j) J[k * 3 + j] += w[k] * ds * dx[j];
        }
    }
}

__device__ bool solve3(const float J[9], const float r[3], float x[3]) {
    float a = J[0], b = J[1], c = J[2], d = J[3], e = J[4], f = J[5], g = J[6], h = J[7], i = J[8];
    float A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    float det = a * A + b * B + c * C;
    if (!(fabsf(det) > 1e-30f)) return false;
    float inv = 1.0f / det;
    float Ji[9] = {A * inv, -(b * i - c * h) * inv, (b * f - c * e) * inv, B * inv, (a * i - c * g) * inv,
                   -(a * f - c * d) * inv, C * inv, -(a * h - b * g) * inv, (a * e - b * d) * inv};
    for (int k = 0; k < 3; ++k) x[k] = Ji[k * 3] * r[0] + Ji[k * 3 + 1] * r[1] + Ji[k * 3 + 2] * r[2];
    return true;
}

__device__ float residualMax(const float c[3], const float target[3]) {
    float rgb[3], J[9];
    reflectedRgbAndJacobian(c, rgb, J);
    return fmaxf(fabsf(target[0] - rgb[0]), fmaxf(fabsf(target[1] - rgb[1]), fabsf(target[2] - rgb[2])));
}

// damped Gauss-Newton on the linear-sRGB residual (halving line search on the max-norm)
__device__ void solveCell(const float target[3], float c[3]) {
    for (int it = 0; it < 16; ++it) {
        float rgb[3], J[9];
        reflectedRgbAndJacobian(c, rgb, J);
        float r[3] = {target[0] - rgb[0], target[1] - rgb[1], target[2] - rgb[2]};
        float rn = fmaxf(fabsf(r[0]), fmaxf(fabsf(r[1]), fabsf(r[2])));
        if (rn < 1e-6f) break;
        float dc[3];
        if (!solve3(J, r, dc)) break;
        float step = 1.0f, trial[3];
        for (int ls = 0; ls < 10; ++ls, step *= 0.5f) {
            for (int q = 0; q < 3; ++q) trial[q] = c[q] + step * dc[q];
            float m = fmaxf(fabsf(trial[0]), fmaxf(fabsf(trial[1]), fabsf(trial[2])));
            if (m > 200.0f)
                for (int q = 0; q < 3; ++q) trial[q] *= 200.0f / m;
            if (residualMax(trial, target) < rn) break;
        }
        for (int q = 0; q < 3; ++q) c[q] = trial[q];
    }
}

__global__ void kRgb2SpecFit(uint32_t res, const float* scale, float* data) {
    uint32_t job = blockIdx.x * blockDim.x + threadIdx.x;
    if (job >= 3u * res * res) return;
    uint32_t l = job / (res * res), j = (job / res) % res, i = job % res;
    float x = float(i) / float(res - 1), y = float(j) / float(res - 1);
    const uint32_t start = res / 5;
    const double c0 = 360.0, c1 = 1.0 / 470.0;
    for (int pass = 0; pass < 2; ++pass) {
        float c[3] = {0.0f, 0.0f, 0.0f};
        int k = int(start), stop = pass == 0 ? int(res) : -1, step = pass == 0 ? 1 : -1;
        float bPrev = scale[start];
        for (int first = 1; k != stop; k += step, first = 0) {
            float b = scale[k];
            // homotopy in brightness: sub-steps of at most 0.02 from the previous level's solution
            int sub = first ? 1 : max(1, int(ceilf(fabsf(b - bPrev) / 0.02f)));
            for (int s = 1; s <= sub; ++s) {
                float bs = bPrev + (b - bPrev) * float(s) / float(sub);
                float target[3];
                target[l] = bs;
                target[(l + 1) % 3] = x * bs;
                target[(l + 2) % 3] = y * bs;
                solveCell(target, c);
            }
            bPrev = b;
            size_t idx = ((((size_t(l) * res + uint32_t(k)) * res + j) * res + i) * 3);
            // polynomial in nanometres from the one in normalised wavelength (FP32 products of FP64 constants)
            float A = c[0], B = c[1], C = c[2];
            data[idx + 0] = float(double(A) * c1 * c1);
            data[idx + 1] = float(double(B) * c1 - 2.0 * double(A) * c0 * c1 * c1);
            data[idx + 2] = float(double(C) - double(B) * c0 * c1 + double(A) * c0 * c0 * c1 * c1);
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------------------------
cudaError_t launchRender(const DeviceScene& sc, const VKRT_CudaSceneData& sd, const RenderParams& rp,
                         const FilmBuffers& film, RenderCounters* counters, uint32_t threadsPerBlock,
                         cudaStream_t stream) {
    (void)threadsPerBlock;
    const uint32_t threads = kDefaultThreads;
    const size_t pixels = size_t(rp.width) * rp.height;
    if (pixels == 0) return cudaSuccess;
    const uint32_t blocks = uint32_t((pixels + threads - 1) / threads);
    const size_t smem = size_t(threads) * VKRT_SMEM_STACK * sizeof(uint2);
    const bool spectral = VKRT_CUDA_RENDER_MODE_OF(sd.packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL;
    const bool features = film.albedoWrite != nullptr;
#define VKRT_MEGA(S, C, F, X) kRenderMega<S, C, F, X><<<blocks, threads, smem, stream>>>(sc, sd, rp, film, counters)
    // full stack when the materials need it, the feature-capturing plain kernel for feature films, else plain
    const bool full = rp.extended != 0u;
    if (spectral) {
        if (full) {
            if (rp.countBytes) VKRT_MEGA(true, true, true, true);
            else VKRT_MEGA(true, false, true, true);
        } else if (features) {
            if (rp.countBytes) VKRT_MEGA(true, true, false, true);
            else VKRT_MEGA(true, false, false, true);
        } else {
            if (rp.countBytes) VKRT_MEGA(true, true, false, false);
            else VKRT_MEGA(true, false, false, false);
        }
    } else {
        if (full) {
            if (rp.countBytes) VKRT_MEGA(false, true, true, true);
            else VKRT_MEGA(false, false, true, true);
        } else if (features) {
            if (rp.countBytes) VKRT_MEGA(false, true, false, true);
            else VKRT_MEGA(false, false, false, true);
        } else {
            if (rp.countBytes) VKRT_MEGA(false, true, false, false);
            else VKRT_MEGA(false, false, false, false);
        }
    }
#undef VKRT_MEGA
    return cudaGetLastError();
}

cudaError_t launchTraceRays(const DeviceScene& sc, const VKRT_CudaRay* rays, uint32_t count, uint32_t anyHit,
                            VKRT_CudaHit* hits, RenderCounters* counters, cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    const uint32_t threads = kDefaultThreads;
    const size_t smem = size_t(threads) * VKRT_SMEM_STACK * sizeof(uint2);
    const bool any = (anyHit & VKRT_CUDA_TRACE_ANY_HIT) != 0u;
    if (anyHit & VKRT_CUDA_TRACE_PERSISTENT) {
        int device = 0, sms = 0;
        cudaError_t e = cudaGetDevice(&device);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e == cudaSuccess) e = cudaMemsetAsync(&counters->workCursor, 0, sizeof(counters->workCursor), stream);
        if (e != cudaSuccess) return e;
        // persistent grid: 8 resident blocks of 128 per SM, as the wavefront's intersect stage
        const uint32_t grid = std::min(uint32_t(sms) * 8u, (count + threads - 1) / threads);
        if (any) kTraceRaysPersistent<true><<<grid, threads, smem, stream>>>(sc, rays, count, hits, counters);
        else kTraceRaysPersistent<false><<<grid, threads, smem, stream>>>(sc, rays, count, hits, counters);
        return cudaGetLastError();
    }
    const uint32_t blocks = (count + threads - 1) / threads;
    if (any) kTraceRays<true><<<blocks, threads, smem, stream>>>(sc, rays, count, hits, counters);
    else kTraceRays<false><<<blocks, threads, smem, stream>>>(sc, rays, count, hits, counters);
    return cudaGetLastError();
}

cudaError_t launchClearFilm(float4* a, float4* b, ushort4* out, size_t pixels, cudaStream_t stream) {
    if (pixels == 0) return cudaSuccess;
    kClearFilm<<<uint32_t((pixels + 255) / 256), 256, 0, stream>>>(a, b, out, pixels);
    return cudaGetLastError();
}

cudaError_t launchBuildEnvDistribution(const float4* texels, uint32_t W, uint32_t H, float* marginal,
                                       float* conditional, float* texelPdf, double* scratch, cudaStream_t stream) {
    double* f = scratch;
    double* rowSum = scratch + size_t(W) * H;
    double* lumSum = rowSum + H;
    double* total = lumSum + 1;
    cudaMemsetAsync(lumSum, 0, sizeof(double) * 2, stream);
    size_t n = size_t(W) * H;
    kEnvLumSum<<<256, 256, 0, stream>>>(texels, W, H, lumSum);
    kEnvImportance<<<uint32_t((n + 255) / 256), 256, 0, stream>>>(texels, W, H, lumSum, f);
    kEnvRows<<<H, 1024, 0, stream>>>(f, W, conditional, rowSum);
    kEnvMarginal<<<1, 32, 0, stream>>>(rowSum, H, marginal, total);
    kEnvTexelPdf<<<uint32_t((n + 255) / 256), 256, 0, stream>>>(f, W, H, total, texelPdf);
    return cudaGetLastError();
}

cudaError_t launchBuildEnvGuides(const float* marginal, const float* conditional, uint32_t W, uint32_t H,
                                 uint32_t* marginalGuide, uint32_t* conditionalGuide, cudaStream_t stream) {
    const uint32_t total = (H + 1u) * (kEnvGuide + 1u);
    kEnvGuides<<<(total + 255u) / 256u, 256, 0, stream>>>(marginal, conditional, W, H, marginalGuide,
                                                          conditionalGuide);
    return cudaGetLastError();
}

cudaError_t launchRepackRgb2Spec(const float* table, uint32_t res, uint32_t dataOffset, float4* cells,
                                 cudaStream_t stream) {
    const uint32_t n = 3u * res * res * res;
    kRepackRgb2Spec<<<(n + 255u) / 256u, 256, 0, stream>>>(table, res, dataOffset, cells);
    return cudaGetLastError();
}

cudaError_t launchRgb2SpecGuide(const float* table, uint32_t res, uint32_t scaleOffset, uint16_t* guide,
                                cudaStream_t stream) {
    if (res < 2 || res > 0xFFFFu) return cudaErrorInvalidValue;
    kBuildRgb2SpecGuide<<<1, 1024, 0, stream>>>(table, res, scaleOffset, guide);
    return cudaGetLastError();
}

cudaError_t launchGenerateRgb2Spec(uint32_t res, float* table, cudaStream_t stream) {
    if (res < 3) return cudaErrorInvalidValue;
    // host quadrature: XYZ (CIE 1931 fits, illuminant E, Y normalised to 1) -> vkrt's display sRGB
    auto cx = [](double l) {
        double t1 = (l - 442.0) * (l < 442.0 ? 0.0624 : 0.0374), t2 = (l - 599.8) * (l < 599.8 ? 0.0264 : 0.0323),
               t3 = (l - 501.1) * (l < 501.1 ? 0.0490 : 0.0382);
        return std::max(0.0, 0.362 * std::exp(-0.5 * t1 * t1) + 1.056 * std::exp(-0.5 * t2 * t2) -
                                 0.065 * std::exp(-0.5 * t3 * t3));
    };
    auto cy = [](double l) {
        double t1 = (l - 568.8) * (l < 568.8 ? 0.0213 : 0.0247), t2 = (l - 530.9) * (l < 530.9 ? 0.0613 : 0.0322);
        return std::max(0.0, 0.821 * std::exp(-0.5 * t1 * t1) + 0.286 * std::exp(-0.5 * t2 * t2));
    };
    auto cz = [](double l) {
        double t1 = (l - 437.0) * (l < 437.0 ? 0.0845 : 0.0278), t2 = (l - 459.0) * (l < 459.0 ? 0.0385 : 0.0725);
        return std::max(0.0, 1.217 * std::exp(-0.5 * t1 * t1) + 0.681 * std::exp(-0.5 * t2 * t2));
    };
    // M = XYZ->sRGB * BradfordInv * diag(E->D65) * Bradford
    const double S[9] = {3.2404542, -1.5371385, -0.4985314, -0.9692660, 1.8760108, 0.0415560, 0.0556434, -0.2040259, 1.0572252};
    const double Bf[9] = {0.8951, 0.2664, -0.1614, -0.7502, 1.7135, 0.0367, 0.0389, -0.0685, 1.0296};
    const double Bi[9] = {0.9869929, -0.1470543, 0.1599627, 0.4323053, 0.5183603, 0.0492912, -0.0085287, 0.0400428, 0.9684867};
    const double D[3] = {0.9413344, 1.0404175, 1.0895327};
    double T[9], U[9], M[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) T[r * 3 + c] = D[r] * Bf[r * 3 + c];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) U[r * 3 + c] = Bi[r * 3 + 0] * T[0 * 3 + c] + Bi[r * 3 + 1] * T[1 * 3 + c] + Bi[r * 3 + 2] * T[2 * 3 + c];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) M[r * 3 + c] = S[r * 3 + 0] * U[0 * 3 + c] + S[r * 3 + 1] * U[1 * 3 + c] + S[r * 3 + 2] * U[2 * 3 + c];
    const double h = 470.0 / double(kFineSamples - 1);
    std::vector<double> w(kFineSamples);
    double ySum = 0.0;
    for (int i = 0; i < kFineSamples; ++i) {
        double wt = 3.0 * h / 8.0 * ((i == 0 || i == kFineSamples - 1) ? 1.0 : (i % 3 == 0 ? 2.0 : 3.0));
        w[i] = wt;
        ySum += wt * cy(360.0 + h * i);
    }
    std::vector<float4> quad(kFineSamples);
    for (int i = 0; i < kFineSamples; ++i) {
        double l = 360.0 + h * i;
        double X = cx(l) * w[i] / ySum, Y = cy(l) * w[i] / ySum, Z = cz(l) * w[i] / ySum;
        quad[i] = make_float4(float((l - 360.0) / 470.0), float(M[0] * X + M[1] * Y + M[2] * Z),
                              float(M[3] * X + M[4] * Y + M[5] * Z), float(M[6] * X + M[7] * Y + M[8] * Z));
    }
    std::vector<float> scale(res);
    for (uint32_t k = 0; k < res; ++k) {
        double x = double(k) / double(res - 1);
        double s1 = x * x * (3.0 - 2.0 * x);
        scale[k] = float(s1 * s1 * (3.0 - 2.0 * s1));
    }
    cudaError_t err = cudaMemcpyToSymbolAsync(cSpecQuad, quad.data(), sizeof(float4) * kFineSamples, 0,
                                              cudaMemcpyHostToDevice, stream);
    if (err != cudaSuccess) return err;
    err = cudaMemcpyAsync(table, scale.data(), sizeof(float) * res, cudaMemcpyHostToDevice, stream);
    if (err != cudaSuccess) return err;
    uint32_t jobs = 3u * res * res;
    kRgb2SpecFit<<<(jobs + 63) / 64, 64, 0, stream>>>(res, table, table + res);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    return cudaStreamSynchronize(stream);  // the host quadrature buffers above go out of scope
}

}  // namespace vkrt
