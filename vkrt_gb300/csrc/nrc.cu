// nrc.cu — neural radiance cache on sm_103a: hash-grid encoding, fused FP16 tensor-core MLP forward and backward
// (FP32 accumulation), weight-gradient reductions, hash-table gradient scatter and Adam.
//
// Training step on n records (inputs + radiance targets), relative L2 loss of Mueller et al. 2021
// ("Real-time Neural Radiance Caching for Path Tracing"): L = mean over records and RGB of
// (y - t)^2 / (sg(y)^2 + 0.01), sg = stop-gradient.
//   encode      n x 64 FP16 inputs from the current table
//   forward     fused 6-layer MLP per 16-row tile, weights in shared memory, activations in registers; stores the
//               five hidden activations, the outputs and dL/dy (scaled by n, so FP16 keeps its precision)
//   backward    fused: dZ of every hidden layer (masked by the stored activations), dL/dx of the 32 hash inputs
//   dW          per layer, dW = dZ^T X as a tensor-core reduction over the records, FP32 atomics
//   table grad  trilinear scatter of dL/dx into the FP32 table gradient
//   Adam        FP32 masters and moments, FP16 working copies
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "nrc.h"

namespace vkrt {

namespace {

constexpr uint32_t kThreads = 128;
constexpr uint32_t kFwdSmemHalves = 5u * 64u * 72u + 16u * 72u;  // row stride 72 halves: conflict-free B loads
constexpr uint32_t kBwdSmemHalves = 5u * 64u * 72u + 64u * 24u;  // transposed weights
constexpr uint32_t kWdChunk = 1024;                              // records per weight-gradient block

VKRT_DEV uint32_t ld32(const __half* p) { return *reinterpret_cast<const uint32_t*>(p); }
VKRT_DEV void st32(__half* p, uint32_t v) { *reinterpret_cast<uint32_t*>(p) = v; }
VKRT_DEV uint32_t pack2(__half lo, __half hi) {
    __half2 h = __halves2half2(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}

VKRT_DEV uint32_t hashU32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
VKRT_DEV float hashUniform(uint32_t seed, uint32_t i) {
    return float(hashU32(hashU32(seed) ^ (i * 0x9e3779b9u) ^ 0x85ebca6bu) >> 8) * (1.0f / 16777216.0f);
}

// weights: He-uniform hidden layers, small output layer with rows 3..15 zero; table: uniform +-1e-4
__global__ void kNrcInit(float* wMaster, __half* wHalf, float* tMaster, __half* tHalf, uint32_t seed) {
    const uint32_t total = kNrcWeightCount + kNrcTableParams;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        if (i < kNrcWeightCount) {
            float bound = sqrtf(6.0f / 64.0f);
            float v = (2.0f * hashUniform(seed, i) - 1.0f) * bound;
            if (i >= 20480u) v = ((i - 20480u) / 64u) < 3u ? v * 0.1f : 0.0f;
            wMaster[i] = v;
            wHalf[i] = __float2half_rn(v);
        } else {
            uint32_t k = i - kNrcWeightCount;
            float v = (2.0f * hashUniform(seed ^ 0x5bd1e995u, k) - 1.0f) * 1e-4f;
            tMaster[k] = v;
            tHalf[k] = __float2half_rn(v);
        }
    }
}

__global__ void kHalfToFloat(const __half* src, float* dst, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dst[i] = __half2float(src[i]);
}

__global__ void kNrcEncode(NrcGridInfo gi, const __half2* __restrict__ table, const NrcInput* __restrict__ in,
                           const uint32_t* count, uint32_t cap, __half* __restrict__ x0) {
    const uint32_t n = count ? min(*count, cap) : cap;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        __align__(16) __half row[64];
        nrcEncode(gi, table, in[r], row);
        const uint4* s = reinterpret_cast<const uint4*>(row);
        uint4* d = reinterpret_cast<uint4*>(x0 + size_t(r) * 64u);
#pragma unroll
        for (int k = 0; k < 8; ++k) d[k] = s[k];
    }
}

// Fused forward. kTrain: also stores the hidden activations (acts, 5 x cap x 64), dL/dy (dy, cap x 16) and the loss.
template <bool kTrain>
__global__ void __launch_bounds__(kThreads) kNrcForward(const __half* __restrict__ W, const __half* __restrict__ x0,
                                                        const uint32_t* count, uint32_t cap, float4* __restrict__ out,
                                                        __half* __restrict__ acts, const float4* __restrict__ targets,
                                                        __half* __restrict__ dy, float* __restrict__ loss) {
    extern __shared__ __half wsm[];
    for (uint32_t i = threadIdx.x; i < kNrcWeightCount / 2u; i += blockDim.x) {
        const uint32_t e = 2u * i;
        const uint32_t layer = e < 20480u ? e / 4096u : 5u;
        const uint32_t within = e < 20480u ? e % 4096u : e - 20480u;
        st32(wsm + layer * 4608u + (within / 64u) * 72u + within % 64u, ld32(W + e));
    }
    __syncthreads();
    const uint32_t n = count ? min(*count, cap) : cap;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    float lossAcc = 0.0f;
    for (uint32_t tile = blockIdx.x * 4u + warp; tile * 16u < n; tile += gridDim.x * 4u) {
        const uint32_t ra = tile * 16u + g, rb = ra + 8u;
        const bool va = ra < n, vb = rb < n;
        uint32_t a[4][4];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            a[s][0] = va ? ld32(x0 + size_t(ra) * 64u + 16u * s + 2u * t) : 0u;
            a[s][1] = vb ? ld32(x0 + size_t(rb) * 64u + 16u * s + 2u * t) : 0u;
            a[s][2] = va ? ld32(x0 + size_t(ra) * 64u + 16u * s + 8u + 2u * t) : 0u;
            a[s][3] = vb ? ld32(x0 + size_t(rb) * 64u + 16u * s + 8u + 2u * t) : 0u;
        }
#pragma unroll 1
        for (int l = 0; l < kNrcHidden; ++l) {
            float acc[8][4];
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
            const __half* wl = wsm + l * 4608;
#pragma unroll
            for (int s = 0; s < 4; ++s)
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const __half* wr = wl + (8u * j + g) * 72u + 16u * s + 2u * t;
                    mma16816(acc[j], a[s], ld32(wr), ld32(wr + 8));
                }
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                a[s][0] = packHalf2(fmaxf(acc[2 * s][0], 0.0f), fmaxf(acc[2 * s][1], 0.0f));
                a[s][1] = packHalf2(fmaxf(acc[2 * s][2], 0.0f), fmaxf(acc[2 * s][3], 0.0f));
                a[s][2] = packHalf2(fmaxf(acc[2 * s + 1][0], 0.0f), fmaxf(acc[2 * s + 1][1], 0.0f));
                a[s][3] = packHalf2(fmaxf(acc[2 * s + 1][2], 0.0f), fmaxf(acc[2 * s + 1][3], 0.0f));
            }
            if (kTrain) {
                __half* dst = acts + size_t(l) * cap * 64u;
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    if (va) {
                        st32(dst + size_t(ra) * 64u + 16u * s + 2u * t, a[s][0]);
                        st32(dst + size_t(ra) * 64u + 16u * s + 8u + 2u * t, a[s][2]);
                    }
                    if (vb) {
                        st32(dst + size_t(rb) * 64u + 16u * s + 2u * t, a[s][1]);
                        st32(dst + size_t(rb) * 64u + 16u * s + 8u + 2u * t, a[s][3]);
                    }
                }
            }
        }
        float y[2][4];
#pragma unroll
        for (int j = 0; j < 2; ++j) y[j][0] = y[j][1] = y[j][2] = y[j][3] = 0.0f;
        const __half* w5 = wsm + 5 * 4608;
#pragma unroll
        for (int s = 0; s < 4; ++s)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const __half* wr = w5 + (8u * j + g) * 72u + 16u * s + 2u * t;
                mma16816(y[j], a[s], ld32(wr), ld32(wr + 8));
            }
        // outputs: columns 0..3 live in tile j = 0 on lanes t = 0, 1
        if (t <= 1u) {
            if (va) {
                reinterpret_cast<float*>(out + ra)[2u * t] = y[0][0];
                reinterpret_cast<float*>(out + ra)[2u * t + 1u] = y[0][1];
            }
            if (vb) {
                reinterpret_cast<float*>(out + rb)[2u * t] = y[0][2];
                reinterpret_cast<float*>(out + rb)[2u * t + 1u] = y[0][3];
            }
        }
        if (kTrain) {
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint32_t row = h ? rb : ra;
                    if (!(h ? vb : va)) continue;
                    __half d[2];
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const uint32_t c = 8u * j + 2u * t + e;
                        float grad = 0.0f;
                        if (c < 3u) {
                            const float yv = y[j][2 * h + e];
                            const float tv = reinterpret_cast<const float*>(targets + row)[c];
                            const float den = yv * yv + 0.01f, diff = yv - tv;
                            lossAcc += diff * diff / den;
                            grad = fminf(fmaxf(2.0f * diff / (3.0f * den), -1024.0f), 1024.0f);
                        }
                        d[e] = __float2half_rn(grad);
                    }
                    st32(dy + size_t(row) * 16u + 8u * j + 2u * t, pack2(d[0], d[1]));
                }
        }
    }
    if (kTrain && loss) {
        for (int off = 16; off > 0; off >>= 1) lossAcc += __shfl_xor_sync(0xFFFFFFFFu, lossAcc, off);
        if (lane == 0u && lossAcc != 0.0f) atomicAdd(loss, lossAcc / (3.0f * float(max(n, 1u))));
    }
}

// Fused backward: dZ of the five hidden layers (dz, 5 x cap x 64) and dL/dx of the 32 hash inputs (dx0, cap x 32).
__global__ void __launch_bounds__(kThreads) kNrcBackward(const __half* __restrict__ W, const __half* __restrict__ acts,
                                                         const __half* __restrict__ dy, uint32_t n, uint32_t cap,
                                                         __half* __restrict__ dz, float* __restrict__ dx0) {
    extern __shared__ __half wt[];  // transposed: [in][out], stride 72 (hidden), 24 (output layer)
    for (uint32_t e = threadIdx.x; e < kNrcWeightCount; e += blockDim.x) {
        const uint32_t layer = e < 20480u ? e / 4096u : 5u;
        const uint32_t within = e < 20480u ? e % 4096u : e - 20480u;
        const uint32_t o = within / 64u, i = within % 64u;
        wt[layer < 5u ? layer * 4608u + i * 72u + o : 5u * 4608u + i * 24u + o] = W[e];
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    for (uint32_t tile = blockIdx.x * 4u + warp; tile * 16u < n; tile += gridDim.x * 4u) {
        const uint32_t ra = tile * 16u + g, rb = ra + 8u;
        const bool va = ra < n, vb = rb < n;
        uint32_t a[4][4];
        a[0][0] = va ? ld32(dy + size_t(ra) * 16u + 2u * t) : 0u;
        a[0][1] = vb ? ld32(dy + size_t(rb) * 16u + 2u * t) : 0u;
        a[0][2] = va ? ld32(dy + size_t(ra) * 16u + 8u + 2u * t) : 0u;
        a[0][3] = vb ? ld32(dy + size_t(rb) * 16u + 8u + 2u * t) : 0u;
        float acc[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
            const __half* wr = wt + 5u * 4608u + (8u * j + g) * 24u + 2u * t;
            mma16816(acc[j], a[0], ld32(wr), ld32(wr + 8));
        }
#pragma unroll 1
        for (int l = kNrcHidden - 1; l >= 0; --l) {
            // dZ = dX (in acc) masked by the layer's ReLU output
            const __half* x = acts + size_t(l) * cap * 64u;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const uint32_t c = 8u * j + 2u * t;
                const float2 xa = va ? unpackHalf2(ld32(x + size_t(ra) * 64u + c)) : make_float2(0.0f, 0.0f);
                const float2 xb = vb ? unpackHalf2(ld32(x + size_t(rb) * 64u + c)) : make_float2(0.0f, 0.0f);
                acc[j][0] = xa.x > 0.0f ? acc[j][0] : 0.0f;
                acc[j][1] = xa.y > 0.0f ? acc[j][1] : 0.0f;
                acc[j][2] = xb.x > 0.0f ? acc[j][2] : 0.0f;
                acc[j][3] = xb.y > 0.0f ? acc[j][3] : 0.0f;
            }
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                a[s][0] = packHalf2(acc[2 * s][0], acc[2 * s][1]);
                a[s][1] = packHalf2(acc[2 * s][2], acc[2 * s][3]);
                a[s][2] = packHalf2(acc[2 * s + 1][0], acc[2 * s + 1][1]);
                a[s][3] = packHalf2(acc[2 * s + 1][2], acc[2 * s + 1][3]);
            }
            __half* d = dz + size_t(l) * cap * 64u;
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                if (va) {
                    st32(d + size_t(ra) * 64u + 16u * s + 2u * t, a[s][0]);
                    st32(d + size_t(ra) * 64u + 16u * s + 8u + 2u * t, a[s][2]);
                }
                if (vb) {
                    st32(d + size_t(rb) * 64u + 16u * s + 2u * t, a[s][1]);
                    st32(d + size_t(rb) * 64u + 16u * s + 8u + 2u * t, a[s][3]);
                }
            }
            // dX of the layer's input = dZ * W (K = out, N = in)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
            const __half* wl = wt + l * 4608;
#pragma unroll
            for (int s = 0; s < 4; ++s)
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const __half* wr = wl + (8u * j + g) * 72u + 16u * s + 2u * t;
                    mma16816(acc[j], a[s], ld32(wr), ld32(wr + 8));
                }
        }
        // acc = dL/dX0; the hash features are columns 0..31
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t c = 8u * j + 2u * t;
            if (va) {
                dx0[size_t(ra) * 32u + c] = acc[j][0];
                dx0[size_t(ra) * 32u + c + 1u] = acc[j][1];
            }
            if (vb) {
                dx0[size_t(rb) * 32u + c] = acc[j][2];
                dx0[size_t(rb) * 32u + c + 1u] = acc[j][3];
            }
        }
    }
}

// dW of layer blockIdx.y over records [blockIdx.x * kWdChunk, +kWdChunk): dW[o][i] += sum_r dZ[r][o] X[r][i] / n
__global__ void __launch_bounds__(kThreads) kNrcWeightGrad(const __half* __restrict__ x0, const __half* __restrict__ acts,
                                                           const __half* __restrict__ dz, const __half* __restrict__ dy,
                                                           uint32_t n, uint32_t cap, float* __restrict__ dW) {
    const uint32_t layer = blockIdx.y;
    const __half* D = layer < 5u ? dz + size_t(layer) * cap * 64u : dy;
    const uint32_t dStride = layer < 5u ? 64u : 16u, M = layer < 5u ? 64u : 16u;
    const __half* X = layer == 0u ? x0 : acts + size_t(layer - 1u) * cap * 64u;
    float* out = dW + layer * 4096u;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    const uint32_t o0 = 16u * warp;
    if (o0 >= M) return;
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const uint32_t r0 = blockIdx.x * kWdChunk, r1 = min(r0 + kWdChunk, n);
    auto h = [&](const __half* p, uint32_t stride, uint32_t r, uint32_t c) {
        return r < r1 ? p[size_t(r) * stride + c] : __float2half_rn(0.0f);
    };
    for (uint32_t k0 = r0; k0 < r1; k0 += 16u) {
        uint32_t a[4];
        a[0] = pack2(h(D, dStride, k0 + 2u * t, o0 + g), h(D, dStride, k0 + 2u * t + 1u, o0 + g));
        a[1] = pack2(h(D, dStride, k0 + 2u * t, o0 + g + 8u), h(D, dStride, k0 + 2u * t + 1u, o0 + g + 8u));
        a[2] = pack2(h(D, dStride, k0 + 2u * t + 8u, o0 + g), h(D, dStride, k0 + 2u * t + 9u, o0 + g));
        a[3] = pack2(h(D, dStride, k0 + 2u * t + 8u, o0 + g + 8u), h(D, dStride, k0 + 2u * t + 9u, o0 + g + 8u));
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = 8u * j + g;
            const uint32_t b0 = pack2(h(X, 64u, k0 + 2u * t, i), h(X, 64u, k0 + 2u * t + 1u, i));
            const uint32_t b1 = pack2(h(X, 64u, k0 + 2u * t + 8u, i), h(X, 64u, k0 + 2u * t + 9u, i));
            mma16816(acc[j], a, b0, b1);
        }
    }
    const float inv = 1.0f / float(max(n, 1u));
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t c = 8u * j + 2u * t;
        atomicAdd(out + (o0 + g) * 64u + c, acc[j][0] * inv);
        atomicAdd(out + (o0 + g) * 64u + c + 1u, acc[j][1] * inv);
        atomicAdd(out + (o0 + g + 8u) * 64u + c, acc[j][2] * inv);
        atomicAdd(out + (o0 + g + 8u) * 64u + c + 1u, acc[j][3] * inv);
    }
}

__global__ void kNrcTableGrad(NrcGridInfo gi, const NrcInput* __restrict__ in, const float* __restrict__ dx0,
                              uint32_t n, float* __restrict__ tGrad) {
    const float inv = 1.0f / float(max(n, 1u));
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const float3 u = nrcUnit(gi, xyz(in[r].posRough));
        for (int l = 0; l < kNrcLevels; ++l) {
            const float d0 = dx0[size_t(r) * 32u + 2u * l] * inv, d1 = dx0[size_t(r) * 32u + 2u * l + 1u] * inv;
            if (d0 == 0.0f && d1 == 0.0f) continue;
            uint32_t c[3];
            float f[3];
            nrcCell(gi, l, u, c, f);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const uint32_t dx = k & 1u, dy = (k >> 1) & 1u, dzz = (k >> 2) & 1u;
                const float w = (dx ? f[0] : 1.0f - f[0]) * (dy ? f[1] : 1.0f - f[1]) * (dzz ? f[2] : 1.0f - f[2]);
                const size_t e = (size_t(l) * kNrcTable + nrcIndex(gi, l, c[0] + dx, c[1] + dy, c[2] + dzz)) * 2u;
                atomicAdd(tGrad + e, w * d0);
                atomicAdd(tGrad + e + 1u, w * d1);
            }
        }
    }
}

__global__ void kNrcAdam(float* __restrict__ master, float* __restrict__ m, float* __restrict__ v,
                         const float* __restrict__ grad, __half* __restrict__ half, uint32_t count, float lr, float b1,
                         float b2, float eps, float bc1, float bc2) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float gr = grad[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gr;
        const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        const float w = master[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        master[i] = w;
        half[i] = __float2half_rn(w);
    }
}

template <class T>
cudaError_t alloc(T*& p, size_t n) {
    if (p) cudaFree(p);
    p = nullptr;
    return cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1));
}

uint32_t gridFor(uint32_t work, uint32_t per) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint32_t want = (work + per - 1u) / per;
    return std::max(1u, std::min(want, uint32_t(std::max(sms, 1)) * 8u));
}

}  // namespace

NrcEngine::NrcEngine() {}

NrcEngine::~NrcEngine() {
    void* ptrs[] = {wHalf_, wMaster_, wM_,  wV_, wGrad_, table_, tMaster_,  tM_,
                    tV_,    tGrad_,   x0_,  acts_, dz_,  dy_,   dx0_,   out_, x0Infer_};
    for (void* p : ptrs)
        if (p) cudaFree(p);
}

cudaError_t NrcEngine::reset(const NrcSettings& s, float3 lo, float3 hi, cudaStream_t stream) {
    s_ = s;
    step_ = 0;
    grid_.lo = lo;
    float3 ext = make_float3(fmaxf(hi.x - lo.x, 1e-6f), fmaxf(hi.y - lo.y, 1e-6f), fmaxf(hi.z - lo.z, 1e-6f));
    grid_.invExtent = make_float3(1.0f / ext.x, 1.0f / ext.y, 1.0f / ext.z);
    for (int l = 0; l < kNrcLevels; ++l) {
        double res = std::floor(double(kNrcBaseRes) * std::pow(double(kNrcGrowth), double(l)));
        grid_.res[l] = uint32_t(res);
        double cells = (res + 1.0) * (res + 1.0) * (res + 1.0);
        grid_.dense[l] = cells <= double(kNrcTable) ? 1u : 0u;
    }
    cudaError_t e = cudaSuccess;
    if (!wHalf_) {
        if (e == cudaSuccess) e = alloc(wHalf_, kNrcWeightCount);
        if (e == cudaSuccess) e = alloc(wMaster_, kNrcWeightCount);
        if (e == cudaSuccess) e = alloc(wM_, kNrcWeightCount);
        if (e == cudaSuccess) e = alloc(wV_, kNrcWeightCount);
        if (e == cudaSuccess) e = alloc(wGrad_, kNrcWeightCount);
        if (e == cudaSuccess) e = alloc(table_, kNrcTableParams / 2u);
        if (e == cudaSuccess) e = alloc(tMaster_, kNrcTableParams);
        if (e == cudaSuccess) e = alloc(tM_, kNrcTableParams);
        if (e == cudaSuccess) e = alloc(tV_, kNrcTableParams);
        if (e == cudaSuccess) e = alloc(tGrad_, kNrcTableParams);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(kNrcForward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(kFwdSmemHalves * sizeof(__half)));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kNrcForward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(kFwdSmemHalves * sizeof(__half)));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kNrcBackward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(kBwdSmemHalves * sizeof(__half)));
        if (e != cudaSuccess) return e;
    }
    cudaMemsetAsync(wM_, 0, sizeof(float) * kNrcWeightCount, stream);
    cudaMemsetAsync(wV_, 0, sizeof(float) * kNrcWeightCount, stream);
    cudaMemsetAsync(wGrad_, 0, sizeof(float) * kNrcWeightCount, stream);
    cudaMemsetAsync(tM_, 0, sizeof(float) * kNrcTableParams, stream);
    cudaMemsetAsync(tV_, 0, sizeof(float) * kNrcTableParams, stream);
    cudaMemsetAsync(tGrad_, 0, sizeof(float) * kNrcTableParams, stream);
    kNrcInit<<<gridFor(kNrcWeightCount + kNrcTableParams, 256), 256, 0, stream>>>(
        wMaster_, wHalf_, tMaster_, reinterpret_cast<__half*>(table_), s.seed);
    return cudaGetLastError();
}

cudaError_t NrcEngine::syncMasters(cudaStream_t stream) {
    kHalfToFloat<<<gridFor(kNrcWeightCount, 256), 256, 0, stream>>>(wHalf_, wMaster_, kNrcWeightCount);
    kHalfToFloat<<<gridFor(kNrcTableParams, 256), 256, 0, stream>>>(reinterpret_cast<const __half*>(table_), tMaster_,
                                                                    kNrcTableParams);
    return cudaGetLastError();
}

cudaError_t NrcEngine::ensureScratch(uint32_t n) {
    if (n <= cap_ && x0_) return cudaSuccess;
    cudaError_t e = alloc(x0_, size_t(n) * 64u);
    if (e == cudaSuccess) e = alloc(acts_, size_t(kNrcHidden) * n * 64u);
    if (e == cudaSuccess) e = alloc(dz_, size_t(kNrcHidden) * n * 64u);
    if (e == cudaSuccess) e = alloc(dy_, size_t(n) * 16u);
    if (e == cudaSuccess) e = alloc(dx0_, size_t(n) * 32u);
    if (e == cudaSuccess) e = alloc(out_, n);
    if (e == cudaSuccess) cap_ = n;
    return e;
}

cudaError_t NrcEngine::reserveInference(uint32_t capacity) {
    if (capacity <= capInfer_ && x0Infer_) return cudaSuccess;
    cudaError_t e = alloc(x0Infer_, size_t(capacity) * 64u);
    if (e == cudaSuccess) capInfer_ = capacity;
    return e;
}

cudaError_t NrcEngine::infer(const NrcInput* inputs, uint32_t n, float4* out, cudaStream_t stream) {
    return inferCounted(inputs, nullptr, n, out, stream);
}

cudaError_t NrcEngine::inferCounted(const NrcInput* inputs, const uint32_t* count, uint32_t capacity, float4* out,
                                    cudaStream_t stream) {
    if (capacity == 0) return cudaSuccess;
    cudaError_t e = reserveInference(capacity);
    if (e != cudaSuccess) return e;
    kNrcEncode<<<gridFor(capacity, 128), 128, 0, stream>>>(grid_, table_, inputs, count, capacity, x0Infer_);
    kNrcForward<false><<<gridFor(capacity, 64), kThreads, kFwdSmemHalves * sizeof(__half), stream>>>(
        wHalf_, x0Infer_, count, capacity, out, nullptr, nullptr, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t NrcEngine::train(const NrcInput* inputs, const float4* targets, uint32_t n, float* lossOut,
                             bool applyUpdate, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = ensureScratch(n);
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(wGrad_, 0, sizeof(float) * kNrcWeightCount, stream);
    cudaMemsetAsync(tGrad_, 0, sizeof(float) * kNrcTableParams, stream);
    kNrcEncode<<<gridFor(n, 128), 128, 0, stream>>>(grid_, table_, inputs, nullptr, n, x0_);
    kNrcForward<true><<<gridFor(n, 64), kThreads, kFwdSmemHalves * sizeof(__half), stream>>>(
        wHalf_, x0_, nullptr, n, out_, acts_, targets, dy_, lossOut);
    kNrcBackward<<<gridFor(n, 64), kThreads, kBwdSmemHalves * sizeof(__half), stream>>>(wHalf_, acts_, dy_, n, n,
                                                                                        dz_, dx0_);
    // the scratch layout uses cap_ as the row stride of acts / dz; train() always allocates with n <= cap_ and
    // writes with stride n, so pass n as the stride to every kernel of this step
    dim3 wg((n + kWdChunk - 1u) / kWdChunk, kNrcLayers);
    kNrcWeightGrad<<<wg, kThreads, 0, stream>>>(x0_, acts_, dz_, dy_, n, n, wGrad_);
    kNrcTableGrad<<<gridFor(n, 128), 128, 0, stream>>>(grid_, inputs, dx0_, n, tGrad_);
    if (applyUpdate) {
        ++step_;
        const float bc1 = 1.0f - std::pow(s_.beta1, float(step_)), bc2 = 1.0f - std::pow(s_.beta2, float(step_));
        kNrcAdam<<<gridFor(kNrcWeightCount, 256), 256, 0, stream>>>(wMaster_, wM_, wV_, wGrad_, wHalf_,
                                                                    kNrcWeightCount, s_.learningRate, s_.beta1,
                                                                    s_.beta2, s_.epsilon, bc1, bc2);
        kNrcAdam<<<gridFor(kNrcTableParams, 256), 256, 0, stream>>>(tMaster_, tM_, tV_, tGrad_,
                                                                    reinterpret_cast<__half*>(table_), kNrcTableParams,
                                                                    s_.learningRate, s_.beta1, s_.beta2, s_.epsilon,
                                                                    bc1, bc2);
    }
    return cudaGetLastError();
}

}  // namespace vkrt
