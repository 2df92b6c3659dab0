// nrc.cu — neural radiance cache on sm_103a: hash-grid encoding, fused FP16 tensor-core MLP forward and backward
// (FP32 accumulation), weight-gradient reductions, hash-table gradient scatter and Adam.
//
// Training step on n records (inputs + radiance targets), relative L2 loss of Mueller et al. 2021
// ("Real-time Neural Radiance Caching for Path Tracing"): L = mean over records and RGB of
// (y - t)^2 / (sg(y)^2 + 0.01), sg = stop-gradient.
//   encode      n x 64 FP16 inputs from the current table, one thread per (record, level)
//   forward     fused 6-layer MLP per 16-row tile, weights in shared memory, activations in registers; stores the
//               five hidden activations, their ReLU masks, the outputs and dL/dy (scaled by n, so FP16 keeps its
//               precision)
//   backward    fused: dZ of every hidden layer (masked), dL/dx of the 32 hash inputs
//   dW          per layer, dW = dZ^T X as a tensor-core reduction over the records (cp.async slabs, transposed
//               ldmatrix), FP32 atomics
//   table grad  trilinear scatter of dL/dx into the FP32 table gradient, one thread per (record, level)
//   Adam        FP32 masters and moments, FP16 working copies; dense for the weights, sparse for the table
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "nrc.h"
#include "umma.cuh"

namespace vkrt {

namespace {

constexpr uint32_t kMlpThreads = 256;      // eight warps, one 16-row tile each per pass
constexpr uint32_t kMlpBlocksPerSM = 4;    // 48 KB of staged weights per block
constexpr uint32_t kWStride = 72;          // shared-memory row stride of a weight matrix (halves)
constexpr uint32_t kLayerHalves = 64u * kWStride;
constexpr uint32_t kMlpSmemBytes = (5u * kLayerHalves + 16u * kWStride) * sizeof(__half);  // 48,384
constexpr uint32_t kWgThreads = 256;
constexpr uint32_t kWgChunk = 1024;        // records per weight-gradient block
constexpr uint32_t kWgSlab = 64;           // records per staged slab
constexpr uint32_t kWgStages = 3;          // slabs in flight per block
constexpr uint32_t kWgSlabHalves = 2u * kWgSlab * kWStride;  // dZ slab + X slab
constexpr uint32_t kWgSmemBytes = kWgStages * kWgSlabHalves * sizeof(__half);  // 55,296
static_assert(kWgSmemBytes >= 8u * 16u * 72u * sizeof(float), "the reduction reuses the slab buffers");

VKRT_DEV uint32_t ld32(const __half* p) { return *reinterpret_cast<const uint32_t*>(p); }
VKRT_DEV void st32(__half* p, uint32_t v) { *reinterpret_cast<uint32_t*>(p) = v; }
VKRT_DEV uint32_t pack2(__half lo, __half hi) {
    __half2 h = __halves2half2(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}

// 16-byte asynchronous global -> shared copy; ok = false writes zeros and reads nothing
VKRT_DEV void cpAsync16(__half* dst, const __half* src, bool ok) {
    const uint32_t d = uint32_t(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 16 : 0));
}
VKRT_DEV void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int kPending>
VKRT_DEV void cpAsyncWait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(kPending));
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

// One thread per (record, level): the level's two hash features and one pair of the remaining inputs. Sixteen
// threads share a record, so the table gathers of a warp come from two records' sixteen levels.
__global__ void kNrcEncode(NrcGridInfo gi, const __half2* __restrict__ table, const NrcInput* __restrict__ in,
                           const uint32_t* count, uint32_t cap, __half* __restrict__ x0) {
    const uint32_t n = count ? min(*count, cap) : cap;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n * 16u; i += gridDim.x * blockDim.x) {
        const uint32_t r = i >> 4, l = i & 15u;
        const NrcInput v = in[r];
        __half2* row = reinterpret_cast<__half2*>(x0 + size_t(r) * 64u);
        row[l] = nrcEncodeLevel(gi, table, nrcUnit(gi, xyz(v.posRough)), int(l));
        row[16u + l] = nrcEncodeTail(v, int(l));
    }
}

// All six weight matrices into shared memory, row r of the concatenated matrices at r * kWStride (16-byte copies).
VKRT_DEV void stageWeights(__half* wsm, const __half* __restrict__ W) {
    for (uint32_t i = threadIdx.x; i < (kNrcWeightCount / 64u) * 8u; i += blockDim.x) {
        const uint32_t row = i >> 3, piece = i & 7u;
        *reinterpret_cast<uint4*>(wsm + row * kWStride + piece * 8u) = reinterpret_cast<const uint4*>(W)[i];
    }
    __syncthreads();
}

// Fused forward. kTrain: also stores the hidden activations (acts, 5 x cap x 64) for the weight gradients, the ReLU
// masks (masks, 5 x tiles x 32 words: lane L of a tile's warp keeps bit 4j + q for its C-fragment element acc[j][q])
// for the backward pass, dL/dy (dy, cap x 16) and the loss.
template <bool kTrain>
__global__ void __launch_bounds__(kMlpThreads, kMlpBlocksPerSM)
    kNrcForward(const __half* __restrict__ W, const __half* __restrict__ x0, const uint32_t* count, uint32_t cap,
                float4* __restrict__ out, __half* __restrict__ acts, uint32_t* __restrict__ masks,
                const float4* __restrict__ targets, __half* __restrict__ dy, float* __restrict__ loss) {
    extern __shared__ __align__(16) __half wsm[];
    stageWeights(wsm, W);
    const uint32_t n = count ? min(*count, cap) : cap;
    const uint32_t tiles = (cap + 15u) / 16u;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    // B fragments of two adjacent 8-output tiles: rows (outputs) lane % 8 + 8 * (lane / 16), columns + 8 * bit 3
    const uint32_t bOff = ((lane & 7u) + 8u * (lane >> 4)) * kWStride + 8u * ((lane >> 3) & 1u);
    float lossAcc = 0.0f;
    for (uint32_t tile = blockIdx.x * warps + warp; tile * 16u < n; tile += gridDim.x * warps) {
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
            const __half* wl = wsm + l * kLayerHalves + bOff;
#pragma unroll
            for (int s = 0; s < 4; ++s)
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    uint32_t b[4];
                    ldsm4(b, wl + jj * 16u * kWStride + 16u * s);
                    mma16816(acc[2 * jj], a[s], b[0], b[1]);
                    mma16816(acc[2 * jj + 1], a[s], b[2], b[3]);
                }
            if (kTrain) {
                uint32_t mask = 0u;
#pragma unroll
                for (int j = 0; j < 8; ++j)
#pragma unroll
                    for (int q = 0; q < 4; ++q) mask |= (acc[j][q] > 0.0f ? 1u : 0u) << (4 * j + q);
                masks[(size_t(l) * tiles + tile) * 32u + lane] = mask;
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
        const __half* w5 = wsm + 5 * kLayerHalves + bOff;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            uint32_t b[4];
            ldsm4(b, w5 + 16u * s);
            mma16816(y[0], a[s], b[0], b[1]);
            mma16816(y[1], a[s], b[2], b[3]);
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

// Inference on the fifth-generation tensor cores (tcgen05): one 128-record tile per step, the tile's FP16 activations
// (128 x 64) and all six weight matrices in shared memory in the canonical K-major layout, the FP32 accumulator of a
// layer in tensor memory (128 lanes = the tile's rows, 64 columns). Per layer one elected thread issues four
// 128 x N x 16 MMAs (N = 64, then 16 for the output layer) and commits them to an mbarrier; after the wait each warp
// reads its 32 rows from tensor memory (tcgen05.ld), applies ReLU, rounds to FP16 and writes the next layer's
// operand. Same network and arithmetic types as kNrcForward<false>; accumulation order inside the tensor core may
// differ. A wait that does not complete within its bound sets bit 0 of *error and the block stops.
constexpr uint32_t kUmmaThreads = 128;  // four warps: tensor-memory lanes 32 w .. 32 w + 31 of warp w
constexpr uint32_t kUmmaRows = 128;
constexpr uint32_t kUmmaLayerBytes = 64u * 64u * 2u;
constexpr uint32_t kUmmaWBytes = 5u * kUmmaLayerBytes + 16u * 64u * 2u;  // 43,008
constexpr uint32_t kUmmaABytes = kUmmaRows * 64u * 2u;                   // 16,384
constexpr uint32_t kUmmaSmemBytes = kUmmaWBytes + kUmmaABytes + 64u;     // + mbarrier and tensor-memory address
constexpr uint32_t kUmmaBlocksPerSM = 3;
constexpr uint32_t kUmmaColumns = 64;
constexpr uint32_t kUmmaWaitPolls = 1u << 22;

__global__ void __launch_bounds__(kUmmaThreads)
    kNrcInferUmma(const __half* __restrict__ W, const __half* __restrict__ x0, const uint32_t* count, uint32_t cap,
                  float4* __restrict__ out, unsigned int* error) {
    extern __shared__ __align__(128) uint8_t usm[];
    uint8_t* wsm = usm;
    uint8_t* act = usm + kUmmaWBytes;
    uint64_t* bar = reinterpret_cast<uint64_t*>(usm + kUmmaWBytes + kUmmaABytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(usm + kUmmaWBytes + kUmmaABytes + 8u);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t n = count ? min(*count, cap) : cap;
    // the grid follows the capacity; blocks past the device-side count leave before staging anything
    if (blockIdx.x * kUmmaRows >= n) return;
    // weights: 16-byte piece kc of row `row` of the concatenated matrices (5 x 64 rows, then 16); rows run fastest
    // across the threads, so a warp's stores fill whole 128-byte core-matrix rows
    constexpr uint32_t kRows = kNrcWeightCount / 64u;  // 336
    for (uint32_t i = tid; i < kRows * 8u; i += blockDim.x) {
        const uint32_t row = i % kRows, kc = i / kRows;
        const uint32_t l = min(row >> 6, 5u), o = row - l * 64u;
        *reinterpret_cast<uint4*>(wsm + l * kUmmaLayerBytes + ummaOffset(o, kc * 8u)) =
            reinterpret_cast<const uint4*>(W)[row * 8u + kc];
    }
    if (tid == 0) mbarInit(bar, 1u);
    if (warp == 0) tmemAlloc(tslot, kUmmaColumns);
    tcgenFenceBefore();
    __syncthreads();
    tcgenFenceAfter();
    const uint32_t tmem = *tslot;
    const uint32_t taddr = tmem + ((warp * 32u) << 16);
    const uint32_t tiles = (n + kUmmaRows - 1u) / kUmmaRows;
    uint32_t phase = 0u;
    bool failed = false;
    for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const uint32_t row = tile * kUmmaRows + tid;
#pragma unroll
        for (uint32_t kc = 0; kc < 8u; ++kc) {
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (row < n) v = reinterpret_cast<const uint4*>(x0 + size_t(row) * 64u)[kc];
            *reinterpret_cast<uint4*>(act + ummaOffset(tid, kc * 8u)) = v;
        }
        for (uint32_t l = 0; l < 6u && !failed; ++l) {
            fenceProxyAsyncShared();
            tcgenFenceBefore();
            __syncthreads();
            if (tid == 0) {
                tcgenFenceAfter();
                const uint32_t idesc = ummaIdescF16(kUmmaRows, l < 5u ? 64u : 16u);
                const uint32_t aBase = smemAddr(act), bBase = smemAddr(wsm + l * kUmmaLayerBytes);
#pragma unroll
                for (uint32_t s = 0; s < 4u; ++s)
                    ummaF16(tmem, ummaSmemDesc(aBase + 256u * s), ummaSmemDesc(bBase + 256u * s), idesc, s);
                ummaCommit(bar);
            }
            const bool ok = mbarWait(bar, phase, kUmmaWaitPolls);
            tcgenFenceAfter();
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            phase ^= 1u;
            if (l < 5u) {
#pragma unroll
                for (uint32_t c = 0; c < 64u; c += 16u) {
                    uint32_t r[16];
                    tmemLoad16(taddr + c, r);
                    tmemLoadWait();
                    uint32_t h[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        h[j] = packHalf2(fmaxf(__uint_as_float(r[2 * j]), 0.0f), fmaxf(__uint_as_float(r[2 * j + 1]), 0.0f));
                    *reinterpret_cast<uint4*>(act + ummaOffset(tid, c)) = make_uint4(h[0], h[1], h[2], h[3]);
                    *reinterpret_cast<uint4*>(act + ummaOffset(tid, c + 8u)) = make_uint4(h[4], h[5], h[6], h[7]);
                }
            } else {
                uint32_t r[16];
                tmemLoad16(taddr, r);
                tmemLoadWait();
                if (row < n)
                    out[row] = make_float4(__uint_as_float(r[0]), __uint_as_float(r[1]), __uint_as_float(r[2]),
                                           __uint_as_float(r[3]));
            }
        }
    }
    if (failed) {
        // let the MMAs of the phase that did not complete finish (bounded) before the columns are released
        if (tid == 0) atomicOr(error, 1u);
        mbarWait(bar, phase, kUmmaWaitPolls);
    }
    tcgenFenceBefore();
    __syncthreads();
    if (warp == 0) {
        tcgenFenceAfter();
        tmemFree(tmem, kUmmaColumns);
    }
}

// Fused backward: dZ of the five hidden layers (dz, 5 x cap x 64) and dL/dx of the 32 hash inputs (dx0, cap x 32).
// dX = dZ W reads the weights in their forward layout through transposed ldmatrix; the ReLU masks come from the
// forward pass, one coalesced word per lane and layer.
__global__ void __launch_bounds__(kMlpThreads, kMlpBlocksPerSM)
    kNrcBackward(const __half* __restrict__ W, const uint32_t* __restrict__ masks, const __half* __restrict__ dy,
                 uint32_t n, uint32_t cap, __half* __restrict__ dz, float* __restrict__ dx0) {
    extern __shared__ __align__(16) __half wsm[];
    stageWeights(wsm, W);
    const uint32_t tiles = (cap + 15u) / 16u;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    // transposed B fragments of two adjacent 8-input tiles: rows (outputs = K) lane % 8 + 8 * bit 3, columns
    // (inputs) + 8 * (lane / 16)
    const uint32_t tOff = ((lane & 7u) + 8u * ((lane >> 3) & 1u)) * kWStride + 8u * (lane >> 4);
    for (uint32_t tile = blockIdx.x * warps + warp; tile * 16u < n; tile += gridDim.x * warps) {
        const uint32_t ra = tile * 16u + g, rb = ra + 8u;
        const bool va = ra < n, vb = rb < n;
        uint32_t mk = masks[(size_t(kNrcHidden - 1) * tiles + tile) * 32u + lane];
        uint32_t a[4][4];
        a[0][0] = va ? ld32(dy + size_t(ra) * 16u + 2u * t) : 0u;
        a[0][1] = vb ? ld32(dy + size_t(rb) * 16u + 2u * t) : 0u;
        a[0][2] = va ? ld32(dy + size_t(ra) * 16u + 8u + 2u * t) : 0u;
        a[0][3] = vb ? ld32(dy + size_t(rb) * 16u + 8u + 2u * t) : 0u;
        float acc[8][4];
        const __half* w5 = wsm + 5u * kLayerHalves + tOff;
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            uint32_t b[4];
            ldsm4t(b, w5 + 16u * jj);
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[2 * jj][q] = acc[2 * jj + 1][q] = 0.0f;
            mma16816(acc[2 * jj], a[0], b[0], b[1]);
            mma16816(acc[2 * jj + 1], a[0], b[2], b[3]);
        }
#pragma unroll 1
        for (int l = kNrcHidden - 1; l >= 0; --l) {
            const uint32_t mkNext = l > 0 ? masks[(size_t(l - 1) * tiles + tile) * 32u + lane] : 0u;
            // dZ = dX (in acc) where the layer's pre-activation was positive
#pragma unroll
            for (int j = 0; j < 8; ++j)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[j][q] = (mk >> (4 * j + q)) & 1u ? acc[j][q] : 0.0f;
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
            // dX of the layer's input = dZ W (K = outputs, N = inputs)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
            const __half* wl = wsm + l * kLayerHalves + tOff;
#pragma unroll
            for (int s = 0; s < 4; ++s)
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    uint32_t b[4];
                    ldsm4t(b, wl + 16u * s * kWStride + 16u * jj);
                    mma16816(acc[2 * jj], a[s], b[0], b[1]);
                    mma16816(acc[2 * jj + 1], a[s], b[2], b[3]);
                }
            mk = mkNext;
        }
        // acc = dL/dX0; the hash features are columns 0..31
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t c = 8u * j + 2u * t;
            if (va) *reinterpret_cast<float2*>(dx0 + size_t(ra) * 32u + c) = make_float2(acc[j][0], acc[j][1]);
            if (vb) *reinterpret_cast<float2*>(dx0 + size_t(rb) * 32u + c) = make_float2(acc[j][2], acc[j][3]);
        }
    }
}

// dW of layer blockIdx.y over records [blockIdx.x * kWgChunk, +kWgChunk): dW[o][i] += sum_r dZ[r][o] X[r][i] / n.
// Slabs of 64 records of dZ and X stream into shared memory with cp.async (kWgStages in flight); the A (dZ^T) and B
// (X) fragments come from transposed ldmatrix. Hidden layers: warp w owns outputs [16 (w % 4), +16) and half of each
// slab's 16-record steps; output layer (16 rows): warps 0..3 take one step each. Partials of a block are summed in
// shared memory before one float2 atomic per pair of weights.
__global__ void __launch_bounds__(kWgThreads)
    kNrcWeightGrad(const __half* __restrict__ x0, const __half* __restrict__ acts, const __half* __restrict__ dz,
                   const __half* __restrict__ dy, uint32_t n, uint32_t cap, float* __restrict__ dW) {
    extern __shared__ __align__(16) __half sm[];
    const uint32_t layer = blockIdx.y;
    const bool outLayer = layer == uint32_t(kNrcHidden);
    const __half* D = outLayer ? dy : dz + size_t(layer) * cap * 64u;
    const uint32_t dWidth = outLayer ? 16u : 64u;
    const __half* X = layer == 0u ? x0 : acts + size_t(layer - 1u) * cap * 64u;
    const uint32_t r0 = blockIdx.x * kWgChunk, r1 = min(r0 + kWgChunk, n);
    if (r0 >= r1) return;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    const uint32_t mTiles = outLayer ? 1u : 4u, kGroups = 8u / mTiles;
    const uint32_t ot = warp % mTiles, kg = warp / mTiles;
    const uint32_t slabs = (r1 - r0 + kWgSlab - 1u) / kWgSlab;
    auto load = [&](uint32_t slab) {
        __half* ds = sm + (slab % kWgStages) * kWgSlabHalves;
        __half* xs = ds + kWgSlab * kWStride;
        const uint32_t k0 = r0 + slab * kWgSlab;
        for (uint32_t i = threadIdx.x; i < kWgSlab * 8u; i += kWgThreads) {
            const uint32_t row = i >> 3, pc = i & 7u;
            const bool ok = k0 + row < r1;
            cpAsync16(xs + row * kWStride + pc * 8u, ok ? X + size_t(k0 + row) * 64u + pc * 8u : X, ok);
        }
        const uint32_t pieces = dWidth / 8u;
        for (uint32_t i = threadIdx.x; i < kWgSlab * pieces; i += kWgThreads) {
            const uint32_t row = i / pieces, pc = i % pieces;
            const bool ok = k0 + row < r1;
            cpAsync16(ds + row * kWStride + pc * 8u, ok ? D + size_t(k0 + row) * dWidth + pc * 8u : D, ok);
        }
    };
    // A = dZ^T from dZ rows (records = K): rows lane % 8 + 8 * (lane / 16), columns 16 ot + 8 * bit 3;
    // B = X from X rows: rows lane % 8 + 8 * bit 3, columns + 8 * (lane / 16)
    const uint32_t aOff = ((lane & 7u) + 8u * (lane >> 4)) * kWStride + 16u * ot + 8u * ((lane >> 3) & 1u);
    const uint32_t bOff = ((lane & 7u) + 8u * ((lane >> 3) & 1u)) * kWStride + 8u * (lane >> 4);
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
    for (uint32_t p = 0; p < kWgStages - 1u; ++p) {
        if (p < slabs) load(p);
        cpAsyncCommit();
    }
    for (uint32_t sl = 0; sl < slabs; ++sl) {
        if (sl + kWgStages - 1u < slabs) load(sl + kWgStages - 1u);
        cpAsyncCommit();
        cpAsyncWait<kWgStages - 1>();
        __syncthreads();
        const __half* ds = sm + (sl % kWgStages) * kWgSlabHalves;
        const __half* xs = ds + kWgSlab * kWStride;
        for (uint32_t s = kg; s < kWgSlab / 16u; s += kGroups) {
            uint32_t a[4];
            ldsm4t(a, ds + 16u * s * kWStride + aOff);
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                uint32_t b[4];
                ldsm4t(b, xs + 16u * s * kWStride + 16u * jj + bOff);
                mma16816(acc[2 * jj], a, b[0], b[1]);
                mma16816(acc[2 * jj + 1], a, b[2], b[3]);
            }
        }
        __syncthreads();
    }
    cpAsyncWait<0>();
    __syncthreads();
    float* red = reinterpret_cast<float*>(sm);  // 8 warps x 16 rows x 72 floats
    float* mine = red + warp * 16u * 72u;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        *reinterpret_cast<float2*>(mine + g * 72u + 8u * j + 2u * t) = make_float2(acc[j][0], acc[j][1]);
        *reinterpret_cast<float2*>(mine + (g + 8u) * 72u + 8u * j + 2u * t) = make_float2(acc[j][2], acc[j][3]);
    }
    __syncthreads();
    if (kg != 0u) return;
    const uint32_t groups = min(kGroups, kWgSlab / 16u);
    for (uint32_t k = 1; k < groups; ++k) {
        const float* o = red + (ot + mTiles * k) * 16u * 72u;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float2 u = *reinterpret_cast<const float2*>(o + g * 72u + 8u * j + 2u * t);
            const float2 v = *reinterpret_cast<const float2*>(o + (g + 8u) * 72u + 8u * j + 2u * t);
            acc[j][0] += u.x;
            acc[j][1] += u.y;
            acc[j][2] += v.x;
            acc[j][3] += v.y;
        }
    }
    const float inv = 1.0f / float(max(n, 1u));
    float* out = dW + layer * 4096u;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t c = 8u * j + 2u * t;
        atomicAdd(reinterpret_cast<float2*>(out + (16u * ot + g) * 64u + c), make_float2(acc[j][0] * inv, acc[j][1] * inv));
        atomicAdd(reinterpret_cast<float2*>(out + (16u * ot + g + 8u) * 64u + c),
                  make_float2(acc[j][2] * inv, acc[j][3] * inv));
    }
}

// One thread per (record, level): trilinear scatter of the level's two input gradients into the table gradient.
__global__ void kNrcTableGrad(NrcGridInfo gi, const NrcInput* __restrict__ in, const float* __restrict__ dx0,
                              uint32_t n, float* __restrict__ tGrad) {
    const float inv = 1.0f / float(max(n, 1u));
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n * 16u; i += gridDim.x * blockDim.x) {
        const uint32_t r = i >> 4;
        const int l = int(i & 15u);
        const float2 d = *reinterpret_cast<const float2*>(dx0 + size_t(r) * 32u + 2u * l);
        if (d.x == 0.0f && d.y == 0.0f) continue;
        const float3 u = nrcUnit(gi, xyz(in[r].posRough));
        uint32_t c[3];
        float f[3];
        nrcCell(gi, l, u, c, f);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t dx = k & 1u, dy = (k >> 1) & 1u, dzz = (k >> 2) & 1u;
            const float w = (dx ? f[0] : 1.0f - f[0]) * (dy ? f[1] : 1.0f - f[1]) * (dzz ? f[2] : 1.0f - f[2]) * inv;
            const size_t e = (size_t(l) * kNrcTable + nrcIndex(gi, l, c[0] + dx, c[1] + dy, c[2] + dzz)) * 2u;
            atomicAdd(reinterpret_cast<float2*>(tGrad + e), make_float2(w * d.x, w * d.y));
        }
    }
}

VKRT_DEV float adamStep(float& w, float& m, float& v, float gr, float lr, float b1, float b2, float eps, float bc1,
                        float bc2) {
    m = b1 * m + (1.0f - b1) * gr;
    v = b2 * v + (1.0f - b2) * gr * gr;
    w -= lr * (m / bc1) / (sqrtf(v / bc2) + eps);
    return w;
}

// dense Adam (MLP weights)
__global__ void kNrcAdam(float* __restrict__ master, float* __restrict__ m, float* __restrict__ v,
                         const float* __restrict__ grad, __half* __restrict__ half, uint32_t count, float lr, float b1,
                         float b2, float eps, float bc1, float bc2) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        float w = master[i], mi = m[i], vi = v[i];
        adamStep(w, mi, vi, grad[i], lr, b1, b2, eps, bc1, bc2);
        m[i] = mi;
        v[i] = vi;
        master[i] = w;
        half[i] = __float2half_rn(w);
    }
}

// Sparse Adam (hash table), four parameters per thread: a parameter whose gradient is zero in this step keeps its
// value and moments (a step's records touch a small part of the finer levels); the gradient is cleared as it is
// consumed, so the next step starts from zeros without a separate clear.
// Parameter average for inference: avg = decay * avg + (1 - decay) * master, in FP32 arithmetic on FP16 storage
// (decay 0 copies the masters).
__global__ void kNrcAverage(const float4* __restrict__ master, uint2* __restrict__ avg, uint32_t count4, float decay) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count4; i += gridDim.x * blockDim.x) {
        const float4 w = master[i];
        const uint2 a = avg[i];
        const float2 a0 = unpackHalf2(a.x), a1 = unpackHalf2(a.y);
        const float k = 1.0f - decay;
        avg[i] = make_uint2(packHalf2(decay * a0.x + k * w.x, decay * a0.y + k * w.y),
                            packHalf2(decay * a1.x + k * w.z, decay * a1.y + k * w.w));
    }
}

__global__ void kNrcAdamSparse(float4* __restrict__ master, float4* __restrict__ m, float4* __restrict__ v,
                               float4* __restrict__ grad, uint2* __restrict__ half, uint32_t count4, float lr, float b1,
                               float b2, float eps, float bc1, float bc2) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count4; i += gridDim.x * blockDim.x) {
        const float4 gr = grad[i];
        if (gr.x == 0.0f && gr.y == 0.0f && gr.z == 0.0f && gr.w == 0.0f) continue;
        grad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float4 w = master[i], mi = m[i], vi = v[i];
        if (gr.x != 0.0f) adamStep(w.x, mi.x, vi.x, gr.x, lr, b1, b2, eps, bc1, bc2);
        if (gr.y != 0.0f) adamStep(w.y, mi.y, vi.y, gr.y, lr, b1, b2, eps, bc1, bc2);
        if (gr.z != 0.0f) adamStep(w.z, mi.z, vi.z, gr.z, lr, b1, b2, eps, bc1, bc2);
        if (gr.w != 0.0f) adamStep(w.w, mi.w, vi.w, gr.w, lr, b1, b2, eps, bc1, bc2);
        master[i] = w;
        m[i] = mi;
        v[i] = vi;
        half[i] = make_uint2(packHalf2(w.x, w.y), packHalf2(w.z, w.w));
    }
}

template <class T>
cudaError_t alloc(T*& p, size_t n) {
    if (p) cudaFree(p);
    p = nullptr;
    return cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1));
}

uint32_t smCount() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return uint32_t(std::max(sms, 1));
}

uint32_t gridFor(uint32_t work, uint32_t per) {
    uint32_t want = (work + per - 1u) / per;
    return std::max(1u, std::min(want, smCount() * 8u));
}

// MLP kernels: one 16-row tile per warp and pass, at most kMlpBlocksPerSM resident blocks per SM (each block stages
// the weights once and loops over tiles)
uint32_t mlpGrid(uint32_t rows) {
    const uint32_t tiles = (rows + 15u) / 16u, warps = kMlpThreads / 32u;
    return std::max(1u, std::min((tiles + warps - 1u) / warps, smCount() * kMlpBlocksPerSM));
}

// tcgen05 inference: one 128-row tile per block and pass, at most kUmmaBlocksPerSM blocks per SM (192 of the 512
// tensor-memory columns)
uint32_t ummaGrid(uint32_t rows) {
    const uint32_t tiles = (rows + kUmmaRows - 1u) / kUmmaRows;
    return std::max(1u, std::min(tiles, smCount() * kUmmaBlocksPerSM));
}

}  // namespace

NrcEngine::NrcEngine() {}

NrcEngine::~NrcEngine() {
    void* ptrs[] = {wHalf_, wMaster_, wM_, wV_,  wGrad_, table_, tMaster_, tM_,     tV_,      tGrad_,
                    x0_,    acts_,    dz_, dy_,  dx0_,   out_,   masks_,   x0Infer_, error_, wAvg_, tAvg_};
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
        if (e == cudaSuccess) e = alloc(error_, 1);
        if (e == cudaSuccess) e = alloc(wAvg_, kNrcWeightCount);
        if (e == cudaSuccess) e = alloc(tAvg_, kNrcTableParams / 2u);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(kNrcInferUmma, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kUmmaSmemBytes));
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(kNrcForward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMlpSmemBytes));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kNrcForward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMlpSmemBytes));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kNrcBackward, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMlpSmemBytes));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kNrcWeightGrad, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kWgSmemBytes));
        if (e != cudaSuccess) return e;
    }
    cudaMemsetAsync(error_, 0, sizeof(unsigned int), stream);
    cudaMemsetAsync(wM_, 0, sizeof(float) * kNrcWeightCount, stream);
    cudaMemsetAsync(wV_, 0, sizeof(float) * kNrcWeightCount, stream);
    cudaMemsetAsync(wGrad_, 0, sizeof(float) * kNrcWeightCount, stream);
    cudaMemsetAsync(tM_, 0, sizeof(float) * kNrcTableParams, stream);
    cudaMemsetAsync(tV_, 0, sizeof(float) * kNrcTableParams, stream);
    cudaMemsetAsync(tGrad_, 0, sizeof(float) * kNrcTableParams, stream);
    tGradClear_ = true;
    kNrcInit<<<gridFor(kNrcWeightCount + kNrcTableParams, 256), 256, 0, stream>>>(
        wMaster_, wHalf_, tMaster_, reinterpret_cast<__half*>(table_), s.seed);
    return refreshAverage(0.0f, stream);
}

cudaError_t NrcEngine::syncMasters(cudaStream_t stream) {
    kHalfToFloat<<<gridFor(kNrcWeightCount, 256), 256, 0, stream>>>(wHalf_, wMaster_, kNrcWeightCount);
    kHalfToFloat<<<gridFor(kNrcTableParams, 256), 256, 0, stream>>>(reinterpret_cast<const __half*>(table_), tMaster_,
                                                                    kNrcTableParams);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? refreshAverage(0.0f, stream) : e;
}

cudaError_t NrcEngine::refreshAverage(float decay, cudaStream_t stream) {
    kNrcAverage<<<gridFor(kNrcWeightCount / 4u, 256), 256, 0, stream>>>(
        reinterpret_cast<const float4*>(wMaster_), reinterpret_cast<uint2*>(wAvg_), kNrcWeightCount / 4u, decay);
    kNrcAverage<<<gridFor(kNrcTableParams / 4u, 256), 256, 0, stream>>>(
        reinterpret_cast<const float4*>(tMaster_), reinterpret_cast<uint2*>(tAvg_), kNrcTableParams / 4u, decay);
    return cudaGetLastError();
}

cudaError_t NrcEngine::ensureScratch(uint32_t n) {
    if (n <= cap_ && x0_) return cudaSuccess;
    const size_t tiles = (size_t(n) + 15u) / 16u;
    cudaError_t e = alloc(x0_, size_t(n) * 64u);
    if (e == cudaSuccess) e = alloc(acts_, size_t(kNrcHidden) * n * 64u);
    if (e == cudaSuccess) e = alloc(dz_, size_t(kNrcHidden) * n * 64u);
    if (e == cudaSuccess) e = alloc(dy_, size_t(n) * 16u);
    if (e == cudaSuccess) e = alloc(dx0_, size_t(n) * 32u);
    if (e == cudaSuccess) e = alloc(out_, n);
    if (e == cudaSuccess) e = alloc(masks_, size_t(kNrcHidden) * tiles * 32u);
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
    if (capacity > (0xFFFFFFFFu >> 4)) return cudaErrorInvalidValue;  // (record, level) indices stay in 32 bits
    cudaError_t e = reserveInference(capacity);
    if (e != cudaSuccess) return e;
    // inference reads the averaged parameters when averaging is on, else the optimiser's current ones
    const __half2* table = averageDecay_ > 0.0f ? tAvg_ : table_;
    const __half* weights = averageDecay_ > 0.0f ? wAvg_ : wHalf_;
    kNrcEncode<<<gridFor(capacity * 16u, 256), 256, 0, stream>>>(grid_, table, inputs, count, capacity, x0Infer_);
    if (tensorPath_ == kNrcTensorTcgen05)
        kNrcInferUmma<<<ummaGrid(capacity), kUmmaThreads, kUmmaSmemBytes, stream>>>(weights, x0Infer_, count, capacity,
                                                                                    out, error_);
    else
        kNrcForward<false><<<mlpGrid(capacity), kMlpThreads, kMlpSmemBytes, stream>>>(
            weights, x0Infer_, count, capacity, out, nullptr, nullptr, nullptr, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t NrcEngine::train(const NrcInput* inputs, const float4* targets, uint32_t n, float* lossOut,
                             bool applyUpdate, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    if (n > (0xFFFFFFFFu >> 4)) return cudaErrorInvalidValue;
    cudaError_t e = ensureScratch(n);
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(wGrad_, 0, sizeof(float) * kNrcWeightCount, stream);
    if (!tGradClear_) cudaMemsetAsync(tGrad_, 0, sizeof(float) * kNrcTableParams, stream);
    // every kernel of the step uses n as the row stride of its scratch (n <= cap_)
    kNrcEncode<<<gridFor(n * 16u, 256), 256, 0, stream>>>(grid_, table_, inputs, nullptr, n, x0_);
    kNrcForward<true><<<mlpGrid(n), kMlpThreads, kMlpSmemBytes, stream>>>(wHalf_, x0_, nullptr, n, out_, acts_, masks_,
                                                                          targets, dy_, lossOut);
    kNrcBackward<<<mlpGrid(n), kMlpThreads, kMlpSmemBytes, stream>>>(wHalf_, masks_, dy_, n, n, dz_, dx0_);
    dim3 wg((n + kWgChunk - 1u) / kWgChunk, kNrcLayers);
    kNrcWeightGrad<<<wg, kWgThreads, kWgSmemBytes, stream>>>(x0_, acts_, dz_, dy_, n, n, wGrad_);
    kNrcTableGrad<<<gridFor(n * 16u, 256), 256, 0, stream>>>(grid_, inputs, dx0_, n, tGrad_);
    tGradClear_ = false;
    if (applyUpdate) {
        ++step_;
        const float bc1 = 1.0f - std::pow(s_.beta1, float(step_)), bc2 = 1.0f - std::pow(s_.beta2, float(step_));
        kNrcAdam<<<gridFor(kNrcWeightCount, 256), 256, 0, stream>>>(wMaster_, wM_, wV_, wGrad_, wHalf_,
                                                                    kNrcWeightCount, s_.learningRate, s_.beta1,
                                                                    s_.beta2, s_.epsilon, bc1, bc2);
        kNrcAdamSparse<<<gridFor(kNrcTableParams / 4u, 256), 256, 0, stream>>>(
            reinterpret_cast<float4*>(tMaster_), reinterpret_cast<float4*>(tM_), reinterpret_cast<float4*>(tV_),
            reinterpret_cast<float4*>(tGrad_), reinterpret_cast<uint2*>(table_), kNrcTableParams / 4u,
            s_.learningRate, s_.beta1, s_.beta2, s_.epsilon, bc1, bc2);
        tGradClear_ = true;
        if (averageDecay_ > 0.0f) {
            cudaError_t e2 = refreshAverage(averageDecay_, stream);
            if (e2 != cudaSuccess) return e2;
        }
    }
    return cudaGetLastError();
}

cudaError_t NrcEngine::errorWord(unsigned int* out, cudaStream_t stream) {
    *out = 0u;
    if (!error_) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(out, error_, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e;
}

}  // namespace vkrt
