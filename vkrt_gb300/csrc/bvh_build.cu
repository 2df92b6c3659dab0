// bvh_build.cu — device BVH construction for the sm_103a tracer.
//
// Replaces the driver-side BLAS/TLAS builds vkrt records with vkCmdBuildAccelerationStructuresKHR
// (src/core/render/accel/blas.c:14-262, tlas.c:291-346, PREFER_FAST_TRACE). Pipeline, all on the context stream:
//   1. flatten   : mesh-relative triangles -> world-space 48-byte records (global id = mesh order, then primitive)
//   2. bounds    : centroid bounds (block reduction + ordered-int atomics)
//   3. morton    : 63-bit Morton codes (21 bits per axis) of the centroids
//   4. radix sort: stable LSD sort of (code, id) pairs, 8 passes of 8 bits (per-tile histograms, one scan kernel,
//                  warp-match ranked scatter)
//   5. LBVH      : Karras 2012 binary radix tree, ties in the code broken by the sorted position
//   6. refit     : bottom-up boxes, subtree sizes and SAH cost with one atomic arrival flag per node
//   7. treelets  : Karras & Aila 2013 treelet restructuring (7 leaves, exhaustive over partitions by a dynamic
//                  program that a whole warp runs), repeated bottom-up passes (two by default)
//   8. collapse  : binary -> 8-wide compressed nodes, children chosen by the SAH-optimal dynamic program of Ylitie et
//                  al. 2017, level by level, leaves of up to 3 triangles, children placed in
//                  octant slots so traversal visits them near to far (Ylitie et al. 2017)
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "bvh_build.h"
#include "scene.cuh"

namespace vkrt {

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// ---- 1. flatten ---------------------------------------------------------------------------------------------
struct MeshXform {
    float m[12];  // rows 0-2 of the column-major TRS matrix: m[r*4 + c]
    uint32_t identity;
    uint32_t pad[3];
};

__global__ void kFlatten(const VKRT_CudaShaderVertex* __restrict__ verts, const uint32_t* __restrict__ idx,
                         const VKRT_CudaMeshInfo* __restrict__ meshes, const uint32_t* __restrict__ meshTriBase,
                         const MeshXform* __restrict__ xf, uint32_t meshCount, uint32_t triCount,
                         TriRecord* __restrict__ out, float4* __restrict__ boxLo, float4* __restrict__ boxHi) {
    uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= triCount) return;
    // mesh containing gid: last base <= gid
    uint32_t lo = 0, hi = meshCount;  // meshTriBase has meshCount + 1 entries
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (meshTriBase[mid] <= gid) lo = mid;
        else hi = mid;
    }
    uint32_t mi = lo;
    uint32_t prim = gid - meshTriBase[mi];
    const VKRT_CudaMeshInfo m = meshes[mi];
    const MeshXform x = xf[mi];
    float3 w[3];
    for (int k = 0; k < 3; ++k) {
        const float* p = verts[idx[m.indexBase + prim * 3u + k] + m.vertexBase].position;
        if (x.identity) {
            w[k] = make_float3(p[0], p[1], p[2]);
        } else {
            float r[3];
            for (int row = 0; row < 3; ++row) {
                float a = __fmul_rn(x.m[row * 4 + 0], p[0]);
                float b = __fmul_rn(x.m[row * 4 + 1], p[1]);
                float c = __fmul_rn(x.m[row * 4 + 2], p[2]);
                r[row] = __fadd_rn(__fadd_rn(__fadd_rn(a, b), c), x.m[row * 4 + 3]);
            }
            w[k] = make_float3(r[0], r[1], r[2]);
        }
    }
    TriRecord t;
    t.v0 = make_float4(w[0].x, w[0].y, w[0].z, __uint_as_float(gid));
    t.v1 = make_float4(w[1].x, w[1].y, w[1].z, __uint_as_float(mi));
    t.v2 = make_float4(w[2].x, w[2].y, w[2].z, __uint_as_float(prim));
    out[gid] = t;
    boxLo[gid] = make_float4(fminf(w[0].x, fminf(w[1].x, w[2].x)), fminf(w[0].y, fminf(w[1].y, w[2].y)),
                             fminf(w[0].z, fminf(w[1].z, w[2].z)), 0.0f);
    boxHi[gid] = make_float4(fmaxf(w[0].x, fmaxf(w[1].x, w[2].x)), fmaxf(w[0].y, fmaxf(w[1].y, w[2].y)),
                             fmaxf(w[0].z, fmaxf(w[1].z, w[2].z)), 0.0f);
}

// ---- 2. bounds ----------------------------------------------------------------------------------------------
// floats mapped to order-preserving unsigned ints so atomicMin/Max work
__device__ __forceinline__ uint32_t floatToOrdered(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float orderedToFloat(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__global__ void kCentroidBounds(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                                uint32_t* __restrict__ bounds /* 6 ordered ints: min xyz, max xyz */) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = lo[i], b = hi[i];
        float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], c[k]);
            mx[k] = fmaxf(mx[k], c[k]);
        }
    }
    for (int k = 0; k < 3; ++k)
        for (int off = 16; off > 0; off >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], off));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], off));
        }
    if ((threadIdx.x & 31u) == 0u)
        for (int k = 0; k < 3; ++k) {
            atomicMin(&bounds[k], floatToOrdered(mn[k]));
            atomicMax(&bounds[3 + k], floatToOrdered(mx[k]));
        }
}

// ---- 3. morton ----------------------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t spread21(uint64_t v) {
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x1F00000000FFFFull;
    v = (v | (v << 16)) & 0x1F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__global__ void kMorton(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                        const uint32_t* __restrict__ bounds, uint64_t* __restrict__ keys,
                        uint32_t* __restrict__ vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float bmin[3], scale[3];
    for (int k = 0; k < 3; ++k) {
        bmin[k] = orderedToFloat(bounds[k]);
        float ext = orderedToFloat(bounds[3 + k]) - bmin[k];
        scale[k] = ext > 0.0f ? 2097151.0f / ext : 0.0f;
    }
    float4 a = lo[i], b = hi[i];
    float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    uint64_t q[3];
    for (int k = 0; k < 3; ++k) {
        float f = (c[k] - bmin[k]) * scale[k];
        f = fminf(fmaxf(f, 0.0f), 2097151.0f);
        q[k] = uint64_t(f);
    }
    keys[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[i] = i;
}

// ---- 4. radix sort --------------------------------------------------------------------------------------------
constexpr uint32_t kSortThreads = 256;
constexpr uint32_t kSortItems = 16;  // items per thread per tile
constexpr uint32_t kSortTile = kSortThreads * kSortItems;

__global__ void __launch_bounds__(kSortThreads) kRadixHistogram(const uint64_t* __restrict__ keys, uint32_t n,
                                                               uint32_t shift, uint32_t numTiles,
                                                               uint32_t* __restrict__ hist /* [256][numTiles] */) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0u;
    __syncthreads();
    uint32_t base = blockIdx.x * kSortTile;
    for (uint32_t k = 0; k < kSortItems; ++k) {
        uint32_t i = base + k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[uint32_t(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * numTiles + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of `count` values in place with one block of 1024 threads
__global__ void __launch_bounds__(1024) kScanExclusive(uint32_t* __restrict__ data, uint32_t count) {
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (uint32_t base = 0; base < count; base += 1024u) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < count ? data[i] : 0u;
        uint32_t x = v;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
            if ((threadIdx.x & 31u) >= uint32_t(off)) x += y;
        }
        if ((threadIdx.x & 31u) == 31u) warpSums[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32u) {
            uint32_t s = warpSums[threadIdx.x];
            for (int off = 1; off < 32; off <<= 1) {
                uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, off);
                if (threadIdx.x >= uint32_t(off)) s += y;
            }
            warpSums[threadIdx.x] = s;  // inclusive
        }
        __syncthreads();
        uint32_t warpPrefix = (threadIdx.x >> 5) ? warpSums[(threadIdx.x >> 5) - 1u] : 0u;
        uint32_t incl = x + warpPrefix;
        if (i < count) data[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023u) carry += incl;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kSortThreads) kRadixScatter(const uint64_t* __restrict__ keysIn,
                                                             const uint32_t* __restrict__ valsIn, uint32_t n,
                                                             uint32_t shift, uint32_t numTiles,
                                                             const uint32_t* __restrict__ offsets,
                                                             uint64_t* __restrict__ keysOut,
                                                             uint32_t* __restrict__ valsOut) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t warpCount[kSortThreads / 32][256];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    base[threadIdx.x] = offsets[threadIdx.x * numTiles + blockIdx.x];
    for (uint32_t w = 0; w < kSortThreads / 32; ++w) warpCount[w][threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t tile = blockIdx.x * kSortTile;
    for (uint32_t k = 0; k < kSortItems; ++k) {
        uint32_t i = tile + k * kSortThreads + threadIdx.x;
        bool valid = i < n;
        uint64_t key = valid ? keysIn[i] : 0ull;
        uint32_t val = valid ? valsIn[i] : 0u;
        uint32_t digit = valid ? (uint32_t(key >> shift) & 0xFFu) : 256u + lane;  // invalid lanes match nobody
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        uint32_t rankInWarp = __popc(peers & ((1u << lane) - 1u));
        bool leader = rankInWarp == 0u;
        if (valid && leader) warpCount[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t before = 0u;
            for (uint32_t w = 0; w < warp; ++w) before += warpCount[w][digit];
            uint32_t dst = base[digit] + before + rankInWarp;
            keysOut[dst] = key;
            valsOut[dst] = val;
        }
        __syncthreads();
        // advance per-digit bases by this chunk's counts and clear the counters
        uint32_t total = 0u;
        for (uint32_t w = 0; w < kSortThreads / 32; ++w) {
            total += warpCount[w][threadIdx.x];
            warpCount[w][threadIdx.x] = 0u;
        }
        base[threadIdx.x] += total;
        __syncthreads();
    }
}

// ---- 5. LBVH (Karras 2012) ------------------------------------------------------------------------------------
__device__ __forceinline__ int commonPrefix(const uint64_t* keys, uint32_t n, int i, int j) {
    if (j < 0 || j >= int(n)) return -1;
    uint64_t a = keys[i], b = keys[j];
    if (a == b) return 64 + __clz(uint32_t(i) ^ uint32_t(j));
    return __clzll(a ^ b);
}

// binary node arrays: internal nodes 0..n-2, leaves n-1..2n-2 (leaf k at n-1+k holds sorted item k)
__global__ void kKarras(const uint64_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ left,
                        uint32_t* __restrict__ right, uint32_t* __restrict__ parent) {
    int i = int(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= int(n) - 1) return;
    int d = (commonPrefix(keys, n, i, i + 1) - commonPrefix(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = commonPrefix(keys, n, i, i - d);
    int lmax = 2;
    while (commonPrefix(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (commonPrefix(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = commonPrefix(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (commonPrefix(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int split = i + s * d + min(d, 0);
    uint32_t lc = (min(i, j) == split) ? uint32_t(n - 1 + split) : uint32_t(split);
    uint32_t rc = (max(i, j) == split + 1) ? uint32_t(n - 1 + split + 1) : uint32_t(split + 1);
    left[i] = lc;
    right[i] = rc;
    parent[lc] = uint32_t(i);
    parent[rc] = uint32_t(i);
    if (i == 0) parent[0] = kInvalid;
}

__device__ __forceinline__ float halfArea(float4 lo, float4 hi) {
    float dx = fmaxf(hi.x - lo.x, 0.0f), dy = fmaxf(hi.y - lo.y, 0.0f), dz = fmaxf(hi.z - lo.z, 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

// ---- 6. refit ---------------------------------------------------------------------------------------------------
constexpr float kCostNode = 1.2f;  // SAH cost of visiting a node relative to one triangle test
constexpr float kCostTri = 1.0f;

__global__ void kInitLeaves(const uint32_t* __restrict__ sortedIds, const float4* __restrict__ triLo,
                            const float4* __restrict__ triHi, uint32_t n, float4* __restrict__ nodeLo,
                            float4* __restrict__ nodeHi, uint32_t* __restrict__ leafCount,
                            float* __restrict__ cost, uint32_t* __restrict__ flags) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n - 1) flags[k] = 0u;
    if (k >= n) return;
    uint32_t node = n - 1 + k;
    uint32_t id = sortedIds[k];
    nodeLo[node] = triLo[id];
    nodeHi[node] = triHi[id];
    leafCount[node] = 1u;
    cost[node] = kCostTri * halfArea(triLo[id], triHi[id]);
}

__global__ void kRefit(uint32_t n, const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                       const uint32_t* __restrict__ parent, float4* nodeLo, float4* nodeHi, uint32_t* leafCount,
                       float* cost, uint32_t* flags) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t node = parent[n - 1 + k];
    while (node != kInvalid) {
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0u) return;  // first arrival: the sibling finishes this node
        __threadfence();
        uint32_t l = left[node], r = right[node];
        float4 llo = __ldcg(&nodeLo[l]), lhi = __ldcg(&nodeHi[l]), rlo = __ldcg(&nodeLo[r]), rhi = __ldcg(&nodeHi[r]);
        float4 lo = make_float4(fminf(llo.x, rlo.x), fminf(llo.y, rlo.y), fminf(llo.z, rlo.z), 0.0f);
        float4 hi = make_float4(fmaxf(lhi.x, rhi.x), fmaxf(lhi.y, rhi.y), fmaxf(lhi.z, rhi.z), 0.0f);
        nodeLo[node] = lo;
        nodeHi[node] = hi;
        uint32_t cnt = __ldcg(&leafCount[l]) + __ldcg(&leafCount[r]);
        leafCount[node] = cnt;
        float a = halfArea(lo, hi);
        cost[node] = fminf(kCostNode * a + __ldcg(&cost[l]) + __ldcg(&cost[r]), kCostTri * a * float(cnt));
        node = parent[node];
    }
}

// ---- 7. treelet restructuring (Karras & Aila 2013) --------------------------------------------------------------
constexpr int kTreeletLeaves = 7;
constexpr uint32_t kTreeletSubsets = 1u << kTreeletLeaves;
constexpr uint32_t kTreeletThreads = 64;

// A treelet formed by one lane: the root's subtree expanded into up to 7 treelet leaves by repeatedly opening the
// internal leaf of largest area (the opened node's left child takes its place, the right child is appended).
struct TreeletSlot {
    uint32_t node[kTreeletLeaves];
    uint32_t internal[kTreeletLeaves - 1];  // the treelet's internal nodes, root first
    uint32_t leaves;
};

// One warp's dynamic program over the 127 leaf subsets of a treelet, with the treelet's leaf boxes, triangle counts
// and SAH costs
struct TreeletDp {
    float4 lo[kTreeletLeaves], hi[kTreeletLeaves];
    uint32_t count[kTreeletLeaves];
    float cost[kTreeletLeaves];
    float area[kTreeletSubsets];
    float copt[kTreeletSubsets];
    unsigned long long best[kTreeletSubsets];  // (cost bits, 255 - partition): the lowest cost, ties to the larger partition
    float refit[kTreeletSubsets];              // SAH cost of each rebuilt subtree
    uint8_t part[kTreeletSubsets];
};

__device__ __forceinline__ float4 boxMin(float4 a, float4 b) {
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
}
__device__ __forceinline__ float4 boxMax(float4 a, float4 b) {
    return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), 0.0f);
}

// the low bits of i placed, in order, at the set bits of mask
__device__ __forceinline__ uint32_t depositBits(uint32_t i, uint32_t mask) {
    uint32_t r = 0u;
    for (uint32_t b = 1u; mask != 0u; b <<= 1) {
        const uint32_t low = mask & (0u - mask);
        if (i & b) r |= low;
        mask ^= low;
    }
    return r;
}

// Forms the treelet rooted at `root` into the lane's slot; false when it has fewer than 3 leaves.
__device__ bool formTreelet(uint32_t n, uint32_t root, const uint32_t* left, const uint32_t* right,
                            const float4* nodeLo, const float4* nodeHi, TreeletSlot& T) {
    float area[kTreeletLeaves];
    uint32_t nl = 2, ni = 1;
    T.internal[0] = root;
    T.node[0] = __ldcg(&left[root]);
    T.node[1] = __ldcg(&right[root]);
    area[0] = halfArea(__ldcg(&nodeLo[T.node[0]]), __ldcg(&nodeHi[T.node[0]]));
    area[1] = halfArea(__ldcg(&nodeLo[T.node[1]]), __ldcg(&nodeHi[T.node[1]]));
    while (nl < uint32_t(kTreeletLeaves)) {
        int best = -1;
        float bestA = -1.0f;
        for (uint32_t i = 0; i < nl; ++i) {
            if (T.node[i] >= n - 1) continue;  // a triangle
            if (area[i] > bestA) {
                bestA = area[i];
                best = int(i);
            }
        }
        if (best < 0) break;
        const uint32_t x = T.node[best];
        T.internal[ni++] = x;
        const uint32_t l = __ldcg(&left[x]), r = __ldcg(&right[x]);
        T.node[best] = l;
        T.node[nl] = r;
        area[best] = halfArea(__ldcg(&nodeLo[l]), __ldcg(&nodeHi[l]));
        area[nl] = halfArea(__ldcg(&nodeLo[r]), __ldcg(&nodeHi[r]));
        ++nl;
    }
    T.leaves = nl;
    return nl >= 3;
}

// The SAH-optimal partition tree of a treelet's leaves, by all 32 lanes of a warp: subsets in order of size, every
// partition of a subset (its lowest leaf fixed on one side) spread over the lanes, the lowest cost kept by a 64-bit
// shared-memory minimum. Ties go to the larger partition mask, as an enumeration from the largest mask down with a
// strict comparison would choose.
__device__ void treeletDp(const TreeletSlot& T, TreeletDp& dp, const uint8_t* bySize, uint32_t lane,
                          const float4* nodeLo, const float4* nodeHi, const uint32_t* leafCount, const float* cost) {
    const uint32_t nl = T.leaves, full = (1u << nl) - 1u;
    if (lane < nl) {  // the leaves' boxes, counts and costs, one leaf per lane
        const uint32_t x = T.node[lane];
        dp.lo[lane] = __ldcg(&nodeLo[x]);
        dp.hi[lane] = __ldcg(&nodeHi[x]);
        dp.count[lane] = __ldcg(&leafCount[x]);
        dp.cost[lane] = __ldcg(&cost[x]);
    }
    __syncwarp();
    for (uint32_t s = lane + 1u; s < kTreeletSubsets; s += 32u) {
        if (s & ~full) continue;
        float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0.0f), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        for (uint32_t i = 0; i < nl; ++i)
            if (s & (1u << i)) {
                lo = boxMin(lo, dp.lo[i]);
                hi = boxMax(hi, dp.hi[i]);
            }
        dp.area[s] = halfArea(lo, hi);
        dp.best[s] = ~0ull;
        if (__popc(s) == 1) {
            dp.copt[s] = dp.cost[__ffs(s) - 1];
            dp.refit[s] = dp.cost[__ffs(s) - 1];
        }
    }
    __syncwarp();
    // 7-bit subsets of each size k start at bySize[offset[k]]: C(7, k) of them
    const uint32_t offset[kTreeletLeaves + 1] = {0, 0, 7, 28, 63, 98, 119, 126};
    const uint32_t number[kTreeletLeaves + 1] = {0, 7, 21, 35, 35, 21, 7, 1};
#pragma unroll
    for (uint32_t k = 2; k <= uint32_t(kTreeletLeaves); ++k) {
        if (k > nl) break;
        const uint32_t parts = (1u << (k - 1u)) - 1u, items = number[k] * parts;
        for (uint32_t w = lane; w < items; w += 32u) {
            const uint32_t s = bySize[offset[k] + w / parts];
            if (s & ~full) continue;
            const uint32_t low = s & (0u - s), p = low | depositBits(w % parts, s ^ low);
            const float c = dp.copt[p] + dp.copt[s ^ p];
            atomicMin(&dp.best[s], (static_cast<unsigned long long>(__float_as_uint(c)) << 32) | (255u - p));
        }
        __syncwarp();
        for (uint32_t j = lane; j < number[k]; j += 32u) {
            const uint32_t s = bySize[offset[k] + j];
            if (s & ~full) continue;
            const unsigned long long b = dp.best[s];
            dp.copt[s] = kCostNode * dp.area[s] + __uint_as_float(uint32_t(b >> 32));
            dp.part[s] = uint8_t(255u - uint32_t(b & 0xFFu));
        }
        __syncwarp();
    }
}

// Rewires the treelet's internal nodes to the optimal partition tree (depth first, parents before children) and
// refits them (children before parents). The original topology is among the candidates, so the SAH cost never rises.
__device__ void rewireTreelet(const TreeletSlot& T, TreeletDp& dp, uint32_t* left, uint32_t* right, uint32_t* parent,
                              float4* nodeLo, float4* nodeHi, uint32_t* leafCount, float* cost) {
    const uint32_t nl = T.leaves, full = (1u << nl) - 1u;
    uint32_t order[kTreeletLeaves - 1], subset[kTreeletLeaves - 1];
    uint32_t stackNode[kTreeletLeaves], stackSet[kTreeletLeaves];
    int sp = 0, used = 1, no = 0;
    stackNode[sp] = T.internal[0];
    stackSet[sp++] = full;
    while (sp > 0) {
        --sp;
        const uint32_t node = stackNode[sp], s = stackSet[sp];
        order[no] = node;
        subset[no++] = s;
        const uint32_t p = dp.part[s], sides[2] = {p, s ^ p};
        uint32_t child[2];
        for (int k = 0; k < 2; ++k) {
            if (__popc(sides[k]) == 1) {
                child[k] = T.node[__ffs(sides[k]) - 1];
            } else {
                child[k] = T.internal[used++];
                stackNode[sp] = child[k];
                stackSet[sp++] = sides[k];
            }
            parent[child[k]] = node;
        }
        left[node] = child[0];
        right[node] = child[1];
    }
    for (int k = no - 1; k >= 0; --k) {
        const uint32_t node = order[k], s = subset[k];
        float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0.0f), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        uint32_t cnt = 0;
        for (uint32_t i = 0; i < nl; ++i)
            if (s & (1u << i)) {
                lo = boxMin(lo, dp.lo[i]);
                hi = boxMax(hi, dp.hi[i]);
                cnt += dp.count[i];
            }
        nodeLo[node] = lo;
        nodeHi[node] = hi;
        leafCount[node] = cnt;
        const float a = halfArea(lo, hi);
        const uint32_t p = dp.part[s];
        const float c = fminf(kCostNode * a + dp.refit[p] + dp.refit[s ^ p], kCostTri * a * float(cnt));
        dp.refit[s] = c;
        cost[node] = c;
    }
}

// Bottom-up pass like the refit: a node is restructured once both of its subtrees are final. Each round, the lanes
// that arrive second at a node with enough leaves form their treelets at once; the warp then runs their dynamic
// programs one after another, and the owning lane rewires each.
__global__ void __launch_bounds__(kTreeletThreads) kTreelets(uint32_t n, uint32_t minLeaves, uint32_t* left,
                                                             uint32_t* right, uint32_t* parent, float4* nodeLo,
                                                             float4* nodeHi, uint32_t* leafCount, float* cost,
                                                             uint32_t* flags) {
    __shared__ TreeletSlot slots[kTreeletThreads];
    __shared__ TreeletDp dps[kTreeletThreads / 32];
    __shared__ uint8_t bySize[kTreeletSubsets];
    // the 127 non-empty 7-bit subsets ordered by size, ascending within a size
    for (uint32_t s = threadIdx.x + 1u; s < kTreeletSubsets; s += blockDim.x) {
        const uint32_t start[kTreeletLeaves + 1] = {0, 0, 7, 28, 63, 98, 119, 126};
        uint32_t rank = 0;
        for (uint32_t t = 1; t < s; ++t) rank += __popc(t) == __popc(s) ? 1u : 0u;
        bySize[start[__popc(s)] + rank] = uint8_t(s);
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    TreeletDp& dp = dps[threadIdx.x >> 5];
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t node = k < n ? __ldcg(&parent[n - 1 + k]) : kInvalid;
    bool active = node != kInvalid;
    while (__any_sync(0xFFFFFFFFu, active)) {
        bool work = false;
        if (active) {
            __threadfence();
            if (atomicAdd(&flags[node], 1u) == 0u) {
                active = false;
            } else {
                __threadfence();
                work = __ldcg(&leafCount[node]) >= minLeaves &&
                       formTreelet(n, node, left, right, nodeLo, nodeHi, slots[threadIdx.x]);
            }
        }
        uint32_t pending = __ballot_sync(0xFFFFFFFFu, work);
        __syncwarp();  // the slots formed above, visible to the whole warp
        // the leaves' data was final when the owning lane arrived: every lane reads it after a fence of its own
        if (pending != 0u) __threadfence();
        for (; pending != 0u; pending &= pending - 1u) {
            const uint32_t leader = __ffs(pending) - 1u;
            treeletDp(slots[(threadIdx.x & ~31u) + leader], dp, bySize, lane, nodeLo, nodeHi, leafCount, cost);
            if (lane == leader)
                rewireTreelet(slots[threadIdx.x], dp, left, right, parent, nodeLo, nodeHi, leafCount, cost);
            __syncwarp();
        }
        if (active) {
            __threadfence();
            node = __ldcg(&parent[node]);
            active = node != kInvalid;
        }
    }
}

__global__ void kRootSah(const float4* nodeLo, const float4* nodeHi, const float* cost, float* out) {
    float a = halfArea(nodeLo[0], nodeHi[0]);
    *out = a > 0.0f ? cost[0] / a : 0.0f;
}

// ---- 8. collapse to 8-wide compressed nodes -------------------------------------------------------------------
// SAH-optimal collapse (Ylitie, Karras, Laine 2017, section 3.1), bottom-up over the binary tree: C(n, i) is the
// lowest cost of representing the subtree of binary node n as at most i children of a wide node,
//   C(n, 1) = min(C_leaf(n), C_internal(n)),  C(n, i) = min(C(n, i - 1), C_distribute(n, i))  for i > 1,
//   C_distribute(n, j) = min over 0 < k < j of C(left, k) + C(right, j - k),
//   C_internal(n) = c_node A(n) + C_distribute(n, 8),  C_leaf(n) = c_tri A(n) p(n) when p(n) <= 3 triangles,
// A the box's half area, p the triangle count. The choices are kept per node in eight bytes: byte 0 is 0 for a leaf
// or the split k of C_distribute(n, 8) for an internal wide node; byte i - 1 (i > 1) is 0 when C(n, i) = C(n, i - 1)
// or the split k of C_distribute(n, i).
constexpr float kWideCostNode = 1.0f;  // a wide node visit (eight box tests)
constexpr float kWideCostTri = 1.0f;   // one triangle test (a traversal step, like a node visit)
constexpr uint32_t kWideLeafMax = 3u;  // triangles per leaf child (three triangle-mask bits per child)

__device__ __forceinline__ void wideLeafCost(float a, float* c, uint8_t* d) {
    for (int i = 0; i < 8; ++i) {
        c[i] = kWideCostTri * a;
        d[i] = 0u;
    }
}

__global__ void kWideCostLeaves(uint32_t n, const float4* __restrict__ nodeLo, const float4* __restrict__ nodeHi,
                                float4* __restrict__ wideCost, uint2* __restrict__ wideDec, uint32_t* __restrict__ flags) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n - 1) flags[k] = 0u;
    if (k >= n) return;
    const uint32_t node = n - 1 + k;
    float c[8];
    uint8_t d[8];
    wideLeafCost(halfArea(nodeLo[node], nodeHi[node]), c, d);
    wideCost[2 * node] = make_float4(c[0], c[1], c[2], c[3]);
    wideCost[2 * node + 1] = make_float4(c[4], c[5], c[6], c[7]);
    wideDec[node] = make_uint2(0u, 0u);
}

// one thread per binary leaf walks up; the second arrival at a node computes its costs (as the refit does)
__global__ void kWideCost(uint32_t n, const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                          const uint32_t* __restrict__ parent, const float4* __restrict__ nodeLo,
                          const float4* __restrict__ nodeHi, const uint32_t* __restrict__ leafCount,
                          float4* wideCost, uint2* wideDec, uint32_t* flags) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t node = parent[n - 1 + k];
    while (node != kInvalid) {
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0u) return;
        __threadfence();
        const uint32_t l = left[node], r = right[node];
        float cl[8], cr[8];
        const float4 l0 = __ldcg(&wideCost[2 * l]), l1 = __ldcg(&wideCost[2 * l + 1]);
        const float4 r0 = __ldcg(&wideCost[2 * r]), r1 = __ldcg(&wideCost[2 * r + 1]);
        cl[0] = l0.x, cl[1] = l0.y, cl[2] = l0.z, cl[3] = l0.w, cl[4] = l1.x, cl[5] = l1.y, cl[6] = l1.z, cl[7] = l1.w;
        cr[0] = r0.x, cr[1] = r0.y, cr[2] = r0.z, cr[3] = r0.w, cr[4] = r1.x, cr[5] = r1.y, cr[6] = r1.z, cr[7] = r1.w;
        // C_distribute(node, j) for j = 2..8 (cl[i - 1] = C(left, i))
        float dist[9];
        uint8_t split[9];
        for (int j = 2; j <= 8; ++j) {
            float best = INFINITY;
            uint8_t bk = 1u;
            for (int kk = 1; kk < j; ++kk) {
                const float v = cl[kk - 1] + cr[j - kk - 1];
                if (v < best) {
                    best = v;
                    bk = uint8_t(kk);
                }
            }
            dist[j] = best;
            split[j] = bk;
        }
        const float a = halfArea(__ldcg(&nodeLo[node]), __ldcg(&nodeHi[node]));
        const uint32_t cnt = leafCount[node];
        const float cInternal = kWideCostNode * a + dist[8];
        const float cLeaf = cnt <= kWideLeafMax ? kWideCostTri * a * float(cnt) : INFINITY;
        float c[8];
        uint8_t d[8];
        if (cnt <= kWideLeafMax && cLeaf <= cInternal) {
            c[0] = cLeaf;
            d[0] = 0u;
        } else {
            c[0] = cInternal;
            d[0] = split[8];
        }
        for (int i = 2; i <= 8; ++i) {
            if (c[i - 2] <= dist[i]) {
                c[i - 1] = c[i - 2];
                d[i - 1] = 0u;
            } else {
                c[i - 1] = dist[i];
                d[i - 1] = split[i];
            }
        }
        wideCost[2 * node] = make_float4(c[0], c[1], c[2], c[3]);
        wideCost[2 * node + 1] = make_float4(c[4], c[5], c[6], c[7]);
        wideDec[node] = make_uint2(uint32_t(d[0]) | (uint32_t(d[1]) << 8) | (uint32_t(d[2]) << 16) |
                                       (uint32_t(d[3]) << 24),
                                   uint32_t(d[4]) | (uint32_t(d[5]) << 8) | (uint32_t(d[6]) << 16) |
                                       (uint32_t(d[7]) << 24));
        node = parent[node];
    }
}

__device__ __forceinline__ uint32_t wideChoice(const uint2* wideDec, uint32_t node, uint32_t i) {
    const uint2 d = wideDec[node];
    const uint32_t w = i < 4u ? d.x : d.y;
    return (w >> ((i & 3u) * 8u)) & 0xFFu;
}

struct CollapseItem {
    uint32_t binary;  // binary node index
    uint32_t wide;    // wide node slot to fill
};

__device__ __forceinline__ uint32_t ceilExponentByte(float s) {
    // smallest e with 2^(e-127) >= s, as a biased exponent byte in [1, 254]
    if (!(s > 0.0f)) return 1u;
    uint32_t b = __float_as_uint(s);
    uint32_t e = (b >> 23) & 0xFFu;
    uint32_t m = b & 0x7FFFFFu;
    uint32_t r = e + (m != 0u ? 1u : 0u);
    if (e == 0u) r = 1u;  // denormal scales: use the smallest normal power of two
    return min(max(r, 1u), 254u);
}

__global__ void kCollapse(uint32_t n, const CollapseItem* __restrict__ in, uint32_t inCount,
                          CollapseItem* __restrict__ out, uint32_t* __restrict__ outCount,
                          const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                          const float4* __restrict__ nodeLo, const float4* __restrict__ nodeHi,
                          const uint32_t* __restrict__ leafCount, const uint2* __restrict__ wideDec,
                          const uint32_t* __restrict__ sortedIds,
                          const TriRecord* __restrict__ trisIn, uint32_t* __restrict__ nodeCursor,
                          uint32_t* __restrict__ triCursor, WideNode* __restrict__ nodes,
                          TriRecord* __restrict__ trisOut) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= inCount) return;
    CollapseItem item = in[w];
    const uint32_t firstLeaf = n - 1;
    uint32_t child[8];
    int cnt = 0;
    auto isLeaf = [&](uint32_t b) { return b >= firstLeaf; };
    // a child is internal (another wide node) when the collapse chose so, else a leaf of at most three triangles
    auto isInternal = [&](uint32_t b) { return !isLeaf(b) && wideChoice(wideDec, b, 0u) != 0u; };
    if (isLeaf(item.binary)) {
        child[cnt++] = item.binary;  // single-triangle scene
    } else {
        // the roots of C_distribute(item, 8): (node, i) = the subtree of node as at most i children
        uint32_t stackNode[8], stackI[8];
        int sp = 0;
        // the root of a scene of at most three triangles may have chosen to be a leaf: split it 1 + 7
        const uint32_t k0 = max(wideChoice(wideDec, item.binary, 0u), 1u);
        stackNode[sp] = right[item.binary], stackI[sp++] = 8u - k0;
        stackNode[sp] = left[item.binary], stackI[sp++] = k0;
        while (sp > 0) {
            uint32_t m = stackNode[--sp], i = stackI[sp];
            for (;;) {
                if (i <= 1u || isLeaf(m)) {
                    child[cnt++] = m;
                    break;
                }
                const uint32_t kk = wideChoice(wideDec, m, i - 1u);
                if (kk == 0u) {
                    --i;
                    continue;
                }
                stackNode[sp] = right[m], stackI[sp++] = i - kk;
                stackNode[sp] = left[m], stackI[sp++] = kk;
                break;
            }
        }
    }
    // a leaf child's triangles (at most three) are gathered below
    // octant slot assignment: slot s prefers the child furthest along (+-1,+-1,+-1) with bit set = positive
    float4 plo = make_float4(INFINITY, INFINITY, INFINITY, 0.0f), phi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
    float3 cc[8];
    for (int c = 0; c < cnt; ++c) {
        float4 a = nodeLo[child[c]], b = nodeHi[child[c]];
        plo = make_float4(fminf(plo.x, a.x), fminf(plo.y, a.y), fminf(plo.z, a.z), 0.0f);
        phi = make_float4(fmaxf(phi.x, b.x), fmaxf(phi.y, b.y), fmaxf(phi.z, b.z), 0.0f);
        cc[c] = make_float3(0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z));
    }
    float3 pc = make_float3(0.5f * (plo.x + phi.x), 0.5f * (plo.y + phi.y), 0.5f * (plo.z + phi.z));
    int slotOf[8];
    int childInSlot[8];
    for (int s = 0; s < 8; ++s) childInSlot[s] = -1;
    for (int c = 0; c < 8; ++c) slotOf[c] = -1;
    for (int round = 0; round < cnt; ++round) {
        float bestCost = INFINITY;
        int bc = -1, bs = -1;
        for (int c = 0; c < cnt; ++c) {
            if (slotOf[c] >= 0) continue;
            float3 d = make_float3(cc[c].x - pc.x, cc[c].y - pc.y, cc[c].z - pc.z);
            for (int s = 0; s < 8; ++s) {
                if (childInSlot[s] >= 0) continue;
                float sx = (s & 4) ? 1.0f : -1.0f, sy = (s & 2) ? 1.0f : -1.0f, sz = (s & 1) ? 1.0f : -1.0f;
                float cost = -(d.x * sx + d.y * sy + d.z * sz);
                if (cost < bestCost) {
                    bestCost = cost;
                    bc = c;
                    bs = s;
                }
            }
        }
        if (bc < 0) {  // non-finite centroids: first unassigned child into the first free slot
            for (int c = 0; c < cnt && bc < 0; ++c)
                if (slotOf[c] < 0) bc = c;
            for (int s = 0; s < 8 && bs < 0; ++s)
                if (childInSlot[s] < 0) bs = s;
        }
        slotOf[bc] = bs;
        childInSlot[bs] = bc;
    }
    // count internal children and triangles in slot order
    uint32_t numInternal = 0u, numTris = 0u;
    for (int s = 0; s < 8; ++s) {
        int c = childInSlot[s];
        if (c < 0) continue;
        uint32_t b = child[c];
        if (isInternal(b)) numInternal++;
        else numTris += isLeaf(b) ? 1u : leafCount[b];
    }
    uint32_t childBase = numInternal ? atomicAdd(nodeCursor, numInternal) : 0u;
    uint32_t triBase = numTris ? atomicAdd(triCursor, numTris) : 0u;
    uint32_t outBase = numInternal ? atomicAdd(outCount, numInternal) : 0u;
    // quantisation frame
    // extents rounded up so that 255 quanta always cover the node (conservative boxes)
    float ext[3] = {__fsub_ru(phi.x, plo.x), __fsub_ru(phi.y, plo.y), __fsub_ru(phi.z, plo.z)};
    uint32_t eb[3];
    float inv[3];
    for (int k = 0; k < 3; ++k) {
        eb[k] = ceilExponentByte(__fdiv_ru(ext[k], 255.0f));
        inv[k] = __uint_as_float((254u - eb[k]) << 23);  // 1 / 2^(e-127)
    }
    uint8_t meta[8], qlo[3][8], qhi[3][8];
    uint32_t imask = 0u;
    uint32_t nextInternal = 0u, nextTri = 0u;
    for (int s = 0; s < 8; ++s) {
        int c = childInSlot[s];
        if (c < 0) {
            meta[s] = 0u;
            for (int k = 0; k < 3; ++k) {
                qlo[k][s] = 0u;
                qhi[k][s] = 0u;
            }
            continue;
        }
        uint32_t b = child[c];
        float4 a = nodeLo[b], bh = nodeHi[b];
        float lo3[3] = {a.x, a.y, a.z}, hi3[3] = {bh.x, bh.y, bh.z}, o3[3] = {plo.x, plo.y, plo.z};
        for (int k = 0; k < 3; ++k) {
            float ql = floorf(__fmul_rd(__fsub_rd(lo3[k], o3[k]), inv[k]));
            float qh = ceilf(__fmul_ru(__fsub_ru(hi3[k], o3[k]), inv[k]));
            qlo[k][s] = uint8_t(fminf(fmaxf(ql, 0.0f), 255.0f));
            qhi[k][s] = uint8_t(fminf(fmaxf(qh, 0.0f), 255.0f));
        }
        if (isInternal(b)) {
            meta[s] = uint8_t((1u << 5) | (24u + uint32_t(s)));
            imask |= 1u << s;
            out[outBase + nextInternal] = CollapseItem{b, childBase + nextInternal};
            nextInternal++;
        } else {
            // gather the subtree's triangles (at most 3) in left-to-right order
            uint32_t stack[4];
            int sp = 0;
            stack[sp++] = b;
            uint32_t first = nextTri;
            while (sp > 0) {
                uint32_t x = stack[--sp];
                if (isLeaf(x)) {
                    uint32_t id = sortedIds[x - firstLeaf];
                    trisOut[triBase + nextTri] = trisIn[id];
                    nextTri++;
                } else {
                    stack[sp++] = right[x];
                    stack[sp++] = left[x];
                }
            }
            uint32_t tcount = nextTri - first;
            uint32_t unary = tcount == 1u ? 1u : (tcount == 2u ? 3u : 7u);
            meta[s] = uint8_t((unary << 5) | first);
        }
    }
    WideNode node;
    node.w[0] = make_uint4(__float_as_uint(plo.x), __float_as_uint(plo.y), __float_as_uint(plo.z),
                           eb[0] | (eb[1] << 8) | (eb[2] << 16) | (imask << 24));
    auto pack4 = [](const uint8_t* v) {
        return uint32_t(v[0]) | (uint32_t(v[1]) << 8) | (uint32_t(v[2]) << 16) | (uint32_t(v[3]) << 24);
    };
    node.w[1] = make_uint4(childBase, triBase, pack4(meta), pack4(meta + 4));
    node.w[2] = make_uint4(pack4(qlo[0]), pack4(qlo[0] + 4), pack4(qlo[1]), pack4(qlo[1] + 4));
    node.w[3] = make_uint4(pack4(qlo[2]), pack4(qlo[2] + 4), pack4(qhi[0]), pack4(qhi[0] + 4));
    node.w[4] = make_uint4(pack4(qhi[1]), pack4(qhi[1] + 4), pack4(qhi[2]), pack4(qhi[2] + 4));
    nodes[item.wide] = node;
}

template <class T>
T* dalloc(size_t count, cudaError_t& err) {
    T* p = nullptr;
    if (err != cudaSuccess) return nullptr;
    err = cudaMalloc(&p, sizeof(T) * (count ? count : 1));
    return p;
}

}  // namespace

// ---- host orchestration ----------------------------------------------------------------------------------------
cudaError_t buildBvh(const BvhBuildInput& in, BvhBuffers& out, BvhBuildStats* stats, cudaStream_t stream) {
    cudaError_t err = cudaSuccess;
    out.release();
    const uint32_t n = in.triCount;
    if (n == 0) return cudaSuccess;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, stream);

    // per-mesh transforms and triangle bases on the host (meshCount is small)
    std::vector<MeshXform> xf(in.meshCount);
    std::vector<uint32_t> triBase(in.meshCount + 1);
    uint32_t acc = 0;
    for (uint32_t i = 0; i < in.meshCount; ++i) {
        triBase[i] = acc;
        acc += in.hostMeshes[i].indexCount / 3u;
        const float* m = in.hostWorld + size_t(i) * 16;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) xf[i].m[r * 4 + c] = m[c * 4 + r];
        xf[i].identity = in.hostIdentity[i];
    }
    triBase[in.meshCount] = acc;

    MeshXform* dXf = dalloc<MeshXform>(in.meshCount, err);
    uint32_t* dTriBase = dalloc<uint32_t>(in.meshCount + 1, err);
    TriRecord* dTrisFlat = dalloc<TriRecord>(n, err);
    float4* dLo = dalloc<float4>(2 * n, err);
    float4* dHi = dalloc<float4>(2 * n, err);
    float4* dTriLo = dalloc<float4>(n, err);
    float4* dTriHi = dalloc<float4>(n, err);
    uint32_t* dBounds = dalloc<uint32_t>(8, err);
    uint64_t* dKeys[2] = {dalloc<uint64_t>(n, err), dalloc<uint64_t>(n, err)};
    uint32_t* dVals[2] = {dalloc<uint32_t>(n, err), dalloc<uint32_t>(n, err)};
    uint32_t numTiles = (n + kSortTile - 1) / kSortTile;
    uint32_t* dHist = dalloc<uint32_t>(size_t(256) * numTiles, err);
    uint32_t* dLeft = dalloc<uint32_t>(n, err);
    uint32_t* dRight = dalloc<uint32_t>(n, err);
    uint32_t* dParent = dalloc<uint32_t>(2 * n, err);
    uint32_t* dLeafCount = dalloc<uint32_t>(2 * n, err);
    float* dCost = dalloc<float>(2 * n, err);
    float4* dWideCost = dalloc<float4>(4 * size_t(n), err);  // C(node, 1..8) as two float4 per binary node
    uint2* dWideDec = dalloc<uint2>(2 * size_t(n), err);
    uint32_t* dFlags = dalloc<uint32_t>(n, err);
    float* dSah = dalloc<float>(2, err);
    // wide nodes: at most one per internal binary node
    uint32_t maxWide = n;  // internal binary nodes = n - 1, plus the root of a one-triangle scene
    out.nodes = dalloc<WideNode>(maxWide, err);
    out.tris = dalloc<TriRecord>(n, err);
    CollapseItem* dQueue[2] = {dalloc<CollapseItem>(maxWide, err), dalloc<CollapseItem>(maxWide, err)};
    uint32_t* dCounters = dalloc<uint32_t>(4, err);  // nodeCursor, triCursor, outCount
    if (err != cudaSuccess) goto done;

    cudaMemcpyAsync(dXf, xf.data(), sizeof(MeshXform) * in.meshCount, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(dTriBase, triBase.data(), sizeof(uint32_t) * (in.meshCount + 1), cudaMemcpyHostToDevice, stream);
    {
        uint32_t b = 256, g = (n + b - 1) / b;
        kFlatten<<<g, b, 0, stream>>>(in.vertices, in.indices, in.meshes, dTriBase, dXf, in.meshCount, n, dTrisFlat,
                                      dTriLo, dTriHi);
        uint32_t init[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u, 0u};
        cudaMemcpyAsync(dBounds, init, sizeof(init), cudaMemcpyHostToDevice, stream);
        kCentroidBounds<<<std::min<uint32_t>(g, 1024u), b, 0, stream>>>(dTriLo, dTriHi, n, dBounds);
        kMorton<<<g, b, 0, stream>>>(dTriLo, dTriHi, n, dBounds, dKeys[0], dVals[0]);
    }
    {
        int cur = 0;
        for (uint32_t pass = 0; pass < 8; ++pass) {
            uint32_t shift = pass * 8u;
            kRadixHistogram<<<numTiles, kSortThreads, 0, stream>>>(dKeys[cur], n, shift, numTiles, dHist);
            kScanExclusive<<<1, 1024, 0, stream>>>(dHist, 256u * numTiles);
            kRadixScatter<<<numTiles, kSortThreads, 0, stream>>>(dKeys[cur], dVals[cur], n, shift, numTiles, dHist,
                                                                 dKeys[cur ^ 1], dVals[cur ^ 1]);
            cur ^= 1;
        }
        // 8 passes: sorted data is back in buffer 0
    }
    {
        uint32_t b = 256;
        if (n > 1) kKarras<<<(n - 1 + b - 1) / b, b, 0, stream>>>(dKeys[0], n, dLeft, dRight, dParent);
        else {
            uint32_t inv = kInvalid;
            cudaMemcpyAsync(dParent, &inv, sizeof(uint32_t), cudaMemcpyHostToDevice, stream);
        }
        kInitLeaves<<<(n + b - 1) / b, b, 0, stream>>>(dVals[0], dTriLo, dTriHi, n, dLo, dHi, dLeafCount, dCost, dFlags);
        if (n > 1) kRefit<<<(n + b - 1) / b, b, 0, stream>>>(n, dLeft, dRight, dParent, dLo, dHi, dLeafCount, dCost, dFlags);
        if (n > 2) {
            kRootSah<<<1, 1, 0, stream>>>(dLo, dHi, dCost, dSah);
            // each pass rewires parent[] along with the children, so the next one walks the restructured tree
            for (uint32_t pass = 0; pass < in.treeletPasses; ++pass) {
                cudaMemsetAsync(dFlags, 0, sizeof(uint32_t) * n, stream);
                kTreelets<<<(n + kTreeletThreads - 1) / kTreeletThreads, kTreeletThreads, 0, stream>>>(
                    n, kTreeletLeaves, dLeft, dRight, dParent, dLo, dHi, dLeafCount, dCost, dFlags);
            }
            kRootSah<<<1, 1, 0, stream>>>(dLo, dHi, dCost, dSah + 1);
        }
        // SAH-optimal choice of each wide node's children
        kWideCostLeaves<<<(n + b - 1) / b, b, 0, stream>>>(n, dLo, dHi, dWideCost, dWideDec, dFlags);
        if (n > 1)
            kWideCost<<<(n + b - 1) / b, b, 0, stream>>>(n, dLeft, dRight, dParent, dLo, dHi, dLeafCount, dWideCost,
                                                         dWideDec, dFlags);
    }
    {
        // level-by-level collapse; the root wide node is slot 0
        uint32_t rootBinary = n > 1 ? 0u : 0u;  // internal root is node 0; a single leaf is node n-1 = 0
        CollapseItem root{rootBinary, 0u};
        cudaMemcpyAsync(dQueue[0], &root, sizeof(root), cudaMemcpyHostToDevice, stream);
        uint32_t counters[4] = {1u, 0u, 0u, 0u};
        cudaMemcpyAsync(dCounters, counters, sizeof(counters), cudaMemcpyHostToDevice, stream);
        uint32_t inCount = 1;
        int q = 0;
        for (int level = 0; level < 128 && inCount > 0; ++level) {
            uint32_t zero = 0u;
            cudaMemcpyAsync(dCounters + 2, &zero, sizeof(zero), cudaMemcpyHostToDevice, stream);
            kCollapse<<<(inCount + 127) / 128, 128, 0, stream>>>(n, dQueue[q], inCount, dQueue[q ^ 1], dCounters + 2,
                                                                 dLeft, dRight, dLo, dHi, dLeafCount, dWideDec,
                                                                 dVals[0],
                                                                 dTrisFlat, dCounters, dCounters + 1, out.nodes,
                                                                 out.tris);
            err = cudaMemcpyAsync(&inCount, dCounters + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
            if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
            if (err != cudaSuccess) goto done;
            q ^= 1;
        }
        uint32_t finalCounters[2];
        err = cudaMemcpyAsync(finalCounters, dCounters, sizeof(finalCounters), cudaMemcpyDeviceToHost, stream);
        if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
        if (err != cudaSuccess) goto done;
        out.nodeCount = finalCounters[0];
        out.triCount = finalCounters[1];
    }
    cudaEventRecord(e1, stream);
    err = cudaEventSynchronize(e1);
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->buildMs = ms;
        stats->nodeCount = out.nodeCount;
        stats->triCount = out.triCount;
        float sah[2] = {0.0f, 0.0f};
        if (n > 2 && cudaMemcpy(sah, dSah, sizeof(sah), cudaMemcpyDeviceToHost) == cudaSuccess) {
            stats->sahLbvh = sah[0];
            stats->sahTreelets = sah[1];
        }
    }
    if (err == cudaSuccess && out.triCount != n) err = cudaErrorUnknown;

done:
    cudaFree(dXf);
    cudaFree(dTriBase);
    cudaFree(dTrisFlat);
    cudaFree(dLo);
    cudaFree(dHi);
    cudaFree(dTriLo);
    cudaFree(dTriHi);
    cudaFree(dBounds);
    cudaFree(dKeys[0]);
    cudaFree(dKeys[1]);
    cudaFree(dVals[0]);
    cudaFree(dVals[1]);
    cudaFree(dHist);
    cudaFree(dLeft);
    cudaFree(dRight);
    cudaFree(dParent);
    cudaFree(dLeafCount);
    cudaFree(dCost);
    cudaFree(dWideCost);
    cudaFree(dWideDec);
    cudaFree(dFlags);
    cudaFree(dSah);
    cudaFree(dQueue[0]);
    cudaFree(dQueue[1]);
    cudaFree(dCounters);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) out.release();
    return err;
}

void BvhBuffers::release() {
    if (nodes) cudaFree(nodes);
    if (tris) cudaFree(tris);
    nodes = nullptr;
    tris = nullptr;
    nodeCount = 0;
    triCount = 0;
}

}  // namespace vkrt
