// wavefront.cu — batched wavefront path tracing on sm_103a.
//
// One call renders one frame of every scene of a batch (one or many contexts of uneven size) with the same per-vertex
// arithmetic as the megakernel (path.cuh), restructured into persistent stage kernels over compacted queues:
//
//   setup, init                      reset counters; every path slot takes a (pixel, sample) item and starts it
//   while (paths remain)             one conditional-while CUDA graph node, two ping-pong iterations per body:
//     begin                          reset the output queues (and the material histogram)
//     intersect                      closest hit of every queued path; material key + histogram when sorting
//     sort (optional)                counting sort of the queue by (scene, class) with class = miss /
//                                    dielectric / metal; or, in class mode, the intersect kernel itself files
//                                    each path under its class (no scene grouping, no extra kernels)
//     shade                          pending shadow results applied, vertex shaded, shadow requests queued,
//                                    continuing paths queued, finished ones handed to finalize
//     shadow                         any-hit rays; visible requests flagged on their slot
//     finalize                       the sample's result stored in its item's place; the slot takes the next item
//     condition                      cudaGraphSetConditional(more work && iteration < bound)
//   resolve                          per pixel, results summed in sample order, blended into the running mean,
//                                    encoded for display
//
// Items are handed out from one cursor over all scenes of the batch; the items of a pixel are consecutive and pixels
// follow a tile order (tileWidth x tileHeight, row-major). Every slot stays busy until the cursor runs out, and
// because each pixel's samples are summed in sample order by one thread of the resolve kernel the image is
// deterministic, needs no atomics on the film, and equals the megakernel's bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "adjoint.cuh"
#include "nrc.h"
#include "wavefront.h"

namespace vkrt {

namespace {

constexpr uint32_t kWfThreads = 128;
// counts[]: queue lengths (queue0, queue1, shadow, finished), the item cursor, the iteration, the fetch cursors
enum : uint32_t {
    kCntActive0 = 0,
    kCntActive1 = 1,
    kCntShadow = 2,
    kCntFinished = 3,
    kCntCursor = 4,
    kCntIteration = 5,
    kCntFetchIntersect = 6,
    kCntFetchShadow = 7,
    kCntClass0 = 8,  // class-partitioned shade queue: misses, dielectric hits, metal hits
    kCntQueries = 11,  // radiance-cache queries of the iteration
    kCntBin0 = 16,     // with rayOrder: entries per direction-octant bin, kRayBins for queue 0 then for queue 1
    kCntCount = 32,
};
constexpr uint32_t kPendCache = 16u;        // pendFlags: the path ended at a radiance-cache query
constexpr uint32_t kPendUnsupported = 32u;  // pendFlags: an NEE shadow ray met a transmissive surface
// sortByMaterial (0: as traced); 1 counting-sorts by (scene, class), 3 by material (both kSortMaterial in the
// kernels, with WfGlobals::keyByMaterial telling the keys apart); 2 files hits into class queues
constexpr uint32_t kSortMaterial = 1, kSortClass = 2, kSortMaterialIndex = 3;


struct WfGlobals {
    uint32_t mode;  // WavefrontMode
    // forward frames: the shade kernel writes the result of a path that ends with nothing pending (no shadow ray, no
    // cache query); with refills (fewer slots than items) the slot still goes to the finalize kernel, marked
    // kFinishedDone, only to take its next item
    uint32_t directFinish;
    uint32_t refills;
    // no tile padding, so slot s starts item s for every slot (Q never exceeds the item count): the first queue is the
    // slot order itself, filled without atomics, which keeps the camera rays in tile order for the first traversal
    uint32_t identityStart;
    // radiance-cache training pass (kWavefrontTrain): per slot up to kNrcTrainVerts surface vertices, then records
    NrcInput* trainIn;     // Q x kNrcTrainVerts: the cache inputs of each vertex
    float4* trainThr;      // the throughput that reached each vertex
    float4* trainRad;      // the path radiance after each vertex's emission, before its light samples
    uint32_t* trainCount;  // vertices recorded per slot
    NrcInput* recIn;       // training records of the frame
    float4* recTarget;
    uint32_t* recCount;
    uint32_t maxRecords;
    uint32_t trainSeed, trainFrame;
    const WfScene* scenes;
    const uint32_t* itemBases;  // scenes[i].itemBase, contiguous for the item -> scene search
    const uint32_t* workBases;  // scenes[i].workBase
    uint32_t sceneCount;
    uint32_t totalWork;   // padded pixels of all scenes
    uint32_t totalItems;  // (pixel, sample) items of all scenes
    uint32_t Q;
    uint32_t maxIter;
    uint32_t sort;
    int refill;  // persistent traversal refill threshold
    uint32_t keyCount;
    uint32_t keyByMaterial;  // sort keys: 0 (scene, class), 1 0 for misses and 1 + materialKeyBase + material index
    uint32_t rngMode;
    uint64_t rngSeed;
    // path record: one 128-byte line per slot (kRec* words of 16 bytes), so a record read through a queue of scattered
    // slots touches one line
    float4* rec;
    uint32_t* slotScene;
    uint32_t* slotItem;    // (pixel, sample) item within the scene
    float4* sampleBuf;     // one result per item, summed per pixel in sample order by the resolve kernel
    uint32_t* hitKey;
    float4* pend0;
    float4* pend1;
    uint32_t* pendFlags;  // bit 0/1: request 0/1 pending, bit 2/3: request 0/1 visible
    // queues
    uint32_t* queue0;       // traversal queues: Q entries, or kRayBins bins of Q entries with rayOrder
    uint32_t* queue1;
    uint32_t rayOrder;
    uint32_t* finished;
    uint32_t* sorted;
    uint32_t* classQueue;  // 3 * Q: the shade queue partitioned by class (kSortClass)
    float4* shadowA;  // origin, tmax
    float4* shadowB;  // direction, slot | request << 31
    uint32_t* keyHist;
    uint32_t* counts;
    RenderCounters* counters;
    uint32_t launchesOutsideLoop;  // setup/clear/init/resolve kernels of one render call
    uint32_t launchesPerBody;      // stage kernels of two iterations plus the condition kernel
    cudaGraphConditionalHandle cond;
    // adjoint pass (one scene): parameters and, per slot, the pending vertex's gradient factors
    AdjointParams adj;
    float4* adjDelta;   // d(loss)/d(sample radiance) of the slot's item
    float4* adjTotal;   // the item's radiance from the primal pass
    float4* adjUv;      // uv0.xy, uv1.xy of the pending vertex
    float4* adjColor;   // its vertex colour
    float4* adjReq0;    // request 0: delta * factor * Le * df/dbase (xyz), roughness term (w)
    float4* adjReq1;
    float4* adjEm0;     // request 0: delta * factor * f (xyz), emissive mesh (w bits)
    float4* adjEm1;
    float4* adjRatioB;  // (df/dbase) / f (xyz), material index (w bits)
    float4* adjRatioR;  // (df/droughness) / f (xyz), kAdjFlag* bits (w)
    // radiance cache: paths end at surface depth cacheDepth (0xFFFFFFFF = off) with a query
    uint32_t cacheDepth;
    float cacheSpread;  // > 0: paths also end at the cache by the area-spread rule with this constant
    NrcInput* nrcQueries;  // Q inputs of the iteration's queries
    uint32_t* slotQuery;   // query position of a slot whose path ended at the cache
    float4* nrcPred;       // predictions, by query position
    // denoiser features (forward frames of scenes with feature films): per (pixel, sample) item, albedo and shading
    // normal of the first non-specular vertex, .w = 1 once taken
    uint32_t features;
    float4* itemFeatA;
    float4* itemFeatN;
    // scenes with transmissive materials: per slot, hero lanes 1-3 of the technique pdfs and the medium's absorption
    // (extA = techYZW + sigma.x, extB = prevVertexYZW + sigma.y, extC = prevBsdfYZW + sigma.z, extD = sigma.w)
    uint32_t transmissive;
    uint32_t alpha;        // some scene has alpha-tested materials: per slot, the alpha seed of the slot's ray
    uint32_t* alphaSeed;
    float4* extA;
    float4* extB;
    float4* extC;
    float* extD;
};

// finished-queue entries whose result the shade kernel has written already (slot numbers stay below 2^28)
constexpr uint32_t kFinishedDone = 0x80000000u;

VKRT_DEV uint32_t warpPush(uint32_t* counter, bool want) {
    unsigned mask = __activemask();
    unsigned ballot = __ballot_sync(mask, want);
    if (!ballot) return 0xFFFFFFFFu;
    int lane = threadIdx.x & 31;
    int leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(ballot));
    base = __shfl_sync(mask, base, leader);
    return want ? base + __popc(ballot & ((1u << lane) - 1u)) : 0xFFFFFFFFu;
}

// warp-aggregated counter increment; every stage loop keeps whole warps together, so the warp is reconverged first
VKRT_DEV void warpCount(unsigned long long* counter, uint32_t v) {
    __syncwarp();
    uint32_t total = __reduce_add_sync(0xFFFFFFFFu, v);
    if ((threadIdx.x & 31u) == 0u && total) atomicAdd(counter, (unsigned long long)total);
}

VKRT_DEV uint32_t sceneOfWork(const WfGlobals& g, uint32_t w) {
    uint32_t lo = 0, hi = g.sceneCount;
    while (hi - lo > 1u) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(g.workBases + mid) <= w) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Position among the converged lanes that hold the same key, with one atomic per distinct key: counters[key] is
// advanced by the number of such lanes.
VKRT_DEV uint32_t warpAggregatedSlot(uint32_t* counters, uint32_t key) {
    const unsigned active = __activemask();
    const unsigned same = __match_any_sync(active, key);
    const uint32_t lane = threadIdx.x & 31u;
    const int leader = __ffs(same) - 1;
    uint32_t base = 0u;
    if (lane == uint32_t(leader)) base = atomicAdd(counters + key, uint32_t(__popc(same)));
    base = __shfl_sync(same, base, leader);
    return base + __popc(same & ((1u << lane) - 1u));
}

constexpr uint32_t kRayBins = 8;  // direction octants

// octant of a direction: bit k set when component k is negative
VKRT_DEV uint32_t dirOctant(float3 d) {
    return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
}

// Files slot `slot`, whose next ray has direction `dir`, into traversal queue `queue` when `want`; whole warps call
// it. With rayOrder the queue is kRayBins bins of Q entries, one per direction octant, and counts[queue] keeps the
// total.
VKRT_DEV void queuePush(const WfGlobals& g, uint32_t queue, bool want, uint32_t slot, float3 dir) {
    uint32_t* q = queue == 0 ? g.queue0 : g.queue1;
    const uint32_t pos = warpPush(&g.counts[queue], want);
    if (!want) return;
    if (!g.rayOrder) {
        q[pos] = slot;
        return;
    }
    const uint32_t b = dirOctant(dir);
    q[size_t(b) * g.Q + warpAggregatedSlot(&g.counts[kCntBin0 + kRayBins * queue], b)] = slot;
}

// The running ends of queue `queue`'s bins, written by thread 0 into `binEnd` (shared memory; the caller
// synchronises the block before use).
VKRT_DEV void loadBinEnds(const WfGlobals& g, uint32_t queue, uint32_t* binEnd) {
    if (threadIdx.x != 0u || !g.rayOrder) return;
    uint32_t s = 0;
    for (uint32_t b = 0; b < kRayBins; ++b) {
        s += g.counts[kCntBin0 + kRayBins * queue + b];
        binEnd[b] = s;
    }
}

// entry i of a traversal queue read as one sequence (bins in octant order with rayOrder)
VKRT_DEV uint32_t queueEntry(const WfGlobals& g, const uint32_t* q, const uint32_t* binEnd, uint32_t i) {
    if (!g.rayOrder) return q[i];
    uint32_t b = 0, start = 0;
    while (b + 1u < kRayBins && i >= binEnd[b]) {
        start = binEnd[b];
        ++b;
    }
    return q[size_t(b) * g.Q + (i - start)];
}

// the scene of a slot; frames of one scene neither write nor read the per-slot array (a scattered 4-byte access per
// item, in front of each shadow ray's traversal)
VKRT_DEV uint32_t sceneOfSlot(const WfGlobals& g, uint32_t slot) {
    return g.sceneCount == 1u ? 0u : g.slotScene[slot];
}

// miss / dielectric / metal
VKRT_DEV uint32_t hitClass(const DeviceScene& sc, const TraceHit& h) {
    if (h.mesh == VKRT_CUDA_INVALID_INDEX) return 0u;
    return sc.materials[sc.meshes[h.mesh].materialIndex].metallic >= 0.5f ? 2u : 1u;
}

// tile-ordered work item -> viewport pixel; false for padding items outside the viewport
VKRT_DEV bool workPixel(const WfScene& S, uint32_t local, int& px, int& py) {
    uint32_t tileArea = S.tileW * S.tileH;
    uint32_t t = local / tileArea, i = local % tileArea;
    uint32_t tx = t % S.tilesX, ty = t / S.tilesX;
    uint32_t x = tx * S.tileW + i % S.tileW, y = ty * S.tileH + i / S.tileW;
    if (x >= S.vw || y >= S.vh) return false;
    px = int(S.vx0 + x);
    py = int(S.vy0 + y);
    return true;
}

// words of a slot's record: origin + depth, direction + flags (together one 32-byte sector, all the traversal reads),
// RNG state, throughput, radiance, MIS terms (lamUnit, techPath, prevVertexTech, prevBsdfTech), previous BSDF pdf with
// the cache's area-spread terms and the closest hit's v, the closest hit (mesh, primitive, t, u). The traversal writes
// the hit into the record's last sector, which the shade kernel reads with the path state.
enum : uint32_t { kRecOrigin = 0, kRecDir, kRecRng, kRecThr, kRecRad, kRecMis, kRecPdf, kRecHit, kRecWords };

VKRT_DEV float4* record(const WfGlobals& g, uint32_t s) { return g.rec + size_t(s) * kRecWords; }

VKRT_DEV void packRecord(float4* r, const PathState& p) {
    r[kRecRng] = make_float4(__uint_as_float(uint32_t(p.rng.state)), __uint_as_float(uint32_t(p.rng.state >> 32)),
                             __uint_as_float(uint32_t(p.rng.inc)), __uint_as_float(uint32_t(p.rng.inc >> 32)));
    r[kRecOrigin] = make_float4(p.o.x, p.o.y, p.o.z, __uint_as_float(p.depth));
    r[kRecDir] = make_float4(p.d.x, p.d.y, p.d.z, __uint_as_float(p.flags));
    r[kRecThr] = p.thr;
    r[kRecRad] = p.radiance;
    r[kRecMis] = make_float4(p.lamUnit, p.techPath, p.prevVertexTech, p.prevBsdfTech);
    r[kRecPdf] = make_float4(p.prevBsdfPdf, p.spread, p.spreadA0, 0.0f);
}

VKRT_DEV void storePath(const WfGlobals& g, uint32_t s, const PathState& p) { packRecord(record(g, s), p); }

VKRT_DEV PathState loadPath(const WfGlobals& g, uint32_t s) {
    PathState p;
    const float4* rp = record(g, s);
    const float4 r = rp[kRecRng];
    p.rng.state = uint64_t(__float_as_uint(r.x)) | (uint64_t(__float_as_uint(r.y)) << 32);
    p.rng.inc = uint64_t(__float_as_uint(r.z)) | (uint64_t(__float_as_uint(r.w)) << 32);
    const float4 o = rp[kRecOrigin], d = rp[kRecDir];
    p.o = make_float3(o.x, o.y, o.z);
    p.depth = __float_as_uint(o.w);
    p.d = make_float3(d.x, d.y, d.z);
    p.flags = __float_as_uint(d.w);
    p.thr = rp[kRecThr];
    p.radiance = rp[kRecRad];
    const float4 m = rp[kRecMis];
    p.lamUnit = m.x;
    p.techPath = m.y;
    p.prevVertexTech = m.z;
    p.prevBsdfTech = m.w;
    const float4 pd = rp[kRecPdf];
    p.prevBsdfPdf = pd.x;
    p.spread = pd.y;
    p.spreadA0 = pd.z;
    return p;
}

// The full instantiations' part of the slot state. Without transmissive materials the hero lanes stay equal and no
// medium is entered, so lanes 1-3 repeat lane 0.
VKRT_DEV void storePathExt(const WfGlobals& g, uint32_t s, const PathState& p) {
    if (!g.transmissive) return;
    g.extA[s] = make_float4(p.techYZW.x, p.techYZW.y, p.techYZW.z, p.sigma.x);
    g.extB[s] = make_float4(p.prevVertexYZW.x, p.prevVertexYZW.y, p.prevVertexYZW.z, p.sigma.y);
    g.extC[s] = make_float4(p.prevBsdfYZW.x, p.prevBsdfYZW.y, p.prevBsdfYZW.z, p.sigma.z);
    g.extD[s] = p.sigma.w;
}

VKRT_DEV void loadPathExt(const WfGlobals& g, uint32_t s, PathState& p) {
    if (!g.transmissive) {
        p.techYZW = f3(p.techPath);
        p.prevVertexYZW = f3(p.prevVertexTech);
        p.prevBsdfYZW = f3(p.prevBsdfTech);
        p.sigma = f4(0.0f);
        return;
    }
    const float4 a = g.extA[s], b = g.extB[s], c = g.extC[s];
    p.techYZW = xyz(a);
    p.prevVertexYZW = xyz(b);
    p.prevBsdfYZW = xyz(c);
    p.sigma = make_float4(a.w, b.w, c.w, g.extD[s]);
}

VKRT_DEV StepConfig stepConfig(const WfGlobals& g, const WfScene& S) {
    StepConfig cfg{S.spectral != 0u, S.neeEnabled != 0u, S.envNee != 0u, g.rngMode, g.rngSeed, g.cacheDepth};
    cfg.cacheSpread = g.cacheSpread;
    cfg.single = S.spectral != 0u && singleWavelength(S.sd);
    return cfg;
}

VKRT_DEV SpecTable specTable(const WfScene& S) {
    return makeSpecTable(S.sc, S.sd);
}

// starts sample `sample` of the slot's pixel; returns false for a padding work item
template <bool kSpectral>
VKRT_DEV bool startSample(const WfGlobals& g, const WfScene* scenes, uint32_t slot, uint32_t sceneId, uint32_t work,
                          uint32_t sample, PathState* held) {
    const WfScene& S = scenes[sceneId];
    int px, py;
    PathState p;
    uint32_t pix = 0;
    if (g.mode == kWavefrontTrain) {
        // training path `work`: a hashed pixel of the viewport and its own random stream (sample index 2^30 + work),
        // as the one-thread-per-path training kernel chooses them
        if (S.vw == 0u || S.vh == 0u) return false;
        const uint32_t h0 = wellonsHash(g.trainSeed ^ (g.trainFrame * 0x9e3779b9u) ^ (work * 0x85ebca6bu));
        px = int(S.vx0 + h0 % S.vw);
        py = int(S.vy0 + wellonsHash(h0) % S.vh);
        p = beginPath<kSpectral>(stepConfig(g, S), S.sd, px, py, 0x40000000u + work);
        g.trainCount[slot] = 0u;
    } else {
        if (!workPixel(S, work, px, py)) return false;
        pix = uint32_t(py) * S.filmWidth + uint32_t(px);
        // a frame continues the film's sample count; the primal and adjoint passes replay the samples from sampleBase
        uint32_t first = g.mode == kWavefrontForward ? uint32_t(S.film.accumRead[pix].w + 0.5f) : g.adj.sampleBase;
        p = beginPath<kSpectral>(stepConfig(g, S), S.sd, px, py, first + sample);
    }
    if (held) *held = p;
    else storePath(g, slot, p);
    storePathExt(g, slot, p);
    g.pendFlags[slot] = 0u;
    if (g.mode == kWavefrontAdjoint) {
        float inv = 1.0f / float(g.adj.sampleBase + S.spp);
        g.adjDelta[slot] = g.adj.dImage[pix] * inv;
        g.adjRatioR[slot] = f4(0.0f);  // no pending vertex
    }
    return true;
}

VKRT_DEV uint32_t sceneOfItem(const WfGlobals& g, uint32_t w) {
    uint32_t lo = 0, hi = g.sceneCount;
    while (hi - lo > 1u) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(g.itemBases + mid) <= w) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Takes (pixel, sample) items from the cursor, starting with `w`, until one lies inside a viewport; false when the
// batch is exhausted. Items of one pixel are consecutive (item = pixel work index * spp + sample). With `held` the
// new path's record is returned there instead of stored.
template <bool kSpectral>
VKRT_DEV bool acquireItem(const WfGlobals& g, const WfScene* scenes, uint32_t slot, uint32_t w,
                          PathState* held = nullptr) {
    for (;;) {
        if (w >= g.totalItems) return false;
        uint32_t sceneId = sceneOfItem(g, w);
        const WfScene& S = scenes[sceneId];
        uint32_t local = w - S.itemBase;
        if (startSample<kSpectral>(g, scenes, slot, sceneId, local / S.spp, local % S.spp, held)) {
            if (g.sceneCount != 1u) g.slotScene[slot] = sceneId;
            g.slotItem[slot] = local;
            if (g.features) {
                g.itemFeatA[size_t(S.itemBase) + local] = f4(0.0f);
                g.itemFeatN[size_t(S.itemBase) + local] = f4(0.0f);
            }
            if (g.mode == kWavefrontAdjoint) g.adjTotal[slot] = g.sampleBuf[size_t(S.itemBase) + local];
            return true;
        }
        w = atomicAdd(&g.counts[kCntCursor], 1u);
    }
}

__global__ void kWfSetup(WfGlobals g) {
    if (threadIdx.x < kCntCount) g.counts[threadIdx.x] = 0u;
    if (threadIdx.x == 0u) {
        if (g.identityStart) g.counts[kCntActive0] = g.Q;
        g.counts[kCntCursor] = min(g.Q, g.totalItems);
        atomicAdd(&g.counters->kernelLaunches, (unsigned long long)g.launchesOutsideLoop);
    }
}

// A warp starts 32 consecutive slots, whose records are one contiguous 4 KB run: the records are assembled in shared
// memory (rows of kRecWords + 1 words, so the 16-byte writes of 8 lanes fall on distinct banks) and stored as 8
// coalesced warp-wide stores instead of 8 stores that each touch 32 lines.
template <bool kSpectral>
__global__ void __launch_bounds__(kWfThreads) kWfInit(WfGlobals g) {
    constexpr uint32_t kRow = kRecWords + 1u;
    __shared__ float4 stage[kWfThreads * kRow];
    const WfScene* scenes = g.scenes;
    const uint32_t lane = threadIdx.x & 31u;
    float4* ws = stage + (threadIdx.x >> 5) * 32u * kRow;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < g.Q; base += stride) {
        const uint32_t s = base + lane;
        PathState p;
        bool ok = false;
        if (s < g.Q) ok = acquireItem<kSpectral>(g, scenes, s, s < g.totalItems ? s : g.totalItems, &p);
        if (ok) packRecord(ws + lane * kRow, p);
        const unsigned okMask = __ballot_sync(0xFFFFFFFFu, ok);
        __syncwarp();
        float4* out = g.rec + size_t(base) * kRecWords;
#pragma unroll
        for (uint32_t k = 0; k < kRecWords; ++k) {
            const uint32_t j = k * 32u + lane, owner = j / kRecWords;
            if ((okMask >> owner) & 1u) out[j] = ws[owner * kRow + j % kRecWords];
        }
        __syncwarp();
        if (g.identityStart) {  // every slot below Q starts its own item
            if (s < g.Q) g.queue0[s] = s;
        } else {
            queuePush(g, 0u, ok, s, p.d);
        }
    }
}

// Per pixel: the samples' results summed in sample order (as one thread summing its pixel's samples would), blended
// into the running mean (writeback.slang:72-114) and encoded for display.
template <bool kSpectral>
__global__ void kWfResolve(WfGlobals g) {
    const WfScene* scenes = g.scenes;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < g.totalWork; w += gridDim.x * blockDim.x) {
        const WfScene& S = scenes[sceneOfWork(g, w)];
        uint32_t local = w - S.workBase;
        int px, py;
        if (!workPixel(S, local, px, py)) continue;
        const float4* r = g.sampleBuf + size_t(S.itemBase) + size_t(local) * S.spp;
        float3 sum = f3(0.0f);
        for (uint32_t s = 0; s < S.spp; ++s) sum += xyz(r[s]);
        uint32_t pix = uint32_t(py) * S.filmWidth + uint32_t(px);
        float4 prev = S.film.accumRead[pix];
        float pw = float(uint32_t(prev.w + 0.5f)), tw = pw + float(S.spp);
        float3 cur = sum / float(S.spp);
        float3 acc = tw <= 0.0f ? f3(0.0f) : (xyz(prev) * pw + cur * float(S.spp)) / tw;
        S.film.accumWrite[pix] = make_float4(acc.x, acc.y, acc.z, tw);
        S.film.output[pix] = encodeOutput(S.sd, acc, kSpectral);
        if (g.features && S.film.albedoWrite) {
            const float4* fa = g.itemFeatA + size_t(S.itemBase) + size_t(local) * S.spp;
            const float4* fn = g.itemFeatN + size_t(S.itemBase) + size_t(local) * S.spp;
            float3 as = f3(0.0f), ns = f3(0.0f);
            float wsum = 0.0f;
            for (uint32_t s = 0; s < S.spp; ++s) {
                as += xyz(fa[s]);
                ns += xyz(fn[s]);
                wsum += fa[s].w;
            }
            blendFeature(S.film.albedoRead, S.film.albedoWrite, pix, as, wsum);
            blendFeature(S.film.normalRead, S.film.normalWrite, pix, ns, wsum);
        }
    }
}

// screen-space clear of film pixels outside each scene's viewport (writeback of raygen for !insideViewport)
__global__ void kWfClearOutside(WfGlobals g) {
    for (uint32_t si = blockIdx.y; si < g.sceneCount; si += gridDim.y) {
        const WfScene& S = g.scenes[si];
        uint32_t n = S.filmWidth * S.filmHeight;
        if (S.vx0 == 0u && S.vy0 == 0u && S.vw == S.filmWidth && S.vh == S.filmHeight) continue;
        for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
            uint32_t x = p % S.filmWidth, y = p / S.filmWidth;
            if (x >= S.vx0 && y >= S.vy0 && x < S.vx0 + S.vw && y < S.vy0 + S.vh) continue;
            S.film.accumWrite[p] = f4(0.0f);
            S.film.output[p] = make_ushort4(0, 0, 0, 0);
            if (S.film.albedoWrite) S.film.albedoWrite[p] = S.film.normalWrite[p] = f4(0.0f);
        }
    }
}

__global__ void kWfBegin(WfGlobals g, uint32_t outQueue) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        g.counts[outQueue] = 0u;
        g.counts[kCntShadow] = 0u;
        g.counts[kCntFinished] = 0u;
        g.counts[kCntFetchIntersect] = 0u;
        g.counts[kCntFetchShadow] = 0u;
        g.counts[kCntClass0] = g.counts[kCntClass0 + 1] = g.counts[kCntClass0 + 2] = 0u;
        g.counts[kCntQueries] = 0u;
        for (uint32_t b = 0; b < kRayBins; ++b) g.counts[kCntBin0 + kRayBins * outQueue + b] = 0u;
    }
    if (g.sort == kSortMaterial)
        for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < g.keyCount; k += gridDim.x * blockDim.x)
            g.keyHist[k] = 0u;
}

// node (80 B) and triangle (48 B) fetch bytes of a warp's traversals, for the profiling frames
VKRT_DEV void warpCountBytes(unsigned long long* nodeBytes, unsigned long long* triBytes, uint32_t nodes,
                             uint32_t tris) {
    __syncwarp();
    uint32_t n = __reduce_add_sync(0xFFFFFFFFu, nodes), t = __reduce_add_sync(0xFFFFFFFFu, tris);
    if ((threadIdx.x & 31u) == 0u) {
        if (n) atomicAdd(nodeBytes, 80ull * n);
        if (t) atomicAdd(triBytes, 48ull * t);
    }
}

// kMinBlocks: resident blocks per SM the register allocation must allow (the launch grid's blocks per SM)
// The closest hit of queue entry i (slot `slot`): hit records, and the sort key or class queue entry
VKRT_DEV void storeHit(const WfGlobals& g, uint32_t i, uint32_t slot, const TraceHit& h) {
    float4* r = record(g, slot);
    r[kRecHit] = make_float4(__uint_as_float(h.mesh), __uint_as_float(h.prim), h.t, h.u);
    reinterpret_cast<float*>(r + kRecPdf)[3] = h.v;
    if (g.sort == kSortMaterial) {  // histogram of (scene, class) or material keys for the counting sort
        const uint32_t sceneId = sceneOfSlot(g, slot);
        const WfScene& S = g.scenes[sceneId];
        const uint32_t key = !g.keyByMaterial ? 3u * sceneId + hitClass(S.sc, h)
                             : h.mesh == VKRT_CUDA_INVALID_INDEX
                                 ? 0u
                                 : 1u + S.materialKeyBase + S.sc.meshes[h.mesh].materialIndex;
        g.hitKey[i] = key;
        warpAggregatedSlot(g.keyHist, key);
    } else if (g.sort == kSortClass) {  // filed straight into the class queues
        const uint32_t c = hitClass(g.scenes[sceneOfSlot(g, slot)].sc, h);
        const uint32_t pos = warpAggregatedSlot(&g.counts[kCntClass0], c);
        g.classQueue[size_t(c) * g.Q + pos] = slot;
    }
}

template <bool kCount, int kMinBlocks>
__global__ void __launch_bounds__(kWfThreads, kMinBlocks) kWfIntersect(WfGlobals g, uint32_t inQueue) {
    extern __shared__ uint2 smemStack[];
    __shared__ uint32_t binEnd[kRayBins];
    const uint32_t* q = inQueue == 0 ? g.queue0 : g.queue1;
    const uint32_t n = g.counts[inQueue];
    loadBinEnds(g, inQueue, binEnd);
    __syncthreads();
    uint32_t primary = 0, ext = 0, nodeVisits = 0, triTests = 0;
    persistentTraceVote<false, kCount>(
        n, &g.counts[kCntFetchIntersect], smemStack + threadIdx.x, blockDim.x, &g.counters->errorFlags, g.refill,
        [&](uint32_t i, TraceRay& r, const WideNode*& nodes, const TriRecord*& tris, uint32_t& nodeCount) {
            uint32_t slot = queueEntry(g, q, binEnd, i);
            const DeviceScene& sc = g.scenes[sceneOfSlot(g, slot)].sc;
            const float4* rp = record(g, slot);
            float4 o = rp[kRecOrigin], d = rp[kRecDir];
            r = TraceRay{make_float3(o.x, o.y, o.z), make_float3(d.x, d.y, d.z), kTMin, kTMax};
            nodes = sc.nodes;
            tris = sc.tris;
            nodeCount = sc.nodeCount;
            if (__float_as_uint(o.w) == 0u) ++primary;
            else ++ext;
        },
        [&](uint32_t i, const TraceHit& h) { storeHit(g, i, queueEntry(g, q, binEnd, i), h); }, nodeVisits,
        triTests);
    warpCount(&g.counters->primaryRays, primary);
    warpCount(&g.counters->extensionRays, ext);
    if (kCount) warpCountBytes(&g.counters->nodeBytes, &g.counters->triBytes, nodeVisits, triTests);
}

// Closest hits of scenes with alpha-tested materials: one ray per thread through traceBvh's alpha mode, seeded from
// the slot's random stream (the shade kernel keeps the seed for the vertex's shadow rays).
template <bool kCount>
__global__ void __launch_bounds__(kWfThreads) kWfIntersectAlpha(WfGlobals g, uint32_t inQueue) {
    extern __shared__ uint2 smemStack[];
    __shared__ uint32_t binEnd[kRayBins];
    const uint32_t* q = inQueue == 0 ? g.queue0 : g.queue1;
    const uint32_t n = g.counts[inQueue];
    loadBinEnds(g, inQueue, binEnd);
    __syncthreads();
    uint32_t primary = 0, ext = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        if (i < n) {
            const uint32_t slot = queueEntry(g, q, binEnd, i);
            const DeviceScene& sc = g.scenes[sceneOfSlot(g, slot)].sc;
            const float4* rp = record(g, slot);
            const float4 o = rp[kRecOrigin], d = rp[kRecDir], rf = rp[kRecRng];
            const uint4 rs = make_uint4(__float_as_uint(rf.x), __float_as_uint(rf.y), __float_as_uint(rf.z),
                                        __float_as_uint(rf.w));
            const TraceRay r{make_float3(o.x, o.y, o.z), make_float3(d.x, d.y, d.z), kTMin, kTMax};
            const TraceHit h = traceBvh<false, kCount, false, false, true>(
                sc, r, smemStack + threadIdx.x, blockDim.x, kCount ? g.counters : nullptr, 0u, rs.x ^ rs.y);
            if (__float_as_uint(o.w) == 0u) ++primary;
            else ++ext;
            storeHit(g, i, slot, h);
        }
    }
    warpCount(&g.counters->primaryRays, primary);
    warpCount(&g.counters->extensionRays, ext);
}

__global__ void __launch_bounds__(1024) kWfSortScan(WfGlobals g) {
    // exclusive scan of the key histogram in place (one block)
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (uint32_t base = 0; base < g.keyCount; base += 1024u) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < g.keyCount ? g.keyHist[i] : 0u;
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
            warpSums[threadIdx.x] = s;
        }
        __syncthreads();
        uint32_t incl = x + ((threadIdx.x >> 5) ? warpSums[(threadIdx.x >> 5) - 1u] : 0u);
        if (i < g.keyCount) g.keyHist[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023u) carry += incl;
        __syncthreads();
    }
}

__global__ void kWfSortScatter(WfGlobals g, uint32_t inQueue) {
    __shared__ uint32_t binEnd[kRayBins];
    const uint32_t* q = inQueue == 0 ? g.queue0 : g.queue1;
    const uint32_t n = g.counts[inQueue];
    loadBinEnds(g, inQueue, binEnd);
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t pos = warpAggregatedSlot(g.keyHist, g.hitKey[i]);
        g.sorted[pos] = queueEntry(g, q, binEnd, i);
    }
}

VKRT_DEV void applyPending(const WfGlobals& g, uint32_t slot, float4& radiance) {
    uint32_t f = g.pendFlags[slot];
    if ((f & 1u) && (f & 4u)) radiance += g.pend0[slot];
    if ((f & 2u) && (f & 8u)) radiance += g.pend1[slot];
}

// radiance-cache inputs of a vertex: world position, outgoing direction (toward the previous vertex), shading normal,
// roughness, base colour, metallic
VKRT_DEV NrcInput nrcInputOf(const Surface& s, const ShadeMaterial& m, float3 rayDir) {
    NrcInput in;
    in.posRough = make_float4(s.hitPoint.x, s.hitPoint.y, s.hitPoint.z, m.roughness);
    in.dirMetal = make_float4(-rayDir.x, -rayDir.y, -rayDir.z, m.metallic);
    in.normal = make_float4(s.shadingNormal.x, s.shadingNormal.y, s.shadingNormal.z, 0.0f);
    in.albedo = make_float4(m.baseColor.x, m.baseColor.y, m.baseColor.z, 0.0f);
    return in;
}

// forward-pass hook: records the radiance-cache query of a path that ends at the cache, and the denoiser feature
// (feat = null when features are off)
struct CacheHook : NoVertexHook {
    NrcInput* in;
    bool* queried;
    float3 rayDir;
    DenoiserFeature* feat;
    VKRT_DEV void surface(const Surface& s, const ShadeMaterial& m, const Bsdf&) {
        if (feat) captureFeature(*feat, s, m);
    }
    VKRT_DEV void cacheQuery(const Surface& s, const ShadeMaterial& m) {
        *in = nrcInputOf(s, m, rayDir);
        *queried = true;
    }
};

// training-path hook: records the cache inputs of every surface vertex
struct TrainHook : NoVertexHook {
    NrcInput* in;
    bool* has;
    float3 rayDir;
    VKRT_DEV void surface(const Surface& s, const ShadeMaterial& m, const Bsdf&) {
        *in = nrcInputOf(s, m, rayDir);
        *has = true;
    }
};

constexpr uint32_t kNrcTrainVerts = 16;  // vertices of a training path that become records

// Radiance-cache training paths: full-length paths from random pixels of scene 0 (their own random streams, sample
// indices from 2^30), traced and shaded like render paths. Each surface vertex j becomes a record whose target is
// the radiance the path gathered after the vertex's own emission, divided by the throughput that reached it: an
// unbiased estimate of what the vertex scatters toward the previous one (linear sRGB; hero paths convert the four
// wavelengths as a sample result is converted).
template <bool kSpectral, bool kExt>
__global__ void __launch_bounds__(kWfThreads) kNrcTrainPaths(const WfScene* __restrict__ scenes, uint32_t paths,
                                                             uint32_t frame, uint32_t seed, uint32_t rngMode,
                                                             uint64_t rngSeed, uint32_t maxRecords,
                                                             NrcInput* __restrict__ recIn,
                                                             float4* __restrict__ recTarget, uint32_t* recCount,
                                                             RenderCounters* counters) {
    extern __shared__ uint2 smemStack[];
    const WfScene& S = scenes[0];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t primary = 0, ext = 0, shadow = 0;
    if (i < paths && S.vw > 0u && S.vh > 0u) {
        const uint32_t h0 = wellonsHash(seed ^ (frame * 0x9e3779b9u) ^ (i * 0x85ebca6bu));
        const int px = int(S.vx0 + h0 % S.vw), py = int(S.vy0 + wellonsHash(h0) % S.vh);
        const StepConfig cfg{kSpectral, S.neeEnabled != 0u, S.envNee != 0u, rngMode, rngSeed};
        KernelCtx k{S.sc, S.sd, smemStack + threadIdx.x, blockDim.x, counters};
        const SpecTable tab = makeSpecTable(S.sc, S.sd);
        PathState p = beginPath<kSpectral>(cfg, S.sd, px, py, 0x40000000u + i);
        NrcInput vin[kNrcTrainVerts];
        float4 vthr[kNrcTrainVerts], vrad[kNrcTrainVerts];
        uint32_t nv = 0;
        for (;;) {
            TraceHit hit = closest<false>(k, p.o, p.d);
            if (p.depth == 0u) ++primary;
            else ++ext;
            NrcInput in;
            bool has = false;
            const float4 thrBefore = p.thr;
            ShadowRequest sh[2];
            uint32_t ns;
            bool cont = shadePathVertex<kSpectral, TrainHook, kExt>(S.sc, S.sd, cfg, tab, p, hit, sh, ns,
                                                                    TrainHook{{}, &in, &has, p.d});
            if (has && nv < kNrcTrainVerts) {
                vin[nv] = in;
                vthr[nv] = thrBefore;
                vrad[nv] = p.radiance;  // emission of the vertex included, its light samples not yet
                ++nv;
            }
            for (uint32_t r = 0; r < ns; ++r) {
                ++shadow;
                TraceRay ray{sh[r].origin, sh[r].dir, kTMin, sh[r].tmax};
                if (traceBvh<true, false>(S.sc, ray, k.stackColumn, k.stackStride, counters).mesh ==
                    VKRT_CUDA_INVALID_INDEX)
                    p.radiance += sh[r].contribution;
            }
            if (!cont) break;
        }
        const float4 total = p.radiance;
        for (uint32_t j = 0; j < nv; ++j) {
            float4 suf;
            suf.x = vthr[j].x > 0.0f ? (total.x - vrad[j].x) / vthr[j].x : 0.0f;
            suf.y = vthr[j].y > 0.0f ? (total.y - vrad[j].y) / vthr[j].y : 0.0f;
            suf.z = vthr[j].z > 0.0f ? (total.z - vrad[j].z) / vthr[j].z : 0.0f;
            suf.w = vthr[j].w > 0.0f ? (total.w - vrad[j].w) / vthr[j].w : 0.0f;
            const float3 rgb = kSpectral ? xyzToLinearSrgb(spectral4ToXYZ(suf, heroLambdas(p.lamUnit), kLambdaRange))
                                         : xyz(suf);
            const uint32_t pos = atomicAdd(recCount, 1u);
            if (pos < maxRecords) {
                recIn[pos] = vin[j];
                recTarget[pos] = make_float4(rgb.x, rgb.y, rgb.z, 0.0f);
            }
        }
    }
    warpCount(&counters->primaryRays, primary);
    warpCount(&counters->extensionRays, ext);
    warpCount(&counters->shadowRays, shadow);
}

// the vertex gradient factors recorded by the hook, kept per slot until the vertex's shadow rays are traced
VKRT_DEV void adjStoreVertex(const WfGlobals& g, uint32_t slot, const AdjVertex& av, bool cont) {
    if (!av.hasSurface) {
        g.adjRatioR[slot] = f4(0.0f);
        return;
    }
    uint32_t flags = kAdjFlagSurface | (cont && av.sampled ? kAdjFlagContinued : 0u) |
                     (av.reqValid[0] ? kAdjFlagReq0 : 0u) | (av.reqValid[1] ? kAdjFlagReq1 : 0u);
    g.adjUv[slot] = make_float4(av.tex.uv0.x, av.tex.uv0.y, av.tex.uv1.x, av.tex.uv1.y);
    g.adjColor[slot] = av.tex.color;
    if (av.reqValid[0]) {
        g.adjReq0[slot] = make_float4(av.reqBase[0].x, av.reqBase[0].y, av.reqBase[0].z, av.reqRough[0]);
        g.adjEm0[slot] = make_float4(av.reqEmit[0].x, av.reqEmit[0].y, av.reqEmit[0].z, __uint_as_float(av.reqLight[0]));
    }
    if (av.reqValid[1]) {
        g.adjReq1[slot] = make_float4(av.reqBase[1].x, av.reqBase[1].y, av.reqBase[1].z, av.reqRough[1]);
        g.adjEm1[slot] = make_float4(av.reqEmit[1].x, av.reqEmit[1].y, av.reqEmit[1].z, __uint_as_float(av.reqLight[1]));
    }
    g.adjRatioB[slot] = make_float4(av.ratioBase.x, av.ratioBase.y, av.ratioBase.z, __uint_as_float(av.materialIndex));
    g.adjRatioR[slot] = make_float4(av.ratioRough.x, av.ratioRough.y, av.ratioRough.z, __uint_as_float(flags));
}

// Finishes the slot's pending vertex: pendFlags carries its requests' visibility, radiance the path radiance with
// them applied.
VKRT_DEV void adjFinishPending(const WfGlobals& g, const WfScene& S, uint32_t slot, uint32_t pendFlags,
                               float4 radiance, MaterialGradient* smemMat) {
    float4 rr = g.adjRatioR[slot];
    uint32_t flags = __float_as_uint(rr.w);
    if (!(flags & kAdjFlagSurface)) return;
    AdjVertex av;
    float4 rb = g.adjRatioB[slot], uv = g.adjUv[slot];
    av.materialIndex = __float_as_uint(rb.w);
    av.tex.uv0 = make_float2(uv.x, uv.y);
    av.tex.uv1 = make_float2(uv.z, uv.w);
    av.tex.color = g.adjColor[slot];
    av.hasSurface = true;
    av.emitted = false;
    av.sampled = true;
    av.ratioBase = xyz(rb);
    av.ratioRough = xyz(rr);
    av.reqValid[0] = (flags & kAdjFlagReq0) != 0u;
    av.reqValid[1] = (flags & kAdjFlagReq1) != 0u;
    if (av.reqValid[0]) {
        float4 a = g.adjReq0[slot], e = g.adjEm0[slot];
        av.reqBase[0] = xyz(a);
        av.reqRough[0] = a.w;
        av.reqEmit[0] = xyz(e);
        av.reqLight[0] = __float_as_uint(e.w);
    }
    if (av.reqValid[1]) {
        float4 a = g.adjReq1[slot], e = g.adjEm1[slot];
        av.reqBase[1] = xyz(a);
        av.reqRough[1] = a.w;
        av.reqEmit[1] = xyz(e);
        av.reqLight[1] = __float_as_uint(e.w);
    }
    bool vis[2] = {(pendFlags & 1u) && (pendFlags & 4u), (pendFlags & 2u) && (pendFlags & 8u)};
    finishVertex(S.sc, g.adj, smemMat, av, vis, (flags & kAdjFlagContinued) != 0u, xyz(g.adjDelta[slot]),
                 xyz(g.adjTotal[slot]), xyz(radiance));
}

// kFull: vkrt's whole material stack (and alpha tests); kFeatures: the denoiser features (taken when g.features is
// set). Separate instantiations, so frames that need neither keep the register budget of the plain kernel.
// kTrain: the cache's training pass, whose surface vertices are recorded for the training records.
template <bool kSpectral, bool kAdjoint, int kMinBlocks, bool kFull = false, bool kFeatures = kFull, bool kTrain = false>
__global__ void __launch_bounds__(kWfThreads, kMinBlocks) kWfShade(WfGlobals g, uint32_t inQueue, uint32_t outQueue) {
    const WfScene* scenes = g.scenes;
    MaterialGradient* smemMat = nullptr;
    if constexpr (kAdjoint) {
        __shared__ MaterialGradient smemMatStorage[kSmemMaterials];
        const uint32_t mc = scenes[0].sc.materialCount;
        smemMat = mc <= kSmemMaterials ? smemMatStorage : nullptr;
        clearMaterialSmem(smemMat, mc);
        __syncthreads();
    }
    __shared__ uint32_t binEnd[kRayBins];
    const uint32_t* q = g.sort == kSortMaterial ? g.sorted : (inQueue == 0 ? g.queue0 : g.queue1);
    const uint32_t n = g.counts[inQueue];
    if (g.sort == 0u) loadBinEnds(g, inQueue, binEnd);
    __syncthreads();
    const uint32_t nMiss = g.counts[kCntClass0], nDiel = g.counts[kCntClass0 + 1];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        uint32_t i = base + threadIdx.x;
        bool valid = i < n;
        bool cont = false;
        uint32_t slot = 0, ns = 0;
        ShadowRequest sh[2];
        NrcInput query{};
        bool queried = false, done = false;
        float3 nextDir = f3(0.0f);
        if (valid) {
            if (g.sort == kSortClass)  // the three class queues read as one
                slot = i < nMiss ? g.classQueue[i]
                                 : (i < nMiss + nDiel ? g.classQueue[g.Q + (i - nMiss)]
                                                      : g.classQueue[2u * size_t(g.Q) + (i - nMiss - nDiel)]);
            else
                slot = g.sort == 0u ? queueEntry(g, q, binEnd, i) : q[i];
            const WfScene& S = scenes[sceneOfSlot(g, slot)];
            PathState p = loadPath(g, slot);
            const uint32_t pf = g.pendFlags[slot];
            applyPending(g, slot, p.radiance);
            if constexpr (kFull) {
                loadPathExt(g, slot, p);
                if (pf & kPendUnsupported) p.flags &= ~kPathPrevNee;  // the previous vertex's NEE was unsupported
                if (g.alpha) g.alphaSeed[slot] = alphaSeedOf(p.rng);  // the seed the intersect kernel used
            }
            if constexpr (kAdjoint) adjFinishPending(g, S, slot, pf, p.radiance, smemMat);
            g.pendFlags[slot] = 0u;
            const float4 a = record(g, slot)[kRecHit];
            const TraceHit h{__float_as_uint(a.x), __float_as_uint(a.y), 0u, a.z, a.w, record(g, slot)[kRecPdf].w};
            StepConfig cfg = stepConfig(g, S);
            if constexpr (kAdjoint) {
                AdjVertex av;
                av.hasSurface = av.emitted = av.sampled = false;
                av.reqValid[0] = av.reqValid[1] = false;
                cont = shadePathVertex<kSpectral, AdjointHook>(S.sc, S.sd, cfg, specTable(S), p, h, sh, ns,
                                                               AdjointHook{&av, xyz(g.adjDelta[slot])});
                if (g.adj.wantEmission && av.emitted) scatterHitEmission(S.sc, g.adj, smemMat, av);
                adjStoreVertex(g, slot, av, cont);
            } else if constexpr (kTrain) {
                // the vertex's cache inputs, the throughput that reached it and the radiance after its emission
                NrcInput tin;
                bool has = false;
                const float4 thrBefore = p.thr;
                cont = shadePathVertex<kSpectral, TrainHook, kFull>(S.sc, S.sd, cfg, specTable(S), p, h, sh, ns,
                                                                    TrainHook{{}, &tin, &has, p.d});
                const uint32_t nv = g.trainCount[slot];
                if (has && nv < kNrcTrainVerts) {
                    const size_t v = size_t(slot) * kNrcTrainVerts + nv;
                    g.trainIn[v] = tin;
                    g.trainThr[v] = thrBefore;
                    g.trainRad[v] = p.radiance;
                    g.trainCount[slot] = nv + 1u;
                }
            } else {
                const bool featDone = (p.flags & kPathFeatureDone) != 0u;
                DenoiserFeature feat{f3(0.0f), f3(0.0f), featDone ? 1.0f : 0.0f};
                cont = shadePathVertex<kSpectral, CacheHook, kFull>(
                    S.sc, S.sd, cfg, specTable(S), p, h, sh, ns,
                    CacheHook{{}, &query, &queried, p.d, (kFeatures && g.features) ? &feat : nullptr});
                if (kFeatures && g.features && !featDone && feat.weight > 0.0f) {
                    const size_t item = size_t(S.itemBase) + g.slotItem[slot];
                    g.itemFeatA[item] = make_float4(feat.albedo.x, feat.albedo.y, feat.albedo.z, 1.0f);
                    g.itemFeatN[item] = make_float4(feat.normal.x, feat.normal.y, feat.normal.z, 0.0f);
                    p.flags |= kPathFeatureDone;
                }
            }
            // not in the full-stack kernels: bound by instruction fetch, they ran 10% slower with this code inside
            if constexpr (!kAdjoint && !kFull) {
                if (g.directFinish && !cont && ns == 0 && !queried) {  // the sample result, as finalize writes it
                    const float3 res = pathResult<kSpectral>(cfg, p);
                    g.sampleBuf[size_t(S.itemBase) + g.slotItem[slot]] = make_float4(res.x, res.y, res.z, 0.0f);
                    done = true;
                }
            }
            if (!done) {
                storePath(g, slot, p);
                if constexpr (kFull) storePathExt(g, slot, p);
            }
            nextDir = p.d;
            uint32_t flags = queried ? kPendCache : 0u;
            if (ns > 0) {
                g.pend0[slot] = sh[0].contribution;
                flags |= 1u;
            }
            if (ns > 1) {
                g.pend1[slot] = sh[1].contribution;
                flags |= 2u;
            }
            g.pendFlags[slot] = flags;
        }
        // continuing paths to the next queue, finished ones to finalize (one atomic per warp and queue)
        __syncwarp();
        queuePush(g, outQueue, valid && cont, slot, nextDir);
        const bool toFinalize = valid && !cont && (!done || g.refills);
        uint32_t pos = warpPush(&g.counts[kCntFinished], toFinalize);
        if (toFinalize) g.finished[pos] = slot | (done ? kFinishedDone : 0u);
        if constexpr (!kAdjoint)
            if (g.directFinish) warpCount(&g.counters->pathSamples, done ? 1u : 0u);
        if (g.cacheDepth != 0xFFFFFFFFu) {
            pos = warpPush(&g.counts[kCntQueries], valid && queried);
            if (valid && queried) {
                g.nrcQueries[pos] = query;
                g.slotQuery[slot] = pos;
            }
        }
        for (uint32_t r = 0; r < 2; ++r) {
            bool want = valid && r < ns;
            pos = warpPush(&g.counts[kCntShadow], want);
            if (want) {
                g.shadowA[pos] = make_float4(sh[r].origin.x, sh[r].origin.y, sh[r].origin.z, sh[r].tmax);
                g.shadowB[pos] = make_float4(sh[r].dir.x, sh[r].dir.y, sh[r].dir.z, __uint_as_float(slot | (r << 31)));
            }
        }
    }
    if constexpr (kAdjoint) {
        __syncthreads();
        flushMaterialSmem(g.adj, smemMat, scenes[0].sc.materialCount);
    }
}

template <bool kCount, int kMinBlocks>
__global__ void __launch_bounds__(kWfThreads, kMinBlocks) kWfShadow(WfGlobals g) {
    extern __shared__ uint2 smemStack[];
    const uint32_t n = g.counts[kCntShadow];
    uint32_t traced = 0, nodeVisits = 0, triTests = 0;
    persistentTraceVote<true, kCount>(
        n, &g.counts[kCntFetchShadow], smemStack + threadIdx.x, blockDim.x, &g.counters->errorFlags, g.refill,
        [&](uint32_t i, TraceRay& r, const WideNode*& nodes, const TriRecord*& tris, uint32_t& nodeCount) {
            float4 a = g.shadowA[i], b = g.shadowB[i];
            uint32_t slot = __float_as_uint(b.w) & 0x7FFFFFFFu;
            const DeviceScene& sc = g.scenes[sceneOfSlot(g, slot)].sc;
            r = TraceRay{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), kTMin, a.w};
            nodes = sc.nodes;
            tris = sc.tris;
            nodeCount = sc.nodeCount;
            ++traced;
        },
        [&](uint32_t i, const TraceHit& h) {
            if (h.mesh != VKRT_CUDA_INVALID_INDEX) return;
            uint32_t tag = __float_as_uint(g.shadowB[i].w);
            atomicOr(&g.pendFlags[tag & 0x7FFFFFFFu], 4u << (tag >> 31));
        },
        nodeVisits, triTests);
    warpCount(&g.counters->shadowRays, traced);
    if (kCount) warpCountBytes(&g.counters->shadowNodeBytes, &g.counters->shadowTriBytes, nodeVisits, triTests);
}

// Shadow rays of scenes with transmissive or alpha-tested materials: one ray per thread through traceBvh's
// transmissive any-hit mode (and alpha mode); a ray whose segment meets only transmissive surfaces marks its
// request unsupported.
template <bool kCount, bool kAlpha>
__global__ void __launch_bounds__(kWfThreads) kWfShadowScan(WfGlobals g) {
    extern __shared__ uint2 smemStack[];
    const uint32_t n = g.counts[kCntShadow];
    uint32_t traced = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        if (i < n) {
            const float4 a = g.shadowA[i], b = g.shadowB[i];
            const uint32_t tag = __float_as_uint(b.w);
            const uint32_t slot = tag & 0x7FFFFFFFu;
            const DeviceScene& sc = g.scenes[sceneOfSlot(g, slot)].sc;
            const TraceRay r{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), kTMin, a.w};
            const TraceHit h = traceBvh<true, kCount, false, true, kAlpha>(
                sc, r, smemStack + threadIdx.x, blockDim.x, kCount ? g.counters : nullptr, 0u,
                kAlpha ? alphaShadowSeed(g.alphaSeed[slot], tag >> 31) : 0u);
            ++traced;
            if (h.mesh == VKRT_CUDA_INVALID_INDEX)
                atomicOr(&g.pendFlags[slot], h.prim == kShadowThroughTransmission ? kPendUnsupported : 4u << (tag >> 31));
        }
    }
    warpCount(&g.counters->shadowRays, traced);
}

// kTrain: the cache's training pass, which turns the recorded vertices of a finished path into training records
template <bool kSpectral, bool kAdjoint, bool kTrain = false>
__global__ void __launch_bounds__(kWfThreads) kWfFinalize(WfGlobals g, uint32_t outQueue) {
    const WfScene* scenes = g.scenes;
    MaterialGradient* smemMat = nullptr;
    if constexpr (kAdjoint) {
        __shared__ MaterialGradient smemMatStorage[kSmemMaterials];
        const uint32_t mc = scenes[0].sc.materialCount;
        smemMat = mc <= kSmemMaterials ? smemMatStorage : nullptr;
        clearMaterialSmem(smemMat, mc);
        __syncthreads();
    }
    const uint32_t n = g.counts[kCntFinished];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        uint32_t i = base + threadIdx.x;
        bool valid = i < n;
        bool requeue = false;
        uint32_t slot = 0, samples = 0;
        bool done = false;  // the shade kernel wrote the result; the slot only takes its next item here
        if (valid) {
            slot = g.finished[i];
            done = (slot & kFinishedDone) != 0u;
            slot &= ~kFinishedDone;
        }
        if (valid && !done) {
            uint32_t sceneId = sceneOfSlot(g, slot);
            const WfScene& S = scenes[sceneId];
            PathState p = loadPath(g, slot);
            const uint32_t pf = g.pendFlags[slot];
            applyPending(g, slot, p.radiance);
            g.pendFlags[slot] = 0u;
            if constexpr (kAdjoint) {
                adjFinishPending(g, S, slot, pf, p.radiance, smemMat);
            } else if constexpr (kTrain) {
                // each recorded vertex j: the radiance the rest of the path gathered after the vertex's emission,
                // over the throughput that reached it (hero lanes converted like a sample result), in linear sRGB
                const float4 total = p.radiance;
                const uint32_t nv = g.trainCount[slot];
                for (uint32_t j = 0; j < nv; ++j) {
                    const size_t v = size_t(slot) * kNrcTrainVerts + j;
                    const float4 vt = g.trainThr[v], vr = g.trainRad[v];
                    float4 suf;
                    suf.x = vt.x > 0.0f ? (total.x - vr.x) / vt.x : 0.0f;
                    suf.y = vt.y > 0.0f ? (total.y - vr.y) / vt.y : 0.0f;
                    suf.z = vt.z > 0.0f ? (total.z - vr.z) / vt.z : 0.0f;
                    suf.w = vt.w > 0.0f ? (total.w - vr.w) / vt.w : 0.0f;
                    const float3 rgb = kSpectral ? xyzToLinearSrgb(spectral4ToXYZ(suf, heroLambdas(p.lamUnit),
                                                                                  kLambdaRange))
                                                 : xyz(suf);
                    const uint32_t pos = atomicAdd(g.recCount, 1u);
                    if (pos < g.maxRecords) {
                        g.recIn[pos] = g.trainIn[v];
                        g.recTarget[pos] = make_float4(rgb.x, rgb.y, rgb.z, 0.0f);
                    }
                }
            } else {
                if (pf & kPendCache) {  // the cache's radiance times the path throughput completes the path
                    const float3 pred = fmax3(xyz(g.nrcPred[g.slotQuery[slot]]), f3(0.0f));
                    // hero lanes carry the balance weight of four equal techniques, as every other term does
                    if (kSpectral)
                        p.radiance += p.thr * spectral4(specTable(S), pred, heroLambdas(p.lamUnit)) *
                                      (p.techPath > 0.0f ? 0.25f : 0.0f);
                    else p.radiance += make_float4(p.thr.x * pred.x, p.thr.y * pred.y, p.thr.z * pred.z, 0.0f);
                }
                StepConfig cfg = stepConfig(g, S);
                float3 res = pathResult<kSpectral>(cfg, p);
                g.sampleBuf[size_t(S.itemBase) + g.slotItem[slot]] = make_float4(res.x, res.y, res.z, 0.0f);
            }
            samples = kTrain ? 0u : 1u;  // training paths are not samples of the frame
        }
        // the next items for this warp's finished slots: one cursor fetch per warp, none once the cursor is past the
        // last item (always, with one slot per item); the counter only grows, so a stale read is conservative
        __syncwarp();
        const unsigned fin = __ballot_sync(0xFFFFFFFFu, valid);
        if (fin) {
            const uint32_t lane = threadIdx.x & 31u, leader = uint32_t(__ffs(fin) - 1);
            uint32_t item0 = g.totalItems;
            if (lane == leader && __ldcg(&g.counts[kCntCursor]) < g.totalItems)
                item0 = atomicAdd(&g.counts[kCntCursor], uint32_t(__popc(fin)));
            item0 = __shfl_sync(0xFFFFFFFFu, item0, int(leader));
            if (valid) {
                const uint32_t w = item0 >= g.totalItems ? g.totalItems : item0 + __popc(fin & ((1u << lane) - 1u));
                requeue = acquireItem<kSpectral>(g, scenes, slot, w);
            }
        }
        __syncwarp();
        float3 dir = f3(0.0f);
        if (g.rayOrder && valid && requeue) dir = xyz(record(g, slot)[kRecDir]);
        queuePush(g, outQueue, valid && requeue, slot, dir);
        warpCount(&g.counters->pathSamples, samples);
    }
    if constexpr (kAdjoint) {
        __syncthreads();
        flushMaterialSmem(g.adj, smemMat, scenes[0].sc.materialCount);
    }
}

__global__ void kWfCondition(WfGlobals g, uint32_t useGraph) {
    uint32_t it = g.counts[kCntIteration] + 1u;
    g.counts[kCntIteration] = it;
    g.counters->wfBodies = it;
    g.counters->kernelLaunches += g.launchesPerBody;
    bool more = g.counts[kCntActive0] > 0u;
    if (more && it >= g.maxIter) {
        g.counters->errorFlags |= 2u;  // iteration bound reached with work left (never expected)
        more = false;
    }
    if (useGraph) cudaGraphSetConditional(g.cond, more ? 1u : 0u);
}

constexpr uint32_t kSlotsDefault = 1u << 26;  // path slots when the configuration leaves the count open

template <class T>
cudaError_t grow(T*& p, size_t& cap, size_t n) {
    if (n <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1));
    if (e == cudaSuccess) cap = n;
    return e;
}

}  // namespace

// ---------------------------------------------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------------------------------------------
// one instantiated graph per mode, rebuilt when the launch shape or the kernel arguments change
struct WfGraphCache {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool spectral = false;
    WavefrontConfig cfg{};
    uint32_t Q = 0, keys = 0, maxIter = 0, total = 0, sceneCount = 0;
    WfGlobals g{};  // kernel arguments baked into the graph (conditional handle zeroed)
};

struct WavefrontEngine::Buffers {
    WfGlobals g{};
    size_t capQ = 0, capKeys = 0, capScenes = 0;
    size_t c_rec = 0, c_scene = 0, c_work = 0,
           c_sample = 0, c_sum = 0, c_key = 0, c_p0 = 0, c_p1 = 0, c_pf = 0, c_q0 = 0,
           c_q1 = 0, c_fin = 0, c_sorted = 0, c_sA = 0, c_sB = 0, c_hist = 0, c_counts = 0, c_sc = 0, c_class = 0,
           c_fA = 0, c_fN = 0, c_eA = 0, c_eB = 0, c_eC = 0, c_eD = 0, c_as = 0;
    size_t c_aD = 0, c_aT = 0, c_aU = 0, c_aC = 0, c_aR0 = 0, c_aR1 = 0, c_aE0 = 0, c_aE1 = 0, c_aRB = 0, c_aRR = 0;
    WfScene* scenes = nullptr;
    uint32_t* bases = nullptr;  // itemBase of every scene, then workBase
    size_t c_bases = 0;
    WfGraphCache graphs[4];  // by WavefrontMode
    float stageMs[kStageCount] = {};
    uint32_t* hostCount = nullptr;  // pinned word the stage-by-stage loop polls
    // radiance cache: queries, predictions, training records
    size_t c_nq = 0, c_sq = 0, c_np = 0, c_ri = 0, c_rt = 0, c_rc = 0, c_ti = 0, c_tt = 0, c_tr = 0, c_tc = 0;
    NrcInput* recIn = nullptr;
    float4* recTarget = nullptr;
    uint32_t* recCount = nullptr;
    uint32_t lastRecords = 0;
};

uint32_t WavefrontEngine::lastCacheRecords() const { return b_->lastRecords; }

cudaError_t WavefrontEngine::readTrainingRecords(void* inputs, void* targets, uint32_t capacity, uint32_t* count,
                                                 cudaStream_t stream) const {
    const uint32_t n = std::min(capacity, b_->lastRecords);
    if (count) *count = b_->lastRecords;
    if (!n) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(inputs, b_->recIn, sizeof(NrcInput) * n, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(targets, b_->recTarget, sizeof(float4) * n, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e;
}

const float* WavefrontEngine::lastStageMs() const { return b_->stageMs; }

WavefrontEngine::WavefrontEngine() : b_(new Buffers()) {}

WavefrontEngine::~WavefrontEngine() {
    release();
    delete b_;
}

void WavefrontEngine::release() {
    if (!b_) return;
    for (WfGraphCache& gc : b_->graphs) {
        if (gc.exec) cudaGraphExecDestroy(gc.exec);
        if (gc.graph) cudaGraphDestroy(gc.graph);
        gc.exec = nullptr;
        gc.graph = nullptr;
    }
    WfGlobals& g = b_->g;
    void* ptrs[] = {g.rec, g.slotScene, g.slotItem, g.sampleBuf,
                    g.hitKey, g.pend0, g.pend1, g.pendFlags, g.queue0, g.queue1, g.finished,
                    g.sorted, g.classQueue, g.shadowA, g.shadowB, g.keyHist, g.counts, b_->scenes, b_->bases,
                    g.nrcQueries, g.slotQuery, g.nrcPred, b_->recIn, b_->recTarget, b_->recCount, g.adjDelta,
                    g.adjTotal,
                    g.adjUv, g.adjColor, g.adjReq0, g.adjReq1, g.adjEm0, g.adjEm1, g.adjRatioB, g.adjRatioR,
                    g.itemFeatA, g.itemFeatN, g.extA, g.extB, g.extC, g.extD, g.alphaSeed,
                    g.trainIn, g.trainThr, g.trainRad, g.trainCount};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b_->hostCount) cudaFreeHost(b_->hostCount);
    Buffers* fresh = new Buffers();
    std::swap(*b_, *fresh);
    delete fresh;
}

// The frame's training records (counted on the device) feed `trainingSteps` optimiser steps over 64K-record batches.
cudaError_t WavefrontEngine::trainOnRecords(const WfCacheFrame& cache, cudaStream_t stream) {
    Buffers& B = *b_;
    const uint32_t maxRecords = cache.trainingPaths * kNrcTrainVerts;
    cudaError_t e = cudaSuccess;
    if (!B.hostCount) e = cudaMallocHost(&B.hostCount, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpyAsync(B.hostCount, B.recCount, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return e;
    const uint32_t records = std::min(*B.hostCount, maxRecords);
    B.lastRecords = records;
    const uint32_t batch = std::min<uint32_t>(records, 1u << 16);
    for (uint32_t k = 0; batch && k < cache.trainingSteps; ++k) {
        const uint32_t off = uint32_t((uint64_t(k) * batch) % records);
        const uint32_t n = std::min(batch, records - off);
        e = cache.engine->train(B.recIn + off, B.recTarget + off, n, nullptr, true, stream);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t WavefrontEngine::render(const std::vector<WfScene>& scenesIn, bool spectral, const WavefrontConfig& cfgIn,
                                    uint32_t rngMode, uint64_t rngSeed, RenderCounters* counters,
                                    cudaStream_t stream, WavefrontMode mode, const AdjointParams* adjoint,
                                    const WfCacheFrame* cache) {
    Buffers& B = *b_;
    const bool adjMode = mode == kWavefrontAdjoint;
    if (adjMode && (!adjoint || spectral || scenesIn.size() != 1)) return cudaErrorInvalidValue;
    const bool useCache = cache && cache->engine && cache->engine->ready() && mode == kWavefrontForward;
    if (useCache && scenesIn.size() != 1) return cudaErrorInvalidValue;
    const bool trainMode = mode == kWavefrontTrain;
    if (trainMode && (!cache || scenesIn.size() != 1)) return cudaErrorInvalidValue;
    // a cache frame traces its training paths first, as a wavefront pass of their own over the same scene, and
    // trains the cache on their records before rendering with it
    const bool wavefrontTraining = useCache && cache->trainingPaths && cache->trainingTracer == 1u;
    if (wavefrontTraining) {
        cudaError_t e = grow(B.recCount, B.c_rc, 1);
        if (e == cudaSuccess) e = cudaMemsetAsync(B.recCount, 0, sizeof(uint32_t), stream);
        if (e == cudaSuccess) e = render(scenesIn, spectral, cfgIn, rngMode, rngSeed, counters, stream, kWavefrontTrain,
                                         nullptr, cache);
        if (e == cudaSuccess) e = trainOnRecords(*cache, stream);
        if (e != cudaSuccess) return e;
    }
    WavefrontConfig cfg = cfgIn;
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (sms <= 0) sms = 1;
    std::vector<WfScene> scenes = scenesIn;
    uint32_t total = 0, maxSpp = 1, maxDepth = 1;
    uint32_t keys = 3u * uint32_t(scenesIn.size());  // (scene, class) sort keys
    if (cfg.sortByMaterial == kSortMaterialIndex) {   // one key for misses, then one per material of every scene
        keys = 1u;
        for (WfScene& S : scenes) {
            S.materialKeyBase = keys - 1u;
            keys += S.sc.materialCount;
        }
    }
    uint64_t items = 0;
    for (WfScene& S : scenes) {
        S.tileW = std::max(1u, cfg.tileWidth);
        S.tileH = std::max(1u, cfg.tileHeight);
        if (trainMode) {  // one work item (one sample) per training path
            S.tilesX = 0;
            S.workBase = S.itemBase = 0;
            S.workCount = total = cache->trainingPaths;
            S.spp = 1;
            items = S.workCount;
            maxDepth = std::max(maxDepth, S.sd.rrMaxDepth);
            continue;
        }
        S.tilesX = (S.vw + S.tileW - 1) / S.tileW;
        uint32_t tilesY = (S.vh + S.tileH - 1) / S.tileH;
        S.workBase = total;
        S.workCount = S.tilesX * tilesY * S.tileW * S.tileH;
        total += S.workCount;
        S.itemBase = uint32_t(items);
        items += uint64_t(S.workCount) * S.spp;
        maxSpp = std::max(maxSpp, S.spp);
        maxDepth = std::max(maxDepth, S.sd.rrMaxDepth);
    }
    if (items >= 0xFFFFFFF0ull) return cudaErrorInvalidValue;  // item indices are 32-bit
    const uint32_t totalItems = uint32_t(items);
    // default: one slot per item up to 64M slots (about 17 GB of slot state and queues). A slot that is refilled with
    // a new item sits wherever the finished path left it, so refills scatter the slot-indexed state accesses of the
    // next bounces; with a slot per item there are no refills. (A slot per item for the 266M items of the 64-scene
    // batch, about 70 GB, measured no faster than 64M refilled slots: 122.3 against 121.8 ms.)
    uint32_t Q = cfg.queueCapacity ? cfg.queueCapacity : std::min<uint32_t>(totalItems, kSlotsDefault);
    Q = std::max(1u, std::min(Q, std::max(totalItems, 1u)));
    // until the item cursor runs out every slot is busy, so the bounces of all items bound the iteration count;
    // the condition kernel counts two-iteration bodies
    uint64_t bodies = (uint64_t(totalItems) * (maxDepth + 1u) + Q - 1) / Q / 2u + maxDepth + 64u;
    uint32_t maxIter = uint32_t(std::min<uint64_t>(bodies, 0x7FFFFFFFull));

    cudaError_t e = cudaSuccess;
    WfGlobals& g = B.g;
#define WF_GROW(field, cap, n) \
    if (e == cudaSuccess) e = grow(g.field, B.cap, (n))
    WF_GROW(rec, c_rec, size_t(kRecWords) * Q);
    WF_GROW(slotScene, c_scene, Q);
    WF_GROW(slotItem, c_work, Q);
    WF_GROW(sampleBuf, c_sum, std::max<size_t>(totalItems, 1));
    bool features = false;  // forward frames render denoiser features when any scene has feature films
    bool extended = false;      // some scene's materials use the full material stack
    bool transmissive = false;  // ... with transmission (media and per-lane hero state per slot)
    bool alpha = false;         // ... with alpha tests
    for (const WfScene& S : scenes) {
        if (mode == kWavefrontForward && S.film.albedoWrite) features = true;
        if (S.extended) extended = true;
        if (S.transmissive) transmissive = true;
        if (S.alpha) alpha = true;
    }
    if (alpha) WF_GROW(alphaSeed, c_as, Q);
    if (transmissive) {
        WF_GROW(extA, c_eA, Q);
        WF_GROW(extB, c_eB, Q);
        WF_GROW(extC, c_eC, Q);
        WF_GROW(extD, c_eD, Q);
    }
    if (features) {
        WF_GROW(itemFeatA, c_fA, std::max<size_t>(totalItems, 1));
        WF_GROW(itemFeatN, c_fN, std::max<size_t>(totalItems, 1));
    }
    if (cfg.sortByMaterial == kSortMaterial || cfg.sortByMaterial == kSortMaterialIndex) {
        WF_GROW(hitKey, c_key, Q);
        WF_GROW(sorted, c_sorted, Q);
    }
    WF_GROW(pend0, c_p0, Q);
    WF_GROW(pend1, c_p1, Q);
    WF_GROW(pendFlags, c_pf, Q);
    WF_GROW(queue0, c_q0, size_t(cfg.rayOrder ? kRayBins : 1u) * Q);
    WF_GROW(queue1, c_q1, size_t(cfg.rayOrder ? kRayBins : 1u) * Q);
    WF_GROW(finished, c_fin, Q);
    if (cfg.sortByMaterial == kSortClass) WF_GROW(classQueue, c_class, 3 * size_t(Q));
    WF_GROW(shadowA, c_sA, 2 * size_t(Q));
    WF_GROW(shadowB, c_sB, 2 * size_t(Q));
    WF_GROW(keyHist, c_hist, keys);
    WF_GROW(counts, c_counts, kCntCount);
    if (trainMode) {
        WF_GROW(trainIn, c_ti, size_t(Q) * kNrcTrainVerts);
        WF_GROW(trainThr, c_tt, size_t(Q) * kNrcTrainVerts);
        WF_GROW(trainRad, c_tr, size_t(Q) * kNrcTrainVerts);
        WF_GROW(trainCount, c_tc, Q);
        const size_t maxRecords = size_t(cache->trainingPaths) * kNrcTrainVerts;
        if (e == cudaSuccess) e = grow(B.recIn, B.c_ri, maxRecords);
        if (e == cudaSuccess) e = grow(B.recTarget, B.c_rt, maxRecords);
        if (e == cudaSuccess) e = grow(B.recCount, B.c_rc, 1);
    }
    if (useCache) {
        WF_GROW(nrcQueries, c_nq, Q);
        WF_GROW(slotQuery, c_sq, Q);
        WF_GROW(nrcPred, c_np, Q);
        const size_t maxRecords = size_t(cache->trainingPaths) * kNrcTrainVerts;
        if (e == cudaSuccess) e = grow(B.recIn, B.c_ri, maxRecords);
        if (e == cudaSuccess) e = grow(B.recTarget, B.c_rt, maxRecords);
        if (e == cudaSuccess) e = grow(B.recCount, B.c_rc, 1);
        if (e == cudaSuccess) e = cache->engine->reserveInference(Q);
    }
    if (adjMode) {
        WF_GROW(adjDelta, c_aD, Q);
        WF_GROW(adjTotal, c_aT, Q);
        WF_GROW(adjUv, c_aU, Q);
        WF_GROW(adjColor, c_aC, Q);
        WF_GROW(adjReq0, c_aR0, Q);
        WF_GROW(adjReq1, c_aR1, Q);
        WF_GROW(adjEm0, c_aE0, Q);
        WF_GROW(adjEm1, c_aE1, Q);
        WF_GROW(adjRatioB, c_aRB, Q);
        WF_GROW(adjRatioR, c_aRR, Q);
    }
#undef WF_GROW
    if (e == cudaSuccess) e = grow(B.scenes, B.c_sc, scenes.size());
    if (e == cudaSuccess) e = grow(B.bases, B.c_bases, 2 * scenes.size());
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(B.scenes, scenes.data(), sizeof(WfScene) * scenes.size(), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    {
        std::vector<uint32_t> bases(2 * scenes.size());
        for (size_t i = 0; i < scenes.size(); ++i) {
            bases[i] = scenes[i].itemBase;
            bases[scenes.size() + i] = scenes[i].workBase;
        }
        // pageable source: the call returns once the bytes are staged, so the vector may go out of scope
        e = cudaMemcpyAsync(B.bases, bases.data(), sizeof(uint32_t) * bases.size(), cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return e;
    }
    g.mode = uint32_t(mode);
    g.directFinish = mode == kWavefrontForward ? 1u : 0u;
    g.refills = Q < totalItems ? 1u : 0u;
    bool padded = false;  // some tile reaches past its viewport, so some items are padding
    for (const WfScene& S : scenes)
        if (uint64_t(S.workCount) != uint64_t(S.vw) * S.vh) padded = true;
    g.identityStart = !padded && totalItems > 0u && !cfg.rayOrder ? 1u : 0u;
    g.features = features ? 1u : 0u;
    g.transmissive = transmissive ? 1u : 0u;
    g.alpha = alpha ? 1u : 0u;
    g.adj = adjoint ? *adjoint : AdjointParams{};
    g.recIn = B.recIn;
    g.recTarget = B.recTarget;
    g.recCount = B.recCount;
    g.maxRecords = trainMode ? cache->trainingPaths * kNrcTrainVerts : 0u;
    g.trainSeed = trainMode ? cache->seed : 0u;
    g.trainFrame = trainMode ? cache->frame : 0u;
    g.cacheDepth = useCache ? cache->cacheDepth : 0xFFFFFFFFu;
    g.cacheSpread = useCache ? cache->cacheSpread : 0.0f;
    g.scenes = B.scenes;
    g.itemBases = B.bases;
    g.workBases = B.bases + scenes.size();
    g.sceneCount = uint32_t(scenes.size());
    g.totalWork = total;
    g.totalItems = totalItems;
    g.Q = Q;
    g.maxIter = maxIter;
    g.sort = cfg.sortByMaterial <= kSortClass ? cfg.sortByMaterial : kSortMaterial;
    g.keyByMaterial = cfg.sortByMaterial == kSortMaterialIndex ? 1u : 0u;
    g.refill = int(std::min(std::max(cfg.refillLanes, 1u), 32u));
    g.rayOrder = cfg.rayOrder ? 1u : 0u;
    g.keyCount = keys;
    g.rngMode = rngMode;
    g.rngSeed = rngSeed;
    g.counters = counters;
    g.launchesOutsideLoop = 2u + (mode == kWavefrontForward ? 2u : 0u);
    g.launchesPerBody = 2u * (5u + (g.sort == kSortMaterial ? 2u : 0u) + (useCache ? 2u : 0u)) + 1u;
    const bool profile = cfg.profileStages != 0u;
    if (profile) cfg.useGraph = 0u;
    for (float& t : B.stageMs) t = 0.0f;
    // profiling: an event pair around every stage launch, summed per stage after the frame
    std::vector<std::pair<uint32_t, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    auto stage = [&](uint32_t st, auto&& launch) {
        if (!profile) {
            launch();
            return;
        }
        cudaEvent_t a = nullptr, b = nullptr;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, stream);
        launch();
        cudaEventRecord(b, stream);
        marks.push_back({st, {a, b}});
    };

    const uint32_t gridI = uint32_t(sms) * std::max(1u, cfg.intersectBlocksPerSM);
    const uint32_t gridS = uint32_t(sms) * std::max(1u, cfg.shadeBlocksPerSM);
    const uint32_t grid3 = uint32_t(sms) * 3u, grid4 = uint32_t(sms) * 4u;
    const uint32_t shadeMin = cfg.shadeBlocksPerSM;
    const size_t smem = size_t(kWfThreads) * VKRT_SMEM_STACK * sizeof(uint2);

    auto body = [&](uint32_t in, uint32_t out, bool useGraph) {
        stage(kStageBegin, [&] { kWfBegin<<<4, 1024, 0, stream>>>(g, out); });
        stage(kStageIntersect, [&] {
            if (alpha && profile) kWfIntersectAlpha<true><<<gridS, kWfThreads, smem, stream>>>(g, in);
            else if (alpha) kWfIntersectAlpha<false><<<gridS, kWfThreads, smem, stream>>>(g, in);
            else if (profile) kWfIntersect<true, 8><<<gridI, kWfThreads, smem, stream>>>(g, in);
            else kWfIntersect<false, 8><<<gridI, kWfThreads, smem, stream>>>(g, in);
        });
        if (g.sort == kSortMaterial) {
            stage(kStageSort, [&] {
                kWfSortScan<<<1, 1024, 0, stream>>>(g);
                kWfSortScatter<<<gridS, 256, 0, stream>>>(g, in);
            });
        }
        stage(kStageShade, [&] {
            // register budget follows the requested residency: 168 (3 blocks/SM, no spills), 128 (4), 80 (6) or
            // 64 (8) registers; kernels compiled for one residency run on a grid of that many blocks per SM
            if (adjMode) kWfShade<false, true, 4><<<grid4, kWfThreads, 0, stream>>>(g, in, out);
            else if (trainMode && extended && spectral)
                kWfShade<true, false, 3, true, false, true><<<grid3, kWfThreads, 0, stream>>>(g, in, out);
            else if (trainMode && extended)
                kWfShade<false, false, 3, true, false, true><<<grid3, kWfThreads, 0, stream>>>(g, in, out);
            else if (trainMode && spectral)
                kWfShade<true, false, 4, false, false, true><<<grid4, kWfThreads, 0, stream>>>(g, in, out);
            else if (trainMode) kWfShade<false, false, 4, false, false, true><<<grid4, kWfThreads, 0, stream>>>(g, in, out);
            else if (extended && spectral) kWfShade<true, false, 3, true><<<grid3, kWfThreads, 0, stream>>>(g, in, out);
            else if (extended) kWfShade<false, false, 3, true><<<grid3, kWfThreads, 0, stream>>>(g, in, out);
            else if (features && spectral)  // reflection-only materials with feature films
                kWfShade<true, false, 3, false, true><<<grid3, kWfThreads, 0, stream>>>(g, in, out);
            else if (features) kWfShade<false, false, 3, false, true><<<grid3, kWfThreads, 0, stream>>>(g, in, out);
            else if (spectral && shadeMin >= 8) kWfShade<true, false, 8><<<gridS, kWfThreads, 0, stream>>>(g, in, out);
            else if (spectral && shadeMin >= 6) kWfShade<true, false, 6><<<gridS, kWfThreads, 0, stream>>>(g, in, out);
            else if (spectral && shadeMin >= 4) kWfShade<true, false, 4><<<gridS, kWfThreads, 0, stream>>>(g, in, out);
            else if (spectral) kWfShade<true, false, 3><<<gridS, kWfThreads, 0, stream>>>(g, in, out);
            else if (shadeMin >= 8) kWfShade<false, false, 8><<<gridS, kWfThreads, 0, stream>>>(g, in, out);
            else if (shadeMin >= 6) kWfShade<false, false, 6><<<gridS, kWfThreads, 0, stream>>>(g, in, out);
            else if (shadeMin >= 4) kWfShade<false, false, 4><<<gridS, kWfThreads, 0, stream>>>(g, in, out);
            else kWfShade<false, false, 3><<<gridS, kWfThreads, 0, stream>>>(g, in, out);
        });
        stage(kStageShadow, [&] {
            if (alpha && profile) kWfShadowScan<true, true><<<gridS, kWfThreads, smem, stream>>>(g);
            else if (alpha) kWfShadowScan<false, true><<<gridS, kWfThreads, smem, stream>>>(g);
            else if (transmissive && profile) kWfShadowScan<true, false><<<gridS, kWfThreads, smem, stream>>>(g);
            else if (transmissive) kWfShadowScan<false, false><<<gridS, kWfThreads, smem, stream>>>(g);
            else if (profile) kWfShadow<true, 8><<<gridI, kWfThreads, smem, stream>>>(g);
            else kWfShadow<false, 8><<<gridI, kWfThreads, smem, stream>>>(g);
        });
        if (useCache)  // predictions for the paths that ended at the cache in this iteration
            stage(kStageShade, [&] { cache->engine->inferCounted(g.nrcQueries, g.counts + kCntQueries, Q, g.nrcPred, stream); });
        stage(kStageFinalize, [&] {
            if (adjMode) kWfFinalize<false, true><<<gridS, kWfThreads, 0, stream>>>(g, out);
            else if (trainMode && spectral) kWfFinalize<true, false, true><<<gridS, kWfThreads, 0, stream>>>(g, out);
            else if (trainMode) kWfFinalize<false, false, true><<<gridS, kWfThreads, 0, stream>>>(g, out);
            else if (spectral) kWfFinalize<true, false><<<gridS, kWfThreads, 0, stream>>>(g, out);
            else kWfFinalize<false, false><<<gridS, kWfThreads, 0, stream>>>(g, out);
        });
        (void)useGraph;
    };
    auto resolve = [&]() {  // the film is written by forward frames only
        if (mode != kWavefrontForward) return;
        stage(kStageResolve, [&] {
            if (spectral) kWfResolve<true><<<gridS, 256, 0, stream>>>(g);
            else kWfResolve<false><<<gridS, 256, 0, stream>>>(g);
        });
    };
    auto prologue = [&]() {
        stage(kStagePrologue, [&] {
            kWfSetup<<<1, 32, 0, stream>>>(g);
            dim3 cg(std::max(1, sms), std::min<uint32_t>(g.sceneCount, 64u));
            if (mode == kWavefrontForward) kWfClearOutside<<<cg, 256, 0, stream>>>(g);
            if (spectral) kWfInit<true><<<gridS, kWfThreads, 0, stream>>>(g);
            else kWfInit<false><<<gridS, kWfThreads, 0, stream>>>(g);
        });
    };

    if (!wavefrontTraining && !trainMode) B.lastRecords = 0;
    if (useCache && !wavefrontTraining) {
        // train the cache on this frame's training paths, one thread per path, before rendering with it
        e = cudaMemsetAsync(B.recCount, 0, sizeof(uint32_t), stream);
        if (e != cudaSuccess) return e;
        const uint32_t maxRecords = cache->trainingPaths * kNrcTrainVerts;
        const uint32_t tb = (cache->trainingPaths + kWfThreads - 1u) / kWfThreads;
        if (cache->trainingPaths) {
#define VKRT_TRAIN(S, X)                                                                                            \
    kNrcTrainPaths<S, X><<<tb, kWfThreads, smem, stream>>>(B.scenes, cache->trainingPaths, cache->frame, cache->seed, \
                                                          rngMode, rngSeed, maxRecords, B.recIn, B.recTarget,       \
                                                          B.recCount, counters)
            if (spectral && extended) VKRT_TRAIN(true, true);
            else if (spectral) VKRT_TRAIN(true, false);
            else if (extended) VKRT_TRAIN(false, true);
            else VKRT_TRAIN(false, false);
#undef VKRT_TRAIN
        }
        e = trainOnRecords(*cache, stream);
        if (e != cudaSuccess) return e;
    }

    if (!cfg.useGraph) {
        prologue();
        if (!B.hostCount) e = cudaMallocHost(&B.hostCount, sizeof(uint32_t));
        if (e != cudaSuccess) return e;
        uint32_t* hostCount = B.hostCount;
        for (uint32_t bodyIndex = 0; bodyIndex < maxIter; ++bodyIndex) {
            body(0, 1, false);
            body(1, 0, false);
            kWfCondition<<<1, 1, 0, stream>>>(g, 0u);
            if ((bodyIndex & 3u) == 3u || bodyIndex + 1 >= maxIter) {
                e = cudaMemcpyAsync(hostCount, g.counts + kCntActive0, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                    stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
                if (e != cudaSuccess || *hostCount == 0u) break;
            }
        }
        resolve();
        if (e == cudaSuccess) e = cudaGetLastError();
        if (profile) {
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
            for (auto& m : marks) {
                float ms = 0.0f;
                if (e == cudaSuccess && cudaEventElapsedTime(&ms, m.second.first, m.second.second) == cudaSuccess)
                    B.stageMs[m.first] += ms;
                cudaEventDestroy(m.second.first);
                cudaEventDestroy(m.second.second);
            }
        }
        return e;
    }

    // one graph per engine shape and mode: setup/init kernels then a conditional while node over the two-iteration
    // body
    WfGraphCache& GC = B.graphs[uint32_t(mode)];
    bool rebuild = !GC.exec || GC.spectral != spectral || std::memcmp(&GC.cfg, &cfg, sizeof(cfg)) != 0 ||
                   GC.Q != Q || GC.keys != keys || GC.maxIter != maxIter || GC.total != total ||
                   GC.sceneCount != g.sceneCount;
    {
        WfGlobals a = g, b = GC.g;
        a.cond = 0;
        b.cond = 0;
        if (std::memcmp(&a, &b, sizeof(a)) != 0) rebuild = true;
    }
    if (rebuild) {
        if (GC.exec) cudaGraphExecDestroy(GC.exec);
        if (GC.graph) cudaGraphDestroy(GC.graph);
        GC.exec = nullptr;
        GC.graph = nullptr;
        e = cudaGraphCreate(&GC.graph, 0);
        if (e != cudaSuccess) return e;
        e = cudaGraphConditionalHandleCreate(&g.cond, GC.graph, 1u, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return e;
        // prologue captured into the top-level graph
        e = cudaStreamBeginCaptureToGraph(stream, GC.graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) return e;
        prologue();
        cudaGraph_t captured = nullptr;
        e = cudaStreamEndCapture(stream, &captured);
        if (e != cudaSuccess) return e;
        // the conditional node depends on every node of the prologue
        size_t numNodes = 0;
        cudaGraphGetNodes(GC.graph, nullptr, &numNodes);
        std::vector<cudaGraphNode_t> nodes(numNodes);
        if (numNodes) cudaGraphGetNodes(GC.graph, nodes.data(), &numNodes);
        // zero-filled storage: the parameter union has no usable default constructor
        alignas(cudaGraphNodeParams) unsigned char cpStorage[sizeof(cudaGraphNodeParams)];
        std::memset(cpStorage, 0, sizeof(cpStorage));
        cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cpStorage);
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = g.cond;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t condNode;
        e = cudaGraphAddNode(&condNode, GC.graph, nodes.data(), nullptr, numNodes, &cp);
        if (e != cudaSuccess) return e;
        cudaGraph_t bodyGraph = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(stream, bodyGraph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) return e;
        body(0, 1, true);
        body(1, 0, true);
        kWfCondition<<<1, 1, 0, stream>>>(g, 1u);
        e = cudaStreamEndCapture(stream, &bodyGraph);
        if (e != cudaSuccess) return e;
        // the resolve kernel runs once the loop has drained every item
        e = cudaStreamBeginCaptureToGraph(stream, GC.graph, &condNode, nullptr, 1, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) return e;
        resolve();
        e = cudaStreamEndCapture(stream, &captured);
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&GC.exec, GC.graph, 0);
        if (e != cudaSuccess) return e;
        GC.spectral = spectral;
        GC.cfg = cfg;
        GC.Q = Q;
        GC.keys = keys;
        GC.maxIter = maxIter;
        GC.total = total;
        GC.sceneCount = g.sceneCount;
        GC.g = g;
        GC.g.cond = 0;
    }
    e = cudaGraphLaunch(GC.exec, stream);
    return e;
}

}  // namespace vkrt
