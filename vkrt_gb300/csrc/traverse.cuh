// traverse.cuh — software ray traversal of the 8-wide compressed BVH on sm_103a.
//
// Replaces the driver's hardware TraceRay behind vkrt's scene and shadow queries
// (src/shaders/rt/queries/scene_query.slang:10-42, shadow_query.slang:8-28). Semantics kept from those queries:
// no face culling (RAY_FLAG_NONE), hits accepted for tMin <= t <= tMax, the closest hit reports
// {mesh, primitive, t, barycentrics of vertices 1 and 2}, the shadow query ends at the first accepted hit.
// Ties in t resolve to the smaller global triangle id so the answer does not depend on visiting order.
//
// Design (Ylitie, Karras, Laine 2017, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs"):
// node groups and triangle groups as 32-bit hit masks, children visited near-to-far through the octant-ordered slots
// written by the builder, a traversal stack whose top entries live in shared memory (spilling to local memory),
// and a warp-vote that postpones triangle tests while too few lanes of the warp want them.
// The ray/triangle test is the watertight test of Woop, Benthin, Wald 2013 with every FP32 operation explicitly
// rounded (no FMA contraction), so results are bit-identical to the CPU oracle's FP32 restatement.
#pragma once

#include "shading.cuh"

namespace vkrt {

#ifndef VKRT_SMEM_STACK
#define VKRT_SMEM_STACK 8  // stack entries per thread kept in shared memory
#endif
#define VKRT_LOCAL_STACK 56  // further entries per thread in local memory
#define VKRT_POSTPONE_FRACTION 0.2f


struct TraceRay {
    float3 org;
    float3 dir;
    float tmin;
    float tmax;
};

struct TraceHit {
    uint32_t mesh;  // VKRT_CUDA_INVALID_INDEX on miss
    uint32_t prim;
    uint32_t gid;
    float t, u, v;
};

// Per-ray constants of the watertight test
struct WatertightRay {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

VKRT_DEV WatertightRay watertightSetup(float3 d) {
    WatertightRay w;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    w.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    w.kx = w.kz == 2 ? 0 : w.kz + 1;
    w.ky = w.kx == 2 ? 0 : w.kx + 1;
    float dk[3] = {d.x, d.y, d.z};
    float dz = dk[w.kz];
    if (dz < 0.0f) {
        int t = w.kx;
        w.kx = w.ky;
        w.ky = t;
    }
    w.Sx = __fdiv_rn(dk[w.kx], dz);
    w.Sy = __fdiv_rn(dk[w.ky], dz);
    w.Sz = __fdiv_rn(1.0f, dz);
    return w;
}

VKRT_DEV float comp(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Woop/Benthin/Wald watertight test; true with t, b1, b2 when tmin <= t <= tmax.
VKRT_DEV bool watertightHit(const WatertightRay& w, float3 org, float3 v0, float3 v1, float3 v2, float tmin,
                            float tmax, float& t, float& b1, float& b2) {
    float3 A = make_float3(__fsub_rn(v0.x, org.x), __fsub_rn(v0.y, org.y), __fsub_rn(v0.z, org.z));
    float3 B = make_float3(__fsub_rn(v1.x, org.x), __fsub_rn(v1.y, org.y), __fsub_rn(v1.z, org.z));
    float3 C = make_float3(__fsub_rn(v2.x, org.x), __fsub_rn(v2.y, org.y), __fsub_rn(v2.z, org.z));
    float Akz = comp(A, w.kz), Bkz = comp(B, w.kz), Ckz = comp(C, w.kz);
    float Ax = __fsub_rn(comp(A, w.kx), __fmul_rn(w.Sx, Akz));
    float Ay = __fsub_rn(comp(A, w.ky), __fmul_rn(w.Sy, Akz));
    float Bx = __fsub_rn(comp(B, w.kx), __fmul_rn(w.Sx, Bkz));
    float By = __fsub_rn(comp(B, w.ky), __fmul_rn(w.Sy, Bkz));
    float Cx = __fsub_rn(comp(C, w.kx), __fmul_rn(w.Sx, Ckz));
    float Cy = __fsub_rn(comp(C, w.ky), __fmul_rn(w.Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double CxBy = __dmul_rn(double(Cx), double(By)), CyBx = __dmul_rn(double(Cy), double(Bx));
        double AxCy = __dmul_rn(double(Ax), double(Cy)), AyCx = __dmul_rn(double(Ay), double(Cx));
        double BxAy = __dmul_rn(double(Bx), double(Ay)), ByAx = __dmul_rn(double(By), double(Ax));
        U = __double2float_rn(__dsub_rn(CxBy, CyBx));
        V = __double2float_rn(__dsub_rn(AxCy, AyCx));
        W = __double2float_rn(__dsub_rn(BxAy, ByAx));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    float Az = __fmul_rn(w.Sz, Akz), Bz = __fmul_rn(w.Sz, Bkz), Cz = __fmul_rn(w.Sz, Ckz);
    float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    float tt = __fdiv_rn(T, det);
    if (!(tt >= tmin && tt <= tmax)) return false;
    t = tt;
    b1 = __fdiv_rn(V, det);
    b2 = __fdiv_rn(W, det);
    return true;
}

VKRT_DEV uint32_t byteOf(uint32_t word, uint32_t i) { return (word >> (i * 8u)) & 0xFFu; }

// Intersects the ray with the 8 child boxes of `node`; returns the child hit masks in Ylitie's encoding:
// bits 24-31 internal children (bit 24 + (slot ^ octInv)), bits 0-23 triangles relative to the node's first one.
VKRT_DEV uint32_t intersectWideNode(const WideNode* __restrict__ nodes, uint32_t nodeIndex, float3 org, float3 idir,
                                    uint32_t octInv4, float tmin, float tmax, uint32_t& childBase,
                                    uint32_t& triBase, uint32_t& imask) {
    const uint4* p = reinterpret_cast<const uint4*>(nodes + nodeIndex);
    uint4 n0 = __ldg(p + 0);
    uint4 n1 = __ldg(p + 1);
    uint4 n2 = __ldg(p + 2);
    uint4 n3 = __ldg(p + 3);
    uint4 n4 = __ldg(p + 4);
    float px = __uint_as_float(n0.x), py = __uint_as_float(n0.y), pz = __uint_as_float(n0.z);
    uint32_t ex = byteOf(n0.w, 0), ey = byteOf(n0.w, 1), ez = byteOf(n0.w, 2);
    imask = byteOf(n0.w, 3);
    childBase = n1.x;
    triBase = n1.y;
    // adjusted ray: t = q * (2^e * idir) + (p - org) * idir
    float sx = __uint_as_float(ex << 23) * idir.x;
    float sy = __uint_as_float(ey << 23) * idir.y;
    float sz = __uint_as_float(ez << 23) * idir.z;
    float ox = (px - org.x) * idir.x;
    float oy = (py - org.y) * idir.y;
    float oz = (pz - org.z) * idir.z;
    uint32_t hitmask = 0u;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        uint32_t meta4 = half == 0 ? n1.z : n1.w;
        uint32_t isInner4 = (meta4 & (meta4 << 1)) & 0x10101010u;
        uint32_t innerMask4 = (isInner4 >> 4) * 0xFFu;  // 0xFF in each byte that is an internal child
        uint32_t bitIndex4 = (meta4 ^ (octInv4 & innerMask4)) & 0x1F1F1F1Fu;
        uint32_t childBits4 = (meta4 >> 5) & 0x07070707u;
        uint32_t qlox = half == 0 ? n2.x : n2.y, qloy = half == 0 ? n2.z : n2.w;
        uint32_t qloz = half == 0 ? n3.x : n3.y, qhix = half == 0 ? n3.z : n3.w;
        uint32_t qhiy = half == 0 ? n4.x : n4.y, qhiz = half == 0 ? n4.z : n4.w;
        // near/far planes picked by the ray direction sign per axis
        uint32_t nx = idir.x >= 0.0f ? qlox : qhix, fx = idir.x >= 0.0f ? qhix : qlox;
        uint32_t ny = idir.y >= 0.0f ? qloy : qhiy, fy = idir.y >= 0.0f ? qhiy : qloy;
        uint32_t nz = idir.z >= 0.0f ? qloz : qhiz, fz = idir.z >= 0.0f ? qhiz : qloz;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float tnx = fmaf(float(byteOf(nx, j)), sx, ox);
            float tny = fmaf(float(byteOf(ny, j)), sy, oy);
            float tnz = fmaf(float(byteOf(nz, j)), sz, oz);
            float tfx = fmaf(float(byteOf(fx, j)), sx, ox);
            float tfy = fmaf(float(byteOf(fy, j)), sy, oy);
            float tfz = fmaf(float(byteOf(fz, j)), sz, oz);
            float tnear = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
            float tfar = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
            bool hit = tnear <= tfar * 1.0000004f;  // conservative widening against FP32 rounding of the slabs
            uint32_t bits = byteOf(childBits4, j);
            if (hit && bits) hitmask |= bits << byteOf(bitIndex4, j);
        }
    }
    return hitmask;
}

VKRT_DEV float3 safeInverse(float3 d) {
    const float eps = 1e-20f;
    float x = fabsf(d.x) < eps ? copysignf(eps, d.x) : d.x;
    float y = fabsf(d.y) < eps ? copysignf(eps, d.y) : d.y;
    float z = fabsf(d.z) < eps ? copysignf(eps, d.z) : d.z;
    return make_float3(1.0f / x, 1.0f / y, 1.0f / z);
}

// Traversal stack: VKRT_SMEM_STACK entries per thread in shared memory (strided by blockDim.x so a warp hits
// 32 different banks), the rest in local memory.
struct TraversalStack {
    uint2* smem;  // this thread's column: smem[i * stride]
    uint32_t stride;
    uint2 local[VKRT_LOCAL_STACK];
    int sp;
    VKRT_DEV void push(uint2 v, unsigned int* errorFlags, bool& overflow) {
        if (sp < VKRT_SMEM_STACK) smem[sp * stride] = v;
        else if (sp < VKRT_SMEM_STACK + VKRT_LOCAL_STACK) local[sp - VKRT_SMEM_STACK] = v;
        else {
            overflow = true;
            if (errorFlags) atomicOr(errorFlags, kErrorStackOverflow);
            return;
        }
        ++sp;
    }
    VKRT_DEV uint2 pop() {
        --sp;
        return sp < VKRT_SMEM_STACK ? smem[sp * stride] : local[sp - VKRT_SMEM_STACK];
    }
};

// prim of a kTransmissive any-hit answer whose segment met transmissive surfaces only
constexpr uint32_t kShadowThroughTransmission = 0xFFFFFFFEu;

// Closest hit (anyHit = false) or first accepted hit (anyHit = true).
// kMeshFilter: only triangles of mesh `meshFilter` count as hits (the selection-mask rays, which vkrt traces
// against a TLAS holding the selected mesh alone).
// kTransmissive (any-hit shadow rays of scenes with transmissive materials, rt/payloads/shadow_payload.slang): hits on
// meshes whose material has transmission > 0 do not end the search but leave prim = kShadowThroughTransmission;
// an opaque hit anywhere on the segment answers occluded (vkrt reports whichever hit the driver accepts first).
// kAlpha 1 (scenes with alpha-tested materials, entry/path/any_hit.slang and entry/shadow/any_hit.slang): a candidate
// hit on such a material counts only when alphaAccepts it, with the ray's `alphaSeed`; kAlpha 2 (selection and pick
// rays, entry/select/any_hit.slang): mask cut-outs are dropped (selectionAlphaAccepts).
// kRuntime: the any-hit, transmissive and alpha (mode 1) behaviours are also chosen per call by rtAnyHit,
// rtTransmissive and rtAlpha, so one inlined copy of the traversal serves closest-hit and shadow rays (the megakernel's
// single trace site); with kRuntime = false the runtime flags are ignored and the template flags alone decide.
template <bool kAnyHit, bool kCount, bool kMeshFilter = false, bool kTransmissive = false, int kAlpha = 0,
          bool kRuntime = false>
VKRT_DEV TraceHit traceBvh(const DeviceScene& sc, const TraceRay& ray, uint2* smemColumn, uint32_t smemStride,
                           RenderCounters* counters, uint32_t meshFilter = 0u, uint32_t alphaSeed = 0u,
                           bool rtAnyHit = false, bool rtTransmissive = false, bool rtAlpha = false) {
    const bool anyHit = kAnyHit || (kRuntime && rtAnyHit);
    const bool transmissive = kTransmissive || (kRuntime && rtTransmissive);
    const bool alphaTest = kAlpha == 1 || (kRuntime && rtAlpha);
    TraceHit best;
    best.mesh = VKRT_CUDA_INVALID_INDEX;
    best.prim = VKRT_CUDA_INVALID_INDEX;
    best.gid = 0xFFFFFFFFu;
    best.t = 0.0f;
    best.u = 0.0f;
    best.v = 0.0f;
    if (sc.nodeCount == 0u) return best;
    const float3 org = ray.org, dir = ray.dir;
    const float3 idir = safeInverse(dir);
    const uint32_t oct = (dir.x < 0.0f ? 4u : 0u) | (dir.y < 0.0f ? 2u : 0u) | (dir.z < 0.0f ? 1u : 0u);
    const uint32_t octInv = 7u - oct;
    const uint32_t octInv4 = octInv * 0x01010101u;
    const WatertightRay wr = watertightSetup(dir);
    float tmax = ray.tmax;
    const float tmin = ray.tmin;
    TraversalStack stack;
    stack.smem = smemColumn;
    stack.stride = smemStride;
    stack.sp = 0;
    bool overflow = false;
    uint32_t nodeBytes = 0, triBytes = 0;

    uint2 nodeGroup = make_uint2(0u, 0x80000000u);  // root = first child of a virtual node, slot 7 ^ octInv
    // the root is stored at index 0: encode it as child bit 31 with a base such that the lookup yields 0
    uint32_t rootSlot = 7u ^ octInv;
    uint32_t rootImask = 1u << rootSlot;  // relative index 0
    uint32_t groupImask = rootImask;
    uint2 triGroup = make_uint2(0u, 0u);
    // node groups carry the parent's imask in the low 8 bits of .y (bits 0-7 are unused by internal-child hits)
    nodeGroup.y = 0x80000000u | groupImask;

    for (;;) {
        if (nodeGroup.y > 0x00FFFFFFu) {
            uint32_t hits = nodeGroup.y;
            uint32_t bit = 31u - __clz(hits);
            uint32_t slot = (bit - 24u) ^ octInv;
            uint32_t parentImask = hits & 0xFFu;
            uint32_t rel = __popc(parentImask & ((1u << slot) - 1u));
            uint32_t child = nodeGroup.x + rel;
            nodeGroup.y &= ~(1u << bit);
            if (nodeGroup.y > 0x00FFFFFFu) stack.push(nodeGroup, counters ? &counters->errorFlags : nullptr, overflow);
            if (overflow) break;
            uint32_t cbase, tbase, imask;
            uint32_t hm = intersectWideNode(sc.nodes, child, org, idir, octInv4, tmin, tmax, cbase, tbase, imask);
            if (kCount) nodeBytes += 80u;
            nodeGroup.x = cbase;
            nodeGroup.y = (hm & 0xFF000000u) | imask;
            triGroup.x = tbase;
            triGroup.y = hm & 0x00FFFFFFu;
        } else {
            triGroup = nodeGroup;
            triGroup.y &= 0x00FFFFFFu;
            nodeGroup = make_uint2(0u, 0u);
        }

        while (triGroup.y != 0u) {
            // warp vote: while this lane still has child nodes to visit, postpone triangle tests that too few
            // lanes of the warp would run together (a postponed group is tested unconditionally once popped)
            uint32_t active = __popc(__activemask());
            if (nodeGroup.y > 0x00FFFFFFu && float(active) < VKRT_POSTPONE_FRACTION * 32.0f) {
                stack.push(triGroup, counters ? &counters->errorFlags : nullptr, overflow);
                break;
            }
            uint32_t tbit = 31u - __clz(triGroup.y);
            triGroup.y &= ~(1u << tbit);
            uint32_t ti = triGroup.x + tbit;
            const float4* tp = reinterpret_cast<const float4*>(sc.tris + ti);
            float4 a = __ldg(tp + 0), b = __ldg(tp + 1), c = __ldg(tp + 2);
            if (kCount) triBytes += 48u;
            if (kMeshFilter && __float_as_uint(b.w) != meshFilter) continue;
            float t, b1, b2;
            if (watertightHit(wr, org, make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z),
                              make_float3(c.x, c.y, c.z), tmin, tmax, t, b1, b2)) {
                uint32_t gid = __float_as_uint(a.w);
                if (alphaTest && !alphaAccepts(sc, __float_as_uint(b.w), __float_as_uint(c.w), b1, b2, alphaSeed, gid))
                    continue;
                if (kAlpha == 2 && !selectionAlphaAccepts(sc, __float_as_uint(b.w), __float_as_uint(c.w), b1, b2))
                    continue;
                if (transmissive && sc.materials[sc.meshes[__float_as_uint(b.w)].materialIndex].transmission > 0.0f) {
                    best.prim = kShadowThroughTransmission;
                    continue;
                }
                if (t < tmax || gid < best.gid) {
                    tmax = t;
                    best.t = t;
                    best.u = b1;
                    best.v = b2;
                    best.gid = gid;
                    best.mesh = __float_as_uint(b.w);
                    best.prim = __float_as_uint(c.w);
                    if (anyHit) {
                        triGroup.y = 0u;
                        nodeGroup.y = 0u;
                        stack.sp = 0;
                        break;
                    }
                }
            }
        }
        if (overflow) break;
        if (anyHit && best.mesh != VKRT_CUDA_INVALID_INDEX) break;

        if (nodeGroup.y <= 0x00FFFFFFu) {
            if (stack.sp > 0) {
                nodeGroup = stack.pop();
            } else {
                break;
            }
        }
    }
    if (kCount && counters) {
        atomicAdd(anyHit ? &counters->shadowNodeBytes : &counters->nodeBytes, (unsigned long long)nodeBytes);
        atomicAdd(anyHit ? &counters->shadowTriBytes : &counters->triBytes, (unsigned long long)triBytes);
    }
    if (overflow) {
        best.mesh = VKRT_CUDA_INVALID_INDEX;
        best.prim = VKRT_CUDA_INVALID_INDEX;
    }
    return best;
}

// ---------------------------------------------------------------------------------------------------------------
// Resumable traversal state for persistent kernels with dynamic ray fetch (Aila & Laine 2009): a lane advances its
// ray one step at a time, and lanes whose ray finished fetch a new one while the others keep traversing, so the warp
// stays full on incoherent rays.
// ---------------------------------------------------------------------------------------------------------------
struct TravState {
    const WideNode* nodes;
    const TriRecord* tris;
    float3 org, idir;
    float tmin, tmax;
    WatertightRay wr;
    uint32_t octInv, octInv4;
    uint2 nodeGroup, triGroup;
    TraceHit best;
    bool overflow;
    uint32_t nodeVisits, triTests;  // counted when the caller asks (persistentTraceVote<..., kCount = true>)
};

VKRT_DEV void travBegin(TravState& s, const WideNode* nodes, const TriRecord* tris, uint32_t nodeCount,
                        const TraceRay& ray, TraversalStack& stack) {
    s.nodes = nodes;
    s.tris = tris;
    s.org = ray.org;
    s.idir = safeInverse(ray.dir);
    s.tmin = ray.tmin;
    s.tmax = ray.tmax;
    s.wr = watertightSetup(ray.dir);
    uint32_t oct = (ray.dir.x < 0.0f ? 4u : 0u) | (ray.dir.y < 0.0f ? 2u : 0u) | (ray.dir.z < 0.0f ? 1u : 0u);
    s.octInv = 7u - oct;
    s.octInv4 = s.octInv * 0x01010101u;
    s.best.mesh = VKRT_CUDA_INVALID_INDEX;
    s.best.prim = VKRT_CUDA_INVALID_INDEX;
    s.best.gid = 0xFFFFFFFFu;
    s.best.t = s.best.u = s.best.v = 0.0f;
    s.overflow = false;
    s.nodeVisits = s.triTests = 0u;
    s.triGroup = make_uint2(0u, 0u);
    s.nodeGroup = nodeCount ? make_uint2(0u, 0x80000000u | (1u << (7u ^ s.octInv))) : make_uint2(0u, 0u);
    stack.sp = 0;
}

// Node visit of the vote-scheduled traversal: takes the nearest remaining child of the lane's node group, pushes the
// rest, intersects the child's eight boxes; a new triangle group replaces the pending one, which is pushed.
template <bool kCount>
VKRT_DEV void voteNodeVisit(TravState& s, TraversalStack& stack, unsigned int* errorFlags) {
    uint32_t hits = s.nodeGroup.y;
    uint32_t bit = 31u - __clz(hits);
    uint32_t slot = (bit - 24u) ^ s.octInv;
    uint32_t rel = __popc((hits & 0xFFu) & ((1u << slot) - 1u));
    uint32_t child = s.nodeGroup.x + rel;
    s.nodeGroup.y &= ~(1u << bit);
    if (s.nodeGroup.y > 0x00FFFFFFu) stack.push(s.nodeGroup, errorFlags, s.overflow);
    uint32_t cbase, tbase, imask;
    uint32_t hm = intersectWideNode(s.nodes, child, s.org, s.idir, s.octInv4, s.tmin, s.tmax, cbase, tbase, imask);
    if (kCount) s.nodeVisits++;
    s.nodeGroup = make_uint2(cbase, (hm & 0xFF000000u) | imask);
    uint32_t tri = hm & 0x00FFFFFFu;
    if (tri) {
        if (s.triGroup.y) stack.push(s.triGroup, errorFlags, s.overflow);
        s.triGroup = make_uint2(tbase, tri);
    }
}

// One triangle of the lane's pending group; true when an any-hit query is answered.
template <bool kAnyHit, bool kCount>
VKRT_DEV bool voteTriangleTest(TravState& s) {
    uint32_t tbit = 31u - __clz(s.triGroup.y);
    s.triGroup.y &= ~(1u << tbit);
    const float4* tp = reinterpret_cast<const float4*>(s.tris + s.triGroup.x + tbit);
    float4 a = __ldg(tp + 0), b = __ldg(tp + 1), c = __ldg(tp + 2);
    if (kCount) s.triTests++;
    float t, b1, b2;
    if (watertightHit(s.wr, s.org, make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), make_float3(c.x, c.y, c.z),
                      s.tmin, s.tmax, t, b1, b2)) {
        uint32_t gid = __float_as_uint(a.w);
        if (t < s.tmax || gid < s.best.gid) {
            s.tmax = t;
            s.best.t = t;
            s.best.u = b1;
            s.best.v = b2;
            s.best.gid = gid;
            s.best.mesh = __float_as_uint(b.w);
            s.best.prim = __float_as_uint(c.w);
            if (kAnyHit) return true;
        }
    }
    return false;
}

// Persistent traversal with dynamic fetch and a warp vote per step: every step the warp runs one kind of work only,
// a node visit on the lanes that hold a node group or one triangle test on the lanes that hold triangles, whichever
// more lanes want (triangles on ties), so node and triangle code never diverge within a step. Lanes with neither
// pop their stack or finish; the warp refills once fewer than `refill` lanes are busy. Same tests and tie rule as
// traceBvh: closest hits are identical.
template <bool kAnyHit, bool kCount, class Load, class Store>
VKRT_DEV void persistentTraceVote(uint32_t n, uint32_t* fetch, uint2* smemColumn, uint32_t smemStride,
                                  unsigned int* errorFlags, int refill, Load load, Store store,
                                  uint32_t& nodeVisits, uint32_t& triTests) {
    TraversalStack stack;
    stack.smem = smemColumn;
    stack.stride = smemStride;
    stack.sp = 0;
    TravState s;
    bool busy = false;
    bool exhausted = false;  // warp-uniform
    uint32_t mine = 0;
    const uint32_t lane = threadIdx.x & 31u;
    auto finish = [&](bool miss) {
        if (miss) {
            s.best.mesh = VKRT_CUDA_INVALID_INDEX;
            s.best.prim = VKRT_CUDA_INVALID_INDEX;
        }
        store(mine, s.best);
        if (kCount) {
            nodeVisits += s.nodeVisits;
            triTests += s.triTests;
        }
        busy = false;
    };
    for (;;) {
        if (!exhausted) {
            unsigned idle = __ballot_sync(0xFFFFFFFFu, !busy);
            if (idle) {
                uint32_t base = 0;
                if (lane == 0u) base = atomicAdd(fetch, uint32_t(__popc(idle)));
                base = __shfl_sync(0xFFFFFFFFu, base, 0);
                if (base + uint32_t(__popc(idle)) >= n) exhausted = true;
                if (!busy) {
                    uint32_t i = base + uint32_t(__popc(idle & ((1u << lane) - 1u)));
                    if (i < n) {
                        TraceRay r;
                        const WideNode* nodes;
                        const TriRecord* tris;
                        uint32_t nodeCount;
                        load(i, r, nodes, tris, nodeCount);
                        travBegin(s, nodes, tris, nodeCount, r, stack);
                        mine = i;
                        busy = true;
                    }
                }
            }
        }
        const int minBusy = exhausted ? 1 : refill;
        for (;;) {
            // lanes without pending work take the next stack entry or finish their ray
            if (busy && s.nodeGroup.y <= 0x00FFFFFFu && s.triGroup.y == 0u) {
                if (stack.sp > 0) {
                    uint2 e = stack.pop();
                    if (e.y > 0x00FFFFFFu) s.nodeGroup = e;
                    else s.triGroup = e;
                } else {
                    finish(false);
                }
            }
            const unsigned busyMask = __ballot_sync(0xFFFFFFFFu, busy);
            if (__popc(busyMask) < minBusy) break;
            const bool wantNode = busy && s.nodeGroup.y > 0x00FFFFFFu;
            const bool wantTri = busy && s.triGroup.y != 0u;
            const int nNode = __popc(__ballot_sync(0xFFFFFFFFu, wantNode));
            const int nTri = __popc(__ballot_sync(0xFFFFFFFFu, wantTri));
            if (nTri >= nNode) {
                if (wantTri && voteTriangleTest<kAnyHit, kCount>(s)) finish(false);
            } else if (wantNode) {
                voteNodeVisit<kCount>(s, stack, errorFlags);
                if (s.overflow) finish(true);
            }
        }
        if (exhausted && !__any_sync(0xFFFFFFFFu, busy)) break;
    }
}

}  // namespace vkrt
