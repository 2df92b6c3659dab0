// oracle.cpp — TEST INFRASTRUCTURE ONLY (the oracle). CPU restatement of vkrt's path-tracing shaders and the
// FP64 intersector used to check the CUDA backend. Each function names the vkrt source it restates (paths are
// relative to the vkrt repository). Compiled with -ffp-contract=off so FP32 expressions round exactly as written.
#include "oracle.h"

#include <array>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle_math.h"
#include "vkrt_cuda.h"

using namespace oracle;

namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kTMin = 0.001f;          // scene/constants.slang:6
constexpr float kTMax = 10000.0f;        // scene/constants.slang:7
constexpr float kShadowOrigin = 0.001f;  // scene/constants.slang:8
constexpr float kShadowDist = 0.002f;    // scene/constants.slang:9
constexpr float kRRMin = 0.05f, kRRMax = 0.95f;  // scene/constants.slang:11-12
constexpr float kSafeEps = 1e-12f;       // scene/constants.slang:14
constexpr float kTangentParallel = 0.999f;
constexpr float kGgxMinAlpha = 1e-3f, kGgxEps = 1e-6f;  // bsdf/lobes/ggx.slang:16-17
constexpr float kLambdaMin = 360.0f, kLambdaRange = 470.0f;  // sampling/wavelength.slang:10-12
constexpr float kCieY = 106.9461715f;    // utility/spectral.slang:21

unsigned hwThreads(unsigned t) {
    if (t) return t;
    unsigned h = std::thread::hardware_concurrency();
    return h ? h : 1;
}

template <class F>
void parallelFor(uint32_t n, unsigned threads, F&& fn) {
    threads = hwThreads(threads);
    if (threads <= 1 || n < 2) {
        for (uint32_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<uint32_t> next(0);
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                uint32_t i = next.fetch_add(1);
                if (i >= n) break;
                fn(i);
            }
        });
    for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------------------------------------
// RNG: Wellons hash (sampling/random.slang:7-27) and PCG32
// ---------------------------------------------------------------------------------------------------------
uint32_t hash32(uint32_t v) {
    v ^= v >> 16;
    v *= 0x7feb352du;
    v ^= v >> 15;
    v *= 0x846ca68bu;
    v ^= v >> 16;
    return v;
}

uint32_t pixelSeed(int32_t x, int32_t y, uint32_t frame, uint32_t sampleIndex) {
    uint32_t s = uint32_t(x) * 73856093u;
    s ^= uint32_t(y) * 19349663u;
    s ^= frame * 83492791u;
    s ^= sampleIndex * 2654435761u;
    return hash32(s);
}

uint32_t pcgNext(uint64_t& state, uint64_t inc) {
    uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    uint32_t xorshifted = uint32_t(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = uint32_t(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

struct Rng {
    uint32_t mode;
    uint32_t h;
    uint64_t state, inc;
    float next() {
        if (mode == VKRT_CUDA_RNG_REFERENCE) {
            h = hash32(h + 0x9e3779b9u);
            return float(h & 0x00ffffffu) * (1.0f / 16777216.0f);
        }
        return float(pcgNext(state, inc) >> 8) * (1.0f / 16777216.0f);
    }
};

// PCG32 stream for one (pixel, frame, sample): srandom(initstate, initseq) with the seed mixed with the frame
Rng makeRng(uint32_t mode, uint64_t seed, int32_t x, int32_t y, uint32_t frame, uint32_t sampleIndex) {
    Rng r{};
    r.mode = mode;
    if (mode == VKRT_CUDA_RNG_REFERENCE) {
        r.h = pixelSeed(x, y, frame, sampleIndex);
        return r;
    }
    uint64_t initstate = seed + uint64_t(frame) * 0x9E3779B97F4A7C15ull;
    uint64_t initseq = (uint64_t(uint32_t(y)) << 48) ^ (uint64_t(uint32_t(x)) << 32) ^ uint64_t(sampleIndex);
    r.inc = (initseq << 1u) | 1u;
    r.state = 0u;
    pcgNext(r.state, r.inc);
    r.state += initstate;
    pcgNext(r.state, r.inc);
    return r;
}

uint32_t reverseBits(uint32_t v) {
    v = ((v & 0x55555555u) << 1u) | ((v >> 1u) & 0x55555555u);
    v = ((v & 0x33333333u) << 2u) | ((v >> 2u) & 0x33333333u);
    v = ((v & 0x0f0f0f0fu) << 4u) | ((v >> 4u) & 0x0f0f0f0fu);
    v = ((v & 0x00ff00ffu) << 8u) | ((v >> 8u) & 0x00ff00ffu);
    return (v << 16u) | (v >> 16u);
}

// ---------------------------------------------------------------------------------------------------------
// Spectral utilities (utility/spectral.slang, utility/rgb2spec.slang, sampling/wavelength.slang)
// ---------------------------------------------------------------------------------------------------------
struct Rgb2Spec {
    const float* table = nullptr;
    uint32_t res = 0;
    uint32_t scaleOffset = 0;
    uint32_t dataOffset = 0;
};

// rgb2specFindInterval (rgb2spec.slang:14-31)
uint32_t rgb2specInterval(const Rgb2Spec& t, float x) {
    int left = 0;
    int size = int(t.res) - 2;
    while (size > 0) {
        int half = size >> 1;
        int middle = left + half + 1;
        if (t.table[t.scaleOffset + uint32_t(middle)] <= x) {
            left = middle;
            size -= half + 1;
        } else {
            size = half;
        }
    }
    return std::min(uint32_t(left), t.res - 2u);
}

template <class R>
V3<R> rgb2specFetch(const Rgb2Spec& t, V3<R> rgb) {  // rgb2spec.slang:33-81
    R z = std::max(rgb.x, std::max(rgb.y, rgb.z));
    if (z <= R(1e-8) || !t.table) return V3<R>(R(0));
    uint32_t dom = 0;
    for (uint32_t c = 1; c < 3; ++c)
        if (rgb[int(c)] >= rgb[int(dom)]) dom = c;
    R xyScale = R(t.res - 1u) / z;
    R x = rgb[int((dom + 1u) % 3u)] * xyScale;
    R y = rgb[int((dom + 2u) % 3u)] * xyScale;
    uint32_t xi = std::min(uint32_t(x), t.res - 2u);
    uint32_t yi = std::min(uint32_t(y), t.res - 2u);
    uint32_t zi = rgb2specInterval(t, float(z));
    uint32_t off = ((((dom * t.res + zi) * t.res + yi) * t.res + xi) * 3u);
    uint32_t dx = 3u, dy = dx * t.res, dz = dy * t.res;
    R x1 = x - R(xi), y1 = y - R(yi), x0 = R(1) - x1, y0 = R(1) - y1;
    R s0 = t.table[t.scaleOffset + zi], s1 = t.table[t.scaleOffset + zi + 1u];
    R z1 = (z - s0) / std::max(s1 - s0, R(1e-8)), z0 = R(1) - z1;
    V3<R> c;
    for (uint32_t j = 0; j < 3; ++j) {
        const float* d = t.table + t.dataOffset + off + j;
        c[int(j)] = ((R(d[0]) * x0 + R(d[dx]) * x1) * y0 + (R(d[dy]) * x0 + R(d[dy + dx]) * x1) * y1) * z0 +
                    ((R(d[dz]) * x0 + R(d[dz + dx]) * x1) * y0 + (R(d[dz + dy]) * x0 + R(d[dz + dy + dx]) * x1) * y1) * z1;
    }
    return c;
}

template <class R>
R rgb2specEval(V3<R> c, R lambda) {  // rgb2spec.slang:83-86
    R x = (c.x * lambda + c.y) * lambda + c.z;
    return R(0.5) * x * rsqrtr(x * x + R(1)) + R(0.5);
}

template <class R>
R spectralScalar(const Rgb2Spec& t, V3<R> rgb, R lambda) {  // spectral.slang:37-48
    R m = maxc(rgb);
    if (m <= R(0)) return R(0);
    if (m <= R(1)) return rgb2specEval(rgb2specFetch(t, rgb), lambda);
    return m * rgb2specEval(rgb2specFetch(t, rgb / m), lambda);
}

template <class R>
V4<R> spectralScalar4(const Rgb2Spec& t, V3<R> rgb, V4<R> l) {  // spectral.slang:50-64
    R m = maxc(rgb);
    if (m <= R(0)) return V4<R>(R(0));
    R scale = m <= R(1) ? R(1) : m;
    V3<R> c = rgb2specFetch(t, rgb / scale);
    return scale * V4<R>(rgb2specEval(c, l.x), rgb2specEval(c, l.y), rgb2specEval(c, l.z), rgb2specEval(c, l.w));
}

// CIE 1931 analytic fits (spectral.slang:66-87)
template <class R>
V3<R> cieXYZ(R l) {
    R t1 = (l - R(442.0)) * (l < R(442.0) ? R(0.0624) : R(0.0374));
    R t2 = (l - R(599.8)) * (l < R(599.8) ? R(0.0264) : R(0.0323));
    R t3 = (l - R(501.1)) * (l < R(501.1) ? R(0.0490) : R(0.0382));
    R X = R(0.362) * std::exp(R(-0.5) * t1 * t1) + R(1.056) * std::exp(R(-0.5) * t2 * t2) -
          R(0.065) * std::exp(R(-0.5) * t3 * t3);
    R u1 = (l - R(568.8)) * (l < R(568.8) ? R(0.0213) : R(0.0247));
    R u2 = (l - R(530.9)) * (l < R(530.9) ? R(0.0613) : R(0.0322));
    R Y = R(0.821) * std::exp(R(-0.5) * u1 * u1) + R(0.286) * std::exp(R(-0.5) * u2 * u2);
    R v1 = (l - R(437.0)) * (l < R(437.0) ? R(0.0845) : R(0.0278));
    R v2 = (l - R(459.0)) * (l < R(459.0) ? R(0.0385) : R(0.0725));
    R Z = R(1.217) * std::exp(R(-0.5) * v1 * v1) + R(0.681) * std::exp(R(-0.5) * v2 * v2);
    return vmax(V3<R>(X, Y, Z), V3<R>(R(0)));
}

template <class R>
V3<R> mat3mul(const double m[9], V3<R> v) {  // row-major 3x3 times column vector (HLSL mul(M, v))
    return {R(m[0]) * v.x + R(m[1]) * v.y + R(m[2]) * v.z, R(m[3]) * v.x + R(m[4]) * v.y + R(m[5]) * v.z,
            R(m[6]) * v.x + R(m[7]) * v.y + R(m[8]) * v.z};
}
// spectral.slang:14-20
const double kXyzToSrgb[9] = {3.2404542, -1.5371385, -0.4985314, -0.9692660, 1.8760108, 0.0415560,
                              0.0556434, -0.2040259, 1.0572252};
const double kBradford[9] = {0.8951, 0.2664, -0.1614, -0.7502, 1.7135, 0.0367, 0.0389, -0.0685, 1.0296};
const double kBradfordInv[9] = {0.9869929, -0.1470543, 0.1599627, 0.4323053, 0.5183603,
                                0.0492912, -0.0085287, 0.0400428, 0.9684867};
const double kEtoD65[3] = {0.9413344, 1.0404175, 1.0895327};

template <class R>
V3<R> xyzToLinearSrgb(V3<R> xyz) {  // spectral.slang:89-97
    V3<R> lms = mat3mul(kBradford, xyz);
    lms = lms * V3<R>(R(kEtoD65[0]), R(kEtoD65[1]), R(kEtoD65[2]));
    return mat3mul(kXyzToSrgb, mat3mul(kBradfordInv, lms));
}

template <class R>
V3<R> spectral4ToXYZ(V4<R> s, V4<R> l, V4<R> invPdf) {  // spectral.slang:104-113
    V3<R> xyz(R(0));
    for (int i = 0; i < 4; ++i) xyz += cieXYZ(l[i]) * ((s[i] * invPdf[i]) / R(kCieY));
    return xyz;
}

template <class R> R heroBalance(V4<R> p) {  // spectral.slang:115-118
    R c = sum4(p);
    return c > R(0) ? p.x / c : R(0);
}

// ---------------------------------------------------------------------------------------------------------
// Scene
// ---------------------------------------------------------------------------------------------------------
struct Tex {
    std::vector<float> rgba;
    uint32_t w = 0, h = 0;
};

struct WorldTri {
    float v[3][3];
    uint32_t mesh, prim, gid;
};

struct BvhNode {
    float lo[3], hi[3];
    uint32_t left;   // internal: left child index; leaf: first triangle
    uint32_t count;  // 0 = internal (right = left + 1), else triangle count
};

struct EnvDist {
    bool valid = false;
    uint32_t w = 0, h = 0;
    std::vector<float> marginal;     // h + 1
    std::vector<float> conditional;  // h * (w + 1)
    std::vector<float> texelWeight;  // w * h luminance*sin(theta) (normalised to pdf over the unit square)
};

struct Scene {
    std::vector<VKRT_CudaShaderVertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<VKRT_CudaMeshInfo> meshes;
    std::vector<VKRT_CudaMaterial> materials;
    std::vector<VKRT_CudaEmissiveMesh> emeshes;
    std::vector<VKRT_CudaEmissiveTriangle> etris;
    std::vector<float> meshQ, triQ;
    std::vector<uint32_t> meshIdx, triIdx;
    std::vector<Tex> textures;
    std::vector<float> rgb2spec;
    std::vector<float> sheenLtc;  // 3 x 32 x 32 (transform a, transform b, albedo), empty: no sheen lobe
    std::vector<WorldTri> tris;        // BVH order after build
    std::vector<uint32_t> meshTriBase; // global id of the first triangle of each mesh
    std::vector<BvhNode> nodes;
    uint32_t envSampling = 0;
    uint32_t envTexture = VKRT_CUDA_INVALID_INDEX;
    EnvDist env;
};

// column-major TRS world matrix (src/core/scene/transform.c:26-35), same rounding as the host library
void meshWorldMatrix(const VKRT_CudaMeshInfo& m, float out[16]);


void mat4MulCM(const float a[16], const float b[16], float out[16]) {
    float r[16];
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            float acc = 0.0f;
            for (int k = 0; k < 4; ++k) acc += a[k * 4 + row] * b[c * 4 + k];
            r[c * 4 + row] = acc;
        }
    std::memcpy(out, r, sizeof(r));
}

void axisRotation(int axis, float rad, float m[16]) {
    for (int i = 0; i < 16; ++i) m[i] = 0.0f;
    m[0] = m[5] = m[10] = m[15] = 1.0f;
    float c = std::cos(rad), s = std::sin(rad);
    int i = (axis + 1) % 3, j = (axis + 2) % 3;
    m[i * 4 + i] = c;
    m[j * 4 + j] = c;
    m[i * 4 + j] = s;
    m[j * 4 + i] = -s;
}

void meshWorldMatrix(const VKRT_CudaMeshInfo& mi, float out[16]) {
    const float deg = 0.01745329251994329577f;
    float m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}, r[16];
    m[12] = mi.position[0];
    m[13] = mi.position[1];
    m[14] = mi.position[2];
    axisRotation(2, mi.rotation[2] * deg, r);
    mat4MulCM(m, r, m);
    axisRotation(1, mi.rotation[1] * deg, r);
    mat4MulCM(m, r, m);
    axisRotation(0, mi.rotation[0] * deg, r);
    mat4MulCM(m, r, m);
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 4; ++row) m[c * 4 + row] *= mi.scale[c];
    std::memcpy(out, m, sizeof(m));
}

bool isIdentityTRS(const VKRT_CudaMeshInfo& m) {
    return m.position[0] == 0.0f && m.position[1] == 0.0f && m.position[2] == 0.0f && m.rotation[0] == 0.0f &&
           m.rotation[1] == 0.0f && m.rotation[2] == 0.0f && m.scale[0] == 1.0f && m.scale[1] == 1.0f &&
           m.scale[2] == 1.0f;
}

// world position p' = M p, each row summed left to right from unfused products (the device flattening uses the
// same order with round-to-nearest intrinsics, so both produce identical FP32 vertices)
void worldPoint(const float m[16], const float p[3], float out[3]) {
    for (int r = 0; r < 3; ++r) {
        float a = m[0 * 4 + r] * p[0];
        float b = m[1 * 4 + r] * p[1];
        float c = m[2 * 4 + r] * p[2];
        out[r] = ((a + b) + c) + m[3 * 4 + r];
    }
}

// ---------------------------------------------------------------------------------------------------------
// Watertight ray/triangle test (Woop, Benthin, Wald 2013), FP32 or FP64
// ---------------------------------------------------------------------------------------------------------
template <class R>
struct RayPre {
    V3<R> org, dir;
    int kx, ky, kz;
    R Sx, Sy, Sz;
    R tmin, tmax;
};

template <class R>
RayPre<R> prepRay(V3<R> o, V3<R> d, R tmin, R tmax) {
    RayPre<R> r;
    r.org = o;
    r.dir = d;
    R ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    r.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    r.kx = (r.kz + 1) % 3;
    r.ky = (r.kx + 1) % 3;
    if (d[r.kz] < R(0)) std::swap(r.kx, r.ky);
    r.Sx = d[r.kx] / d[r.kz];
    r.Sy = d[r.ky] / d[r.kz];
    r.Sz = R(1) / d[r.kz];
    r.tmin = tmin;
    r.tmax = tmax;
    return r;
}

// returns true with t, b1 (weight of v1), b2 (weight of v2) when tmin <= t <= tmax
template <class R>
bool watertight(const RayPre<R>& r, const R* v0, const R* v1, const R* v2, R& t, R& b1, R& b2) {
    R A[3] = {v0[0] - r.org.x, v0[1] - r.org.y, v0[2] - r.org.z};
    R B[3] = {v1[0] - r.org.x, v1[1] - r.org.y, v1[2] - r.org.z};
    R C[3] = {v2[0] - r.org.x, v2[1] - r.org.y, v2[2] - r.org.z};
    R Ax = A[r.kx] - r.Sx * A[r.kz], Ay = A[r.ky] - r.Sy * A[r.kz];
    R Bx = B[r.kx] - r.Sx * B[r.kz], By = B[r.ky] - r.Sy * B[r.kz];
    R Cx = C[r.kx] - r.Sx * C[r.kz], Cy = C[r.ky] - r.Sy * C[r.kz];
    R U = Cx * By - Cy * Bx;
    R V = Ax * Cy - Ay * Cx;
    R W = Bx * Ay - By * Ax;
    if (sizeof(R) == 4 && (U == R(0) || V == R(0) || W == R(0))) {
        double CxBy = double(Cx) * double(By), CyBx = double(Cy) * double(Bx);
        double AxCy = double(Ax) * double(Cy), AyCx = double(Ay) * double(Cx);
        double BxAy = double(Bx) * double(Ay), ByAx = double(By) * double(Ax);
        U = R(CxBy - CyBx);
        V = R(AxCy - AyCx);
        W = R(BxAy - ByAx);
    }
    if ((U < R(0) || V < R(0) || W < R(0)) && (U > R(0) || V > R(0) || W > R(0))) return false;
    R det = U + V + W;
    if (det == R(0)) return false;
    R Az = r.Sz * A[r.kz], Bz = r.Sz * B[r.kz], Cz = r.Sz * C[r.kz];
    R T = U * Az + V * Bz + W * Cz;
    R tt = T / det;
    if (!(tt >= r.tmin && tt <= r.tmax)) return false;
    t = tt;
    b1 = V / det;
    b2 = W / det;
    return true;
}

// ---------------------------------------------------------------------------------------------------------
// BVH2 (binned SAH) over world triangles, FP32 traversal
// ---------------------------------------------------------------------------------------------------------
struct BuildItem {
    float lo[3], hi[3], c[3];
    uint32_t tri;
};

// Right child indices are kept separately because the recursive build interleaves subtrees.
struct Bvh {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> right;
};

uint32_t buildBvh2(Bvh& bvh, std::vector<BuildItem>& items, uint32_t begin, uint32_t end) {
    uint32_t idx = uint32_t(bvh.nodes.size());
    bvh.nodes.push_back(BvhNode{});
    bvh.right.push_back(0);
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = begin; i < end; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], items[i].lo[k]);
            hi[k] = std::max(hi[k], items[i].hi[k]);
            clo[k] = std::min(clo[k], items[i].c[k]);
            chi[k] = std::max(chi[k], items[i].c[k]);
        }
    for (int k = 0; k < 3; ++k) {
        bvh.nodes[idx].lo[k] = lo[k];
        bvh.nodes[idx].hi[k] = hi[k];
    }
    uint32_t n = end - begin;
    if (n <= 4) {
        bvh.nodes[idx].left = begin;
        bvh.nodes[idx].count = n;
        return idx;
    }
    constexpr int kBins = 16;
    float bestCost = INFINITY;
    int bestAxis = -1, bestSplit = -1;
    auto area = [](const float* l, const float* h) {
        float d[3] = {std::max(0.0f, h[0] - l[0]), std::max(0.0f, h[1] - l[1]), std::max(0.0f, h[2] - l[2])};
        return d[0] * d[1] + d[1] * d[2] + d[2] * d[0];
    };
    for (int axis = 0; axis < 3; ++axis) {
        float ext = chi[axis] - clo[axis];
        if (!(ext > 0.0f)) continue;
        float blo[kBins][3], bhi[kBins][3];
        uint32_t bcnt[kBins] = {};
        for (int b = 0; b < kBins; ++b)
            for (int k = 0; k < 3; ++k) {
                blo[b][k] = INFINITY;
                bhi[b][k] = -INFINITY;
            }
        for (uint32_t i = begin; i < end; ++i) {
            int b = std::min(kBins - 1, std::max(0, int((items[i].c[axis] - clo[axis]) / ext * kBins)));
            bcnt[b]++;
            for (int k = 0; k < 3; ++k) {
                blo[b][k] = std::min(blo[b][k], items[i].lo[k]);
                bhi[b][k] = std::max(bhi[b][k], items[i].hi[k]);
            }
        }
        float rlo[kBins][3], rhi[kBins][3];
        uint32_t rcnt[kBins];
        float alo[3] = {INFINITY, INFINITY, INFINITY}, ahi[3] = {-INFINITY, -INFINITY, -INFINITY};
        uint32_t acnt = 0;
        for (int b = kBins - 1; b >= 0; --b) {
            for (int k = 0; k < 3; ++k) {
                alo[k] = std::min(alo[k], blo[b][k]);
                ahi[k] = std::max(ahi[k], bhi[b][k]);
                rlo[b][k] = alo[k];
                rhi[b][k] = ahi[k];
            }
            acnt += bcnt[b];
            rcnt[b] = acnt;
        }
        float llo[3] = {INFINITY, INFINITY, INFINITY}, lhi[3] = {-INFINITY, -INFINITY, -INFINITY};
        uint32_t lcnt = 0;
        for (int b = 0; b < kBins - 1; ++b) {
            for (int k = 0; k < 3; ++k) {
                llo[k] = std::min(llo[k], blo[b][k]);
                lhi[k] = std::max(lhi[k], bhi[b][k]);
            }
            lcnt += bcnt[b];
            if (lcnt == 0 || rcnt[b + 1] == 0) continue;
            float cost = area(llo, lhi) * float(lcnt) + area(rlo[b + 1], rhi[b + 1]) * float(rcnt[b + 1]);
            if (cost < bestCost) {
                bestCost = cost;
                bestAxis = axis;
                bestSplit = b;
            }
        }
    }
    uint32_t mid;
    if (bestAxis < 0) {
        mid = begin + n / 2;
    } else {
        float ext = chi[bestAxis] - clo[bestAxis];
        auto it = std::partition(items.begin() + begin, items.begin() + end, [&](const BuildItem& e) {
            int b = std::min(kBins - 1, std::max(0, int((e.c[bestAxis] - clo[bestAxis]) / ext * kBins)));
            return b <= bestSplit;
        });
        mid = uint32_t(it - items.begin());
        if (mid == begin || mid == end) mid = begin + n / 2;
    }
    uint32_t l = buildBvh2(bvh, items, begin, mid);
    uint32_t r = buildBvh2(bvh, items, mid, end);
    bvh.nodes[idx].left = l;
    bvh.nodes[idx].count = 0;
    bvh.right[idx] = r;
    return idx;
}

struct SceneFull : Scene {
    Bvh bvh;
};

// slab test with the same conservative widening the device uses on its far distance
bool boxHit(const BvhNode& n, const V3<float>& org, const V3<float>& inv, float tmin, float tmax) {
    float t0 = tmin, t1 = tmax;
    for (int k = 0; k < 3; ++k) {
        float a = (n.lo[k] - org[k]) * inv[k];
        float b = (n.hi[k] - org[k]) * inv[k];
        if (a > b) std::swap(a, b);
        if (std::isnan(a) || std::isnan(b)) {  // zero direction and origin on the slab plane: keep the box
            continue;
        }
        t0 = std::max(t0, a);
        t1 = std::min(t1, b);
    }
    return t0 <= t1 * 1.0000004f;
}

struct HitRec {
    uint32_t mesh = VKRT_CUDA_INVALID_INDEX, prim = VKRT_CUDA_INVALID_INDEX, gid = 0xFFFFFFFFu;
    float t = 0.0f, b1 = 0.0f, b2 = 0.0f;
    bool hit() const { return mesh != VKRT_CUDA_INVALID_INDEX; }
};

// Alpha test of a candidate hit (rt/alpha_test.slang), defined with the texture sampler below. vkrt draws its
// stochastic decisions from the path stream in any-hit order, which the driver leaves unspecified; here a triangle's
// decision hashes the ray's seed (the path stream's state when the ray starts, salted per shadow request) with the
// triangle id, so the closest accepted hit does not depend on traversal order.
bool alphaAccepts(const Scene& s, uint32_t mesh, uint32_t prim, float u, float v, uint32_t seed, uint32_t gid);
bool selectionAlphaAccepts(const Scene& s, uint32_t mesh, uint32_t prim, float u, float v);
bool sceneAlphaTested(const Scene& s);
uint32_t alphaShadowSeed(uint32_t seed, uint32_t request) { return seed ^ (0x68bc21ebu * (request + 1u)); }
float alphaRandom(uint32_t seed, uint32_t gid) {
    return float(hash32(seed ^ hash32(gid + 0x632be5abu)) & 0x00ffffffu) * (1.0f / 16777216.0f);
}

// closest hit (anyHit = false) or first accepted hit; ties on t go to the smaller global triangle id; with `alpha`,
// candidate hits must pass alphaAccepts under `alphaSeed`
HitRec traceFp32(const SceneFull& s, V3<float> o, V3<float> d, float tmin, float tmax, bool anyHit, bool alpha = false,
                 uint32_t alphaSeed = 0u, bool selection = false) {
    HitRec best;
    if (s.bvh.nodes.empty()) return best;
    RayPre<float> rp = prepRay(o, d, tmin, tmax);
    V3<float> inv(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    float bestT = tmax;
    while (sp > 0) {
        uint32_t ni = stack[--sp];
        const BvhNode& n = s.bvh.nodes[ni];
        if (!boxHit(n, o, inv, tmin, bestT)) continue;
        if (n.count == 0) {
            stack[sp++] = s.bvh.right[ni];
            stack[sp++] = n.left;
            continue;
        }
        for (uint32_t i = 0; i < n.count; ++i) {
            const WorldTri& tr = s.tris[n.left + i];
            RayPre<float> r2 = rp;
            r2.tmax = bestT;
            float t, b1, b2;
            if (!watertight(r2, tr.v[0], tr.v[1], tr.v[2], t, b1, b2)) continue;
            if (alpha && !alphaAccepts(s, tr.mesh, tr.prim, b1, b2, alphaSeed, tr.gid)) continue;
            if (selection && !selectionAlphaAccepts(s, tr.mesh, tr.prim, b1, b2)) continue;
            if (t < bestT || (t == bestT && tr.gid < best.gid)) {
                bestT = t;
                best.mesh = tr.mesh;
                best.prim = tr.prim;
                best.gid = tr.gid;
                best.t = t;
                best.b1 = b1;
                best.b2 = b2;
                if (anyHit) return best;
            }
        }
    }
    return best;
}

const float* sheenTable(const Scene& s) { return s.sheenLtc.empty() ? nullptr : s.sheenLtc.data(); }

bool meshTransmissive(const Scene& s, uint32_t mesh) {
    return s.materials[s.meshes[mesh].materialIndex].transmission > 0.0f;
}

// Shadow query of a scene with transmissive materials (rt/payloads/shadow_payload.slang, entry/shadow/closest_hit.slang):
// a shadow ray whose reported hit is transmissive answers "unsupported" instead of "occluded". vkrt reports the first
// hit the driver accepts, in an unspecified order; here an opaque hit anywhere on the segment wins, and the segment
// is unsupported when its only hits are transmissive.
enum : int { kShadowVisible = 0, kShadowOccluded = 1, kShadowTransmission = 2 };
int shadowFp32(const SceneFull& s, V3<float> o, V3<float> d, float tmin, float tmax, bool alpha = false,
               uint32_t alphaSeed = 0u) {
    if (s.bvh.nodes.empty()) return kShadowVisible;
    RayPre<float> rp = prepRay(o, d, tmin, tmax);
    V3<float> inv(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    bool sawTransmissive = false;
    while (sp > 0) {
        uint32_t ni = stack[--sp];
        const BvhNode& n = s.bvh.nodes[ni];
        if (!boxHit(n, o, inv, tmin, tmax)) continue;
        if (n.count == 0) {
            stack[sp++] = s.bvh.right[ni];
            stack[sp++] = n.left;
            continue;
        }
        for (uint32_t i = 0; i < n.count; ++i) {
            const WorldTri& tr = s.tris[n.left + i];
            float t, b1, b2;
            if (!watertight(rp, tr.v[0], tr.v[1], tr.v[2], t, b1, b2)) continue;
            if (alpha && !alphaAccepts(s, tr.mesh, tr.prim, b1, b2, alphaSeed, tr.gid)) continue;
            if (!meshTransmissive(s, tr.mesh)) return kShadowOccluded;
            sawTransmissive = true;
        }
    }
    return sawTransmissive ? kShadowTransmission : kShadowVisible;
}

// FP64 brute-force closest hit over world triangles (optionally reporting ambiguity)
HitRec traceFp64Brute(const SceneFull& s, const std::vector<std::array<double, 9>>& tri64, V3<double> o,
                      V3<double> d, double tmin, double tmax, bool* ambiguous, double eps) {
    RayPre<double> rp = prepRay(o, d, tmin, tmax);
    HitRec best;
    double bestT = INFINITY;
    double secondT = INFINITY;
    double bestMinBary = 0.0;
    bool nearEdgeCloser = false;
    double nearestUncertainT = INFINITY;
    for (size_t i = 0; i < tri64.size(); ++i) {
        const double* v = tri64[i].data();
        // full barycentrics without the range rejection, for the ambiguity classifier
        double A[3] = {v[0] - o.x, v[1] - o.y, v[2] - o.z}, B[3] = {v[3] - o.x, v[4] - o.y, v[5] - o.z},
               C[3] = {v[6] - o.x, v[7] - o.y, v[8] - o.z};
        double Ax = A[rp.kx] - rp.Sx * A[rp.kz], Ay = A[rp.ky] - rp.Sy * A[rp.kz];
        double Bx = B[rp.kx] - rp.Sx * B[rp.kz], By = B[rp.ky] - rp.Sy * B[rp.kz];
        double Cx = C[rp.kx] - rp.Sx * C[rp.kz], Cy = C[rp.ky] - rp.Sy * C[rp.kz];
        double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
        double det = U + V + W;
        double Az = rp.Sz * A[rp.kz], Bz = rp.Sz * B[rp.kz], Cz = rp.Sz * C[rp.kz];
        double T = U * Az + V * Bz + W * Cz;
        double sumAbs = std::fabs(U) + std::fabs(V) + std::fabs(W);
        if (!(sumAbs > 0.0)) continue;
        double bu = U / sumAbs, bv = V / sumAbs, bw = W / sumAbs;
        bool allPos = bu >= 0 && bv >= 0 && bw >= 0, allNeg = bu <= 0 && bv <= 0 && bw <= 0;
        double minB = allNeg ? std::min(-bu, std::min(-bv, -bw)) : std::min(bu, std::min(bv, bw));
        double t = det != 0.0 ? T / det : INFINITY;
        bool inside = (allPos || allNeg) && det != 0.0;
        bool inRange = t >= tmin && t <= tmax;
        // edge-adjacent candidate: barycentric margin below eps on either side
        double margin = (allPos || allNeg) ? minB : -std::max(std::max(allNeg ? bu : -bu, allNeg ? bv : -bv), allNeg ? bw : -bw);
        (void)margin;
        double edgeDist;
        if (allPos || allNeg) edgeDist = minB;
        else {
            // distance outside: most negative (sign-normalised) barycentric
            double s0 = (U + V + W) >= 0 ? 1.0 : -1.0;
            edgeDist = -std::min(s0 * bu, std::min(s0 * bv, s0 * bw));
        }
        // uncertain: the ray passes within eps (relative to the triangle) of an edge, or through the triangle at a
        // distance within eps of tmin / tmax; a triangle the ray passes well outside of is never uncertain, whatever
        // distance its plane is crossed at
        bool nearOrInside = allPos || allNeg || edgeDist < eps;
        bool uncertain = nearOrInside && (std::fabs(edgeDist) < eps ||
                                          (det != 0.0 && (std::fabs(t - tmin) < eps * std::max(1.0, tmin) ||
                                                          std::fabs(t - tmax) < eps * std::max(1.0, tmax))));
        if (uncertain && det != 0.0 && t > tmin - eps && t < tmax + eps) nearestUncertainT = std::min(nearestUncertainT, t);
        if (!inside || !inRange) continue;
        if (t < bestT || (t == bestT && s.tris[i].gid < best.gid)) {
            secondT = bestT;
            bestT = t;
            best.mesh = s.tris[i].mesh;
            best.prim = s.tris[i].prim;
            best.gid = s.tris[i].gid;
            best.t = float(t);
            best.b1 = float(V / det);
            best.b2 = float(W / det);
            bestMinBary = minB;
        } else if (t < secondT) {
            secondT = t;
        }
    }
    (void)bestMinBary;
    (void)nearEdgeCloser;
    if (ambiguous) {
        bool amb = false;
        if (std::isfinite(nearestUncertainT) &&
            nearestUncertainT <= (std::isfinite(bestT) ? bestT * (1.0 + eps) + eps : INFINITY))
            amb = true;
        if (std::isfinite(bestT) && std::isfinite(secondT) && std::fabs(secondT - bestT) <= eps * std::max(1.0, bestT)) amb = true;
        *ambiguous = amb;
    }
    return best;
}

// ---------------------------------------------------------------------------------------------------------
// Geometry reconstruction (geometry/packing.slang, geometry/surface/*.slang)
// ---------------------------------------------------------------------------------------------------------
template <class R>
V3<R> decodeOct(R px, R py) {  // packing.slang:13-21
    R z = R(1) - std::fabs(px) - std::fabs(py);
    if (z < R(0)) {
        R ox = px;
        px = (R(1) - std::fabs(py)) * (ox >= R(0) ? R(1) : R(-1));
        py = (R(1) - std::fabs(ox)) * (py >= R(0) ? R(1) : R(-1));
    }
    return normalize(V3<R>(px, py, z));
}

template <class R>
V3<R> unpackNormal(uint32_t p) {  // packing.slang:23-29
    R x = R(float(int32_t(p << 16) >> 16) / 32767.0f);
    R y = R(float(int32_t(p) >> 16) / 32767.0f);
    return decodeOct(x, y);
}

template <class R>
R unpackSnorm15(uint32_t v) {  // packing.slang:44-50
    int32_t s = int32_t(v & 0x7fffu);
    if (s & 0x4000) s |= ~int32_t(0x7fffu);
    return clampr(R(float(s) / 16383.0f), R(-1), R(1));
}

template <class R>
V4<R> unpackTangent(uint32_t p) {  // packing.slang:52-56
    V3<R> d = decodeOct(unpackSnorm15<R>(p), unpackSnorm15<R>(p >> 15u));
    return V4<R>(d.x, d.y, d.z, (p & 0x80000000u) ? R(-1) : R(1));
}

template <class R>
V4<R> unpackColor(uint32_t p) {  // packing.slang:31-42
    return V4<R>(R(float(p & 0xffu) * (1.0f / 255.0f)), R(float((p >> 8) & 0xffu) * (1.0f / 255.0f)),
                 R(float((p >> 16) & 0xffu) * (1.0f / 255.0f)), R(float((p >> 24) & 0xffu) * (1.0f / 255.0f)));
}

template <class R>
V3<R> safeNormalize(V3<R> v) {  // camera/ray.slang:32-39
    R l2 = dot(v, v);
    if (l2 <= R(kSafeEps)) return V3<R>(R(0), R(0), R(1));
    return v * rsqrtr(l2);
}

template <class R>
V3<R> rotX(V3<R> v, R a) { R s = std::sin(a), c = std::cos(a); return {v.x, c * v.y - s * v.z, s * v.y + c * v.z}; }
template <class R>
V3<R> rotY(V3<R> v, R a) { R s = std::sin(a), c = std::cos(a); return {c * v.x + s * v.z, v.y, -s * v.x + c * v.z}; }
template <class R>
V3<R> rotZ(V3<R> v, R a) { R s = std::sin(a), c = std::cos(a); return {c * v.x - s * v.y, s * v.x + c * v.y, v.z}; }

template <class R>
V3<R> rotateMesh(V3<R> v, const float* deg) {  // transform.slang:27-30
    V3<R> r = V3<R>(R(deg[0]), R(deg[1]), R(deg[2])) * R(0.01745329251994329577);
    return rotZ(rotY(rotX(v, r.x), r.y), r.z);
}

template <class R>
R safeRcp(R v) {  // transform.slang:32-38
    if (std::fabs(v) > R(1e-6)) return R(1) / v;
    return v < R(0) ? R(-1) / R(1e-6) : R(1) / R(1e-6);
}

template <class R>
V3<R> meshVector(const VKRT_CudaMeshInfo& m, V3<R> v) {  // transform.slang:40-42
    return rotateMesh(v * V3<R>(R(m.scale[0]), R(m.scale[1]), R(m.scale[2])), m.rotation);
}

template <class R>
V3<R> meshNormal(const VKRT_CudaMeshInfo& m, V3<R> n) {  // transform.slang:44-51
    V3<R> inv(safeRcp(R(m.scale[0])), safeRcp(R(m.scale[1])), safeRcp(R(m.scale[2])));
    return safeNormalize(rotateMesh(n * inv, m.rotation));
}

template <class R>
struct TexData {
    V4<R> color = V4<R>(R(1));
    R uv0[2] = {0, 0};
    R uv1[2] = {0, 0};
};

template <class R>
struct SurfaceData {
    uint32_t materialIndex = VKRT_CUDA_INVALID_INDEX;
    uint32_t frontFace = 0;
    V3<R> shadingNormal{R(0), R(0), R(1)};
    V3<R> geometricNormal{R(0), R(0), R(1)};
    V4<R> tangent{R(1), R(0), R(0), R(1)};
    TexData<R> tex;
};

template <class R>
V3<R> interp3(V3<R> a, V3<R> b, V3<R> c, R u, R v) {
    R w = R(1) - u - v;
    return a * w + b * u + c * v;
}
template <class R>
V4<R> interp4(V4<R> a, V4<R> b, V4<R> c, R u, R v) {
    R w = R(1) - u - v;
    return a * w + b * u + c * v;
}

template <class R>
SurfaceData<R> reconstruct(const Scene& s, const VKRT_CudaMeshInfo& m, uint32_t prim, R u, R v, V3<R> dir) {
    // reconstruct.slang:8-49 with loadTriangleVertices (interpolation.slang:8-25)
    uint32_t base = m.indexBase + prim * 3u;
    const VKRT_CudaShaderVertex& a = s.vertices[s.indices[base + 0] + m.vertexBase];
    const VKRT_CudaShaderVertex& b = s.vertices[s.indices[base + 1] + m.vertexBase];
    const VKRT_CudaShaderVertex& c = s.vertices[s.indices[base + 2] + m.vertexBase];
    V3<R> on = safeNormalize(interp3(unpackNormal<R>(a.packedNormal), unpackNormal<R>(b.packedNormal),
                                     unpackNormal<R>(c.packedNormal), u, v));
    V4<R> ot = interp4(unpackTangent<R>(a.packedTangent), unpackTangent<R>(b.packedTangent),
                       unpackTangent<R>(c.packedTangent), u, v);
    R hand = ot.w < R(0) ? R(-1) : R(1);
    V3<R> sn = meshNormal(m, on);
    R facing = dot(sn, dir) > R(0) ? R(-1) : R(1);
    V3<R> pa(R(a.position[0]), R(a.position[1]), R(a.position[2]));
    V3<R> pb(R(b.position[0]), R(b.position[1]), R(b.position[2]));
    V3<R> pc(R(c.position[0]), R(c.position[1]), R(c.position[2]));
    V3<R> e1 = meshVector(m, pb - pa), e2 = meshVector(m, pc - pa);
    V3<R> gn = safeNormalize(cross(e1, e2));
    if (m.scale[0] * m.scale[1] * m.scale[2] < 0.0f) gn = -gn;
    SurfaceData<R> h;
    h.materialIndex = m.materialIndex;
    h.frontFace = dot(gn, dir) < R(0) ? 1u : 0u;
    h.shadingNormal = sn * facing;
    h.geometricNormal = h.frontFace ? gn : -gn;
    V3<R> tw = safeNormalize(meshVector(m, V3<R>(ot.x, ot.y, ot.z))) * facing;
    h.tangent = V4<R>(tw.x, tw.y, tw.z, hand);
    h.tex.color = interp4(unpackColor<R>(a.packedColor), unpackColor<R>(b.packedColor), unpackColor<R>(c.packedColor), u, v);
    R w = R(1) - u - v;
    for (int k = 0; k < 2; ++k) {
        h.tex.uv0[k] = R(a.texcoord0[k]) * w + R(b.texcoord0[k]) * u + R(c.texcoord0[k]) * v;
        h.tex.uv1[k] = R(a.texcoord1[k]) * w + R(b.texcoord1[k]) * u + R(c.texcoord1[k]) * v;
    }
    return h;
}

// ---------------------------------------------------------------------------------------------------------
// Textures (material/textures.slang, bilinear sampler of src/core/scene/textures.c:141-164)
// ---------------------------------------------------------------------------------------------------------
int wrapCoord(int i, int n, uint32_t mode) {
    if (mode == VKRT_CUDA_TEXTURE_WRAP_CLAMP_TO_EDGE) return std::min(std::max(i, 0), n - 1);
    if (mode == VKRT_CUDA_TEXTURE_WRAP_MIRRORED_REPEAT) {
        int p = ((i % (2 * n)) + 2 * n) % (2 * n);
        return p < n ? p : 2 * n - 1 - p;
    }
    return ((i % n) + n) % n;
}

uint32_t wrapAxisMode(uint32_t m) {
    if (m == VKRT_CUDA_TEXTURE_WRAP_CLAMP_TO_EDGE || m == VKRT_CUDA_TEXTURE_WRAP_MIRRORED_REPEAT) return m;
    return VKRT_CUDA_TEXTURE_WRAP_REPEAT;
}

template <class R>
V4<R> sampleBilinear(const Tex& t, R u, R v, uint32_t wrapU, uint32_t wrapV) {
    R x = u * R(t.w) - R(0.5), y = v * R(t.h) - R(0.5);
    R fx0 = std::floor(x), fy0 = std::floor(y);
    int x0 = int(fx0), y0 = int(fy0);
    R ax = x - fx0, ay = y - fy0;
    int xs[2] = {wrapCoord(x0, int(t.w), wrapU), wrapCoord(x0 + 1, int(t.w), wrapU)};
    int ys[2] = {wrapCoord(y0, int(t.h), wrapV), wrapCoord(y0 + 1, int(t.h), wrapV)};
    V4<R> r(R(0));
    for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
            R wgt = (i ? ax : R(1) - ax) * (j ? ay : R(1) - ay);
            const float* p = &t.rgba[(size_t(ys[j]) * t.w + size_t(xs[i])) * 4];
            r += V4<R>(R(p[0]), R(p[1]), R(p[2]), R(p[3])) * wgt;
        }
    return r;
}

template <class R>
V4<R> sampleMaterialTexture(const Scene& s, uint32_t idx, uint32_t wrap, const float* xf, float rot, uint32_t set,
                            const TexData<R>& td, V4<R> fallback) {  // textures.slang:37-73
    if (idx == VKRT_CUDA_INVALID_INDEX || idx >= s.textures.size() || s.textures[idx].rgba.empty()) return fallback;
    const R* uv = set == 1u ? td.uv1 : td.uv0;
    R sx = uv[0] * R(xf[0]), sy = uv[1] * R(xf[1]);
    R sn = std::sin(R(rot)), cs = std::cos(R(rot));
    R tu = cs * sx - sn * sy + R(xf[2]);
    R tv = sn * sx + cs * sy + R(xf[3]);
    return sampleBilinear(s.textures[idx], tu, tv, wrapAxisMode(wrap & 0xffffu), wrapAxisMode((wrap >> 16) & 0xffffu));
}

bool alphaAccepts(const Scene& s, uint32_t mesh, uint32_t prim, float u, float v, uint32_t seed, uint32_t gid) {
    const VKRT_CudaMeshInfo& m = s.meshes[mesh];
    const VKRT_CudaMaterial& mat = s.materials[m.materialIndex];
    const uint32_t mask = 1u, blend = 2u;  // VKRT_MATERIAL_ALPHA_MODE_MASK / _BLEND (shared/constants.h:56-58)
    if (!(mat.alphaMode == mask || mat.alphaMode == blend || mat.opacity < 0.999f || m.opacity < 0.999f)) return true;
    // evaluateSurfaceTextureData (geometry/surface/interpolation.slang:46-60)
    uint32_t base = m.indexBase + prim * 3u;
    const VKRT_CudaShaderVertex& a = s.vertices[s.indices[base + 0] + m.vertexBase];
    const VKRT_CudaShaderVertex& b = s.vertices[s.indices[base + 1] + m.vertexBase];
    const VKRT_CudaShaderVertex& c = s.vertices[s.indices[base + 2] + m.vertexBase];
    TexData<float> td;
    td.color = interp4(unpackColor<float>(a.packedColor), unpackColor<float>(b.packedColor),
                       unpackColor<float>(c.packedColor), u, v);
    float w = 1.0f - u - v;
    for (int k = 0; k < 2; ++k) {
        td.uv0[k] = a.texcoord0[k] * w + b.texcoord0[k] * u + c.texcoord0[k] * v;
        td.uv1[k] = a.texcoord1[k] * w + b.texcoord1[k] * u + c.texcoord1[k] * v;
    }
    // evaluateMaterialTextureAlpha, alphaPass (rt/alpha_test.slang:19-57)
    float texAlpha = td.color.w;
    if (mat.alphaMode != VKRT_CUDA_ALPHA_MODE_OPAQUE)
        texAlpha *= sampleMaterialTexture(s, mat.baseColorTextureIndex, mat.baseColorTextureWrap,
                                          mat.baseColorTextureTransform, mat.textureRotations[0],
                                          mat.textureTexcoordSets & 0xffu, td, V4<float>(1.0f)).w;
    if (mat.alphaMode == mask) {
        if (texAlpha < mat.alphaCutoff) return false;
        float o = sat(m.opacity * mat.opacity * td.color.w);
        if (o >= 1.0f) return true;
        if (o <= 0.0f) return false;
        return alphaRandom(seed, gid) <= o;
    }
    float o = sat(m.opacity * mat.opacity * texAlpha);
    if (o <= 0.0f) return false;
    if (o >= 1.0f) return true;
    return alphaRandom(seed, gid) <= o;
}

// selectionAlphaHitAccepted (rt/alpha_test.slang:68-76): only mask cut-outs are dropped
bool selectionAlphaAccepts(const Scene& s, uint32_t mesh, uint32_t prim, float u, float v) {
    const VKRT_CudaMeshInfo& m = s.meshes[mesh];
    const VKRT_CudaMaterial& mat = s.materials[m.materialIndex];
    if (mat.alphaMode != 1u) return true;
    uint32_t base = m.indexBase + prim * 3u;
    const VKRT_CudaShaderVertex& a = s.vertices[s.indices[base + 0] + m.vertexBase];
    const VKRT_CudaShaderVertex& b = s.vertices[s.indices[base + 1] + m.vertexBase];
    const VKRT_CudaShaderVertex& c = s.vertices[s.indices[base + 2] + m.vertexBase];
    TexData<float> td;
    td.color = interp4(unpackColor<float>(a.packedColor), unpackColor<float>(b.packedColor),
                       unpackColor<float>(c.packedColor), u, v);
    float w = 1.0f - u - v;
    for (int k = 0; k < 2; ++k) {
        td.uv0[k] = a.texcoord0[k] * w + b.texcoord0[k] * u + c.texcoord0[k] * v;
        td.uv1[k] = a.texcoord1[k] * w + b.texcoord1[k] * u + c.texcoord1[k] * v;
    }
    float texAlpha = td.color.w * sampleMaterialTexture(s, mat.baseColorTextureIndex, mat.baseColorTextureWrap,
                                                        mat.baseColorTextureTransform, mat.textureRotations[0],
                                                        mat.textureTexcoordSets & 0xffu, td, V4<float>(1.0f)).w;
    return texAlpha >= mat.alphaCutoff;
}

bool sceneAlphaTested(const Scene& s) {
    for (const VKRT_CudaMeshInfo& m : s.meshes) {
        if (m.materialIndex >= s.materials.size()) continue;
        const VKRT_CudaMaterial& mat = s.materials[m.materialIndex];
        if (mat.alphaMode != VKRT_CUDA_ALPHA_MODE_OPAQUE || mat.opacity < 0.999f || m.opacity < 0.999f) return true;
    }
    return false;
}

template <class R>
struct MaterialR {  // Material fields the restated lobes read, after texturing
    V3<R> baseColor;
    R roughness, metallic, anisotropic, specular, specularTint, ior, transmission, subsurface, clearcoat;
    R clearcoatGloss, diffuseRoughness;
    R sheenWeight, sheenRoughness;
    V3<R> sheenTint;
    V3<R> eta, k;
    V3<R> emissionColor;
    R emissionLuminance;
    R abbe;
    R absorptionCoefficient;
    V3<R> attenuationColor;
};

template <class R>
void applySurfaceTextures(const Scene& s, const VKRT_CudaMaterial& m, const TexData<R>& td, MaterialR<R>& out) {
    // textures.slang:123-141
    V4<R> bc = sampleMaterialTexture(s, m.baseColorTextureIndex, m.baseColorTextureWrap, m.baseColorTextureTransform,
                                     m.textureRotations[0], (m.textureTexcoordSets >> 0) & 0xffu, td, V4<R>(R(1)));
    out.baseColor = out.baseColor * V3<R>(bc.x, bc.y, bc.z) * V3<R>(td.color.x, td.color.y, td.color.z);
    V4<R> mr = sampleMaterialTexture(s, m.metallicRoughnessTextureIndex, m.metallicRoughnessTextureWrap,
                                     m.metallicRoughnessTextureTransform, m.textureRotations[1],
                                     (m.textureTexcoordSets >> 8) & 0xffu, td, V4<R>(R(1)));
    out.roughness = sat(out.roughness * mr.y);
    out.metallic = sat(out.metallic * mr.z);
    V4<R> em = sampleMaterialTexture(s, m.emissiveTextureIndex, m.emissiveTextureWrap, m.emissiveTextureTransform,
                                     m.textureRotations[3], (m.textureTexcoordSets >> 24) & 0xffu, td, V4<R>(R(1)));
    V3<R> e = out.emissionColor * out.emissionLuminance * V3<R>(em.x, em.y, em.z);
    R emax = maxc(e);
    if (emax > R(0)) {
        out.emissionColor = e / emax;
        out.emissionLuminance = emax;
    } else {
        out.emissionColor = V3<R>(R(1));
        out.emissionLuminance = R(0);
    }
}

// ---------------------------------------------------------------------------------------------------------
// Shading basis (bsdf/base/basis.slang)
// ---------------------------------------------------------------------------------------------------------
template <class R>
struct Basis {
    V3<R> t, b, n;
};

template <class R>
Basis<R> makeBasis(V3<R> normal, V4<R> td) {
    Basis<R> B;
    B.n = safeNormalize(normal);
    V3<R> tv(td.x, td.y, td.z);
    V3<R> t = tv - B.n * dot(tv, B.n);
    if (dot(t, t) <= R(kSafeEps)) {
        V3<R> up = std::fabs(B.n.z) < R(kTangentParallel) ? V3<R>(R(0), R(0), R(1)) : V3<R>(R(1), R(0), R(0));
        t = safeNormalize(cross(up, B.n));
    } else {
        t = safeNormalize(t);
    }
    R hand = td.w < R(0) ? R(-1) : R(1);
    B.t = t;
    B.b = cross(B.n, B.t) * hand;
    return B;
}

template <class R>
V3<R> sanitizeNormal(V3<R> sn, V3<R> gn, V3<R> out) {
    V3<R> n = safeNormalize(sn), g = safeNormalize(gn), o = safeNormalize(out);
    if (dot(n, g) <= R(1e-4) || dot(n, o) <= R(1e-4)) return g;
    return n;
}

template <class R> V3<R> toWorld(V3<R> l, const Basis<R>& B) { return B.t * l.x + B.b * l.y + B.n * l.z; }
template <class R> V3<R> toLocal(V3<R> w, const Basis<R>& B) { return V3<R>(dot(w, B.t), dot(w, B.b), dot(w, B.n)); }

template <class R>
V3<R> applyNormalTexture(const Scene& s, const VKRT_CudaMaterial& m, const TexData<R>& td, const Basis<R>& B) {
    if (m.normalTextureIndex == VKRT_CUDA_INVALID_INDEX) return B.n;  // textures.slang:143-155
    V4<R> smp = sampleMaterialTexture(s, m.normalTextureIndex, m.normalTextureWrap, m.normalTextureTransform,
                                      m.textureRotations[2], (m.textureTexcoordSets >> 16) & 0xffu, td,
                                      V4<R>(R(0.5), R(0.5), R(1), R(1)));
    V3<R> n(smp.x * R(2) - R(1), smp.y * R(2) - R(1), smp.z * R(2) - R(1));
    n.x *= R(m.normalTextureScale);
    n.y *= R(m.normalTextureScale);
    n = safeNormalize(n);
    return safeNormalize(B.t * n.x + B.b * n.y + B.n * n.z);
}

// ---------------------------------------------------------------------------------------------------------
// Principled BSDF, glTF metallic-roughness subset (bsdf/**)
// ---------------------------------------------------------------------------------------------------------
template <class R> R lum(V3<R> c) { return R(0.2126) * c.x + R(0.7152) * c.y + R(0.0722) * c.z; }
template <class R> R pow5(R v) { R v2 = v * v; return v2 * v2 * v; }
template <class R> R schlickW(R c) { return pow5(R(1) - sat(c)); }

template <class R> R dielectricF0(R eta) {  // fresnel.slang:4-9
    R num = eta - R(1), den = eta + R(1);
    R f = num / std::max(den, R(1e-6));
    return f * f;
}
template <class R> V3<R> tintColor(V3<R> bc) {  // material.slang:58-61
    R l = lum(bc);
    return l <= R(0) ? V3<R>(R(1)) : bc / l;
}
template <class R> V3<R> dielSpecF0(const MaterialR<R>& m) {  // fresnel.slang:15-20
    R d = dielectricF0(m.ior);
    R sc = m.specular / R(0.5);
    V3<R> tint = V3<R>(R(1)) + (tintColor(m.baseColor) - V3<R>(R(1))) * sat(m.specularTint);
    return sat(tint * (d * sc));
}
template <class R> V3<R> schlick(R c, V3<R> f0) {  // fresnel.slang:26-29
    R w = schlickW(c);
    return f0 + (V3<R>(R(1)) - f0) * w;
}
template <class R> V3<R> fresnelConductor(R cosT, V3<R> eta, V3<R> k) {  // fresnel.slang:50-68
    R ci = sat(cosT), c2 = ci * ci, s2 = std::max(R(1) - c2, R(0));
    V3<R> r;
    for (int i = 0; i < 3; ++i) {
        R e2 = eta[i] * eta[i], k2 = k[i] * k[i];
        R t0 = e2 - k2 - s2;
        R ab = std::sqrt(std::max(t0 * t0 + R(4) * e2 * k2, R(0)));
        R t1 = ab + c2;
        R a = std::sqrt(std::max(R(0.5) * (ab + t0), R(0)));
        R t2 = R(2) * ci * a;
        R rs = (t1 - t2) / std::max(t1 + t2, R(1e-6));
        R t3 = c2 * ab + s2 * s2;
        R t4 = t2 * s2;
        R rp = rs * ((t3 - t4) / std::max(t3 + t4, R(1e-6)));
        r[i] = R(0.5) * (rp + rs);
    }
    return r;
}
template <class R> R fresnelDielectric(R cosT, R eta) {  // fresnel.slang:31-48
    R ci = clampr(cosT, R(-1), R(1));
    if (ci < R(0)) {
        eta = R(1) / std::max(eta, R(1e-6));
        ci = -ci;
    }
    R s2i = std::max(R(1) - ci * ci, R(0));
    R s2t = s2i / std::max(eta * eta, R(1e-6));
    if (s2t >= R(1)) return R(1);
    R ct = std::sqrt(std::max(R(1) - s2t, R(0)));
    R rpa = (eta * ci - ct) / std::max(eta * ci + ct, R(1e-6));
    R rpe = (ci - eta * ct) / std::max(ci + eta * ct, R(1e-6));
    return R(0.5) * (rpa * rpa + rpe * rpe);
}

template <class R>
struct Ggx {
    R ax, ay, vndfK, projLen;
};
template <class R> Ggx<R> makeGgx(const MaterialR<R>& m, V3<R> wo) {  // ggx.slang:25-72
    Ggx<R> g;
    R r = std::max(m.roughness, R(kGgxMinAlpha));
    R aspect = std::sqrt(std::max(R(1) - R(0.9) * m.anisotropic, R(kGgxMinAlpha)));
    R a = r * r;
    g.ax = std::max(a / aspect, R(kGgxMinAlpha));
    g.ay = std::max(a * aspect, R(kGgxMinAlpha));
    R am = sat(std::min(g.ax, g.ay));
    R s = R(1) + std::sqrt(wo.x * wo.x + wo.y * wo.y);
    R a2 = am * am, s2 = s * s;
    g.vndfK = (R(1) - a2) * s2 / std::max(s2 + a2 * wo.z * wo.z, R(kGgxEps));
    R sx = g.ax * wo.x, sy = g.ay * wo.y;
    g.projLen = std::sqrt(sx * sx + sy * sy + wo.z * wo.z);
    return g;
}
template <class R> R ggxLambda(V3<R> w, const Ggx<R>& g) {
    R z2 = std::max(w.z * w.z, R(kGgxEps));
    R slope2 = (g.ax * g.ax * w.x * w.x + g.ay * g.ay * w.y * w.y) / z2;
    return R(0.5) * (std::sqrt(R(1) + slope2) - R(1));
}
template <class R> R ggxD(V3<R> m, const Ggx<R>& g) {
    if (m.z <= R(0)) return R(0);
    R c = (m.x * m.x) / (g.ax * g.ax) + (m.y * m.y) / (g.ay * g.ay) + m.z * m.z;
    return R(1) / (R(kPi) * g.ax * g.ay * c * c);
}
template <class R> R ggxG(V3<R> wo, V3<R> wi, const Ggx<R>& g) { return R(1) / (R(1) + ggxLambda(wo, g) + ggxLambda(wi, g)); }
template <class R> R ggxG1(V3<R> w, const Ggx<R>& g) { return R(1) / (R(1) + ggxLambda(w, g)); }
template <class R> bool halfVector(V3<R> wo, V3<R> wi, V3<R>& m, R& woDotM) {
    V3<R> h = wo + wi;
    R h2 = dot(h, h);
    if (h2 <= R(kGgxEps)) return false;
    m = h * rsqrtr(h2);
    woDotM = dot(wo, m);
    return woDotM > R(0);
}
template <class R> R visibleNormalPdf(V3<R> wo, V3<R> m, const Ggx<R>& g) {
    R wm = dot(wo, m);
    if (wo.z <= R(0) || m.z <= R(0) || wm <= R(0)) return R(0);
    return ggxD(m, g) * ggxG1(wo, g) * wm / std::max(wo.z, R(kGgxEps));
}
template <class R> R reflectionPdf(V3<R> wo, V3<R> m, const Ggx<R>& g) {
    return visibleNormalPdf(wo, m, g) / std::max(R(4) * std::fabs(dot(wo, m)), R(kGgxEps));
}
template <class R> bool sampleVndf(V3<R> wo, const Ggx<R>& g, R u1, R u2, V3<R>& m) {  // ggx.slang:180-209
    if (g.projLen <= R(kGgxEps)) return false;
    V3<R> ws(wo.x * g.ax / g.projLen, wo.y * g.ay / g.projLen, wo.z / g.projLen);
    R phi = R(2) * R(kPi) * u1;
    R b = g.vndfK * ws.z;
    R z = (R(1) - u2) * (R(1) + b) - b;
    R st = std::sqrt(sat(R(1) - z * z));
    V3<R> wi(st * std::cos(phi), st * std::sin(phi), z);
    V3<R> ms = ws + wi;
    if (dot(ms, ms) <= R(kGgxEps)) return false;
    V3<R> um(ms.x * g.ax, ms.y * g.ay, ms.z);
    R um2 = dot(um, um);
    if (um2 <= R(kGgxEps)) return false;
    m = um * rsqrtr(um2);
    return m.z > R(0);
}

template <class R>
struct Weights {
    R metal = 0, dielectric = 0, diffuse = 0, coat = 0, subsurface = 0, sheen = 0;
};

// Disney clearcoat (bsdf/lobes/clearcoat.slang) and the coat's directional attenuation (attenuation.slang:13-24)
template <class R> R clearcoatAlpha(const MaterialR<R>& m) {
    R g = sat(m.clearcoatGloss);
    return std::max(R(0.1) + (R(0.001) - R(0.1)) * g, R(1e-3));
}
template <class R> R clearcoatG1(R c, R a) {
    R a2 = a * a, c2 = std::max(c * c, R(1e-6));
    R t2 = std::max(R(1) - c2, R(0)) / c2;
    return R(2) / (R(1) + std::sqrt(R(1) + a2 * t2));
}
template <class R> R clearcoatD(R cm, R a) {
    R a2 = a * a;
    if (a2 >= R(1) - R(1e-6)) return R(kInvPi);
    R den = R(kPi) * std::log(a2) * (R(1) + (a2 - R(1)) * cm * cm);
    return (a2 - R(1)) / std::min(den, R(-1e-6));
}
template <class R> R evalClearcoat(R weight, R a, V3<R> wo, V3<R> wi, R& pdf) {
    pdf = R(0);
    if (weight <= R(0) || wo.z <= R(0) || wi.z <= R(0)) return R(0);
    V3<R> h = safeNormalize(wo + wi);
    R woh = sat(dot(wo, h));
    if (woh <= R(0)) return R(0);
    R D = clearcoatD(sat(h.z), a);
    R F = R(0.04) + (R(1) - R(0.04)) * schlickW(woh);
    R G = clearcoatG1(wo.z, R(0.25)) * clearcoatG1(wi.z, R(0.25));
    pdf = D * sat(h.z) / std::max(R(4) * woh, R(1e-6));
    return R(0.25) * weight * D * F * G / std::max(R(4) * wo.z * wi.z, R(1e-6));
}
template <class R> R coatDirAtten(const MaterialR<R>& m, V3<R> w) {
    if (m.clearcoat <= R(0)) return R(1);
    R c = std::fabs(w.z);
    if (c <= R(0)) return R(0);
    return R(1) - sat(R(0.25) * m.clearcoat * (R(0.04) + (R(1) - R(0.04)) * schlickW(c)));
}

// Oren-Nayar and the Disney fake subsurface for a unit colour (bsdf/lobes/diffuse.slang:20-53, subsurface.slang)
template <class R> R orenNayarUnit(R rough, V3<R> wo, V3<R> wi) {
    if (wo.z <= R(0) || wi.z <= R(0)) return R(0);
    R sg = sat(rough) * (R(0.5) * R(kPi)), sg2 = sg * sg;
    R A = R(1) - sg2 / (R(2) * (sg2 + R(0.33)));
    R B = R(0.45) * sg2 / (sg2 + R(0.09));
    R s2i = sat(R(1) - wi.z * wi.z), s2o = sat(R(1) - wo.z * wo.z);
    R si = std::sqrt(s2i), so = std::sqrt(s2o);
    R cphi = R(0);
    if (s2i > R(0) && s2o > R(0))
        cphi = std::min(std::max((wi.x * wo.x + wi.y * wo.y) / std::sqrt(s2i * s2o), R(-1)), R(1));
    R mc = std::max(R(0), cphi);
    bool inSteeper = std::fabs(wi.z) > std::fabs(wo.z);
    R sinA = inSteeper ? so : si;
    R tanB = inSteeper ? si / std::max(std::fabs(wi.z), R(1e-6)) : so / std::max(std::fabs(wo.z), R(1e-6));
    return R(kInvPi) * (A + B * mc * sinA * tanB);
}
template <class R> R fakeSubsurfaceUnit(R rough, V3<R> wo, V3<R> wi) {
    if (wo.z <= R(0) || wi.z <= R(0)) return R(0);
    V3<R> h = safeNormalize(wo + wi);
    R wih = sat(dot(wi, h));
    R f90 = wih * wih * rough;
    R fin = R(1) + (f90 - R(1)) * schlickW(wi.z);
    R fout = R(1) + (f90 - R(1)) * schlickW(wo.z);
    R ss = R(1.25) * (fin * fout * (R(1) / std::max(wi.z + wo.z, R(1e-6)) - R(0.5)) + R(0.5));
    return R(kInvPi) * ss;
}

template <class R> V3<R> dielDirAlbedo(const MaterialR<R>& m, V3<R> w) {  // attenuation.slang:30-47
    if (std::fabs(w.z) <= R(0)) return V3<R>(R(1));
    R rr = sat(m.roughness), ct = sat(std::fabs(w.z));
    R r0 = rr * R(-1.0) + R(1.0), r1 = rr * R(-0.0275) + R(0.0425), r2 = rr * R(-0.572) + R(1.04),
      r3 = rr * R(0.022) + R(-0.04);
    R a004 = std::min(r0 * r0, std::exp2(R(-9.28) * ct)) * r0 + r1;
    R A = sat(R(-1.04) * a004 + r2), Bv = sat(R(1.04) * a004 + r3);
    return sat(dielSpecF0(m) * A + V3<R>(Bv));
}
template <class R> V3<R> dielDirAtten(const MaterialR<R>& m, V3<R> w) { return sat(V3<R>(R(1)) - dielDirAlbedo(m, w)); }

// Dispersion by the Cauchy fit through the Fraunhofer D line and the Abbe number (utility/spectral.slang:124-136)
template <class R> R dispersiveIor(R ior, R abbe, R lambdaNm) {
    if (ior <= R(1) + R(1e-4) || abbe <= R(0)) return std::max(ior, R(1));
    const R cUm = R(0.6562725), dUm = R(0.5875618), fUm = R(0.4861327);
    R lUm = std::max(lambdaNm * R(0.001), R(1e-4));
    R dn = (ior - R(1)) / std::max(abbe, R(1e-6));
    R B = dn / (R(1) / (fUm * fUm) - R(1) / (cUm * cUm));
    R A = ior - B / (dUm * dUm);
    return std::max(A + B / (lUm * lUm), R(1));
}
// bsdf/base/interface.slang:4-32: the interface IOR (dispersive in the spectral modes) and the two eta conventions
template <class R> R interfaceIor(const MaterialR<R>& m, R lambdaNm, bool spectral) {
    R ior = std::max(m.ior, R(1));
    return spectral ? dispersiveIor(ior, m.abbe, lambdaNm) : ior;
}
template <class R> R interfaceEta(const MaterialR<R>& m, uint32_t front, R lambdaNm = R(0), bool spectral = false) {
    R ior = interfaceIor(m, lambdaNm, spectral);
    return front ? ior : R(1) / ior;
}
template <class R> R refractionEta(const MaterialR<R>& m, uint32_t front, R lambdaNm, bool spectral) {
    R ior = interfaceIor(m, lambdaNm, spectral);
    return front ? R(1) / ior : ior;
}
template <class R> bool dielIdentity(const MaterialR<R>& m) { return std::max(m.ior, R(1)) <= R(1) + R(1e-4); }
template <class R> V3<R> transmissionColor(const MaterialR<R>& m) {  // material.slang:75-77
    return m.transmission > R(0) && m.metallic <= R(0) ? V3<R>(R(1)) : m.baseColor;
}
template <class R> R transmissionProbability(const MaterialR<R>& m, R F) {  // dielectric/interface.slang:68-72
    R tw = m.transmission * (R(1) - F), tot = F + tw;
    return tot <= R(0) ? R(0) : tw / tot;
}
template <class R> bool mediumIsRefractive(const MaterialR<R>& m) {  // base/medium.slang:40-42
    return m.transmission > R(0) && std::max(m.ior, R(1)) > R(1) + R(1e-4);
}
template <class R> bool hasAbsorption(const MaterialR<R>& m) {  // base/medium.slang:36-38
    return m.absorptionCoefficient > R(0) &&
           (m.attenuationColor.x < R(0.9999) || m.attenuationColor.y < R(0.9999) || m.attenuationColor.z < R(0.9999));
}
// HLSL refract(i, n, eta): the zero vector on total internal reflection
template <class R> V3<R> refractDir(V3<R> i, V3<R> n, R eta) {
    R c = dot(n, i);
    R k = R(1) - eta * eta * (R(1) - c * c);
    if (k < R(0)) return V3<R>(R(0));
    return i * eta - n * (eta * c + std::sqrt(k));
}

// Microfiber sheen through its LTC fit (bsdf/lobes/sheen.slang): a 32 x 32 table per layer over (cos theta_o,
// roughness), looked up bilinearly (:23-39); the lobe is a linearly transformed cosine in the frame whose tangent
// is wo's projection (:41-85)
template <class R> R lerpr(R a, R b, R t) { return a * (R(1) - t) + b * t; }
template <class R> R sheenLookup(const float* T, R cosT, R rough, uint32_t layer) {
    R ux = sat(cosT) * R(31), uy = sat(rough) * R(31);
    uint32_t x0 = std::min(uint32_t(ux), 31u), y0 = std::min(uint32_t(uy), 31u);
    uint32_t x1 = std::min(x0 + 1u, 31u), y1 = std::min(y0 + 1u, 31u);
    R tx = ux - std::floor(ux), ty = uy - std::floor(uy);
    const float* L = T + layer * 1024u;
    R e00 = R(L[y0 * 32u + x0]), e10 = R(L[y0 * 32u + x1]), e01 = R(L[y1 * 32u + x0]), e11 = R(L[y1 * 32u + x1]);
    return lerpr(lerpr(e00, e10, tx), lerpr(e01, e11, tx), ty);
}
template <class R> V3<R> sheenColor(const MaterialR<R>& m, const float* T) {  // material.slang:63-73
    return T ? sat(m.sheenTint) * sat(m.sheenWeight) : V3<R>(R(0));
}
template <class R> R sheenAlbedo(const float* T, R cosT, R rough) {  // sheenDirectionalAlbedo (sheen.slang:87-89)
    return T ? sheenLookup(T, cosT, std::min(std::max(rough, R(1e-3)), R(1)), 2u) : R(0);
}
template <class R> R sheenAtten(const float* T, R weight, R cosT, R rough) {  // sheenLayerAttenuation (:91-93)
    return sat(R(1) - weight * sheenAlbedo(T, cosT, rough));
}
template <class R> struct SheenLtc {
    Basis<R> basis;
    R a = R(0), b = R(0), albedo = R(0);
};
template <class R> SheenLtc<R> sheenLtcAt(const float* T, V3<R> wo, R sheenRough) {  // makeSheenParams (:41-57)
    SheenLtc<R> p;
    if (!T) return p;  // no table: no sheen lobe (its weight is 0 and the lobe is never evaluated)
    p.basis = makeBasis(V3<R>(R(0), R(0), R(1)), V4<R>(wo.x, wo.y, wo.z, R(1)));
    if (wo.z <= R(0)) return p;
    R r = std::min(std::max(sheenRough, R(1e-3)), R(1));
    p.a = sheenLookup(T, wo.z, r, 0u);
    p.b = sheenLookup(T, wo.z, r, 1u);
    p.albedo = sheenLookup(T, wo.z, r, 2u);
    return p;
}
template <class R> R sheenDistribution(V3<R> lw, const SheenLtc<R>& p) {  // sheenDistributionValue (:59-74)
    R z = std::max(lw.z, R(0));
    if (z <= R(0) || std::fabs(p.a) < R(1e-5) || p.albedo < R(1e-5)) return R(0);
    R axbz = p.a * lw.x + p.b * lw.z;
    R len2 = axbz * axbz + (p.a * lw.y) * (p.a * lw.y) + lw.z * lw.z;
    if (len2 <= R(1e-6)) return R(0);
    R scale = p.a / len2;
    return R(kInvPi) * z * scale * scale;
}
template <class R> R evalSheenUnit(const SheenLtc<R>& p, V3<R> wo, V3<R> wi, R& pdf) {  // evalSheen (:95-111)
    pdf = R(0);
    if (wo.z <= R(0) || wi.z <= R(0)) return R(0);
    R D = sheenDistribution(toLocal(wi, p.basis), p);
    pdf = D;
    return p.albedo * D;
}

template <class R> Weights<R> branchWeights(const MaterialR<R>& m, V3<R> wo, uint32_t frontFace,
                                            const float* sheenT) {  // weights.slang:27-62
    V3<R> diff = m.baseColor * (R(1) - m.metallic);
    R nonMetal = R(1) - m.metallic;
    R baseW = std::max(lum(m.baseColor), R(1e-3));
    R diffW = std::max(lum(diff), R(1e-3));
    R baseScatter = nonMetal * (R(1) - m.transmission);
    R transW = m.transmission * std::max(lum(transmissionColor(m)), R(1e-3));
    R dielSpecW = nonMetal * std::max(sat(lum(dielSpecF0(m))) + transW, R(0));
    Weights<R> w;
    V3<R> sc = sheenColor(m, sheenT);
    if (m.transmission > R(0) && frontFace == 0u) {  // interior side of a transmissive interface
        w.metal = m.metallic * baseW;
        w.dielectric = dielSpecW;
    } else {
        R dielAtt = lum(dielDirAtten(m, wo));
        R viewCoat = coatDirAtten(m, wo);
        R viewSheen = sheenAtten(sheenT, maxc(sc), wo.z, m.sheenRoughness);
        w.sheen = lum(sc);
        w.coat = viewSheen * m.clearcoat * R(0.25);
        w.metal = viewSheen * viewCoat * m.metallic * baseW;
        w.dielectric = viewSheen * viewCoat * dielSpecW;
        w.diffuse = viewSheen * viewCoat * dielAtt * baseScatter * (R(1) - m.subsurface) * diffW;
        w.subsurface = viewSheen * viewCoat * dielAtt * baseScatter * m.subsurface * diffW;
    }
    R total = w.sheen + w.coat + w.metal + w.dielectric + w.diffuse + w.subsurface;
    if (total <= R(0)) {
        w.metal = w.dielectric = w.coat = w.subsurface = w.sheen = R(0);
        w.diffuse = R(1);
        return w;
    }
    w.sheen /= total;
    w.coat /= total;
    w.metal /= total;
    w.dielectric /= total;
    w.diffuse /= total;
    w.subsurface /= total;
    return w;
}

template <class R>
struct BsdfState {
    MaterialR<R> mat;
    V3<R> wo;
    Ggx<R> ggx;
    uint32_t frontFace;
    Weights<R> w;
    bool conductor;
    bool interior;  // useInteriorDielectricInterface (attenuation.slang:4-6)
    const float* sheenT;  // the sheen LTC table, or null
    SheenLtc<R> sheen;    // the sheen lobe's transform at wo
};

template <class R> BsdfState<R> makeBsdf(const MaterialR<R>& m, V3<R> wo, uint32_t frontFace,
                                         const float* sheenT = nullptr) {
    BsdfState<R> s;
    s.mat = m;
    s.wo = wo;
    s.frontFace = frontFace;
    s.ggx = makeGgx(m, wo);
    s.sheenT = sheenT;
    s.sheen = sheenLtcAt(sheenT, wo, m.sheenRoughness);
    s.w = branchWeights(m, wo, frontFace, sheenT);
    s.conductor = m.k.x > R(0) || m.k.y > R(0) || m.k.z > R(0);
    s.interior = m.transmission > R(0) && frontFace == 0u;
    return s;
}

template <class R> V3<R> metalFresnelRgb(const BsdfState<R>& s, R c) {  // ggx.slang:104-116
    return s.conductor ? fresnelConductor(c, vmax(s.mat.eta, V3<R>(R(1e-3))), vmax(s.mat.k, V3<R>(R(0))))
                       : schlick(c, s.mat.baseColor);
}

// One transmission lane (dielectric/eval_rgb.slang:40-95, eval_spectral.slang:45-97): the rough dielectric BTDF of
// Walter et al. 2007 with the Fresnel-weighted choice between reflection and refraction; `color` is the lane's
// transmission colour, `coatAtt` the attenuation of the layers above the interface.
template <class R> R evalTransmissionLane(const BsdfState<R>& s, V3<R> wi, R coatAtt, R color, R lambdaNm,
                                          bool spectral, R& pdf) {
    pdf = R(0);
    if (s.mat.transmission <= R(0) || s.wo.z <= R(0) || wi.z >= R(0)) return R(0);
    if (dielIdentity(s.mat)) {
        if (dot(wi, -s.wo) < R(0.9999)) return R(0);
        pdf = R(1);
        return coatAtt * color / std::max(std::fabs(wi.z), R(kGgxEps));
    }
    R etap = interfaceEta(s.mat, s.frontFace, lambdaNm, spectral);
    V3<R> h = s.wo + wi * etap;
    if (dot(h, h) <= R(kGgxEps)) return R(0);
    V3<R> wm = safeNormalize(h);
    if (wm.z < R(0)) wm = -wm;
    R woM = dot(s.wo, wm), wiM = dot(wi, wm);
    R denom = wiM + woM / etap;
    if (!(woM > R(0) && wiM < R(0) && std::fabs(denom) > R(kGgxEps))) return R(0);
    R F = fresnelDielectric(woM, etap);
    R tprob = transmissionProbability(s.mat, F);
    if (tprob <= R(0)) return R(0);
    R D = ggxD(wm, s.ggx), G = ggxG(s.wo, wi, s.ggx);
    R d2 = denom * denom;
    R scale = R(1) / std::max(etap * etap, R(kGgxEps));
    R term = std::fabs((wiM * woM) / std::max(std::fabs(wi.z) * s.wo.z * d2, R(kGgxEps)));
    R dwm = std::fabs(wiM) / std::max(d2, R(kGgxEps));
    pdf = tprob * visibleNormalPdf(s.wo, wm, s.ggx) * dwm;
    return coatAtt * color * ((R(1) - F) * D * G * term * scale);
}

template <class R> R transmissionCoatAtt(const BsdfState<R>& s) {  // materialTransmissionStackAttenuation
    if (s.interior) return R(1);
    return sheenAtten(s.sheenT, maxc(sheenColor(s.mat, s.sheenT)), s.wo.z, s.mat.sheenRoughness) *
           coatDirAtten(s.mat, s.wo);
}

// The scalar stack (principled/eval_rgb.slang:4-141): RGB (single = false) or one wavelength of the single-wavelength
// path (single = true: colours become spectral scalars at lambda; the dielectric view attenuation stays RGB, as in
// evalScalarReflectionStack, and callers read the first component).
template <class R> void evalScalar(const BsdfState<R>& s, const Rgb2Spec* tab, V3<R> wi, R lambda, bool single,
                                   V3<R>& value, R& pdf) {
    value = V3<R>(R(0));
    pdf = R(0);
    auto spec = [&](V3<R> c) { return single ? V3<R>(spectralScalar(*tab, sat(c), lambda)) : c; };
    if (wi.z <= R(0)) {  // evalDielectricTransmission
        V3<R> tc = transmissionColor(s.mat) * ((R(1) - s.mat.metallic) * s.mat.transmission);
        tc = spec(tc);
        R coatAtt = transmissionCoatAtt(s);
        R tp = R(0);
        for (int i = 0; i < 3; ++i) value[i] = evalTransmissionLane(s, wi, coatAtt, tc[i], lambda, single, tp);
        pdf = tp * s.w.dielectric;
        return;
    }
    R coat = R(0);
    V3<R> metal(R(0)), diel(R(0)), sub(R(0)), sheenV(R(0)), sc(R(0));
    if (s.w.sheen > R(0) || !s.interior) sc = spec(sheenColor(s.mat, s.sheenT));
    if (s.w.sheen > R(0)) {
        R sp;
        sheenV = sc * evalSheenUnit(s.sheen, s.wo, wi, sp);
        pdf += s.w.sheen * sp;
    }
    if (s.w.coat > R(0)) {
        R cp;
        coat = evalClearcoat(s.mat.clearcoat, clearcoatAlpha(s.mat), s.wo, wi, cp);
        pdf += s.w.coat * cp;
    }
    if (s.w.metal > R(0)) {  // evalGGX (ggx.slang:118-152)
        V3<R> m;
        R wom;
        if (s.wo.z > R(0) && halfVector(s.wo, wi, m, wom)) {
            R D = ggxD(m, s.ggx), G = ggxG(s.wo, wi, s.ggx);
            metal = spec(metalFresnelRgb(s, wom)) * (D * G / std::max(R(4) * s.wo.z * wi.z, R(kGgxEps)));
            pdf += s.w.metal * reflectionPdf(s.wo, m, s.ggx);
        }
    }
    if (s.w.dielectric > R(0)) {  // evalDielectricReflection (dielectric/eval_rgb.slang:6-38)
        V3<R> m;
        R wom;
        if (!dielIdentity(s.mat) && s.wo.z > R(0) && halfVector(s.wo, wi, m, wom)) {
            R F = fresnelDielectric(wom, interfaceEta(s.mat, s.frontFace, lambda, single));
            R reflP = R(1) - transmissionProbability(s.mat, F);
            if (reflP > R(0)) {
                R D = ggxD(m, s.ggx), G = ggxG(s.wo, wi, s.ggx);
                V3<R> color = s.mat.transmission > R(0) && s.mat.metallic <= R(0) ? V3<R>(F)
                                                                                  : spec(schlick(wom, dielSpecF0(s.mat)));
                diel = color * (D * G / std::max(R(4) * s.wo.z * wi.z, R(kGgxEps)));
                pdf += s.w.dielectric * (reflP * reflectionPdf(s.wo, m, s.ggx));
            }
        }
    }
    if (s.w.diffuse > R(0) || s.w.subsurface > R(0)) {
        V3<R> dc = spec(s.mat.baseColor * (R(1) - s.mat.metallic));
        if (s.w.diffuse > R(0)) {  // evalLambertian / evalOrenNayar (diffuse.slang:13-53)
            V3<R> dw = dc * ((R(1) - s.mat.transmission) * (R(1) - s.mat.subsurface));
            R unit = s.mat.diffuseRoughness <= R(0) ? R(kInvPi) : orenNayarUnit(s.mat.diffuseRoughness, s.wo, wi);
            sub += dw * unit;
            pdf += s.w.diffuse * (wi.z * R(kInvPi));
        }
        if (s.w.subsurface > R(0)) {  // evalFakeSubsurface (subsurface.slang:12-31)
            V3<R> sw = dc * ((R(1) - s.mat.transmission) * s.mat.subsurface);
            sub += sw * fakeSubsurfaceUnit(s.mat.diffuseRoughness, s.wo, wi);
            pdf += s.w.subsurface * (wi.z * R(kInvPi));
        }
    }
    R nonMetal = R(1) - s.mat.metallic;
    if (s.interior) {
        value = metal * s.mat.metallic + diel * nonMetal;
        return;
    }
    V3<R> viewAtt = dielDirAtten(s.mat, s.wo);
    R att = coatDirAtten(s.mat, s.wo) * coatDirAtten(s.mat, wi);  // reflectionStackAttenuation
    R viewSheen = sheenAtten(s.sheenT, maxc(sc), s.wo.z, s.mat.sheenRoughness);
    value = sheenV + (V3<R>(coat) + (metal * s.mat.metallic + (diel + viewAtt * sub) * nonMetal) * att) * viewSheen;
}

template <class R> void evalRgb(const BsdfState<R>& s, V3<R> wi, V3<R>& value, R& pdf) {
    evalScalar(s, static_cast<const Rgb2Spec*>(nullptr), wi, R(0), false, value, pdf);
}

// 4-lane hero stack (principled/eval_spectral.slang:4-117): per-lane technique pdfs `tp` (they differ across lanes
// only at dispersive interfaces)
template <class R> V4<R> evalSpectral(const BsdfState<R>& s, const Rgb2Spec& tab, V3<R> wi, V4<R> l, V4<R>& tp) {
    tp = V4<R>(R(0));
    if (wi.z <= R(0)) {  // evalSpectralDielectricTransmission
        R coatAtt = transmissionCoatAtt(s);
        V4<R> tc = spectralScalar4(tab, sat(transmissionColor(s.mat)), l) *
                   ((R(1) - s.mat.metallic) * s.mat.transmission);
        V4<R> v;
        for (int i = 0; i < 4; ++i) v[i] = evalTransmissionLane(s, wi, coatAtt, tc[i], l[i], true, tp[i]);
        tp = tp * s.w.dielectric;
        return v;
    }
    R coat = R(0);
    V4<R> metal(R(0)), diel(R(0)), sub(R(0)), sheenV(R(0)), sc(R(0));
    if (s.w.sheen > R(0) || !s.interior) sc = spectralScalar4(tab, sat(sheenColor(s.mat, s.sheenT)), l);
    if (s.w.sheen > R(0)) {
        R sp;
        sheenV = sc * evalSheenUnit(s.sheen, s.wo, wi, sp);
        tp += V4<R>(s.w.sheen * sp);
    }
    if (s.w.coat > R(0)) {
        R cp;
        coat = evalClearcoat(s.mat.clearcoat, clearcoatAlpha(s.mat), s.wo, wi, cp);
        tp += V4<R>(s.w.coat * cp);
    }
    if (s.w.metal > R(0)) {  // evalSpectralGGX
        V3<R> m;
        R wom;
        if (s.wo.z > R(0) && halfVector(s.wo, wi, m, wom)) {
            R D = ggxD(m, s.ggx), G = ggxG(s.wo, wi, s.ggx);
            R p = reflectionPdf(s.wo, m, s.ggx);
            metal = spectralScalar4(tab, sat(metalFresnelRgb(s, wom)), l) *
                    (D * G / std::max(R(4) * s.wo.z * wi.z, R(kGgxEps)));
            tp += V4<R>(s.w.metal * p);
        }
    }
    if (s.w.dielectric > R(0)) {  // evalSpectralDielectricReflection
        V3<R> m;
        R wom;
        if (!dielIdentity(s.mat) && s.wo.z > R(0) && halfVector(s.wo, wi, m, wom)) {
            R D = ggxD(m, s.ggx), G = ggxG(s.wo, wi, s.ggx);
            R base = reflectionPdf(s.wo, m, s.ggx);
            V4<R> F, lanes;
            for (int i = 0; i < 4; ++i) {
                F[i] = fresnelDielectric(wom, interfaceEta(s.mat, s.frontFace, l[i], true));
                lanes[i] = (R(1) - transmissionProbability(s.mat, F[i])) * base;
            }
            if (anyPositive(lanes)) {
                V4<R> color = s.mat.transmission > R(0) && s.mat.metallic <= R(0)
                                  ? F
                                  : spectralScalar4(tab, sat(schlick(wom, dielSpecF0(s.mat))), l);
                diel = color * (D * G / std::max(R(4) * s.wo.z * wi.z, R(kGgxEps)));
                tp += lanes * s.w.dielectric;
            }
        }
    }
    if (s.w.diffuse > R(0) || s.w.subsurface > R(0)) {
        V4<R> dc = spectralScalar4(tab, sat(s.mat.baseColor * (R(1) - s.mat.metallic)), l);
        if (s.w.diffuse > R(0)) {
            R scale = (R(1) - s.mat.transmission) * (R(1) - s.mat.subsurface);
            R unit = s.mat.diffuseRoughness <= R(0) ? R(kInvPi) : orenNayarUnit(s.mat.diffuseRoughness, s.wo, wi);
            sub += dc * (scale * unit);
            tp += V4<R>(s.w.diffuse * (wi.z * R(kInvPi)));
        }
        if (s.w.subsurface > R(0)) {
            R scale = (R(1) - s.mat.transmission) * s.mat.subsurface;
            sub += dc * (scale * fakeSubsurfaceUnit(s.mat.diffuseRoughness, s.wo, wi));
            tp += V4<R>(s.w.subsurface * (wi.z * R(kInvPi)));
        }
    }
    R nonMetal = R(1) - s.mat.metallic;
    if (s.interior) return metal * s.mat.metallic + diel * nonMetal;
    V4<R> viewAtt = spectralScalar4(tab, sat(dielDirAtten(s.mat, s.wo)), l);
    R att = coatDirAtten(s.mat, s.wo) * coatDirAtten(s.mat, wi);
    R alb = sheenAlbedo(s.sheenT, s.wo.z, s.mat.sheenRoughness);
    V4<R> viewSheen;
    for (int i = 0; i < 4; ++i) viewSheen[i] = sat(R(1) - sc[i] * alb);
    return sheenV + (V4<R>(coat) + (metal * s.mat.metallic + (diel + viewAtt * sub) * nonMetal) * att) * viewSheen;
}

// sampleBSDFDirection (principled/sample.slang:4-51) with sampleDielectric (dielectric/sample.slang:7-53); the
// dielectric lobe refracts at the IOR of `lambda` when `spectral`
template <class R> bool sampleDirection(const BsdfState<R>& s, Rng& rng, V3<R>& wi, bool& isTrans, R lambda = R(0),
                                        bool spectral = false) {
    isTrans = false;
    R sel = R(rng.next());
    if (sel < s.w.sheen) {  // sampleSheen (sheen.slang:113-128)
        const SheenLtc<R>& p = s.sheen;
        if (std::fabs(p.a) < R(1e-5) || p.albedo < R(1e-5)) return false;
        R r = std::sqrt(R(rng.next()));
        R phi = R(2) * R(kPi) * R(rng.next());
        R dx = r * std::cos(phi), dy = r * std::sin(phi);
        R dz = std::sqrt(std::max(R(1) - (dx * dx + dy * dy), R(0)));
        V3<R> lw = normalize(V3<R>(dx - dz * p.b, dy, dz * p.a));
        wi = toWorld(lw, p.basis);
        return wi.z > R(0);
    }
    sel -= s.w.sheen;
    if (sel < s.w.coat) {  // sampleClearcoat (clearcoat.slang:73-97)
        R u1 = R(rng.next()), u2 = R(rng.next());
        R a = clearcoatAlpha(s.mat), a2 = a * a, cm;
        if (a2 >= R(1) - R(1e-6)) cm = std::sqrt(std::max(R(0), R(1) - u1));
        else cm = std::sqrt(sat((R(1) - std::pow(a2, R(1) - u1)) / std::max(R(1) - a2, R(1e-6))));
        R sm = std::sqrt(sat(R(1) - cm * cm)), phi = R(2) * R(kPi) * u2;
        V3<R> m(sm * std::cos(phi), sm * std::sin(phi), cm);
        R wom = dot(s.wo, m);
        if (wom <= R(0)) return false;
        wi = m * (R(2) * wom) - s.wo;
        return wi.z > R(0);
    }
    sel -= s.w.coat;
    if (sel < s.w.metal) {  // sampleGGX (ggx.slang:211-227)
        R u1 = R(rng.next()), u2 = R(rng.next());
        V3<R> m;
        if (!sampleVndf(s.wo, s.ggx, u1, u2, m)) return false;
        R wom = dot(s.wo, m);
        if (wom <= R(0)) return false;
        wi = m * (R(2) * wom) - s.wo;
        return wi.z > R(0);
    }
    sel -= s.w.metal;
    if (sel < s.w.dielectric) {  // sampleDielectric
        if (s.wo.z <= R(0)) return false;
        if (dielIdentity(s.mat)) {
            wi = -s.wo;
            isTrans = s.mat.transmission > R(0);
            return s.mat.transmission > R(0);
        }
        R u1 = R(rng.next()), u2 = R(rng.next());
        V3<R> m;
        if (!sampleVndf(s.wo, s.ggx, u1, u2, m)) return false;
        R wom = dot(s.wo, m);
        if (wom <= R(0)) return false;
        R F = fresnelDielectric(wom, interfaceEta(s.mat, s.frontFace, lambda, spectral));
        R tprob = transmissionProbability(s.mat, F);
        if (tprob > R(0) && R(rng.next()) < tprob) {
            V3<R> t = refractDir(-s.wo, m, refractionEta(s.mat, s.frontFace, lambda, spectral));
            if (dot(t, t) > R(0) && t.z < R(0)) {
                wi = t;
                isTrans = true;
                return true;
            }
        }
        wi = m * (R(2) * wom) - s.wo;
        return wi.z > R(0);
    }
    // diffuse, subsurface (and the fallback branch) -> cosine hemisphere (math.slang:42-48)
    R u1 = R(rng.next()), u2 = R(rng.next());
    R r = std::sqrt(u1), phi = R(2) * R(kPi) * u2;
    wi = V3<R>(r * std::cos(phi), r * std::sin(phi), std::sqrt(std::max(R(0), R(1) - u1)));
    return true;
}

// ---------------------------------------------------------------------------------------------------------
// Environment (light/environment.slang) + importance distribution
// ---------------------------------------------------------------------------------------------------------
template <class R>
void envUV(V3<R> d, R rotDeg, R& u, R& v) {  // environment.slang:9-14
    V3<R> n = normalize(d);
    R phi = std::atan2(n.y, n.x) + rotDeg * (R(kPi) / R(180));
    R theta = std::acos(clampr(n.z, R(-1), R(1)));
    u = fracr(phi * (R(0.5) * R(kInvPi)) + R(0.5));
    v = theta * R(kInvPi);
}

template <class R>
V3<R> envRadiance(const Scene& s, const VKRT_CudaSceneData& sd, V3<R> d) {  // environment.slang:16-27
    uint32_t ti = sd.environmentTextureIndex;
    if (ti == VKRT_CUDA_INVALID_INDEX || ti >= s.textures.size() || s.textures[ti].rgba.empty())
        return V3<R>(R(sd.environmentLight[0]), R(sd.environmentLight[1]), R(sd.environmentLight[2]));
    R u, v;
    envUV(d, R(sd.environmentRotation), u, v);
    V4<R> c = sampleBilinear(s.textures[ti], u, v, VKRT_CUDA_TEXTURE_WRAP_REPEAT, VKRT_CUDA_TEXTURE_WRAP_CLAMP_TO_EDGE);
    return V3<R>(c.x, c.y, c.z) * R(sd.environmentLight[3]);
}

// Importance of texel (i, j): the largest luminance in its 3x3 neighbourhood (the bilinear footprint of any
// lookup inside the texel) plus a floor of 1e-3 x the mean, times sin(theta) at the row centre.
void buildEnvDistribution(const float* rgba, uint32_t W, uint32_t H, std::vector<float>& marginal,
                          std::vector<float>& conditional, std::vector<float>& texelPdf, double* totalOut) {
    std::vector<double> lumv(size_t(W) * H);
    double mean = 0.0;
    for (uint32_t j = 0; j < H; ++j)
        for (uint32_t i = 0; i < W; ++i) {
            const float* p = rgba + (size_t(j) * W + i) * 4;
            double l = 0.2126 * double(p[0]) + 0.7152 * double(p[1]) + 0.0722 * double(p[2]);
            l = std::max(l, 0.0);
            lumv[size_t(j) * W + i] = l;
            mean += l;
        }
    mean /= double(W) * double(H);
    std::vector<double> f(size_t(W) * H);
    for (uint32_t j = 0; j < H; ++j) {
        double sinT = std::sin(3.14159265358979323846 * (double(j) + 0.5) / double(H));
        for (uint32_t i = 0; i < W; ++i) {
            double m = 0.0;
            for (int dj = -1; dj <= 1; ++dj) {
                int jj = std::min(std::max(int(j) + dj, 0), int(H) - 1);
                for (int di = -1; di <= 1; ++di) {
                    int ii = ((int(i) + di) % int(W) + int(W)) % int(W);
                    m = std::max(m, lumv[size_t(jj) * W + size_t(ii)]);
                }
            }
            f[size_t(j) * W + i] = (m + 1e-3 * mean + 1e-12) * sinT;
        }
    }
    marginal.assign(H + 1, 0.0f);
    conditional.assign(size_t(H) * (W + 1), 0.0f);
    texelPdf.assign(size_t(W) * H, 0.0f);
    std::vector<double> rowSum(H);
    double total = 0.0;
    for (uint32_t j = 0; j < H; ++j) {
        double acc = 0.0;
        for (uint32_t i = 0; i < W; ++i) acc += f[size_t(j) * W + i];
        rowSum[j] = acc;
        total += acc;
    }
    for (uint32_t j = 0; j < H; ++j) {
        double acc = 0.0;
        float* c = &conditional[size_t(j) * (W + 1)];
        c[0] = 0.0f;
        for (uint32_t i = 0; i < W; ++i) {
            acc += f[size_t(j) * W + i];
            c[i + 1] = float(acc / rowSum[j]);
        }
        c[W] = 1.0f;
    }
    double acc = 0.0;
    marginal[0] = 0.0f;
    for (uint32_t j = 0; j < H; ++j) {
        acc += rowSum[j];
        marginal[j + 1] = float(acc / total);
    }
    marginal[H] = 1.0f;
    for (size_t k = 0; k < size_t(W) * H; ++k) texelPdf[k] = float(f[k] / total * double(W) * double(H));
    if (totalOut) *totalOut = total;
}

// first index i in [0, n) with cdf[i+1] > u (cdf has n+1 entries, cdf[0] = 0, cdf[n] = 1)
uint32_t cdfFind(const float* cdf, uint32_t n, float u) {
    uint32_t lo = 0, hi = n;  // answer in [lo, hi)
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <class R>
R envPdf(const Scene& s, V3<R> d, R rotDeg) {
    if (!s.env.valid) return R(0);
    R u, v;
    envUV(d, rotDeg, u, v);
    uint32_t i = std::min(uint32_t(u * R(s.env.w)), s.env.w - 1u);
    uint32_t j = std::min(uint32_t(v * R(s.env.h)), s.env.h - 1u);
    R sinT = std::sin(v * R(kPi));
    if (sinT <= R(0)) return R(0);
    return R(s.env.texelWeight[size_t(j) * s.env.w + i]) / (R(2) * R(kPi) * R(kPi) * sinT);
}

template <class R>
bool envSample(const Scene& s, R u1, R u2, R rotDeg, V3<R>& dir, R& pdf) {
    if (!s.env.valid) return false;
    const EnvDist& e = s.env;
    uint32_t j = cdfFind(e.marginal.data(), e.h, float(u1));
    float m0 = e.marginal[j], m1 = e.marginal[j + 1];
    R dv = (u1 - R(m0)) / std::max(R(m1) - R(m0), R(1e-20));
    const float* c = &e.conditional[size_t(j) * (e.w + 1)];
    uint32_t i = cdfFind(c, e.w, float(u2));
    R du = (u2 - R(c[i])) / std::max(R(c[i + 1]) - R(c[i]), R(1e-20));
    R u = (R(i) + clampr(du, R(0), R(1))) / R(e.w);
    R v = (R(j) + clampr(dv, R(0), R(1))) / R(e.h);
    R theta = v * R(kPi);
    R phi = (u - R(0.5)) * R(2) * R(kPi) - rotDeg * (R(kPi) / R(180));
    R st = std::sin(theta);
    if (st <= R(0)) return false;
    dir = V3<R>(st * std::cos(phi), st * std::sin(phi), std::cos(theta));
    pdf = R(e.texelWeight[size_t(j) * e.w + i]) / (R(2) * R(kPi) * R(kPi) * st);
    return pdf > R(0);
}

// ---------------------------------------------------------------------------------------------------------
// Integrators (integrator/path/**)
// ---------------------------------------------------------------------------------------------------------
template <class R>
struct FeatureAcc {  // a sample's denoiser feature (integrator/path/state.slang DenoiserFeatures)
    V3<R> albedo{R(0)}, normal{R(0)};
    R weight = R(0);
};

template <class R>
struct Ctx {
    const SceneFull& s;
    const VKRT_CudaSceneData& sd;
    Rgb2Spec tab;
    bool bruteForce;
    const std::vector<std::array<double, 9>>* tri64;
    OracleRenderStats stats{};
    FeatureAcc<R>* feat = nullptr;  // the current sample's feature, when features are rendered
};

// bsdf/principled/denoiser.slang:7-22
template <class R>
bool denoiserFollowsSpecular(const MaterialR<R>& m, uint32_t frontFace) {
    R diffuseW = maxc(m.baseColor * (R(1) - m.metallic)) * (R(1) - m.transmission);
    R subsurfaceW = diffuseW * m.subsurface;
    R sheenW = maxc(sat(m.sheenTint) * sat(m.sheenWeight)) * (R(1) - m.transmission);
    R clearcoatW = frontFace != 0u ? m.clearcoat : R(0);
    const R eps = R(1e-3);
    if (diffuseW > eps || subsurfaceW > eps || sheenW > eps || clearcoatW > eps) return false;
    if (m.transmission > eps && m.ior <= R(1) + R(1e-4)) return true;
    if (m.roughness > R(0.02)) return false;
    return m.transmission > eps || m.metallic >= R(1) - eps || maxc(dielSpecF0(m)) > eps;
}

// bsdf/principled/denoiser.slang:24-44
template <class R>
V3<R> denoiserAlbedo(const MaterialR<R>& m) {
    R nonMetal = R(1) - m.metallic;
    V3<R> diffuse = m.baseColor * nonMetal;
    V3<R> sheen = sat(m.sheenTint) * sat(m.sheenWeight);
    V3<R> f0 = dielSpecF0(m);
    bool conductor = m.k.x > R(0) || m.k.y > R(0) || m.k.z > R(0);
    V3<R> metalF0 = conductor ? fresnelConductor(R(1), vmax(m.eta, V3<R>(R(1e-3))), vmax(m.k, V3<R>(R(0))))
                              : sat(m.baseColor);
    R wd = nonMetal * (R(1) - m.transmission) * (R(1) - m.subsurface);
    R wss = nonMetal * (R(1) - m.transmission) * m.subsurface;
    R ws = nonMetal * (R(1) - m.transmission) * sat(lum(f0));
    R wt = nonMetal * m.transmission;
    R wm = m.metallic;
    R wsh = maxc(sheen) * nonMetal * (R(1) - m.transmission);
    R total = wd + wss + ws + wt + wm + wsh;
    if (total <= R(0)) return sat(diffuse);
    V3<R> a = diffuse * wd + diffuse * wss + f0 * ws + V3<R>(R(1)) * wt + metalF0 * wm + sheen * wsh;
    return sat(a / total);
}

// Alpha-tested scenes take the FP32 traversal with alpha tests, also in brute-force mode.
template <class R>
HitRec traceClosest(Ctx<R>& c, V3<R> o, V3<R> d, bool primary, bool alpha = false, uint32_t alphaSeed = 0u) {
    if (primary) c.stats.primaryRays++;
    else c.stats.extensionRays++;
    if (alpha) return traceFp32(c.s, V3<float>(o), V3<float>(d), kTMin, kTMax, false, true, alphaSeed);
    if (c.bruteForce) {
        return traceFp64Brute(c.s, *c.tri64, V3<double>(o), V3<double>(d), double(kTMin), double(kTMax), nullptr, 0.0);
    }
    return traceFp32(c.s, V3<float>(o), V3<float>(d), kTMin, kTMax, false);
}

template <class R>
bool occluded(Ctx<R>& c, V3<R> o, V3<R> d, R tmax) {
    c.stats.shadowRays++;
    if (c.bruteForce) {
        HitRec h = traceFp64Brute(c.s, *c.tri64, V3<double>(o), V3<double>(d), double(kTMin), double(tmax), nullptr, 0.0);
        return h.hit();
    }
    return traceFp32(c.s, V3<float>(o), V3<float>(d), kTMin, float(tmax), true).hit();
}

template <class R>
struct Vertex {
    V3<R> hitPoint;
    SurfaceData<R> surf;
    MaterialR<R> mat;
    Basis<R> basis;
};

template <class R>
MaterialR<R> toMaterialR(const VKRT_CudaMaterial& m) {
    MaterialR<R> r;
    r.baseColor = V3<R>(R(m.baseColor[0]), R(m.baseColor[1]), R(m.baseColor[2]));
    r.roughness = R(m.roughness);
    r.metallic = R(m.metallic);
    r.anisotropic = R(m.anisotropic);
    r.specular = R(m.specular);
    r.specularTint = R(m.specularTint);
    r.ior = R(m.ior);
    r.transmission = R(m.transmission);
    r.subsurface = R(m.subsurface);
    r.clearcoat = R(m.clearcoat);
    r.clearcoatGloss = R(m.clearcoatGloss);
    r.diffuseRoughness = R(m.diffuseRoughness);
    r.sheenWeight = R(m.sheenTintWeight[3]);
    r.sheenTint = V3<R>(R(m.sheenTintWeight[0]), R(m.sheenTintWeight[1]), R(m.sheenTintWeight[2]));
    r.sheenRoughness = R(m.sheenRoughness);
    r.eta = V3<R>(R(m.eta[0]), R(m.eta[1]), R(m.eta[2]));
    r.k = V3<R>(R(m.k[0]), R(m.k[1]), R(m.k[2]));
    r.emissionColor = V3<R>(R(m.emissionColor[0]), R(m.emissionColor[1]), R(m.emissionColor[2]));
    r.emissionLuminance = R(m.emissionLuminance);
    r.abbe = R(m.abbeNumber);
    r.absorptionCoefficient = R(m.absorptionCoefficient);
    r.attenuationColor = V3<R>(R(m.attenuationColor[0]), R(m.attenuationColor[1]), R(m.attenuationColor[2]));
    return r;
}

template <class R>
Vertex<R> makeVertex(Ctx<R>& c, const HitRec& h, V3<R> o, V3<R> d) {  // surface_state.slang:14-30
    Vertex<R> v;
    v.hitPoint = o + d * R(h.t);
    const VKRT_CudaMeshInfo& mi = c.s.meshes[h.mesh];
    v.surf = reconstruct(c.s, mi, h.prim, R(h.b1), R(h.b2), d);
    const VKRT_CudaMaterial& m = c.s.materials[v.surf.materialIndex];
    Basis<R> b0 = makeBasis(v.surf.shadingNormal, v.surf.tangent);
    v.surf.shadingNormal = applyNormalTexture(c.s, m, v.surf.tex, b0);
    v.surf.shadingNormal = sanitizeNormal(v.surf.shadingNormal, v.surf.geometricNormal, -d);
    v.basis = makeBasis(v.surf.shadingNormal, v.surf.tangent);
    v.mat = toMaterialR<R>(m);
    applySurfaceTextures(c.s, m, v.surf.tex, v.mat);
    return v;
}

// integrator/path/loop.slang:83-103: the first vertex that is not followed through a sharp specular lobe
template <class R>
void captureFeature(Ctx<R>& c, const Vertex<R>& v) {
    if (!c.feat || c.feat->weight > R(0) || denoiserFollowsSpecular(v.mat, v.surf.frontFace)) return;
    c.feat->albedo = denoiserAlbedo(v.mat);
    c.feat->normal = v.surf.shadingNormal;
    c.feat->weight = R(1);
}

template <class R>
V3<R> primaryDir(const VKRT_CudaSceneData& sd, int px, int py, R jx, R jy, V3<R>& origin) {  // camera/ray.slang:15-30
    R vx = R(px - int(sd.viewportRect[0])) + R(0.5) + jx;
    R vy = R(py - int(sd.viewportRect[1])) + R(0.5) + jy;
    R ndcx = vx / R(sd.viewportRect[2]) * R(2) - R(1);
    R ndcy = vy / R(sd.viewportRect[3]) * R(2) - R(1);
    const float(*P)[4] = sd.projInverse;
    const float(*V)[4] = sd.viewInverse;
    R vd[4];
    for (int r = 0; r < 4; ++r) vd[r] = R(P[0][r]) * ndcx + R(P[1][r]) * ndcy + R(P[2][r]) * R(1) + R(P[3][r]) * R(1);
    origin = V3<R>(R(V[3][0]), R(V[3][1]), R(V[3][2]));
    V3<R> d;
    for (int r = 0; r < 3; ++r) d[r] = R(V[0][r]) * vd[0] + R(V[1][r]) * vd[1] + R(V[2][r]) * vd[2];
    return normalize(d);
}

template <class R>
struct LightSampleR {
    bool valid = false;
    V3<R> wi;
    R pdfSA = 0, shadowDist = 0;
    V3<R> emission;
};

// sampleDirectLightSurface (light/direct/light_sampling.slang:9-63)
template <class R>
LightSampleR<R> sampleEmissive(Ctx<R>& c, V3<R> p, Rng& rng) {
    LightSampleR<R> ls;
    uint32_t meshCount = c.sd.emissiveMeshCount;
    if (meshCount == 0u) return ls;
    auto alias = [](float u, uint32_t count, uint32_t off, const float* q, const uint32_t* idx) {
        float scaled = u * float(count);
        uint32_t i = std::min(uint32_t(scaled), count - 1u);
        float rem = scaled - float(i);
        return rem < q[off + i] ? i : idx[off + i];
    };
    uint32_t mi = alias(rng.next(), meshCount, 0u, c.s.meshQ.data(), c.s.meshIdx.data());
    const VKRT_CudaEmissiveMesh& em = c.s.emeshes[mi];
    if (em.triCount == 0u) return ls;
    uint32_t lt = alias(rng.next(), em.triCount, em.triOffset, c.s.triQ.data(), c.s.triIdx.data());
    const VKRT_CudaEmissiveTriangle& tr = c.s.etris[em.triOffset + lt];
    R u1 = R(rng.next()), u2 = R(rng.next());
    R su = std::sqrt(u1);
    R b1 = u2 * su, b2 = (R(1) - u2) * su;
    V3<R> v0(R(tr.v0Area[0]), R(tr.v0Area[1]), R(tr.v0Area[2]));
    V3<R> e1(R(tr.e1Pad[0]), R(tr.e1Pad[1]), R(tr.e1Pad[2]));
    V3<R> e2(R(tr.e2Pad[0]), R(tr.e2Pad[1]), R(tr.e2Pad[2]));
    V3<R> pos = v0 + e1 * b1 + e2 * b2;
    V3<R> n = safeNormalize(cross(e1, e2));
    R pdf = R(em.pmfMesh) * R(em.invTotalArea);
    if (!(pdf > R(0))) return ls;
    V3<R> tl = pos - p;
    R d2 = dot(tl, tl);
    if (d2 <= R(0)) return ls;
    R invD = rsqrtr(d2);
    R dist = d2 * invD;
    ls.wi = tl * invD;
    R cosL = std::fabs(dot(ls.wi, n));
    if (cosL <= R(0)) return ls;
    ls.pdfSA = pdf * d2 / cosL;
    if (ls.pdfSA <= R(0)) return ls;
    ls.shadowDist = dist - R(kShadowDist);
    if (ls.shadowDist <= R(0)) return ls;
    ls.emission = V3<R>(R(em.emission[0]), R(em.emission[1]), R(em.emission[2]));
    ls.valid = true;
    return ls;
}

template <class R>
bool shadowVisible(Ctx<R>& c, V3<R> p, V3<R> gn, V3<R> wi, R tmax) {  // light/direct/common.slang:37-44
    V3<R> off = dot(wi, gn) >= R(0) ? gn : -gn;
    V3<R> o = p + off * R(kShadowOrigin);
    return !occluded(c, o, wi, tmax);
}

struct ModeFlags {
    bool neeEnabled;   // misNeeEnabled && emissiveMeshCount > 0 (state.slang:50-52)
    bool envNee;       // environment importance sampling enabled and a distribution exists
    bool transmissive; // some material has transmission > 0 (environment NEE is then off: vkrt has none)
    bool alpha;        // some mesh is alpha-tested
    bool single;       // spectral mode with one wavelength per path (raygen_spectral_single.slang)
};

// A shadow ray: visible, occluded, or unsupported (through a transmissive surface). Scenes without transmissive or
// alpha-tested materials take the any-hit query above; others scan the segment with shadowFp32 (the FP32 traversal
// also in brute-force mode). `alphaSeed` is the ray's alpha seed (alphaShadowSeed of the vertex's seed).
template <class R>
int shadowResult(Ctx<R>& c, const ModeFlags& mf, V3<R> p, V3<R> gn, V3<R> wi, R tmax, uint32_t alphaSeed) {
    if (!mf.transmissive && !mf.alpha) return shadowVisible(c, p, gn, wi, tmax) ? kShadowVisible : kShadowOccluded;
    c.stats.shadowRays++;
    V3<R> off = dot(wi, gn) >= R(0) ? gn : -gn;
    V3<R> o = p + off * R(kShadowOrigin);
    return shadowFp32(c.s, V3<float>(o), V3<float>(wi), kTMin, float(tmax), mf.alpha, alphaSeed);
}

uint32_t alphaSeedOf(const Rng& r) {  // the seed of a ray that starts with the stream in state r
    if (r.mode == VKRT_CUDA_RNG_REFERENCE) return r.h;
    return uint32_t(r.state) ^ uint32_t(r.state >> 32);
}

// MediumState (bsdf/base/medium.slang:7-33): the medium a path entered through a transmissive interface
template <class R>
struct Medium {
    bool refractive = false, absorbing = false;
    V4<R> sigma = V4<R>(R(0));  // absorption: RGB in xyz, the four hero lanes, or the single wavelength in x
    bool boundary() const { return refractive || absorbing; }
};

template <class R>
R absorptionSigma1(R tint, R coeff) {  // materialAbsorptionSigma (medium.slang:44-64)
    return -std::log(std::max(tint, R(1e-6))) * coeff;
}

// updateMediumStateFromTransmission / ...Spectral (medium.slang:79-115); `mode` 0 RGB, 1 hero lanes, 2 one wavelength
template <class R>
void updateMedium(Medium<R>& med, const Rgb2Spec* tab, const MaterialR<R>& m, uint32_t frontFace, bool isTrans,
                  int mode, V4<R> lam) {
    if (!isTrans) return;
    bool entering = frontFace != 0u;
    med.refractive = entering && mediumIsRefractive(m);
    med.absorbing = entering && hasAbsorption(m);
    med.sigma = V4<R>(R(0));
    if (!med.absorbing) return;
    V3<R> tint = sat(m.attenuationColor);
    if (mode == 0) {
        med.sigma = V4<R>(absorptionSigma1(tint.x, m.absorptionCoefficient),
                          absorptionSigma1(tint.y, m.absorptionCoefficient),
                          absorptionSigma1(tint.z, m.absorptionCoefficient), R(0));
    } else if (mode == 1) {
        V4<R> s4 = spectralScalar4(*tab, tint, lam);
        for (int i = 0; i < 4; ++i) med.sigma[i] = absorptionSigma1(s4[i], m.absorptionCoefficient);
    } else {
        med.sigma = V4<R>(absorptionSigma1(spectralScalar(*tab, tint, lam.x), m.absorptionCoefficient));
    }
}

template <class R>
V4<R> mediumTransmittance(const Medium<R>& med, R dist) {
    if (!med.absorbing) return V4<R>(R(1));
    V4<R> T;
    for (int i = 0; i < 4; ++i) T[i] = std::exp(-med.sigma[i] * dist);
    return T;
}

template <class R>
V3<R> traceRgbSample(Ctx<R>& c, const ModeFlags& mf, int px, int py, uint32_t sampleIndexGlobal, uint32_t rngMode,
                     uint64_t seed) {
    // rgb/integrator.slang:15-113
    Rng rng = makeRng(rngMode, seed, px, py, c.sd.frameNumber, sampleIndexGlobal);
    c.stats.pathSamples++;
    R jx = R(rng.next()) - R(0.5);
    R jy = R(rng.next()) - R(0.5);
    V3<R> o;
    V3<R> d = primaryDir(c.sd, px, py, jx, jy, o);
    V3<R> radiance(R(0)), thr(R(1));
    R prevBsdfPdf = R(0);
    bool prevNee = false;
    Medium<R> med;
    R rot = R(c.sd.environmentRotation);
    for (uint32_t depth = 0; depth < c.sd.rrMaxDepth; ++depth) {
        const uint32_t vseed = alphaSeedOf(rng);  // the ray's alpha seed, reused salted by the vertex's shadow rays
        uint32_t requests = 0;                    // shadow requests of the vertex so far
        HitRec h = traceClosest(c, o, d, depth == 0, mf.alpha, vseed);
        if (!h.hit()) {
            if (med.boundary()) break;  // shouldAccumulateEnvironmentMiss (loop.slang:4-6)
            V3<R> L = envRadiance<R>(c.s, c.sd, d);
            R w = R(1);
            if (mf.envNee && prevNee && depth > 0 && prevBsdfPdf > R(0)) {
                R pe = envPdf(c.s, d, rot);
                if (pe > R(0)) w = (prevBsdfPdf * prevBsdfPdf) / (prevBsdfPdf * prevBsdfPdf + pe * pe);
            }
            radiance += thr * L * w;
            break;
        }
        if (med.absorbing) {  // applyRgbMediumTransmittance (rgb/transport.slang:10-17)
            V4<R> T = mediumTransmittance(med, R(h.t));
            thr = thr * V3<R>(T.x, T.y, T.z);
        }
        if (!anyPositive(thr)) break;
        Vertex<R> v = makeVertex(c, h, o, d);
        captureFeature(c, v);
        BsdfState<R> st = makeBsdf(v.mat, toLocal(-d, v.basis), v.surf.frontFace, sheenTable(c.s));
        V3<R> contrib(R(0));
        const bool neeAllowedHere = !med.refractive;  // rgb/integrator.slang:61
        bool vertexNeeSupported = neeAllowedHere;
        if (mf.neeEnabled && neeAllowedHere && st.wo.z > R(0)) {  // sampleDirectLightRgb (rgb_lighting.slang:7-31)
            LightSampleR<R> ls = sampleEmissive(c, v.hitPoint, rng);
            int vis = ls.valid ? shadowResult(c, mf, v.hitPoint, v.surf.geometricNormal, ls.wi, ls.shadowDist,
                                              alphaShadowSeed(vseed, requests++))
                               : kShadowOccluded;
            if (vis == kShadowTransmission) vertexNeeSupported = false;
            V3<R> wl = toLocal(ls.wi, v.basis);
            if (vis == kShadowVisible && !(mediumIsRefractive(v.mat) && wl.z <= R(0))) {
                V3<R> f;
                R pdf;
                evalRgb(st, wl, f, pdf);
                if (pdf > R(0)) {
                    R mis = (ls.pdfSA * ls.pdfSA) / (ls.pdfSA * ls.pdfSA + pdf * pdf);
                    V4<R> T = mediumTransmittance(med, ls.shadowDist);
                    contrib += V3<R>(T.x, T.y, T.z) * (f * std::fabs(wl.z)) * ls.emission * mis / ls.pdfSA;
                }
            }
        }
        if (mf.envNee && st.wo.z > R(0)) {  // environment NEE with MIS against the BSDF
            V3<R> wi;
            R pe;
            R u1 = R(rng.next()), u2 = R(rng.next());
            if (envSample(c.s, u1, u2, rot, wi, pe)) {
                if (shadowResult(c, mf, v.hitPoint, v.surf.geometricNormal, wi, R(kTMax),
                                 alphaShadowSeed(vseed, requests++)) == kShadowVisible) {
                    V3<R> wl = toLocal(wi, v.basis);
                    V3<R> f;
                    R pdf;
                    evalRgb(st, wl, f, pdf);
                    if (pdf > R(0)) {
                        R mis = (pe * pe) / (pe * pe + pdf * pdf);
                        contrib += (f * std::fabs(wl.z)) * envRadiance<R>(c.s, c.sd, wi) * mis / pe;
                    }
                }
            }
        }
        V3<R> emission = v.mat.emissionColor * v.mat.emissionLuminance;
        if (anyPositive(emission)) {  // loop.slang:62-80
            R w = R(1);
            if (mf.neeEnabled && prevNee && depth > 0 && prevBsdfPdf > R(0)) {
                R lpa = R(c.s.meshes[h.mesh].lightPdfArea);
                R lps = R(0);
                if (lpa > R(0)) {
                    R d2 = R(h.t) * R(h.t);
                    R cl = std::fabs(dot(d, v.surf.geometricNormal));
                    if (d2 > R(0) && cl > R(0)) lps = lpa * d2 / cl;
                }
                w = lps <= R(0) ? R(1) : (prevBsdfPdf * prevBsdfPdf) / (prevBsdfPdf * prevBsdfPdf + lps * lps);
            }
            contrib += emission * w;
        }
        radiance += thr * contrib;
        // sampleRgbNextDirection (rgb/transport.slang:23-45) via sampleBSDF (sample_rgb.slang:6-23)
        if (st.wo.z <= R(0)) break;
        V3<R> wl;
        bool isTrans;
        if (!sampleDirection(st, rng, wl, isTrans)) break;
        V3<R> f;
        R pdf;
        evalRgb(st, wl, f, pdf);
        if (pdf <= R(0)) break;
        V3<R> weight = f * std::fabs(wl.z) / pdf;
        if (!(pdf > R(0) && anyPositive(weight))) break;
        thr *= weight;
        if (!anyPositive(thr)) break;
        prevBsdfPdf = pdf;
        prevNee = vertexNeeSupported && !isTrans;
        updateMedium(med, static_cast<const Rgb2Spec*>(nullptr), v.mat, v.surf.frontFace, isTrans, 0, V4<R>(R(0)));
        if (depth + 1u >= c.sd.rrMinDepth) {  // rgb/integrator.slang:100-106
            R p = clampr(maxc(thr), R(kRRMin), R(kRRMax));
            if (R(rng.next()) > p) break;
            thr /= p;
        }
        // advancePathRay (loop.slang:113-120): a refracted ray starts below the surface
        o = v.hitPoint + (isTrans ? -v.surf.geometricNormal : v.surf.geometricNormal) * R(kShadowOrigin);
        d = toWorld(wl, v.basis);
    }
    return radiance;
}

template <class R>
V3<R> traceHeroSample(Ctx<R>& c, const ModeFlags& mf, int px, int py, uint32_t sampleIndexGlobal, uint32_t rngMode,
                      uint64_t seed) {
    // spectral_hero/integrator.slang:16-172 with spectral_hero/transport.slang: four hero lanes until a dispersive
    // refraction collapses the path to its first lane, which then continues as a single-wavelength path
    Rng rng = makeRng(rngMode, seed, px, py, c.sd.frameNumber, sampleIndexGlobal);
    c.stats.pathSamples++;
    R jx = R(rng.next()) - R(0.5);
    R jy = R(rng.next()) - R(0.5);
    V3<R> o;
    V3<R> d = primaryDir(c.sd, px, py, jx, jy, o);
    // sampleHeroWavelengths4 (wavelength.slang:29-47)
    float radInv = float(reverseBits(sampleIndexGlobal)) * (1.0f / 4294967296.0f);
    float unit = fracr(radInv + rng.next());
    V4<R> lam;
    const float offs[4] = {0.0f, 0.25f, 0.5f, 0.75f};
    for (int i = 0; i < 4; ++i) lam[i] = R(kLambdaMin) + fracr(R(unit) + R(offs[i])) * R(kLambdaRange);
    V4<R> invPdf = V4<R>(R(kLambdaRange));
    V4<R> thr(R(1)), techPath(R(1)), prevVertexTech(R(0)), prevBsdfTech(R(0)), spec(R(0));
    // spectral_single/integrator.slang:15-120 is the collapsed branch from the start: sampleUniformWavelength
    // (wavelength.slang:34-42) draws the same unit sample, so its wavelength is hero lane 0
    bool collapsed = mf.single;  // !spectralHeroPathActive
    R thrS = collapsed ? R(1) : R(0), specS = R(0), prevBsdfPdf = R(0);
    if (collapsed) thr = V4<R>(R(0));
    V3<R> xyzDone(R(0));  // the hero lanes' radiance, moved to XYZ at the collapse
    bool prevNee = false;
    Medium<R> med;
    R rot = R(c.sd.environmentRotation);
    for (uint32_t depth = 0; depth < c.sd.rrMaxDepth; ++depth) {
        const uint32_t vseed = alphaSeedOf(rng);  // the ray's alpha seed, reused salted by the vertex's shadow rays
        uint32_t requests = 0;                    // shadow requests of the vertex so far
        HitRec h = traceClosest(c, o, d, depth == 0, mf.alpha, vseed);
        if (!h.hit()) {
            if (med.boundary()) break;
            V3<R> L = envRadiance<R>(c.s, c.sd, d);
            if (collapsed) {
                specS += thrS * spectralScalar(c.tab, L, lam.x);
                break;
            }
            R w = heroBalance(techPath);
            if (mf.envNee && prevNee && depth > 0) {
                R pe = envPdf(c.s, d, rot);
                V4<R> bt = prevVertexTech * prevBsdfTech, lt = prevVertexTech * pe;
                R den = sum4(bt) + sum4(lt);
                w = den > R(0) ? bt.x / den : R(0);
            }
            spec += thr * (spectralScalar4(c.tab, L, lam) * w);
            break;
        }
        if (med.absorbing) {  // applySpectralHeroMediumTransmittance (spectral_hero/transport.slang:22-35)
            V4<R> T = mediumTransmittance(med, R(h.t));
            if (collapsed) thrS *= T.x;
            else thr = thr * T;
        }
        if (collapsed ? !(thrS > R(0)) : !anyPositive(thr)) break;
        Vertex<R> v = makeVertex(c, h, o, d);
        captureFeature(c, v);
        BsdfState<R> st = makeBsdf(v.mat, toLocal(-d, v.basis), v.surf.frontFace, sheenTable(c.s));
        V4<R> contrib(R(0));
        R contribS = R(0);
        const bool neeAllowedHere = !med.refractive;
        bool vertexNeeSupported = neeAllowedHere;
        if (mf.neeEnabled && neeAllowedHere && st.wo.z > R(0)) {
            // sampleDirectLightSpectralHero / sampleDirectLightSpectralSingle (spectral_lighting.slang:7-64)
            LightSampleR<R> ls = sampleEmissive(c, v.hitPoint, rng);
            int vis = ls.valid ? shadowResult(c, mf, v.hitPoint, v.surf.geometricNormal, ls.wi, ls.shadowDist,
                                              alphaShadowSeed(vseed, requests++))
                               : kShadowOccluded;
            if (vis == kShadowTransmission) vertexNeeSupported = false;
            V3<R> wl = toLocal(ls.wi, v.basis);
            if (vis == kShadowVisible && !(mediumIsRefractive(v.mat) && wl.z <= R(0))) {
                V4<R> T = mediumTransmittance(med, ls.shadowDist);
                if (collapsed) {
                    V3<R> f;
                    R pdf;
                    evalScalar(st, &c.tab, wl, lam.x, true, f, pdf);
                    if (pdf > R(0)) {
                        R value = f.x * std::fabs(wl.z) * spectralScalar(c.tab, ls.emission, lam.x);
                        R mis = (ls.pdfSA * ls.pdfSA) / (ls.pdfSA * ls.pdfSA + pdf * pdf);
                        contribS += mis * T.x * value / ls.pdfSA;
                    }
                } else {
                    V4<R> tp;
                    V4<R> fcos = evalSpectral(st, c.tab, wl, lam, tp) * std::fabs(wl.z);
                    V4<R> lt = techPath * ls.pdfSA, bt = techPath * tp;
                    R den = sum4(lt) + sum4(bt);
                    R mis = den > R(0) ? lt.x / den : R(0);
                    if (mis > R(0))
                        contrib += T * fcos * spectralScalar4(c.tab, ls.emission, lam) * (mis / ls.pdfSA);
                }
            }
        }
        if (mf.envNee && st.wo.z > R(0)) {  // never with transmissive materials, so never on a collapsed path
            V3<R> wi;
            R pe;
            R u1 = R(rng.next()), u2 = R(rng.next());
            if (envSample(c.s, u1, u2, rot, wi, pe)) {
                if (shadowResult(c, mf, v.hitPoint, v.surf.geometricNormal, wi, R(kTMax),
                                 alphaShadowSeed(vseed, requests++)) == kShadowVisible) {
                    V3<R> wl = toLocal(wi, v.basis);
                    V4<R> tp;
                    V4<R> fcos = evalSpectral(st, c.tab, wl, lam, tp) * std::fabs(wl.z);
                    V4<R> lt = techPath * pe, bt = techPath * tp;
                    R den = sum4(lt) + sum4(bt);
                    R mis = den > R(0) ? lt.x / den : R(0);
                    if (mis > R(0))
                        contrib += fcos * spectralScalar4(c.tab, envRadiance<R>(c.s, c.sd, wi), lam) * (mis / pe);
                }
            }
        }
        V3<R> emission = v.mat.emissionColor * v.mat.emissionLuminance;
        if (anyPositive(emission)) {
            R lps = R(0);
            R lpa = R(c.s.meshes[h.mesh].lightPdfArea);
            if (lpa > R(0)) {
                R d2 = R(h.t) * R(h.t);
                R cl = std::fabs(dot(d, v.surf.geometricNormal));
                if (d2 > R(0) && cl > R(0)) lps = lpa * d2 / cl;
            }
            if (collapsed) {  // bsdfEmitterMisWeight (loop.slang:60-80)
                R w = R(1);
                if (mf.neeEnabled && prevNee && depth > 0 && prevBsdfPdf > R(0))
                    w = lps <= R(0) ? R(1) : (prevBsdfPdf * prevBsdfPdf) / (prevBsdfPdf * prevBsdfPdf + lps * lps);
                contribS += spectralScalar(c.tab, emission, lam.x) * w;
            } else {
                R w = heroBalance(techPath);
                if (mf.neeEnabled && prevNee && depth > 0) {
                    V4<R> bt = prevVertexTech * prevBsdfTech, lt = prevVertexTech * lps;
                    R den = sum4(bt) + sum4(lt);
                    w = den > R(0) ? bt.x / den : R(0);
                }
                contrib += spectralScalar4(c.tab, emission, lam) * w;
            }
        }
        if (collapsed) specS += thrS * contribS;
        else spec += thr * contrib;
        // sampleSpectralHeroNextDirection (spectral_hero/transport.slang:49-109)
        if (st.wo.z <= R(0)) break;
        V3<R> wl;
        bool isTrans;
        if (!sampleDirection(st, rng, wl, isTrans, lam.x, true)) break;
        if (collapsed) {
            V3<R> f;
            R pdf;
            evalScalar(st, &c.tab, wl, lam.x, true, f, pdf);
            if (pdf <= R(0)) break;
            V3<R> weight = f * (std::fabs(wl.z) / pdf);
            if (!anyPositive(weight)) break;
            thrS *= weight.x;
            if (!(thrS > R(0))) break;
            prevBsdfPdf = pdf;
        } else {
            V4<R> tp;
            V4<R> val = evalSpectral(st, c.tab, wl, lam, tp);
            if (!(tp.x > R(0))) break;
            V4<R> weight = val * (std::fabs(wl.z) / tp.x);
            if (!anyPositive(weight)) break;
            prevVertexTech = techPath;
            prevBsdfTech = tp;
            techPath *= tp;
            thr *= weight;
            if (!anyPositive(thr)) break;
            if (isTrans && mediumIsRefractive(v.mat) && v.mat.abbe > R(0)) {  // collapse to the first lane
                xyzDone += spectral4ToXYZ(spec, lam, invPdf);
                spec = V4<R>(R(0));
                thrS = thr.x;
                thr = V4<R>(R(0));
                prevBsdfPdf = tp.x;
                collapsed = true;
            }
        }
        prevNee = vertexNeeSupported && !isTrans;
        updateMedium(med, &c.tab, v.mat, v.surf.frontFace, isTrans, collapsed ? 2 : 1, lam);
        if (depth + 1u >= c.sd.rrMinDepth) {
            if (collapsed) {
                R p = clampr(thrS, R(kRRMin), R(kRRMax));
                if (R(rng.next()) > p) break;
                thrS /= p;
            } else {
                R p = clampr(max4(thr), R(kRRMin), R(kRRMax));
                if (R(rng.next()) > p) break;
                techPath = techPath * p;
                thr = thr / p;
            }
        }
        o = v.hitPoint + (isTrans ? -v.surf.geometricNormal : v.surf.geometricNormal) * R(kShadowOrigin);
        d = toWorld(wl, v.basis);
    }
    if (collapsed) return xyzDone + cieXYZ(lam.x) * ((specS * invPdf.x) / R(kCieY));
    return spectral4ToXYZ(spec, lam, invPdf);
}

float srgbEncode(float v) {  // film/tonemap.slang:9-12
    if (v <= 0.0031308f) return 12.92f * v;
    return 1.055f * std::pow(v, 1.0f / 2.4f) - 0.055f;
}

void tonemapPixel(const VKRT_CudaSceneData& sd, V3<float> acc, bool spectral, uint16_t out[4]) {
    // writeback.slang:58-61 + tonemap.slang:14-32
    V3<float> c = spectral ? xyzToLinearSrgb(acc) : acc;
    c = vmax(c * sd.exposure, V3<float>(0.0f));
    if (VKRT_CUDA_TONE_MAPPING_OF(sd.packedRenderSettings) == VKRT_CUDA_TONE_MAPPING_ACES) {
        V3<float> n = c * (c * 2.51f + V3<float>(0.03f));
        V3<float> dd = c * (c * 2.43f + V3<float>(0.59f)) + V3<float>(0.14f);
        c = n / dd;
    }
    c = sat(c);
    for (int i = 0; i < 3; ++i) out[i] = uint16_t(std::lround(sat(srgbEncode(c[i])) * 65535.0f));
    out[3] = 65535;
}

template <class R>
void renderRows(SceneFull& s, const VKRT_CudaSceneData& sd, const OracleRenderParams& p, const float* accIn,
                float* accOut, uint16_t* outImg, OracleRenderStats* statsOut,
                const std::vector<std::array<double, 9>>* tri64, double* accOut64 = nullptr,
                float* albedoOut = nullptr, float* normalOut = nullptr) {
    uint32_t W = sd.viewportRect[0] + sd.viewportRect[2];
    uint32_t H = sd.viewportRect[1] + sd.viewportRect[3];
    uint32_t r0 = p.rowBegin, r1 = p.rowEnd ? std::min(p.rowEnd, H) : H;
    bool spectral = VKRT_CUDA_RENDER_MODE_OF(sd.packedRenderSettings) == VKRT_CUDA_RENDER_MODE_SPECTRAL;
    ModeFlags mf;
    mf.neeEnabled = sd.misNeeEnabled != 0u && sd.emissiveMeshCount > 0u;
    mf.transmissive = false;
    for (const VKRT_CudaMaterial& m : s.materials) mf.transmissive = mf.transmissive || m.transmission > 0.0f;
    mf.alpha = sceneAlphaTested(s);
    mf.single = spectral && VKRT_CUDA_SPECTRAL_MODE_OF(sd.packedRenderSettings) == VKRT_CUDA_SPECTRAL_SINGLE;
    if (mf.single) mf.envNee = false;
    mf.envNee = s.envSampling == VKRT_CUDA_ENV_IMPORTANCE && s.env.valid && sd.misNeeEnabled != 0u &&
                sd.environmentTextureIndex == s.envTexture && !mf.transmissive;
    Rgb2Spec tab;
    if (!s.rgb2spec.empty()) {
        tab.table = s.rgb2spec.data();
        tab.res = uint32_t(sd.rgb2specSRGB.res);
        tab.scaleOffset = sd.rgb2specSRGB.scaleOffset;
        tab.dataOffset = sd.rgb2specSRGB.dataOffset;
    }
    const uint32_t step = std::max(p.rowStep, 1u);
    const uint32_t nRows = r1 > r0 ? (r1 - r0 + step - 1u) / step : 0u;
    std::vector<OracleRenderStats> rowStats(nRows);
    uint32_t spp = std::max(sd.samplesPerPixel, 1u);
    parallelFor(nRows, p.threads, [&](uint32_t ri) {
        uint32_t y = r0 + ri * step;
        Ctx<R> c{s, sd, tab, p.useBruteForce != 0, tri64, {}};
        for (uint32_t x = 0; x < W; ++x) {
            size_t pi = size_t(y) * W + x;
            bool inside = x >= sd.viewportRect[0] && y >= sd.viewportRect[1] && sd.viewportRect[2] > 0 &&
                          sd.viewportRect[3] > 0;
            if (!inside) {
                for (int k = 0; k < 4; ++k) accOut[pi * 4 + k] = 0.0f;
                if (outImg)
                    for (int k = 0; k < 4; ++k) outImg[pi * 4 + k] = 0;
                continue;
            }
            float prev[4] = {accIn[pi * 4 + 0], accIn[pi * 4 + 1], accIn[pi * 4 + 2], accIn[pi * 4 + 3]};
            uint32_t prevN = uint32_t(prev[3] + 0.5f);  // state.slang:72
            V3<R> sum(R(0));
            FeatureAcc<R> fsum;
            for (uint32_t si = 0; si < spp; ++si) {
                uint32_t gi = prevN + si;
                FeatureAcc<R> f;
                c.feat = albedoOut ? &f : nullptr;
                sum += spectral ? traceHeroSample(c, mf, int(x), int(y), gi, p.rngMode, p.rngSeed)
                                : traceRgbSample(c, mf, int(x), int(y), gi, p.rngMode, p.rngSeed);
                fsum.albedo += f.albedo;
                fsum.normal += f.normal;
                fsum.weight += f.weight;
            }
            if (albedoOut && normalOut) {  // the frame's feature means and their weight (writeback.slang:9-22)
                V3<R> a = fsum.weight > R(0) ? fsum.albedo / fsum.weight : V3<R>(R(0));
                V3<R> n = fsum.weight > R(0) ? fsum.normal / fsum.weight : V3<R>(R(0));
                albedoOut[pi * 4 + 0] = float(a.x);
                albedoOut[pi * 4 + 1] = float(a.y);
                albedoOut[pi * 4 + 2] = float(a.z);
                albedoOut[pi * 4 + 3] = float(fsum.weight);
                normalOut[pi * 4 + 0] = float(n.x);
                normalOut[pi * 4 + 1] = float(n.y);
                normalOut[pi * 4 + 2] = float(n.z);
                normalOut[pi * 4 + 3] = float(fsum.weight);
            }
            // writeback.slang:9-22,72-114
            V3<R> cur = sum / R(spp);
            R pw = R(prevN), tw = pw + R(spp);
            V3<R> acc = tw <= R(0) ? V3<R>(R(0))
                                   : (V3<R>(R(prev[0]), R(prev[1]), R(prev[2])) * pw + cur * R(spp)) / tw;
            accOut[pi * 4 + 0] = float(acc.x);
            accOut[pi * 4 + 1] = float(acc.y);
            accOut[pi * 4 + 2] = float(acc.z);
            accOut[pi * 4 + 3] = float(tw);
            if (accOut64) {
                accOut64[pi * 4 + 0] = double(acc.x);
                accOut64[pi * 4 + 1] = double(acc.y);
                accOut64[pi * 4 + 2] = double(acc.z);
                accOut64[pi * 4 + 3] = double(tw);
            }
            if (outImg) tonemapPixel(sd, V3<float>(acc), spectral, &outImg[pi * 4]);
        }
        rowStats[ri] = c.stats;
    });
    if (statsOut) {
        *statsOut = OracleRenderStats{};
        for (auto& rs : rowStats) {
            statsOut->primaryRays += rs.primaryRays;
            statsOut->extensionRays += rs.extensionRays;
            statsOut->shadowRays += rs.shadowRays;
            statsOut->pathSamples += rs.pathSamples;
        }
    }
}

struct SceneHandle {
    SceneFull s;
    std::vector<std::array<double, 9>> tri64;  // FP64 world triangles in global-id order
    std::vector<WorldTri> trisById;
};

}  // namespace

// =========================================================================================================
// C interface
// =========================================================================================================
extern "C" {

void* oracle_scene_create(const OracleSceneDesc* d) {
    if (!d) return nullptr;
    SceneHandle* h = new SceneHandle();
    SceneFull& s = h->s;
    s.vertices.assign(d->vertices, d->vertices + d->vertexCount);
    s.indices.assign(d->indices, d->indices + d->indexCount);
    s.meshes.assign(d->meshes, d->meshes + d->meshCount);
    s.materials.assign(d->materials, d->materials + d->materialCount);
    if (d->emissiveMeshCount) {
        s.emeshes.assign(d->emissiveMeshes, d->emissiveMeshes + d->emissiveMeshCount);
        s.meshQ.assign(d->meshAliasQ, d->meshAliasQ + d->emissiveMeshCount);
        s.meshIdx.assign(d->meshAliasIdx, d->meshAliasIdx + d->emissiveMeshCount);
    }
    if (d->emissiveTriangleCount) {
        s.etris.assign(d->emissiveTriangles, d->emissiveTriangles + d->emissiveTriangleCount);
        s.triQ.assign(d->triAliasQ, d->triAliasQ + d->emissiveTriangleCount);
        s.triIdx.assign(d->triAliasIdx, d->triAliasIdx + d->emissiveTriangleCount);
    }
    s.textures.resize(d->textureCount);
    for (uint32_t i = 0; i < d->textureCount; ++i) {
        const OracleTexture& t = d->textures[i];
        if (!t.rgba) continue;
        s.textures[i].w = t.width;
        s.textures[i].h = t.height;
        s.textures[i].rgba.assign(t.rgba, t.rgba + size_t(t.width) * t.height * 4);
    }
    if (d->rgb2spec && d->rgb2specFloatCount) s.rgb2spec.assign(d->rgb2spec, d->rgb2spec + d->rgb2specFloatCount);
    if (d->sheenLtc && d->sheenLtcFloatCount >= 3072u) s.sheenLtc.assign(d->sheenLtc, d->sheenLtc + 3072);
    s.envSampling = d->environmentSampling;
    s.envTexture = d->envTextureIndex;
    if (s.envSampling == VKRT_CUDA_ENV_IMPORTANCE && d->envTextureIndex < s.textures.size() &&
        !s.textures[d->envTextureIndex].rgba.empty()) {
        const Tex& t = s.textures[d->envTextureIndex];
        s.env.w = t.w;
        s.env.h = t.h;
        buildEnvDistribution(t.rgba.data(), t.w, t.h, s.env.marginal, s.env.conditional, s.env.texelWeight, nullptr);
        s.env.valid = true;
    }
    // flatten to world space in global-id order (mesh order, then primitive order)
    s.meshTriBase.resize(s.meshes.size());
    uint32_t gid = 0;
    std::vector<WorldTri> tris;
    for (uint32_t mi = 0; mi < s.meshes.size(); ++mi) {
        const VKRT_CudaMeshInfo& m = s.meshes[mi];
        s.meshTriBase[mi] = gid;
        float M[16];
        meshWorldMatrix(m, M);
        bool ident = isIdentityTRS(m);
        double M64[16];
        for (int k = 0; k < 16; ++k) M64[k] = double(M[k]);
        uint32_t nt = m.indexCount / 3u;
        for (uint32_t t = 0; t < nt; ++t, ++gid) {
            WorldTri wt;
            std::array<double, 9> t64;
            for (int k = 0; k < 3; ++k) {
                const float* p = s.vertices[s.indices[m.indexBase + 3 * t + k] + m.vertexBase].position;
                if (ident) {
                    wt.v[k][0] = p[0];
                    wt.v[k][1] = p[1];
                    wt.v[k][2] = p[2];
                } else {
                    worldPoint(M, p, wt.v[k]);
                }
                for (int r = 0; r < 3; ++r)
                    t64[k * 3 + r] = ident ? double(p[r])
                                           : M64[0 * 4 + r] * double(p[0]) + M64[1 * 4 + r] * double(p[1]) +
                                                 M64[2 * 4 + r] * double(p[2]) + M64[3 * 4 + r];
            }
            wt.mesh = mi;
            wt.prim = t;
            wt.gid = gid;
            tris.push_back(wt);
            h->tri64.push_back(t64);
        }
    }
    h->trisById = tris;
    std::vector<BuildItem> items(tris.size());
    for (size_t i = 0; i < tris.size(); ++i) {
        for (int k = 0; k < 3; ++k) {
            items[i].lo[k] = std::min(tris[i].v[0][k], std::min(tris[i].v[1][k], tris[i].v[2][k]));
            items[i].hi[k] = std::max(tris[i].v[0][k], std::max(tris[i].v[1][k], tris[i].v[2][k]));
            items[i].c[k] = 0.5f * (items[i].lo[k] + items[i].hi[k]);
        }
        items[i].tri = uint32_t(i);
    }
    if (!items.empty()) buildBvh2(s.bvh, items, 0, uint32_t(items.size()));
    s.tris.resize(items.size());
    for (size_t i = 0; i < items.size(); ++i) s.tris[i] = tris[items[i].tri];
    // the brute-force paths index triangles by global id
    return h;
}

void oracle_scene_destroy(void* p) { delete static_cast<SceneHandle*>(p); }

uint32_t oracle_world_triangles(void* p, float* out, uint32_t capacity) {
    SceneHandle* h = static_cast<SceneHandle*>(p);
    uint32_t n = uint32_t(h->trisById.size());
    if (out)
        for (uint32_t i = 0; i < n && i < capacity; ++i)
            for (int k = 0; k < 3; ++k)
                for (int r = 0; r < 3; ++r) out[size_t(i) * 9 + k * 3 + r] = h->trisById[i].v[k][r];
    return n;
}

static void fillHit(const HitRec& r, VKRT_CudaHit* out) {
    std::memset(out, 0, sizeof(*out));
    out->instanceIndex = r.mesh;
    out->primitiveIndex = r.prim;
    out->t = r.hit() ? r.t : 0.0f;
    out->u = r.hit() ? r.b1 : 0.0f;
    out->v = r.hit() ? r.b2 : 0.0f;
}

int32_t oracle_trace_fp32(void* p, const VKRT_CudaRay* rays, uint32_t count, uint32_t anyHit, VKRT_CudaHit* hits,
                          uint32_t threads) {
    SceneHandle* h = static_cast<SceneHandle*>(p);
    if (!h || (!rays && count)) return -1;
    parallelFor((count + 255) / 256, threads, [&](uint32_t blk) {
        for (uint32_t i = blk * 256; i < std::min(count, blk * 256 + 256); ++i) {
            const VKRT_CudaRay& r = rays[i];
            HitRec hr = traceFp32(h->s, V3<float>(r.origin[0], r.origin[1], r.origin[2]),
                                  V3<float>(r.direction[0], r.direction[1], r.direction[2]), r.tMin, r.tMax,
                                  (anyHit & 1u) != 0, false, 0u, (anyHit & 2u) != 0);
            fillHit(hr, &hits[i]);
        }
    });
    return 0;
}

int32_t oracle_trace_fp64_bruteforce(void* p, const VKRT_CudaRay* rays, uint32_t count, VKRT_CudaHit* hits,
                                     uint8_t* ambiguous, double eps, uint32_t threads) {
    SceneHandle* h = static_cast<SceneHandle*>(p);
    if (!h || (!rays && count)) return -1;
    // brute force iterates triangles in global-id order
    SceneFull byId;
    byId.tris = h->trisById;
    parallelFor((count + 63) / 64, threads, [&](uint32_t blk) {
        for (uint32_t i = blk * 64; i < std::min(count, blk * 64 + 64); ++i) {
            const VKRT_CudaRay& r = rays[i];
            bool amb = false;
            HitRec hr = traceFp64Brute(byId, h->tri64, V3<double>(r.origin[0], r.origin[1], r.origin[2]),
                                       V3<double>(r.direction[0], r.direction[1], r.direction[2]), double(r.tMin),
                                       double(r.tMax), &amb, eps);
            fillHit(hr, &hits[i]);
            if (ambiguous) ambiguous[i] = amb ? 1 : 0;
        }
    });
    return 0;
}

// A spectral frame needs an rgb2spec table that holds the layout SceneData.rgb2specSRGB names (the device's frame
// validation refuses the same frames).
bool spectralTableFits(const Scene& s, const VKRT_CudaSceneData& sd) {
    if (VKRT_CUDA_RENDER_MODE_OF(sd.packedRenderSettings) != VKRT_CUDA_RENDER_MODE_SPECTRAL) return true;
    const uint64_t res = sd.rgb2specSRGB.res, n = s.rgb2spec.size();
    return res >= 2 && uint64_t(sd.rgb2specSRGB.scaleOffset) + res <= n &&
           uint64_t(sd.rgb2specSRGB.dataOffset) + 9ull * res * res * res <= n;
}

int32_t oracle_render(void* p, const VKRT_CudaSceneData* sd, const OracleRenderParams* params, const float* accIn,
                      float* accOut, uint16_t* out, OracleRenderStats* stats) {
    SceneHandle* h = static_cast<SceneHandle*>(p);
    if (!h || !sd || !params || !accIn || !accOut) return -1;
    if (!spectralTableFits(h->s, *sd)) return -2;
    SceneFull& s = h->s;
    // the brute-force path needs triangles by global id
    SceneFull* sp = &s;
    SceneFull byId;
    if (params->useBruteForce) {
        byId = s;
        byId.tris = h->trisById;
        sp = &byId;
    }
    if (params->precision == 64)
        renderRows<double>(*sp, *sd, *params, accIn, accOut, out, stats, &h->tri64);
    else
        renderRows<float>(*sp, *sd, *params, accIn, accOut, out, stats, &h->tri64);
    return 0;
}

int32_t oracle_render_f64(void* p, const VKRT_CudaSceneData* sd, const OracleRenderParams* params, const float* accIn,
                          double* accOut64) {
    SceneHandle* h = static_cast<SceneHandle*>(p);
    if (!h || !sd || !params || !accIn || !accOut64) return -1;
    if (!spectralTableFits(h->s, *sd)) return -2;
    size_t n = size_t(sd->viewportRect[0] + sd->viewportRect[2]) * (sd->viewportRect[1] + sd->viewportRect[3]) * 4;
    std::vector<float> acc32(n);
    if (params->precision == 64)
        renderRows<double>(h->s, *sd, *params, accIn, acc32.data(), nullptr, nullptr, &h->tri64, accOut64);
    else
        renderRows<float>(h->s, *sd, *params, accIn, acc32.data(), nullptr, nullptr, &h->tri64, accOut64);
    return 0;
}

int32_t oracle_render_features(void* p, const VKRT_CudaSceneData* sd, const OracleRenderParams* params,
                               const float* accIn, float* accOut, float* albedoOut, float* normalOut) {
    SceneHandle* h = static_cast<SceneHandle*>(p);
    if (!h || !sd || !params || !accIn || !accOut || !albedoOut || !normalOut) return -1;
    if (!spectralTableFits(h->s, *sd)) return -2;
    if (params->precision == 64)
        renderRows<double>(h->s, *sd, *params, accIn, accOut, nullptr, nullptr, &h->tri64, nullptr, albedoOut,
                           normalOut);
    else
        renderRows<float>(h->s, *sd, *params, accIn, accOut, nullptr, nullptr, &h->tri64, nullptr, albedoOut,
                          normalOut);
    return 0;
}

uint32_t oracle_hash(uint32_t v) { return hash32(v); }
uint32_t oracle_init_pixel_seed(int32_t x, int32_t y, uint32_t frame, uint32_t sampleIndex) {
    return pixelSeed(x, y, frame, sampleIndex);
}
float oracle_rand(uint32_t* state) {
    Rng r{};
    r.mode = VKRT_CUDA_RNG_REFERENCE;
    r.h = *state;
    float v = r.next();
    *state = r.h;
    return v;
}
uint32_t oracle_pcg32(uint64_t* state, uint64_t inc) { return pcgNext(*state, inc); }

int32_t oracle_env_cdf(const float* rgba, uint32_t w, uint32_t h, float* marginal, float* conditional,
                       double* totalOut, float* texelPdf) {
    if (!rgba || !w || !h) return -1;
    std::vector<float> m, c, t;
    buildEnvDistribution(rgba, w, h, m, c, t, totalOut);
    if (marginal) std::memcpy(marginal, m.data(), m.size() * sizeof(float));
    if (conditional) std::memcpy(conditional, c.data(), c.size() * sizeof(float));
    if (texelPdf) std::memcpy(texelPdf, t.data(), t.size() * sizeof(float));
    return 0;
}

float oracle_env_pdf(void* p, const float dir[3], float rot) {
    SceneHandle* h = static_cast<SceneHandle*>(p);
    return envPdf<float>(h->s, V3<float>(dir[0], dir[1], dir[2]), rot);
}

int32_t oracle_env_sample(void* p, float u1, float u2, float rot, float dirOut[3], float* pdfOut) {
    SceneHandle* h = static_cast<SceneHandle*>(p);
    V3<float> d;
    float pdf = 0.0f;
    bool ok = envSample<float>(h->s, u1, u2, rot, d, pdf);
    dirOut[0] = d.x;
    dirOut[1] = d.y;
    dirOut[2] = d.z;
    *pdfOut = pdf;
    return ok ? 0 : -1;
}

void oracle_rgb2spec_fetch(const float* table, uint32_t res, const float rgb[3], float coeff[3]) {
    Rgb2Spec t;
    t.table = table;
    t.res = res;
    t.scaleOffset = 0;
    t.dataOffset = res;
    V3<float> c = rgb2specFetch(t, V3<float>(rgb[0], rgb[1], rgb[2]));
    coeff[0] = c.x;
    coeff[1] = c.y;
    coeff[2] = c.z;
}
float oracle_rgb2spec_eval(const float c[3], float l) { return rgb2specEval(V3<float>(c[0], c[1], c[2]), l); }
void oracle_spectral_to_xyz(float l, float xyz[3]) {
    V3<float> v = cieXYZ(l);
    xyz[0] = v.x;
    xyz[1] = v.y;
    xyz[2] = v.z;
}
void oracle_xyz_to_linear_srgb(const float xyz[3], float rgb[3]) {
    V3<float> v = xyzToLinearSrgb(V3<float>(xyz[0], xyz[1], xyz[2]));
    rgb[0] = v.x;
    rgb[1] = v.y;
    rgb[2] = v.z;
}

int32_t oracle_bsdf_eval_rgb(const VKRT_CudaMaterial* m, const float wo[3], const float wi[3], uint32_t front,
                             float value[3], float* pdf) {
    MaterialR<float> mr = toMaterialR<float>(*m);
    BsdfState<float> st = makeBsdf(mr, V3<float>(wo[0], wo[1], wo[2]), front);
    V3<float> f;
    float p;
    evalRgb(st, V3<float>(wi[0], wi[1], wi[2]), f, p);
    value[0] = f.x;
    value[1] = f.y;
    value[2] = f.z;
    *pdf = p;
    return 0;
}

int32_t oracle_bsdf_sample_rgb(const VKRT_CudaMaterial* m, const float wo[3], uint32_t front, uint32_t rngState,
                               float wi[3], float weight[3], float* pdf) {
    MaterialR<float> mr = toMaterialR<float>(*m);
    BsdfState<float> st = makeBsdf(mr, V3<float>(wo[0], wo[1], wo[2]), front);
    Rng rng{};
    rng.mode = VKRT_CUDA_RNG_REFERENCE;
    rng.h = rngState;
    V3<float> w;
    *pdf = 0.0f;
    bool isTrans;
    if (st.wo.z <= 0.0f || !sampleDirection(st, rng, w, isTrans)) return -1;
    V3<float> f;
    float p;
    evalRgb(st, w, f, p);
    if (p <= 0.0f) return -1;
    V3<float> wt = f * std::fabs(w.z) / p;
    wi[0] = w.x;
    wi[1] = w.y;
    wi[2] = w.z;
    weight[0] = wt.x;
    weight[1] = wt.y;
    weight[2] = wt.z;
    *pdf = p;
    return 0;
}

}  // extern "C"
