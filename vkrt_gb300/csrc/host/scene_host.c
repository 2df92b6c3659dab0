/*
 * Host-side scene preparation (C11). Restates vkrt's host scene layer so that every record handed to the CUDA
 * backend is the one vkrt itself would upload. Each function cites the vkrt routine whose output it reproduces.
 */
#include "vkrt_cuda_host.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---- vertex packing: packShaderVertex (src/core/utility/packing.c:92-156) ------------------------------- */

static float clamp_range(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* normalize3f (packing.c:21-34): zero-length input maps to +Z */
static void unit3(const float in[3], float out[3]) {
    float len2 = in[0] * in[0] + in[1] * in[1] + in[2] * in[2];
    if (len2 <= 1e-20f) {
        out[0] = 0.0f;
        out[1] = 0.0f;
        out[2] = 1.0f;
        return;
    }
    float inv = 1.0f / sqrtf(len2);
    out[0] = in[0] * inv;
    out[1] = in[1] * inv;
    out[2] = in[2] * inv;
}

/* octahedral projection of a unit vector, lower hemisphere folded over the diagonals */
static void octahedral_project(const float n[3], float* px, float* py) {
    float l1 = 1.0f / (fabsf(n[0]) + fabsf(n[1]) + fabsf(n[2]));
    float x = n[0] * l1;
    float y = n[1] * l1;
    if (n[2] < 0.0f) {
        float fx = (1.0f - fabsf(y)) * (x >= 0.0f ? 1.0f : -1.0f);
        float fy = (1.0f - fabsf(x)) * (y >= 0.0f ? 1.0f : -1.0f);
        x = fx;
        y = fy;
    }
    *px = x;
    *py = y;
}

static uint32_t pack_normal_oct16(const float normal[3]) {
    float n[3];
    unit3(normal, n);
    float x, y;
    octahedral_project(n, &x, &y);
    int32_t qx = (int32_t)lroundf(clamp_range(x, -1.0f, 1.0f) * 32767.0f);
    int32_t qy = (int32_t)lroundf(clamp_range(y, -1.0f, 1.0f) * 32767.0f);
    return ((uint32_t)qx & 0xFFFFu) | (((uint32_t)qy & 0xFFFFu) << 16u);
}

static uint32_t snorm15(float v) { return (uint32_t)(int32_t)lroundf(clamp_range(v, -1.0f, 1.0f) * 16383.0f) & 0x7FFFu; }

static uint32_t pack_tangent_oct15(const float tangent[4]) {
    float n[3];
    unit3(tangent, n);
    float x, y;
    octahedral_project(n, &x, &y);
    uint32_t bits = snorm15(x) | (snorm15(y) << 15u);
    if (tangent[3] < 0.0f) bits |= 0x80000000u;
    return bits;
}

static uint32_t unorm8(float v) { return (uint32_t)lroundf(clamp_range(v, 0.0f, 1.0f) * 255.0f); }

void vkrt_host_pack_shader_vertices(const VKRT_CudaVertex* vertices, uint32_t count, VKRT_CudaShaderVertex* out) {
    if (!vertices || !out) return;
    for (uint32_t i = 0; i < count; ++i) {
        const VKRT_CudaVertex* v = &vertices[i];
        VKRT_CudaShaderVertex s;
        memset(&s, 0, sizeof(s));
        memcpy(s.position, v->position, sizeof(s.position));
        memcpy(s.texcoord0, v->texcoord0, sizeof(s.texcoord0));
        memcpy(s.texcoord1, v->texcoord1, sizeof(s.texcoord1));
        s.packedNormal = pack_normal_oct16(v->normal);
        s.packedTangent = pack_tangent_oct15(v->tangent);
        s.packedColor = unorm8(v->color[0]) | (unorm8(v->color[1]) << 8u) | (unorm8(v->color[2]) << 16u) |
                        (unorm8(v->color[3]) << 24u);
        out[i] = s;
    }
}

/* ---- matrices ---------------------------------------------------------------------------------------------- */

/* column-major helpers: m[c * 4 + r] */
static void mat4_identity(float m[16]) {
    memset(m, 0, 16 * sizeof(float));
    m[0] = m[5] = m[10] = m[15] = 1.0f;
}

static void mat4_mul(const float a[16], const float b[16], float out[16]) {
    float r[16];
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            float acc = 0.0f;
            for (int k = 0; k < 4; ++k) acc += a[k * 4 + row] * b[c * 4 + k];
            r[c * 4 + row] = acc;
        }
    memcpy(out, r, sizeof(r));
}

/* rotation about a principal axis (0 = X, 1 = Y, 2 = Z) by `radians`, right-handed */
static void mat4_axis_rotation(int axis, float radians, float m[16]) {
    mat4_identity(m);
    float c = cosf(radians), s = sinf(radians);
    int i = (axis + 1) % 3, j = (axis + 2) % 3;
    m[i * 4 + i] = c;
    m[j * 4 + j] = c;
    m[i * 4 + j] = s;  /* column i, row j */
    m[j * 4 + i] = -s; /* column j, row i */
}

void vkrt_host_mesh_transform(const float position[3], const float rotationDegrees[3], const float scale[3],
                              float out[16]) {
    const float deg = 0.01745329251994329577f;
    float m[16], r[16];
    mat4_identity(m);
    m[12] = position[0];
    m[13] = position[1];
    m[14] = position[2];
    mat4_axis_rotation(2, rotationDegrees[2] * deg, r);
    mat4_mul(m, r, m);
    mat4_axis_rotation(1, rotationDegrees[1] * deg, r);
    mat4_mul(m, r, m);
    mat4_axis_rotation(0, rotationDegrees[0] * deg, r);
    mat4_mul(m, r, m);
    for (int c = 0; c < 3; ++c)
        for (int row = 0; row < 4; ++row) m[c * 4 + row] *= scale[c];
    memcpy(out, m, sizeof(m));
}

/* general inverse through the adjugate (cofactor expansion by 2x2 minors) */
static void mat4_inverse(const float m[16], float out[16]) {
    /* element (row r, column c) = m[c*4 + r] */
#define E(r, c) m[(c) * 4 + (r)]
    float s0 = E(0, 0) * E(1, 1) - E(1, 0) * E(0, 1);
    float s1 = E(0, 0) * E(1, 2) - E(1, 0) * E(0, 2);
    float s2 = E(0, 0) * E(1, 3) - E(1, 0) * E(0, 3);
    float s3 = E(0, 1) * E(1, 2) - E(1, 1) * E(0, 2);
    float s4 = E(0, 1) * E(1, 3) - E(1, 1) * E(0, 3);
    float s5 = E(0, 2) * E(1, 3) - E(1, 2) * E(0, 3);
    float c5 = E(2, 2) * E(3, 3) - E(3, 2) * E(2, 3);
    float c4 = E(2, 1) * E(3, 3) - E(3, 1) * E(2, 3);
    float c3 = E(2, 1) * E(3, 2) - E(3, 1) * E(2, 2);
    float c2 = E(2, 0) * E(3, 3) - E(3, 0) * E(2, 3);
    float c1 = E(2, 0) * E(3, 2) - E(3, 0) * E(2, 2);
    float c0 = E(2, 0) * E(3, 1) - E(3, 0) * E(2, 1);
    float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    float inv = det != 0.0f ? 1.0f / det : 0.0f;
    float r[16];
#define O(r_, c_) r[(c_) * 4 + (r_)]
    O(0, 0) = (E(1, 1) * c5 - E(1, 2) * c4 + E(1, 3) * c3) * inv;
    O(0, 1) = (-E(0, 1) * c5 + E(0, 2) * c4 - E(0, 3) * c3) * inv;
    O(0, 2) = (E(3, 1) * s5 - E(3, 2) * s4 + E(3, 3) * s3) * inv;
    O(0, 3) = (-E(2, 1) * s5 + E(2, 2) * s4 - E(2, 3) * s3) * inv;
    O(1, 0) = (-E(1, 0) * c5 + E(1, 2) * c2 - E(1, 3) * c1) * inv;
    O(1, 1) = (E(0, 0) * c5 - E(0, 2) * c2 + E(0, 3) * c1) * inv;
    O(1, 2) = (-E(3, 0) * s5 + E(3, 2) * s2 - E(3, 3) * s1) * inv;
    O(1, 3) = (E(2, 0) * s5 - E(2, 2) * s2 + E(2, 3) * s1) * inv;
    O(2, 0) = (E(1, 0) * c4 - E(1, 1) * c2 + E(1, 3) * c0) * inv;
    O(2, 1) = (-E(0, 0) * c4 + E(0, 1) * c2 - E(0, 3) * c0) * inv;
    O(2, 2) = (E(3, 0) * s4 - E(3, 1) * s2 + E(3, 3) * s0) * inv;
    O(2, 3) = (-E(2, 0) * s4 + E(2, 1) * s2 - E(2, 3) * s0) * inv;
    O(3, 0) = (-E(1, 0) * c3 + E(1, 1) * c1 - E(1, 2) * c0) * inv;
    O(3, 1) = (E(0, 0) * c3 - E(0, 1) * c1 + E(0, 2) * c0) * inv;
    O(3, 2) = (-E(3, 0) * s3 + E(3, 1) * s1 - E(3, 2) * s0) * inv;
    O(3, 3) = (E(2, 0) * s3 - E(2, 1) * s1 + E(2, 2) * s0) * inv;
#undef O
#undef E
    memcpy(out, r, sizeof(r));
}

void vkrt_host_camera_matrices(const float pos[3], const float target[3], const float up[3], float vfovDegrees,
                               float nearZ, float farZ, uint32_t width, uint32_t height, VKRT_CudaSceneData* sd) {
    if (!sd) return;
    /* right-handed look-at: forward f, side s = f x up, true up u = s x f */
    float f[3] = {target[0] - pos[0], target[1] - pos[1], target[2] - pos[2]};
    float fl = sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (fl > 0.0f) { f[0] /= fl; f[1] /= fl; f[2] /= fl; }
    float s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    float sl = sqrtf(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (sl > 0.0f) { s[0] /= sl; s[1] /= sl; s[2] /= sl; }
    float u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    float view[16];
    memset(view, 0, sizeof(view));
    for (int i = 0; i < 3; ++i) {
        view[i * 4 + 0] = s[i];
        view[i * 4 + 1] = u[i];
        view[i * 4 + 2] = -f[i];
    }
    view[12] = -(s[0] * pos[0] + s[1] * pos[1] + s[2] * pos[2]);
    view[13] = -(u[0] * pos[0] + u[1] * pos[1] + u[2] * pos[2]);
    view[14] = f[0] * pos[0] + f[1] * pos[1] + f[2] * pos[2];
    view[15] = 1.0f;

    uint32_t w = width > 0u ? width : 1u, h = height > 0u ? height : 1u;
    float aspect = (float)w / (float)h;
    float fy = 1.0f / tanf(vfovDegrees * 0.01745329251994329577f * 0.5f);
    float fn = 1.0f / (nearZ - farZ);
    float proj[16];
    memset(proj, 0, sizeof(proj));
    proj[0] = fy / aspect;
    proj[5] = -fy; /* Vulkan Y flip applied to the OpenGL-style projection */
    proj[10] = (nearZ + farZ) * fn;
    proj[11] = -1.0f;
    proj[14] = 2.0f * nearZ * farZ * fn;

    float vi[16], pi[16];
    mat4_inverse(view, vi);
    mat4_inverse(proj, pi);
    memcpy(sd->viewInverse, vi, sizeof(vi));
    memcpy(sd->projInverse, pi, sizeof(pi));
}

void vkrt_host_default_scene_data(uint32_t width, uint32_t height, VKRT_CudaSceneData* sd) {
    if (!sd) return;
    memset(sd, 0, sizeof(*sd));
    sd->samplesPerPixel = 8u;
    sd->rrMaxDepth = 8u;
    sd->rrMinDepth = 4u;
    sd->viewportRect[0] = 0u;
    sd->viewportRect[1] = 0u;
    sd->viewportRect[2] = width;
    sd->viewportRect[3] = height;
    sd->packedRenderSettings =
        VKRT_CUDA_PACK_RENDER_SETTINGS(VKRT_CUDA_TONE_MAPPING_ACES, VKRT_CUDA_RENDER_MODE_RGB, VKRT_CUDA_SPECTRAL_HERO);
    sd->exposure = 1.0f;
    sd->timeBase = -1.0f;
    sd->timeStep = 0.5f;
    sd->environmentLight[0] = 0.25f;
    sd->environmentLight[1] = 0.25f;
    sd->environmentLight[2] = 0.25f;
    sd->environmentLight[3] = 1.0f;
    sd->environmentTextureIndex = VKRT_CUDA_INVALID_INDEX;
    sd->environmentRotation = 0.0f;
    sd->debugMode = VKRT_CUDA_DEBUG_MODE_NONE;
    sd->misNeeEnabled = 1u;
    sd->selectionEnabled = 0u;
    sd->selectedMeshIndex = VKRT_CUDA_INVALID_INDEX;
    const float pos[3] = {-0.5f, 0.2f, -0.2f}, tgt[3] = {0.0f, 0.0f, 0.0f}, up[3] = {0.0f, 0.0f, 1.0f};
    vkrt_host_camera_matrices(pos, tgt, up, 40.0f, 0.001f, 10000.0f, width, height, sd);
}

void vkrt_host_default_material(VKRT_CudaMaterial* m) {
    if (!m) return;
    memset(m, 0, sizeof(*m));
    m->baseColor[0] = m->baseColor[1] = m->baseColor[2] = 0.8f;
    m->roughness = 0.5f;
    m->emissionColor[0] = m->emissionColor[1] = m->emissionColor[2] = 1.0f;
    m->specular = 0.5f;
    m->sheenTintWeight[0] = m->sheenTintWeight[1] = m->sheenTintWeight[2] = 1.0f;
    m->clearcoatGloss = 1.0f;
    m->ior = 1.5f;
    m->sheenRoughness = 0.5f;
    m->attenuationColor[0] = m->attenuationColor[1] = m->attenuationColor[2] = 1.0f;
    m->normalTextureScale = 1.0f;
    m->baseColorTextureIndex = VKRT_CUDA_INVALID_INDEX;
    m->metallicRoughnessTextureIndex = VKRT_CUDA_INVALID_INDEX;
    m->normalTextureIndex = VKRT_CUDA_INVALID_INDEX;
    m->emissiveTextureIndex = VKRT_CUDA_INVALID_INDEX;
    m->opacity = 1.0f;
    m->alphaCutoff = 0.5f;
    m->alphaMode = VKRT_CUDA_ALPHA_MODE_OPAQUE;
    for (int i = 0; i < 4; ++i) {
        float* t[4] = {m->baseColorTextureTransform, m->metallicRoughnessTextureTransform, m->normalTextureTransform,
                       m->emissiveTextureTransform};
        t[i][0] = 1.0f;
        t[i][1] = 1.0f;
    }
}

/* ---- emissive light tables (src/core/scene/lighting.c) ------------------------------------------------------ */

/* Walker/Vose alias table with two LIFO work lists, as buildAliasTable (lighting.c:108-164) fills them: the
 * order in which under-full and over-full bins are paired decides the table contents, so it is kept. */
void vkrt_host_build_alias_table(const float* pmf, uint32_t count, float* outQ, uint32_t* outIdx) {
    if (count == 0u || !pmf || !outQ || !outIdx) return;
    float* weight = (float*)malloc(sizeof(float) * count);
    uint32_t* under = (uint32_t*)malloc(sizeof(uint32_t) * count);
    uint32_t* over = (uint32_t*)malloc(sizeof(uint32_t) * count);
    if (!weight || !under || !over) {
        free(weight);
        free(under);
        free(over);
        for (uint32_t i = 0; i < count; ++i) {
            outQ[i] = 1.0f;
            outIdx[i] = i;
        }
        return;
    }
    uint32_t nUnder = 0, nOver = 0;
    for (uint32_t i = 0; i < count; ++i) {
        weight[i] = pmf[i] * (float)count;
        if (weight[i] < 1.0f) under[nUnder++] = i;
        else over[nOver++] = i;
    }
    while (nUnder > 0u && nOver > 0u) {
        uint32_t lo = under[--nUnder];
        uint32_t hi = over[--nOver];
        outQ[lo] = weight[lo];
        outIdx[lo] = hi;
        weight[hi] = weight[hi] + weight[lo] - 1.0f;
        if (weight[hi] < 1.0f) under[nUnder++] = hi;
        else over[nOver++] = hi;
    }
    while (nOver > 0u) {
        uint32_t i = over[--nOver];
        outQ[i] = 1.0f;
        outIdx[i] = i;
    }
    while (nUnder > 0u) {
        uint32_t i = under[--nUnder];
        outQ[i] = 1.0f;
        outIdx[i] = i;
    }
    free(weight);
    free(under);
    free(over);
}

static float luminance709(const float rgb[3]) { return 0.2126f * rgb[0] + 0.7152f * rgb[1] + 0.0722f * rgb[2]; }

/* materialEmissionWeight (lighting.c:55-60) */
static float emission_weight(const VKRT_CudaMaterial* m) {
    if (!isfinite(m->emissionLuminance) || m->emissionLuminance <= 0.0f) return 0.0f;
    float lum = luminance709(m->emissionColor);
    if (lum <= 0.0f) return 0.0f;
    return lum * m->emissionLuminance;
}

/* materialEligibleForDirectLightSampling (lighting.c:62-67) */
static int light_eligible(const VKRT_CudaMeshInfo* mi, const VKRT_CudaMaterial* m) {
    if (mi->opacity < 0.999f || m->opacity < 0.999f) return 0;
    if (m->emissiveTextureIndex != VKRT_CUDA_INVALID_INDEX) return 0;
    return m->alphaMode == VKRT_CUDA_ALPHA_MODE_OPAQUE;
}

/* world position = 3x4 part of the column-major matrix applied to p, row by row (transformPosition,
 * lighting.c:69-76) */
static void world_position(const float m[16], const float p[4], float out[3]) {
    for (int r = 0; r < 3; ++r) out[r] = (m[0 * 4 + r] * p[0]) + (m[1 * 4 + r] * p[1]) + (m[2 * 4 + r] * p[2]) + m[3 * 4 + r];
}

int32_t vkrt_host_build_light_tables(VKRT_CudaMeshInfo* meshInfos, uint32_t meshCount,
                                     const VKRT_CudaMaterial* materials, uint32_t materialCount,
                                     const VKRT_CudaVertex* vertices, const uint32_t* indices,
                                     VKRT_CudaEmissiveMesh* outMeshes, uint32_t meshCapacity,
                                     VKRT_CudaEmissiveTriangle* outTriangles, uint32_t triangleCapacity,
                                     float* outMeshAliasQ, uint32_t* outMeshAliasIdx, float* outTriAliasQ,
                                     uint32_t* outTriAliasIdx, uint32_t* outEmissiveMeshCount,
                                     uint32_t* outEmissiveTriangleCount) {
    if (!meshInfos || !materials || !vertices || !indices || !outEmissiveMeshCount || !outEmissiveTriangleCount)
        return -1;
    uint32_t nMeshes = 0, nTris = 0;
    float totalSelection = 0.0f;
    float* meshWeight = (float*)malloc(sizeof(float) * (meshCount ? meshCount : 1u));
    uint32_t* sourceMesh = (uint32_t*)malloc(sizeof(uint32_t) * (meshCount ? meshCount : 1u));
    float* pmfScratch = (float*)malloc(sizeof(float) * (triangleCapacity > meshCount ? triangleCapacity : meshCount) + 4);
    if (!meshWeight || !sourceMesh || !pmfScratch) {
        free(meshWeight);
        free(sourceMesh);
        free(pmfScratch);
        return -2;
    }
    for (uint32_t i = 0; i < meshCount; ++i) meshInfos[i].lightPdfArea = 0.0f;

    for (uint32_t mi = 0; mi < meshCount; ++mi) {
        VKRT_CudaMeshInfo* info = &meshInfos[mi];
        if (info->materialIndex >= materialCount) continue;
        const VKRT_CudaMaterial* mat = &materials[info->materialIndex];
        if (!light_eligible(info, mat)) continue;
        float ew = emission_weight(mat);
        if (ew <= 0.0f) continue;
        uint32_t triCount = info->indexCount / 3u;
        if (triCount == 0u) continue;
        if (nMeshes >= meshCapacity) {
            free(meshWeight);
            free(sourceMesh);
            free(pmfScratch);
            return -2;
        }
        float world[16];
        vkrt_host_mesh_transform(info->position, info->rotation, info->scale, world);
        uint32_t first = nTris;
        float area = 0.0f;
        for (uint32_t t = 0; t < triCount; ++t) {
            const uint32_t* tri = &indices[info->indexBase + 3u * t];
            if (tri[0] >= info->vertexCount || tri[1] >= info->vertexCount || tri[2] >= info->vertexCount) continue;
            if (nTris >= triangleCapacity) {
                free(meshWeight);
                free(sourceMesh);
                free(pmfScratch);
                return -2;
            }
            float p0[3], p1[3], p2[3];
            world_position(world, vertices[info->vertexBase + tri[0]].position, p0);
            world_position(world, vertices[info->vertexBase + tri[1]].position, p1);
            world_position(world, vertices[info->vertexBase + tri[2]].position, p2);
            float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
            float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
            float cx = e1[1] * e2[2] - e1[2] * e2[1];
            float cy = e1[2] * e2[0] - e1[0] * e2[2];
            float cz = e1[0] * e2[1] - e1[1] * e2[0];
            float a = 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
            if (a <= 0.0f) continue;
            VKRT_CudaEmissiveTriangle* et = &outTriangles[nTris++];
            memset(et, 0, sizeof(*et));
            for (int k = 0; k < 3; ++k) {
                et->v0Area[k] = p0[k];
                et->e1Pad[k] = e1[k];
                et->e2Pad[k] = e2[k];
            }
            et->v0Area[3] = a;
            area += a;
        }
        uint32_t valid = nTris - first;
        float selection = area * ew;
        if (selection <= 0.0f || valid == 0u) {
            nTris = first;
            continue;
        }
        float invArea = 1.0f / area;
        for (uint32_t t = 0; t < valid; ++t) pmfScratch[t] = outTriangles[first + t].v0Area[3] * invArea;
        vkrt_host_build_alias_table(pmfScratch, valid, &outTriAliasQ[first], &outTriAliasIdx[first]);
        VKRT_CudaEmissiveMesh* em = &outMeshes[nMeshes];
        memset(em, 0, sizeof(*em));
        em->triOffset = first;
        em->triCount = valid;
        em->invTotalArea = invArea;
        for (int k = 0; k < 3; ++k) em->emission[k] = mat->emissionColor[k] * mat->emissionLuminance;
        meshWeight[nMeshes] = selection;
        sourceMesh[nMeshes] = mi;
        totalSelection += selection;
        ++nMeshes;
    }
    if (nMeshes > 0u && totalSelection > 0.0f) {
        float inv = 1.0f / totalSelection;
        for (uint32_t i = 0; i < nMeshes; ++i) {
            float pmf = meshWeight[i] * inv;
            outMeshes[i].pmfMesh = pmf;
            pmfScratch[i] = pmf;
            meshInfos[sourceMesh[i]].lightPdfArea = pmf * outMeshes[i].invTotalArea;
        }
        vkrt_host_build_alias_table(pmfScratch, nMeshes, outMeshAliasQ, outMeshAliasIdx);
    }
    *outEmissiveMeshCount = nMeshes;
    *outEmissiveTriangleCount = nTris;
    free(meshWeight);
    free(sourceMesh);
    free(pmfScratch);
    return 0;
}

/* ---- auto-SPP: VKRT_setAutoSPPTargetFPS (src/core/api/settings.c:68-79), updateAutoSPP (scene/timing.c:121-178) */

void vkrt_host_auto_spp_init(VKRT_CudaAutoSpp* state, uint32_t targetFPS) {
    if (!state) return;
    uint32_t fps = targetFPS ? targetFPS : 60u;
    if (fps < 30u) fps = 30u;
    if (fps > 360u) fps = 360u;
    state->targetFrameMs = 1000.0f / (float)fps;
    state->controlMs = 0.0f;
}

int32_t vkrt_host_auto_spp_update(VKRT_CudaAutoSpp* state, float renderMs, uint32_t* samplesPerPixel) {
    /* exponential smoothing of the cost per sample, a 90% budget, asymmetric deadbands and step limits */
    const float smoothing = 0.35f, budget = 0.90f;
    const float upBand = 0.18f, downBand = 0.08f, upStep = 1.25f, downStep = 0.60f;
    const uint32_t maxSpp = 2048u;
    if (!state || !samplesPerPixel) return -1;
    if (!(state->targetFrameMs > 0.0f) || !(renderMs > 0.0f)) return 0;
    const uint32_t spp = *samplesPerPixel ? *samplesPerPixel : 1u;
    const float sppf = (float)spp;
    const float perSample = renderMs / sppf;
    if (!(perSample > 0.0f)) return 0;
    state->controlMs = state->controlMs <= 0.0f ? perSample
                                                : state->controlMs * (1.0f - smoothing) + perSample * smoothing;
    float desired = state->targetFrameMs * budget / state->controlMs;
    desired = desired < 1.0f ? 1.0f : (desired > (float)maxSpp ? (float)maxSpp : desired);
    const float delta = desired - sppf;
    const float band = fmaxf(sppf * (delta > 0.0f ? upBand : downBand), 1.0f);
    if (fabsf(delta) <= band) return 0;
    uint32_t next;
    if (delta > 0.0f) {
        next = (uint32_t)floorf(fminf(desired, ceilf(sppf * upStep)));
        if (next <= spp && spp < maxSpp) next = spp + 1u;
    } else {
        next = (uint32_t)ceilf(fmaxf(desired, floorf(sppf * downStep)));
        if (next >= spp && spp > 1u) next = spp - 1u;
    }
    next = next < 1u ? 1u : (next > maxSpp ? maxSpp : next);
    if (next == spp) return 0;
    *samplesPerPixel = next;
    return 1;
}

/* ---- PNG scanline filters (PNG specification, section 9) ----------------------------------------------------- */

static uint8_t paeth_predictor(int a, int b, int c) {
    int p = a + b - c;
    int pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    return (uint8_t)(pb <= pc ? b : c);
}

int32_t vkrt_host_png_unfilter(const uint8_t* src, uint32_t height, uint64_t rowBytes, uint32_t bytesPerPixel,
                               uint8_t* dst) {
    if ((!src || !dst) && height > 0u) return -1;
    if (bytesPerPixel == 0u) return -1;
    const size_t n = (size_t)rowBytes, bpp = bytesPerPixel;
    for (uint32_t y = 0; y < height; ++y) {
        const uint8_t* in = src + (size_t)y * (n + 1u);
        uint8_t* out = dst + (size_t)y * n;
        const uint8_t* up = y > 0u ? out - n : NULL; /* the previous reconstructed row; zeros above the first */
        const uint8_t type = in[0];
        ++in;
        switch (type) {
            case 0:
                memcpy(out, in, n);
                break;
            case 1:
                for (size_t i = 0; i < n; ++i) out[i] = (uint8_t)(in[i] + (i >= bpp ? out[i - bpp] : 0));
                break;
            case 2:
                for (size_t i = 0; i < n; ++i) out[i] = (uint8_t)(in[i] + (up ? up[i] : 0));
                break;
            case 3:
                for (size_t i = 0; i < n; ++i) {
                    int a = i >= bpp ? out[i - bpp] : 0, b = up ? up[i] : 0;
                    out[i] = (uint8_t)(in[i] + ((a + b) >> 1));
                }
                break;
            case 4:
                for (size_t i = 0; i < n; ++i) {
                    int a = i >= bpp ? out[i - bpp] : 0, b = up ? up[i] : 0, c = (i >= bpp && up) ? up[i - bpp] : 0;
                    out[i] = (uint8_t)(in[i] + paeth_predictor(a, b, c));
                }
                break;
            default:
                return -1;
        }
    }
    return 0;
}
