/* ref_driver.c — TEST INFRASTRUCTURE ONLY. Linked with vkrt's own src/core/utility/packing.c (compiled from the
 * vkrt checkout by oracle/build.py) and vkrt's vendored header-only cglm, it exposes vkrt's packing and the cglm
 * matrix calls vkrt uses for the camera (src/core/scene/camera.c:128-143) and mesh transforms
 * (src/core/scene/transform.c:26-35) to the tests, which compare them with the backend's host library. */
#include <stdint.h>
#include <string.h>

#include "cglm.h"
#include "packing.h"
#include "types.h"

int32_t ref_sizeof(const char* name) {
    if (!strcmp(name, "Vertex")) return (int32_t)sizeof(Vertex);
    if (!strcmp(name, "ShaderVertex")) return (int32_t)sizeof(ShaderVertex);
    if (!strcmp(name, "MeshInfo")) return (int32_t)sizeof(MeshInfo);
    if (!strcmp(name, "Material")) return (int32_t)sizeof(Material);
    if (!strcmp(name, "EmissiveMesh")) return (int32_t)sizeof(EmissiveMesh);
    if (!strcmp(name, "EmissiveTriangle")) return (int32_t)sizeof(EmissiveTriangle);
    if (!strcmp(name, "SceneData")) return (int32_t)sizeof(SceneData);
    return -1;
}

void ref_pack_vertices(const Vertex* in, uint32_t count, ShaderVertex* out) {
    for (uint32_t i = 0; i < count; ++i) out[i] = packShaderVertex(&in[i]);
}

/* view/proj inverses exactly as syncCameraMatrices computes them */
void ref_camera_matrices(const float pos[3], const float target[3], const float up[3], float vfov, float nearZ,
                         float farZ, uint32_t w, uint32_t h, float viewInverse[16], float projInverse[16]) {
    mat4 view, proj, vi, pi;
    vec3 p = {pos[0], pos[1], pos[2]}, t = {target[0], target[1], target[2]}, u = {up[0], up[1], up[2]};
    glm_lookat(p, t, u, view);
    glm_perspective(glm_rad(vfov), (float)(w ? w : 1u) / (float)(h ? h : 1u), nearZ, farZ, proj);
    proj[1][1] *= -1.0f;
    glm_mat4_inv(view, vi);
    glm_mat4_inv(proj, pi);
    memcpy(viewInverse, vi, sizeof(vi));
    memcpy(projInverse, pi, sizeof(pi));
}

/* T * Rz * Ry * Rx * S as VKRT_buildMeshTransformMatrix builds it */
void ref_mesh_transform(const float position[3], const float rotationDegrees[3], const float scale[3], float out[16]) {
    mat4 m;
    glm_mat4_identity(m);
    glm_translate(m, (vec3){position[0], position[1], position[2]});
    glm_rotate(m, glm_rad(rotationDegrees[2]), (vec3){0.0f, 0.0f, 1.0f});
    glm_rotate(m, glm_rad(rotationDegrees[1]), (vec3){0.0f, 1.0f, 0.0f});
    glm_rotate(m, glm_rad(rotationDegrees[0]), (vec3){1.0f, 0.0f, 0.0f});
    glm_scale(m, (vec3){scale[0], scale[1], scale[2]});
    memcpy(out, m, sizeof(m));
}
