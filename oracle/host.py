"""TEST INFRASTRUCTURE ONLY. A numpy restatement of vkrt's host scene layer, independent of the backend's own host
library: the CPU reference arm of the benchmark builds its scenes with it, so that run loads no product code, and the
CPU tests check it against the vectors vkrt's own packing.c and cglm produced (tests/golden) and against the
backend's host library.

* default_material       VKRT_materialDefault (src/core/api/vkrt_types.h:79-121)
* default_scene_data     initializeDefaultSceneSettings + writeSceneStateUniform (src/core/scene/uniform.c:93-174)
* camera_matrices        syncCameraMatrices (src/core/scene/camera.c:128-143): glm_lookat, glm_perspective with the
                         Vulkan Y flip, glm_mat4_inv of both; computed in FP64 and rounded to FP32
* mesh_transform         VKRT_buildMeshTransformMatrix (src/core/scene/transform.c:26-35): T * Rz * Ry * Rx * S, FP64
* pack_vertices          packShaderVertex (src/core/utility/packing.c:92-156), FP32 as written, bit-exact
* build_light_tables     populateEmissiveLightScratch / appendEmissiveMesh / appendMeshEmissiveTriangles /
                         finalizeMeshSelectionWeights / buildAliasTable (src/core/scene/lighting.c:55-164,267-433)
"""
from __future__ import annotations

import math

import numpy as np

F32 = np.float32
INVALID = 0xFFFFFFFF


def _abi():
    # record layouts only (numpy dtypes); importing the module loads no library
    from vkrt_gb300 import abi
    return abi


def default_material() -> np.ndarray:
    abi = _abi()
    m = np.zeros(1, dtype=abi.MATERIAL)
    m["baseColor"] = (0.8, 0.8, 0.8)
    m["roughness"] = 0.5
    m["emissionColor"] = (1.0, 1.0, 1.0)
    m["specular"] = 0.5
    m["sheenTintWeight"] = (1.0, 1.0, 1.0, 0.0)
    m["clearcoatGloss"] = 1.0
    m["ior"] = 1.5
    m["sheenRoughness"] = 0.5
    m["attenuationColor"] = (1.0, 1.0, 1.0)
    m["normalTextureScale"] = 1.0
    for k in ("baseColorTextureIndex", "metallicRoughnessTextureIndex", "normalTextureIndex",
              "emissiveTextureIndex"):
        m[k] = INVALID
    m["opacity"] = 1.0
    m["alphaCutoff"] = 0.5
    m["alphaMode"] = 0  # VKRT_MATERIAL_ALPHA_MODE_OPAQUE
    for k in ("baseColorTextureTransform", "metallicRoughnessTextureTransform", "normalTextureTransform",
              "emissiveTextureTransform"):
        m[k] = (1.0, 1.0, 0.0, 0.0)
    return m


def default_scene_data(width: int, height: int) -> np.ndarray:
    abi = _abi()
    sd = np.zeros(1, dtype=abi.SCENE_DATA)
    sd["samplesPerPixel"] = 8
    sd["rrMaxDepth"] = 8
    sd["rrMinDepth"] = 4
    sd["viewportRect"] = (0, 0, width, height)
    sd["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES, abi.RENDER_MODE_RGB,
                                                          abi.SPECTRAL_HERO)
    sd["exposure"] = 1.0
    sd["timeBase"] = -1.0
    sd["timeStep"] = 0.5
    sd["environmentLight"] = (0.25, 0.25, 0.25, 1.0)  # colour x strength, strength
    sd["environmentTextureIndex"] = INVALID
    sd["environmentRotation"] = 0.0
    sd["debugMode"] = 0
    sd["misNeeEnabled"] = 1
    sd["selectionEnabled"] = 0
    sd["selectedMeshIndex"] = INVALID
    camera_matrices(sd, (-0.5, 0.2, -0.2), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 40.0)
    return sd


def camera_matrices(sd: np.ndarray, pos, target, up=(0.0, 0.0, 1.0), vfov: float = 40.0, near: float = 0.001,
                    far: float = 10000.0) -> None:
    """Writes viewInverse and projInverse (column-major, as cglm stores mat4) into SceneData `sd`."""
    p = np.asarray(pos, np.float64)
    f = np.asarray(target, np.float64) - p
    f /= np.linalg.norm(f)
    s = np.cross(f, np.asarray(up, np.float64))
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.eye(4)  # row-major here; transposed into cglm's column-major layout below
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[0, 3], view[1, 3], view[2, 3] = -s @ p, -u @ p, f @ p
    w = max(int(sd["viewportRect"][0][2]), 1)
    h = max(int(sd["viewportRect"][0][3]), 1)
    fy = 1.0 / math.tan(math.radians(vfov) * 0.5)
    proj = np.zeros((4, 4))
    proj[0, 0] = fy / (w / h)
    proj[1, 1] = -fy  # Vulkan Y flip (camera.c:140)
    proj[2, 2] = (near + far) / (near - far)
    proj[3, 2] = -1.0
    proj[2, 3] = 2.0 * near * far / (near - far)
    sd["viewInverse"] = np.linalg.inv(view).T.astype(F32)
    sd["projInverse"] = np.linalg.inv(proj).T.astype(F32)


def mesh_transform(position, rotation_deg, scale) -> np.ndarray:
    """Row-major 4x4 world matrix T * Rz * Ry * Rx * S (FP64)."""
    def rot(axis, deg):
        c, s = math.cos(math.radians(deg)), math.sin(math.radians(deg))
        i, j = (axis + 1) % 3, (axis + 2) % 3
        r = np.eye(4)
        r[i, i] = r[j, j] = c
        r[j, i], r[i, j] = s, -s
        return r
    t = np.eye(4)
    t[:3, 3] = np.asarray(position, np.float64)
    sc = np.diag(list(np.asarray(scale, np.float64)) + [1.0])
    rx, ry, rz = (float(v) for v in rotation_deg)
    return t @ rot(2, rz) @ rot(1, ry) @ rot(0, rx) @ sc


def _lround(x: np.ndarray) -> np.ndarray:
    """lroundf of FP32 values: halves away from zero, exact (the FP32 value is widened before rounding)."""
    x = x.astype(np.float64)
    return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)


def _octahedral(v: np.ndarray):
    """normalize3f + the octahedral projection of packOctNormal32 / packTangent32, in FP32 as written."""
    x, y, z = (v[:, k].astype(F32) for k in range(3))
    len2 = (x * x + y * y) + z * z
    small = len2 <= F32(1e-20)
    inv = F32(1.0) / np.sqrt(np.where(small, F32(1.0), len2))
    nx, ny, nz = np.where(small, F32(0), x * inv), np.where(small, F32(0), y * inv), np.where(small, F32(1), z * inv)
    l1 = F32(1.0) / ((np.abs(nx) + np.abs(ny)) + np.abs(nz))
    px, py = nx * l1, ny * l1
    fold = nz < F32(0)
    fx = (F32(1) - np.abs(py)) * np.where(px >= F32(0), F32(1), F32(-1))
    fy = (F32(1) - np.abs(px)) * np.where(py >= F32(0), F32(1), F32(-1))
    return np.where(fold, fx, px).astype(F32), np.where(fold, fy, py).astype(F32)


def pack_vertices(vertices: np.ndarray) -> np.ndarray:
    abi = _abi()
    v = np.ascontiguousarray(vertices, dtype=abi.VERTEX)
    out = np.zeros(len(v), dtype=abi.SHADER_VERTEX)
    out["position"] = v["position"]
    out["texcoord0"] = v["texcoord0"]
    out["texcoord1"] = v["texcoord1"]
    ox, oy = _octahedral(v["normal"][:, :3])
    qx = _lround(np.clip(ox, F32(-1), F32(1)) * F32(32767.0)) & 0xFFFF
    qy = _lround(np.clip(oy, F32(-1), F32(1)) * F32(32767.0)) & 0xFFFF
    out["packedNormal"] = (qx | (qy << 16)).astype(np.uint32)
    tx, ty = _octahedral(v["tangent"][:, :3])
    sx = _lround(np.clip(tx, F32(-1), F32(1)) * F32(16383.0)) & 0x7FFF
    sy = _lround(np.clip(ty, F32(-1), F32(1)) * F32(16383.0)) & 0x7FFF
    out["packedTangent"] = (sx | (sy << 15) | np.where(v["tangent"][:, 3] < 0, 0x80000000, 0)).astype(np.uint32)
    c = _lround(np.clip(v["color"].astype(F32), F32(0), F32(1)) * F32(255.0))
    out["packedColor"] = (c[:, 0] | (c[:, 1] << 8) | (c[:, 2] << 16) | (c[:, 3] << 24)).astype(np.uint32)
    return out


def build_alias_table(pmf: np.ndarray):
    """buildAliasTable: Vose's method with LIFO small / large work lists in vkrt's pairing order, FP32."""
    n = len(pmf)
    q = np.zeros(n, F32)
    idx = np.zeros(n, np.uint32)
    scaled = [F32(p) * F32(n) for p in pmf]
    small = [i for i in range(n) if scaled[i] < F32(1)]
    large = [i for i in range(n) if not scaled[i] < F32(1)]
    while small and large:
        s, l = small.pop(), large.pop()
        q[s], idx[s] = scaled[s], l
        scaled[l] = F32(F32(scaled[l] + scaled[s]) - F32(1))
        (small if scaled[l] < F32(1) else large).append(l)
    for i in large + small:
        q[i], idx[i] = F32(1), i
    return q, idx


def build_light_tables(scene) -> None:
    """Emissive meshes and triangles, their alias tables and MeshInfo.lightPdfArea, as vkrt's lighting.c builds
    them; fills the scene's light fields and SceneData counts."""
    abi = _abi()
    meshes, mats = scene.meshes, scene.materials
    meshes["lightPdfArea"] = 0.0
    em, et, weights, sources, tq_all, ti_all = [], [], [], [], [], []
    for mi in range(len(meshes)):
        info = meshes[mi]
        if info["materialIndex"] >= len(mats):
            continue
        m = mats[info["materialIndex"]]
        # materialEligibleForDirectLightSampling
        if info["opacity"] < F32(0.999) or m["opacity"] < F32(0.999) or m["emissiveTextureIndex"] != INVALID:
            continue
        if m["alphaMode"] != 0:
            continue
        # materialEmissionWeight
        lum_e = F32(m["emissionLuminance"])
        if not np.isfinite(lum_e) or lum_e <= 0:
            continue
        ec = m["emissionColor"].astype(F32)
        lum = F32(F32(F32(0.2126) * ec[0]) + F32(F32(0.7152) * ec[1])) + F32(F32(0.0722) * ec[2])
        if lum <= 0:
            continue
        ew = F32(lum * lum_e)
        n_tri = int(info["indexCount"]) // 3
        if n_tri == 0:
            continue
        world = mesh_transform(info["position"], info["rotation"], info["scale"]).astype(F32)
        ib, vb, vc = int(info["indexBase"]), int(info["vertexBase"]), int(info["vertexCount"])
        tris, area = [], F32(0)
        for t in range(n_tri):
            i3 = scene.indices[ib + 3 * t: ib + 3 * t + 3]
            if (i3 >= vc).any():
                continue
            ps = []
            for k in range(3):
                p = scene.vertices[vb + int(i3[k])]["position"].astype(F32)
                # transformPosition: rows of the 3x4 world matrix, summed left to right
                ps.append(np.array([F32(F32(F32(F32(world[r, 0] * p[0]) + F32(world[r, 1] * p[1]))
                                            + F32(world[r, 2] * p[2])) + world[r, 3]) for r in range(3)], F32))
            e1, e2 = ps[1] - ps[0], ps[2] - ps[0]
            cr = np.array([F32(e1[1] * e2[2]) - F32(e1[2] * e2[1]), F32(e1[2] * e2[0]) - F32(e1[0] * e2[2]),
                           F32(e1[0] * e2[1]) - F32(e1[1] * e2[0])], F32)
            a = F32(F32(0.5) * np.sqrt(F32(F32(F32(cr[0] * cr[0]) + F32(cr[1] * cr[1])) + F32(cr[2] * cr[2]))))
            if a <= 0:
                continue
            tris.append((ps[0], e1, e2, a))
            area = F32(area + a)
        selection = F32(area * ew)
        if selection <= 0 or not tris:
            continue
        inv_area = F32(F32(1) / area)
        q, idx = build_alias_table(np.array([F32(t[3] * inv_area) for t in tris], F32))
        first = len(et)
        for (v0, e1, e2, a) in tris:
            r = np.zeros(1, abi.EMISSIVE_TRIANGLE)
            r["v0Area"] = (v0[0], v0[1], v0[2], a)
            r["e1Pad"][0, :3] = e1
            r["e2Pad"][0, :3] = e2
            et.append(r)
        tq_all.append(q)
        ti_all.append(idx)
        rec = np.zeros(1, abi.EMISSIVE_MESH)
        rec["triOffset"], rec["triCount"], rec["invTotalArea"] = first, len(tris), inv_area
        rec["emission"][0, :3] = ec * lum_e
        em.append(rec)
        weights.append(selection)
        sources.append(mi)
    total = F32(0)
    for w in weights:
        total = F32(total + w)
    mesh_q = mesh_i = None
    if em:
        inv_total = F32(F32(1) / total)
        pmf = np.array([F32(w * inv_total) for w in weights], F32)
        for k, (rec, src) in enumerate(zip(em, sources)):
            rec["pmfMesh"] = pmf[k]
            meshes[src]["lightPdfArea"] = F32(pmf[k] * rec["invTotalArea"][0])
        mesh_q, mesh_i = build_alias_table(pmf)
    scene.emissive_meshes = np.concatenate(em) if em else np.zeros(0, abi.EMISSIVE_MESH)
    scene.emissive_triangles = np.concatenate(et) if et else np.zeros(0, abi.EMISSIVE_TRIANGLE)
    scene.mesh_alias_q = mesh_q if mesh_q is not None else np.zeros(0, F32)
    scene.mesh_alias_idx = mesh_i if mesh_i is not None else np.zeros(0, np.uint32)
    scene.tri_alias_q = np.concatenate(tq_all) if tq_all else np.zeros(0, F32)
    scene.tri_alias_idx = np.concatenate(ti_all) if ti_all else np.zeros(0, np.uint32)
    scene.emissive_mesh_materials = np.ascontiguousarray(meshes["materialIndex"][sources], dtype=np.uint32)
    scene.scene_data["emissiveMeshCount"] = len(em)
    scene.scene_data["emissiveTriangleCount"] = len(et)


class OracleHost:
    """The host-layer interface vkrt_gb300.scenes builds scenes through, backed by this restatement."""
    default_material = staticmethod(default_material)
    default_scene_data = staticmethod(default_scene_data)
    pack_vertices = staticmethod(pack_vertices)
    build_light_tables = staticmethod(build_light_tables)

    @staticmethod
    def camera_matrices(sd, pos, target, up, vfov):
        camera_matrices(sd, pos, target, up, vfov)
