"""vkrt scene files ("format": "vkrt.scene", version 1) into a Scene, following vkrt's loader
(src/app/scene/controller.c:1528-1595 and the steps it calls):

* meshImports (controller.c:1241-1271): each glTF file, resolved against the scene file's folder, is imported with
  vkrt_gb300.gltf; its mesh entries are appended in order, its materials after vkrt's default material 0, its
  textures after the scene's textures so far, its materials' texture indices moved with them
  (mesh/controller.c:159-181, 394-412);
* textureImports (controller.c:1274-1300): each standalone image is loaded in its saved colour space and appended;
  saved materials name textures by their saved index, which is remapped to the new one (controller.c:640-661);
  images of a format this package does not decode (JPEG, EXR) are left out and noted, where vkrt decodes them;
* meshes (controller.c:1314-1455): each saved mesh names (importIndex, importLocalIndex); meshes no saved mesh names are
  dropped, the rest keep their import order; name, material (hasMaterialAssignment ? materialIndex : 0), backface
  rendering and opacity are applied;
* materials (controller.c:585-634, 1375-1408): each entry overwrites vkrt's default material with the fields it gives,
  at its explicit index (else the next contiguous one); the material list grows to the highest index used;
* sceneObjects (controller.c:737-765, 1457-1526; session.c:257-300): local TRS (Euler XYZ degrees) or a localTransform
  matrix, parents listed before children; a mesh's world matrix is the product down its parent chain, decomposed
  into MeshInfo position / rotation / scale as vkrt does (core/scene/transform.c:158-209); meshes without a scene
  object keep their glTF node transform;
* sceneSettings (controller.c:823-890, core/scene/uniform.c:153-174): camera pose and vertical field of view, Russian
  roulette depths, tone mapping / render / spectral sampling modes, exposure, environment colour x strength and
  rotation, MIS/NEE switch.

`missing="skip"` drops imports whose file is absent (and the saved meshes and objects that use them) instead of
failing as vkrt does; the Scene's `notes` lists what was dropped or ignored.
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

from . import abi, gltf
from .context import Scene, build_light_tables

SCENE_FORMAT, SCENE_VERSION = "vkrt.scene", 1

_MATERIAL_FIELDS = {  # JSON field -> (MATERIAL field, components) (controller.c:589-631)
    "baseColor": 3, "roughness": 1, "emissionColor": 3, "emissionLuminance": 1, "eta": 3, "metallic": 1, "k": 3,
    "anisotropic": 1, "specular": 1, "specularTint": 1, "sheenTintWeight": 4, "clearcoat": 1, "clearcoatGloss": 1,
    "ior": 1, "abbeNumber": 1, "diffuseRoughness": 1, "transmission": 1, "subsurface": 1, "sheenRoughness": 1,
    "absorptionCoefficient": 1, "attenuationColor": 3, "normalTextureScale": 1, "baseColorTextureIndex": 1,
    "metallicRoughnessTextureIndex": 1, "normalTextureIndex": 1, "emissiveTextureIndex": 1, "baseColorTextureWrap": 1,
    "metallicRoughnessTextureWrap": 1, "normalTextureWrap": 1, "emissiveTextureWrap": 1, "opacity": 1,
    "alphaCutoff": 1, "alphaMode": 1, "textureTexcoordSets": 1, "baseColorTextureTransform": 4,
    "metallicRoughnessTextureTransform": 4, "normalTextureTransform": 4, "emissiveTextureTransform": 4,
    "textureRotations": 4,
}


class SceneFileError(ValueError):
    pass


# ---- transforms (core/scene/transform.c) --------------------------------------------------------------------------
def mesh_transform_matrix(position, rotation_deg, scale) -> np.ndarray:
    """T * Rz * Ry * Rx * S, column vectors (VKRT_buildMeshTransformMatrix, transform.c:26-35)."""
    rx, ry, rz = (math.radians(float(a)) for a in rotation_deg)
    cx, sx, cy, sy, cz, sz = math.cos(rx), math.sin(rx), math.cos(ry), math.sin(ry), math.cos(rz), math.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    m = np.eye(4)
    m[:3, :3] = Rz @ Ry @ Rx @ np.diag(np.asarray(scale, float))
    m[:3, 3] = position
    return m


def _euler_zyx_deg(r: np.ndarray):
    """Rotation matrix (column vectors) -> XYZ Euler degrees of Rz * Ry * Rx (transform.c:62-80)."""
    sy = -min(max(r[2, 0], -1.0), 1.0)
    y = math.asin(sy)
    if abs(math.cos(y)) > 1e-6:
        x = math.atan2(r[2, 1], r[2, 2])
        z = math.atan2(r[1, 0], r[0, 0])
    else:
        x = math.atan2(-r[1, 2], r[1, 1])
        z = 0.0
    return [math.degrees(x), math.degrees(y), math.degrees(z)]


def decompose_mesh_transform(world: np.ndarray):
    """(position, rotation degrees, scale) reproducing `world` through mesh_transform_matrix; a mirrored matrix tries
    a negative scale on each axis and keeps the best reconstruction (VKRT_decomposeMeshTransform, transform.c:158-209)."""
    pos = world[:3, 3].copy()
    rot = np.eye(3)
    scale = np.ones(3)
    for a in range(3):
        col = world[:3, a]
        s = float(np.linalg.norm(col))
        if s < 1e-6 or not math.isfinite(s):
            continue
        scale[a] = s
        rot[:, a] = col / s
    det = float(np.linalg.det(rot))
    best = None
    for flip in ([0, 1, 2] if det < 0 else [-1]):
        r, sc = rot.copy(), scale.copy()
        if flip >= 0:
            r[:, flip] *= -1
            sc[flip] *= -1
        e = _euler_zyx_deg(r)
        err = float(np.abs(mesh_transform_matrix(pos, e, sc)[:3] - world[:3]).max())
        if best is None or err < best[0]:
            best = (err, e, sc)
    return pos, np.array(best[1]), best[2]


# ---- loading ------------------------------------------------------------------------------------------------------
def _floats(v, n, what):
    a = np.asarray(v, dtype=np.float64).reshape(-1)
    if a.size != n or not np.all(np.isfinite(a)):
        raise SceneFileError(f"{what}: expected {n} finite numbers")
    return a


def _index_or_invalid(v):
    return abi.INVALID_INDEX if v is None else int(v)


def parse_material(obj, base: np.ndarray) -> np.ndarray:
    if not isinstance(obj, dict):
        raise SceneFileError("material must be an object")
    m = base.copy()
    for key, n in _MATERIAL_FIELDS.items():
        if key not in obj:
            continue
        v = obj[key]
        m[key] = _floats(v, n, key) if n > 1 else (float(v) if m.dtype[key].kind == "f" else int(v))
    return m


def scene_data_from_settings(settings, width: int, height: int) -> np.ndarray:
    sd = np.zeros(1, dtype=abi.SCENE_DATA)
    lib = abi.load()
    lib.vkrt_host_default_scene_data(width, height, abi.ptr(sd))
    cam = settings.get("camera")
    if not isinstance(cam, dict):
        raise SceneFileError("sceneSettings.camera is required")
    pos = _floats(cam.get("position", [-0.5, 0.2, -0.2]), 3, "camera.position").astype(np.float32)
    tgt = _floats(cam.get("target", [0.0, 0.0, 0.0]), 3, "camera.target").astype(np.float32)
    up = _floats(cam.get("up", [0.0, 0.0, 1.0]), 3, "camera.up").astype(np.float32)
    vfov = float(cam.get("vfov", 40.0))
    if not (0.0 < vfov < 179.0):
        raise SceneFileError("camera.vfov must be in (0, 179) degrees")
    lib.vkrt_host_camera_matrices(abi.ptr(pos), abi.ptr(tgt), abi.ptr(up), vfov, 0.001, 10000.0, width, height,
                                  abi.ptr(sd))
    sd["rrMinDepth"] = int(settings.get("rrMinDepth", sd["rrMinDepth"][0]))
    sd["rrMaxDepth"] = int(settings.get("rrMaxDepth", sd["rrMaxDepth"][0]))
    packed = int(sd["packedRenderSettings"][0])
    tone = int(settings.get("toneMappingMode", abi.unpack_render_settings(packed)[0]))
    mode = int(settings.get("renderMode", abi.unpack_render_settings(packed)[1]))
    spectral = int(settings.get("spectralSamplingMode", abi.unpack_render_settings(packed)[2]))
    sd["packedRenderSettings"] = abi.pack_render_settings(tone, mode, spectral)
    sd["exposure"] = float(settings.get("exposure", 1.0))
    color = np.maximum(_floats(settings.get("environmentColor", [0.25, 0.25, 0.25]), 3, "environmentColor"), 0.0)
    strength = max(float(settings.get("environmentStrength", 1.0)), 0.0)
    sd["environmentLight"] = [*(color * strength), strength]
    sd["environmentRotation"] = float(settings.get("environmentRotation", 0.0))
    sd["misNeeEnabled"] = 1 if settings.get("misNeeEnabled", True) else 0
    return sd


def load_scene_file(path, width: int = 1280, height: int = 720, missing: str = "error") -> Scene:
    path = Path(path)
    doc = json.loads(path.read_text())
    if (doc.get("format") != SCENE_FORMAT or doc.get("version") != SCENE_VERSION
            or not isinstance(doc.get("meshImports"), list) or not isinstance(doc.get("meshes"), list)
            or not isinstance(doc.get("sceneObjects"), list) or not isinstance(doc.get("sceneSettings"), dict)):
        raise SceneFileError(f"{path}: not a {SCENE_FORMAT} version {SCENE_VERSION} document")
    from .image_decode import ImageDecodeError, UnsupportedImage, decode_image, texture_texels
    notes = []
    base = gltf.default_material()
    materials = [base.copy()]
    images = []   # decoded textures in scene order
    batches = []  # per import: (first loaded mesh, entries) or None when skipped
    loaded = []   # loaded mesh entries in import order: (entry, material index, node world)
    for k, rel in enumerate(doc["meshImports"]):
        f = (path.parent / rel).resolve()
        if not f.exists():
            if missing == "skip":
                notes.append(f"import {k} ({rel}) is missing: skipped")
                batches.append(None)
                continue
            raise SceneFileError(f"{path}: mesh import {rel} not found")
        imp = gltf.load_gltf(f)
        first_material = len(materials)
        first_texture = len(images)
        images.extend(imp.textures)
        for m in imp.materials:
            m = m.reshape(1).copy()
            for slot in ("baseColor", "metallicRoughness", "normal", "emissive"):
                t = int(m[slot + "TextureIndex"][0])
                if t != abi.INVALID_INDEX:
                    m[slot + "TextureIndex"] = first_texture + t if t < len(imp.textures) else abi.INVALID_INDEX
            materials.append(m)
        batches.append((len(loaded), len(imp.entries)))
        for e in imp.entries:
            mat = first_material + e.material if e.material != abi.INVALID_INDEX else 0
            loaded.append((e, mat, imp.node_world[e.node]))
        notes.extend(f"{rel}: {what} ignored" for what in sorted(imp.ignored))
    saved_texture = {}  # saved texture index -> scene texture index
    for k, to in enumerate(doc.get("textureImports") or []):
        if not isinstance(to, dict) or not isinstance(to.get("path"), str):
            raise SceneFileError(f"textureImports {k}: index, colorSpace and path are required")
        idx, cs = int(to["index"]), int(to["colorSpace"])
        f = (path.parent / to["path"]).resolve()
        if not f.exists():
            if missing == "skip":
                notes.append(f"texture {to['path']} is missing: skipped")
                continue
            raise SceneFileError(f"{path}: texture {to['path']} not found")
        try:
            images.append(decode_image(f.read_bytes(), None, cs))
            saved_texture[idx] = len(images) - 1
        except (UnsupportedImage, ImageDecodeError) as e:
            notes.append(f"texture {to['path']} left out ({e})")
    if doc.get("environmentTexturePath"):
        notes.append("environmentTexturePath ignored (HDR / EXR environment images are not decoded here)")

    # saved meshes -> loaded entries
    saved_to_loaded = []
    for k, mo in enumerate(doc["meshes"]):
        ii, li = int(mo["importIndex"]), int(mo["importLocalIndex"])
        if ii >= len(batches):
            raise SceneFileError(f"mesh {k}: import {ii} does not exist")
        if batches[ii] is None:
            saved_to_loaded.append(None)
            continue
        first, count = batches[ii]
        if li >= count:
            raise SceneFileError(f"mesh {k}: import {ii} has no mesh {li}")
        saved_to_loaded.append(first + li)
    keep = sorted({i for i in saved_to_loaded if i is not None})
    new_index = {old: new for new, old in enumerate(keep)}

    # materials: explicit or contiguous indices, list grown to the highest index any mesh or material names
    highest = max([int(mo.get("materialIndex", 0)) for mo in doc["meshes"]] + [0])
    for k, mo in enumerate(doc.get("materials") or []):
        highest = max(highest, int(mo.get("index", k)))
    while len(materials) <= highest:
        materials.append(base.copy())
    for k, mo in enumerate(doc.get("materials") or []):
        if not isinstance(mo.get("name"), str):
            raise SceneFileError(f"material {k}: name is required")
        m = parse_material(mo.get("material"), base)
        for slot in ("baseColor", "metallicRoughness", "normal", "emissive"):
            t = int(m[slot + "TextureIndex"][0])
            if t in saved_texture:
                m[slot + "TextureIndex"] = saved_texture[t]
        materials[int(mo.get("index", k))] = m
    materials = np.concatenate(materials)

    mesh_mat = {old: mat for old, (_, mat, _) in enumerate(loaded)}
    backfaces = {old: e.render_backfaces for old, (e, _, _) in enumerate(loaded)}
    opacity = {old: 1.0 for old in range(len(loaded))}
    names = {old: e.name for old, (e, _, _) in enumerate(loaded)}
    for k, mo in enumerate(doc["meshes"]):
        old = saved_to_loaded[k]
        if old is None:
            continue
        names[old] = str(mo.get("name", names[old]))
        mesh_mat[old] = int(mo["materialIndex"]) if mo.get("hasMaterialAssignment", False) else 0
        backfaces[old] = 1 if mo.get("renderBackfaces", False) else 0
        opacity[old] = float(mo.get("opacity", 1.0))
    world = {old: w for old, (_, _, w) in enumerate(loaded)}

    # scene objects: world matrices down the parent chain
    obj_world = []
    for k, so in enumerate(doc["sceneObjects"]):
        parent = _index_or_invalid(so.get("parentIndex"))
        if parent != abi.INVALID_INDEX and parent >= k:
            raise SceneFileError(f"sceneObject {k}: parent must come first")
        if "localPosition" in so or "localRotation" in so or "localScale" in so:
            local = mesh_transform_matrix(_floats(so["localPosition"], 3, "localPosition"),
                                          _floats(so["localRotation"], 3, "localRotation"),
                                          _floats(so["localScale"], 3, "localScale"))
        else:
            local = _floats(so["localTransform"], 16, "localTransform").reshape(4, 4).T
        w = local if parent == abi.INVALID_INDEX else obj_world[parent] @ local
        obj_world.append(w)
        mref = _index_or_invalid(so.get("meshIndex"))
        if mref == abi.INVALID_INDEX:
            continue
        if mref >= len(saved_to_loaded):
            raise SceneFileError(f"sceneObject {k}: mesh {mref} does not exist")
        if saved_to_loaded[mref] is not None:
            world[saved_to_loaded[mref]] = w

    verts, idxs = [], []
    meshes = np.zeros(len(keep), dtype=abi.MESH_INFO)
    vb = ib = 0
    for new, old in enumerate(keep):
        e = loaded[old][0]
        pos, rot, scl = decompose_mesh_transform(world[old])
        m = meshes[new]
        m["position"], m["rotation"], m["scale"] = pos, rot, scl
        m["vertexBase"], m["vertexCount"] = vb, len(e.vertices)
        m["indexBase"], m["indexCount"] = ib, len(e.indices)
        m["materialIndex"] = mesh_mat[old]
        m["renderBackfaces"] = backfaces[old]
        m["opacity"] = opacity[old]
        verts.append(e.vertices)
        idxs.append(e.indices.astype(np.uint32))
        vb += len(e.vertices)
        ib += len(e.indices)
    if not keep:
        raise SceneFileError(f"{path}: no meshes left to render")
    sd = scene_data_from_settings(doc["sceneSettings"], width, height)
    s = Scene(vertices=np.concatenate(verts), indices=np.concatenate(idxs), meshes=meshes, materials=materials,
              scene_data=sd, name=path.stem, mesh_names=[names[old] for old in keep], notes=notes,
              textures={i: texture_texels(img) for i, img in enumerate(images)})
    build_light_tables(s)
    return s
