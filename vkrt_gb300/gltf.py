"""glTF 2.0 import (.glb and .gltf with embedded or side-by-side buffers) into vkrt's authoring records, following
vkrt's importer (src/app/mesh/loader.c):

* node walk (loader.c:2027-2096): the default scene's roots (else every parentless node), depth first, children in
  order; one mesh entry per triangle primitive of each node with a mesh, in that order;
* vertices (loader.c:1757-1832): glTF's Y-up basis to vkrt's Z-up one, (x, y, z) -> (x, -z, y) for positions, normals
  and tangents; colour defaults to white, texture coordinates to 0;
* normals and tangents (loader.c:1871-1892): generated face-area-weighted normals when the primitive has none;
  otherwise triangles are rewound to agree with their vertex normals; imported tangents are orthonormalised,
  missing ones are built from the tangent texture coordinates, else a fallback frame;
* node transforms (loader.c:1557-1567, core/scene/transform.c:99-117): the local matrix M becomes B M B^-1 with B the
  +90 degree rotation about X;
* materials (loader.c:942-1078, 1472-1556): metallic-roughness or specular-glossiness factors, emission split into
  colour x luminance, KHR_materials_ior / specular / transmission / volume / clearcoat / sheen / emissive_strength
  factors, double-sided -> render backfaces, alpha modes.

* textures (loader.c:309-404, 702-736, 907-1011, 1472-1535): per material in order, the base colour (or
  specular-glossiness diffuse) texture read as sRGB, the metallic-roughness texture, the normal texture (linear) and
  the emissive texture (sRGB), each image decoded once per colour space and numbered in registration order; a texture
  on a texture-coordinate set above 1 is not bound; the sampler's wrap modes (repeat by default), the texture
  coordinate set, KHR_texture_transform scale / offset / rotation and the normal scale go into the material. Images
  come from files beside the glTF document or from buffer views (vkrt decodes no data-URI image); PNG is decoded
  (vkrt_gb300.image_decode), JPEG and EXR images are left unbound.

`GltfImport.ignored` lists what was skipped.
"""
from __future__ import annotations

import base64
import json
import math
import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import abi

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_WIDTH = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}
_NORM_SCALE = {np.int8: 127.0, np.uint8: 255.0, np.int16: 32767.0, np.uint16: 65535.0, np.uint32: 4294967295.0}
ALPHA_MODE_OPAQUE, ALPHA_MODE_MASK, ALPHA_MODE_BLEND = 0, 1, 2
ALPHA_BLEND_CUTOFF = 1.0 / 255.0  # loader.c:29


@dataclass
class MeshEntry:
    name: str
    vertices: np.ndarray          # abi.VERTEX, vkrt basis
    indices: np.ndarray           # uint32, entry-relative
    material: int                 # index into GltfImport.materials, or abi.INVALID_INDEX
    render_backfaces: int
    node: int                     # index into GltfImport.node_world


@dataclass
class GltfImport:
    entries: list
    materials: np.ndarray         # abi.MATERIAL, one per glTF material; texture indices into `textures`
    node_world: list              # per visited node: 4x4 world matrix (vkrt basis, column vectors)
    ignored: set = field(default_factory=set)
    textures: list = field(default_factory=list)  # image_decode.DecodedImage, in registration order


# ---- container ----------------------------------------------------------------------------------------------------
def _read_document(path: Path):
    data = path.read_bytes()
    if data[:4] == b"glTF":
        _, _, length = struct.unpack_from("<III", data, 0)
        off, doc, binchunk = 12, None, None
        while off + 8 <= length:
            clen, ctype = struct.unpack_from("<II", data, off)
            chunk = data[off + 8:off + 8 + clen]
            if ctype == 0x4E4F534A:
                doc = json.loads(chunk.decode("utf-8"))
            elif ctype == 0x004E4942:
                binchunk = chunk
            off += 8 + clen
        if doc is None:
            raise ValueError(f"{path}: GLB without a JSON chunk")
        return doc, binchunk
    return json.loads(data.decode("utf-8")), None


def _buffers(doc, binchunk, base: Path):
    out = []
    for i, b in enumerate(doc.get("buffers", [])):
        uri = b.get("uri")
        if uri is None:
            if binchunk is None:
                raise ValueError("buffer without uri and no GLB binary chunk")
            out.append(binchunk)
        elif uri.startswith("data:"):
            out.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            out.append((base / uri).read_bytes())
    return out


def _accessor(doc, buffers, index):
    """Accessor `index` as float64 (normalised integers mapped to [0, 1] / [-1, 1]) or integer array, (count, width)."""
    a = doc["accessors"][index]
    if "sparse" in a:
        raise ValueError("sparse accessors are not supported")
    dt = _COMPONENT[a["componentType"]]
    width = _WIDTH[a["type"]]
    count = a["count"]
    if "bufferView" not in a:
        arr = np.zeros((count, width), dtype=dt)
    else:
        bv = doc["bufferViews"][a["bufferView"]]
        buf = buffers[bv["buffer"]]
        start = bv.get("byteOffset", 0) + a.get("byteOffset", 0)
        item = np.dtype(dt).itemsize * width
        stride = bv.get("byteStride", 0) or item
        raw = np.frombuffer(buf, dtype=np.uint8, count=(count - 1) * stride + item if count else 0, offset=start)
        rows = np.lib.stride_tricks.as_strided(raw, shape=(count, item), strides=(stride, 1)) if count else raw
        arr = np.ascontiguousarray(rows).view(dt).reshape(count, width)
    if a.get("normalized", False) and dt in _NORM_SCALE:
        f = arr.astype(np.float64) / _NORM_SCALE[dt]
        return np.maximum(f, -1.0) if np.issubdtype(dt, np.signedinteger) else f
    return arr


# ---- transforms ---------------------------------------------------------------------------------------------------
def _quat_matrix(q):
    x, y, z, w = (float(v) for v in q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def node_local_matrix(node) -> np.ndarray:
    """4x4 local matrix of a glTF node (column vectors): `matrix`, else T * R * S."""
    if "matrix" in node:
        return np.array(node["matrix"], dtype=np.float64).reshape(4, 4).T
    m = np.eye(4)
    m[:3, :3] = _quat_matrix(node.get("rotation", [0, 0, 0, 1])) * np.array(node.get("scale", [1, 1, 1]), float)
    m[:3, 3] = node.get("translation", [0, 0, 0])
    return m


_BASIS = np.array([[1, 0, 0, 0], [0, 0, -1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.float64)  # Rx(+90 deg)


def to_vkrt_basis(m: np.ndarray) -> np.ndarray:
    return _BASIS @ m @ _BASIS.T


# ---- geometry -----------------------------------------------------------------------------------------------------
def _yup_to_zup(v):
    return np.stack([v[:, 0], -v[:, 2], v[:, 1]], axis=1)


def _normalise_rows(v, eps=1e-12):
    n2 = (v * v).sum(1)
    ok = n2 > eps
    out = v.copy()
    out[ok] /= np.sqrt(n2[ok])[:, None]
    return out, ok


def _fallback_tangents(normals):
    """loader.c:1418-1446: cross((0,0,1) or (1,0,0) when the normal is nearly +-Z, n), w = +1."""
    n = normals.astype(np.float32).copy()
    n2 = (n * n).sum(1)
    n[n2 <= 1e-12] = (0.0, 0.0, 1.0)
    n, _ = _normalise_rows(n)
    up = np.zeros_like(n)
    near_z = np.abs(n[:, 2]) > 0.999
    up[~near_z] = (0.0, 0.0, 1.0)
    up[near_z] = (1.0, 0.0, 0.0)
    t = np.cross(up, n)
    t, ok = _normalise_rows(t)
    t[~ok] = (1.0, 0.0, 0.0)
    return np.concatenate([t, np.ones((len(t), 1), np.float32)], 1)


def _orthonormal_tangents(normals, tangents, handedness):
    """loader.c:1386-1416; rows that degenerate get the fallback frame."""
    n, nok = _normalise_rows(normals.astype(np.float32))
    t = tangents[:, :3].astype(np.float32)
    tok = (t * t).sum(1) > 1e-12
    t = t - n * (t * n).sum(1, keepdims=True)
    t, pok = _normalise_rows(t)
    good = nok & tok & pok
    out = _fallback_tangents(normals)
    out[good, :3] = t[good]
    out[good, 3] = np.where(handedness[good] < 0, -1.0, 1.0)
    return out


def _generate_normals(pos, idx):
    """loader.c:1599-1644: sum of unnormalised face normals per vertex, normalised; zero -> +Z."""
    tri = idx.reshape(-1, 3)
    p = pos.astype(np.float32)
    fn = np.cross(p[tri[:, 1]] - p[tri[:, 0]], p[tri[:, 2]] - p[tri[:, 0]])
    keep = (fn * fn).sum(1) > 1e-12
    acc = np.zeros_like(p)
    for k in range(3):
        np.add.at(acc, tri[keep, k], fn[keep])
    out, ok = _normalise_rows(acc)
    out[~ok] = (0.0, 0.0, 1.0)
    return out


def _align_winding(pos, normals, idx):
    """loader.c:1343-1384, 1894-1907: swap the last two indices of triangles whose face normal opposes the sum of
    their vertex normals."""
    tri = idx.reshape(-1, 3).copy()
    p = pos.astype(np.float32)
    fn = np.cross(p[tri[:, 1]] - p[tri[:, 0]], p[tri[:, 2]] - p[tri[:, 0]])
    avg = normals[tri[:, 0]] + normals[tri[:, 1]] + normals[tri[:, 2]]
    valid = ((fn * fn).sum(1) > 1e-12) & ((avg * avg).sum(1) > 1e-12)
    flip = valid & ((fn * avg).sum(1) < 0)
    tri[flip, 1], tri[flip, 2] = tri[flip, 2].copy(), tri[flip, 1].copy()
    return tri.reshape(-1)


def _generate_tangents(pos, normals, idx, uv):
    """loader.c:1646-1740: per-triangle UV-gradient tangents summed per vertex, handedness from the bitangent sums."""
    tri = idx.reshape(-1, 3)
    p = pos.astype(np.float32)
    e1, e2 = p[tri[:, 1]] - p[tri[:, 0]], p[tri[:, 2]] - p[tri[:, 0]]
    du1, dv1 = uv[tri[:, 1], 0] - uv[tri[:, 0], 0], uv[tri[:, 1], 1] - uv[tri[:, 0], 1]
    du2, dv2 = uv[tri[:, 2], 0] - uv[tri[:, 0], 0], uv[tri[:, 2], 1] - uv[tri[:, 0], 1]
    det = du1 * dv2 - dv1 * du2
    keep = np.abs(det) > 1e-12
    inv = np.zeros_like(det)
    inv[keep] = 1.0 / det[keep]
    sdir = (dv2[:, None] * e1 - dv1[:, None] * e2) * inv[:, None]
    tdir = (du1[:, None] * e2 - du2[:, None] * e1) * inv[:, None]
    t1 = np.zeros_like(p)
    t2 = np.zeros_like(p)
    for k in range(3):
        np.add.at(t1, tri[keep, k], sdir[keep])
        np.add.at(t2, tri[keep, k], tdir[keep])
    n, _ = _normalise_rows(normals.astype(np.float32))
    hand = np.where((np.cross(n, t1) * t2).sum(1) < 0, -1.0, 1.0)
    out = _orthonormal_tangents(normals, np.concatenate([t1, np.zeros((len(t1), 1), np.float32)], 1), hand)
    bad = ((normals * normals).sum(1) <= 1e-12) | ((t1 * t1).sum(1) <= 1e-12)
    out[bad] = _fallback_tangents(normals[bad]) if bad.any() else out[bad]
    return out


def _texcoord_set(info) -> int:
    if not info:
        return 0
    s = int(info.get("texCoord", 0))
    return s if s <= 1 else 0


def _primitive(doc, buffers, prim, name, node_index, ignored):
    attrs = prim.get("attributes", {})
    if prim.get("mode", 4) != 4 or "POSITION" not in attrs:
        return None
    if prim.get("targets"):
        ignored.add("morph targets")
    pos = _yup_to_zup(_accessor(doc, buffers, attrs["POSITION"]).astype(np.float64)).astype(np.float32)
    n = len(pos)
    if n == 0:
        return None
    normals = _accessor(doc, buffers, attrs["NORMAL"]).astype(np.float32) if "NORMAL" in attrs else None
    tangents = _accessor(doc, buffers, attrs["TANGENT"]).astype(np.float32) if "TANGENT" in attrs else None
    uv0 = _accessor(doc, buffers, attrs["TEXCOORD_0"]).astype(np.float32) if "TEXCOORD_0" in attrs else None
    uv1 = _accessor(doc, buffers, attrs["TEXCOORD_1"]).astype(np.float32) if "TEXCOORD_1" in attrs else None
    color = np.ones((n, 4), np.float32)
    if "COLOR_0" in attrs:
        c = _accessor(doc, buffers, attrs["COLOR_0"]).astype(np.float32)
        if c.shape[1] not in (3, 4):
            raise ValueError(f"{name}: COLOR_0 must have 3 or 4 components")
        color[:, :c.shape[1]] = c
    if "indices" in prim:
        idx = _accessor(doc, buffers, prim["indices"]).reshape(-1).astype(np.int64)
        if idx.size and (idx.min() < 0 or idx.max() >= n):
            raise ValueError(f"{name}: index out of range")
        idx = idx.astype(np.uint32)
    else:
        idx = np.arange(n, dtype=np.uint32)
    idx = idx[:len(idx) // 3 * 3]

    mat_index = prim.get("material", abi.INVALID_INDEX)
    material = doc["materials"][mat_index] if mat_index != abi.INVALID_INDEX else None
    tangent_set = _texcoord_set(material.get("normalTexture")) if material else 0
    tangent_uv = uv1 if tangent_set == 1 else uv0

    v = np.zeros(n, dtype=abi.VERTEX)
    v["position"][:, :3] = pos
    v["position"][:, 3] = 1.0
    v["color"] = color
    if uv0 is not None:
        v["texcoord0"] = uv0
    if uv1 is not None:
        v["texcoord1"] = uv1
    if normals is None:
        nrm = _generate_normals(pos, idx)
        tan = np.zeros((n, 4), np.float32)  # vkrt leaves the tangent of generated-normal primitives untouched
    else:
        nrm = _yup_to_zup(normals.astype(np.float64)).astype(np.float32)
        idx = _align_winding(pos, nrm, idx)
        if tangents is not None:
            t = np.concatenate([_yup_to_zup(tangents[:, :3].astype(np.float64)), tangents[:, 3:4]], 1)
            tan = _orthonormal_tangents(nrm, t.astype(np.float32), np.where(tangents[:, 3] < 0, -1.0, 1.0))
        elif tangent_uv is not None:
            tan = _generate_tangents(pos, nrm, idx, tangent_uv)
        else:
            tan = _fallback_tangents(nrm)
    v["normal"][:, :3] = nrm
    v["tangent"] = tan
    return MeshEntry(name=name, vertices=v, indices=idx, material=mat_index,
                     render_backfaces=1 if material and material.get("doubleSided", False) else 0, node=node_index)


# ---- textures -----------------------------------------------------------------------------------------------------
SLOT_BASE_COLOR, SLOT_METALLIC_ROUGHNESS, SLOT_NORMAL, SLOT_EMISSIVE = 0, 1, 2, 3  # VKRT_MATERIAL_TEXTURE_SLOT_*
_SLOT_FIELDS = {SLOT_BASE_COLOR: "baseColor", SLOT_METALLIC_ROUGHNESS: "metallicRoughness", SLOT_NORMAL: "normal",
                SLOT_EMISSIVE: "emissive"}


class _Textures:
    """Decoded images of one document, each registered once per (image, colour space) (registerImportedTexture)."""

    def __init__(self, doc, buffers, base: Path, ignored: set):
        self.doc, self.buffers, self.base, self.ignored = doc, buffers, base, ignored
        self.images: list = []
        self.cache: dict = {}

    @staticmethod
    def texcoord_set(view) -> int:  # queryTextureViewTexcoordSet (loader.c:380-386)
        t = view.get("extensions", {}).get("KHR_texture_transform", {})
        if "texCoord" in t and int(t["texCoord"]) >= 0:
            return int(t["texCoord"])
        return max(int(view.get("texCoord", 0)), 0)

    def _bytes(self, image):
        uri = image.get("uri")
        if uri and not uri.startswith("data:"):
            return (self.base / uri).read_bytes(), image.get("mimeType")
        if "bufferView" in image:
            bv = self.doc["bufferViews"][image["bufferView"]]
            off, n = bv.get("byteOffset", 0), bv["byteLength"]
            return bytes(self.buffers[bv["buffer"]][off:off + n]), image.get("mimeType")
        return None, None

    def register(self, view, color_space: int):
        """Import-local texture index of `view`, or None when it does not bind."""
        from .image_decode import ImageDecodeError, UnsupportedImage, decode_image
        if not view or "index" not in view:
            return None
        if self.texcoord_set(view) > 1:  # textureViewUsesUnsupportedTransform (loader.c:1183-1186)
            self.ignored.add("textures on texture-coordinate sets above 1")
            return None
        tex = self.doc.get("textures", [])[view["index"]]
        if "source" not in tex:
            return None
        key = (tex["source"], color_space)
        if key not in self.cache:
            data, mime = self._bytes(self.doc["images"][tex["source"]])
            if data is None:
                self.ignored.add("data-URI images")
                self.cache[key] = None
            else:
                try:
                    self.images.append(decode_image(data, mime, color_space))
                    self.cache[key] = len(self.images) - 1
                except (UnsupportedImage, ImageDecodeError) as e:
                    self.ignored.add(f"textures ({e})")
                    self.cache[key] = None
        return self.cache[key]

    def bind(self, m: np.ndarray, slot: int, view, color_space: int) -> None:
        """Binds `view` to material slot `slot`: index, wrap modes, coordinate set, transform and rotation."""
        idx = self.register(view, color_space)
        if idx is None:
            return
        f = _SLOT_FIELDS[slot]
        m[f + "TextureIndex"] = idx
        sampler = self.doc["samplers"][self.doc["textures"][view["index"]]["sampler"]] \
            if "sampler" in self.doc["textures"][view["index"]] else {}
        ws, wt = int(sampler.get("wrapS", abi.WRAP_REPEAT)), int(sampler.get("wrapT", abi.WRAP_REPEAT))
        m[f + "TextureWrap"] = (ws or abi.WRAP_REPEAT) | ((wt or abi.WRAP_REPEAT) << 16)  # packTextureWrapModes
        shift = 8 * slot
        sets = int(m["textureTexcoordSets"][0])
        m["textureTexcoordSets"] = (sets & ~(0xFF << shift)) | ((self.texcoord_set(view) & 0xFF) << shift)
        t = view.get("extensions", {}).get("KHR_texture_transform")
        if t is not None:  # copyTextureTransform (loader.c:388-404)
            sc, of = t.get("scale", [1.0, 1.0]), t.get("offset", [0.0, 0.0])
            m[f + "TextureTransform"] = (sc[0], sc[1], of[0], of[1])
            m["textureRotations"][0, slot] = t.get("rotation", 0.0)


# ---- materials ----------------------------------------------------------------------------------------------------
def _material(src, default, ignored, textures: _Textures | None = None) -> np.ndarray:
    from .abi import COLOR_SPACE_LINEAR, COLOR_SPACE_SRGB
    m = default.copy()
    ext = src.get("extensions", {})
    if "KHR_materials_pbrSpecularGlossiness" in ext:
        sg = ext["KHR_materials_pbrSpecularGlossiness"]
        d = sg.get("diffuseFactor", [1, 1, 1, 1])
        m["baseColor"] = d[:3]
        m["opacity"] = d[3]
        m["roughness"] = 1.0 - sg.get("glossinessFactor", 1.0)
        if textures is not None:
            textures.bind(m, SLOT_BASE_COLOR, sg.get("diffuseTexture"), COLOR_SPACE_SRGB)
    elif "pbrMetallicRoughness" in src:  # without it vkrt keeps its default material factors (loader.c:966)
        pbr = src["pbrMetallicRoughness"]
        c = pbr.get("baseColorFactor", [1, 1, 1, 1])
        m["baseColor"] = c[:3]
        m["opacity"] = c[3]
        m["metallic"] = pbr.get("metallicFactor", 1.0)
        m["roughness"] = pbr.get("roughnessFactor", 1.0)
        if textures is not None:
            textures.bind(m, SLOT_BASE_COLOR, pbr.get("baseColorTexture"), COLOR_SPACE_SRGB)
            textures.bind(m, SLOT_METALLIC_ROUGHNESS, pbr.get("metallicRoughnessTexture"), COLOR_SPACE_LINEAR)
    if "KHR_materials_specular" in ext:
        m["specular"] = ext["KHR_materials_specular"].get("specularFactor", 1.0)
    if "KHR_materials_ior" in ext:
        m["ior"] = ext["KHR_materials_ior"].get("ior", 1.5)
    if "KHR_materials_transmission" in ext:
        m["transmission"] = ext["KHR_materials_transmission"].get("transmissionFactor", 0.0)
    if "KHR_materials_volume" in ext:
        vol = ext["KHR_materials_volume"]
        m["attenuationColor"] = vol.get("attenuationColor", [1, 1, 1])
        dist = vol.get("attenuationDistance", math.inf)
        m["absorptionCoefficient"] = 1.0 / dist if dist > 0 and math.isfinite(dist) else 0.0
    if "KHR_materials_clearcoat" in ext:
        cc = ext["KHR_materials_clearcoat"]
        m["clearcoat"] = cc.get("clearcoatFactor", 0.0)
        m["clearcoatGloss"] = 1.0 - cc.get("clearcoatRoughnessFactor", 0.0)
    if "KHR_materials_sheen" in ext:
        sh = ext["KHR_materials_sheen"]
        col = np.array(sh.get("sheenColorFactor", [0, 0, 0]), np.float32)
        w = float(col.max())
        m["sheenTintWeight"] = [*(col / w), w] if w > 0 else [1, 1, 1, 0]
        m["sheenRoughness"] = sh.get("sheenRoughnessFactor", 0.0)
    scale = ext.get("KHR_materials_emissive_strength", {}).get("emissiveStrength", 1.0)
    e = np.array(src.get("emissiveFactor", [0, 0, 0]), np.float32) * np.float32(scale)
    emax = float(e.max())
    if emax > 0:
        m["emissionColor"] = e / np.float32(emax)
        m["emissionLuminance"] = emax
    else:
        m["emissionColor"] = 1.0
        m["emissionLuminance"] = 0.0
    if textures is not None:
        nt = src.get("normalTexture")
        textures.bind(m, SLOT_NORMAL, nt, COLOR_SPACE_LINEAR)
        if m["normalTextureIndex"][0] != abi.INVALID_INDEX:
            scale = float(nt.get("scale", 1.0))
            m["normalTextureScale"] = scale if scale > 0.0 else 1.0
        textures.bind(m, SLOT_EMISSIVE, src.get("emissiveTexture"), COLOR_SPACE_SRGB)
    if "occlusionTexture" in src:
        ignored.add("occlusion textures")  # vkrt's materials have no occlusion input
    mode = src.get("alphaMode", "OPAQUE")
    if mode == "MASK":
        m["alphaMode"] = ALPHA_MODE_MASK
        m["alphaCutoff"] = src.get("alphaCutoff", 0.5)
    elif mode == "BLEND":
        m["alphaMode"] = ALPHA_MODE_BLEND
        m["alphaCutoff"] = ALPHA_BLEND_CUTOFF
    return m


def default_material() -> np.ndarray:
    m = np.zeros(1, dtype=abi.MATERIAL)
    abi.load().vkrt_host_default_material(abi.ptr(m))
    return m


# ---- import -------------------------------------------------------------------------------------------------------
def load_gltf(path) -> GltfImport:
    path = Path(path)
    doc, binchunk = _read_document(path)
    buffers = _buffers(doc, binchunk, path.parent)
    ignored: set = set()
    for key, label in (("skins", "skinning"), ("animations", "animations"), ("cameras", "cameras")):
        if doc.get(key):
            ignored.add(label)
    base = default_material()
    textures = _Textures(doc, buffers, path.parent, ignored)
    materials = (np.concatenate([_material(src, base, ignored, textures) for src in doc.get("materials", [])])
                 if doc.get("materials") else np.zeros(0, dtype=abi.MATERIAL))
    nodes = doc.get("nodes", [])
    scene = doc.get("scene")
    if scene is not None and doc.get("scenes") and doc["scenes"][scene].get("nodes"):
        roots = list(doc["scenes"][scene]["nodes"])
    else:
        children = {c for nd in nodes for c in nd.get("children", [])}
        roots = [i for i in range(len(nodes)) if i not in children]
    entries, node_world = [], []
    stack = [(r, np.eye(4)) for r in reversed(roots)]
    while stack:
        ni, parent = stack.pop()
        nd = nodes[ni]
        world = parent @ to_vkrt_basis(node_local_matrix(nd))
        node_world.append(world)
        if "mesh" in nd:
            mesh = doc["meshes"][nd["mesh"]]
            for pi, prim in enumerate(mesh.get("primitives", [])):
                base_name = nd.get("name") or mesh.get("name") or f"mesh{nd['mesh']}"
                e = _primitive(doc, buffers, prim, base_name if len(mesh["primitives"]) == 1 else f"{base_name}_{pi}",
                               len(node_world) - 1, ignored)
                if e is not None:
                    entries.append(e)
        for c in reversed(nd.get("children", [])):
            stack.append((c, world))
    if not entries:
        raise ValueError(f"{path}: no triangle mesh primitives")
    return GltfImport(entries=entries, materials=materials, node_world=node_world, ignored=ignored,
                      textures=textures.images)
