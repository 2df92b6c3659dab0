"""Textured glTF imports and standalone texture imports of vkrt scene files (vkrt_gb300.gltf, scene_file) against
hand-built GLB files: textures registered per material in vkrt's order (base colour sRGB, metallic-roughness,
normal, emissive sRGB), each (image, colour space) decoded once, samplers' wrap modes, texture-coordinate sets and
KHR_texture_transform in the material, texture indices moved with the import's place in the scene, standalone
textures remapped from their saved index, and images of formats this package does not decode left unbound."""
import json

import numpy as np

from png_writer import encode_png
from tests.gltf_writer import plane_mesh, write_glb
from vkrt_gb300 import abi, gltf, scene_file
from vkrt_gb300.image_decode import decode_image, texture_texels

INVALID = abi.INVALID_INDEX
CLAMP, MIRROR, REPEAT = abi.WRAP_CLAMP, abi.WRAP_MIRROR, abi.WRAP_REPEAT


def _images(seed=0):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 256, (8, 8, 4))
    b = rng.integers(0, 65536, (4, 4, 1))
    c = rng.integers(0, 256, (4, 4, 3))
    return a, b, c, [(encode_png(a, 8, 6), "image/png"), (encode_png(b, 16, 0), "image/png"),
                     (encode_png(c, 8, 2), "image/png"), (b"\xff\xd8\xff\xe0" + bytes(32), "image/jpeg")]


def _write(path, seed=0):
    a, b, c, images = _images(seed)
    textures = [{"source": 0, "sampler": 0}, {"source": 1}, {"source": 2, "sampler": 1}, {"source": 3}]
    samplers = [{"wrapS": CLAMP, "wrapT": MIRROR}, {}]
    materials = [
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicRoughnessTexture": {"index": 1}},
         "normalTexture": {"index": 2, "scale": 0.5}, "emissiveTexture": {"index": 0}},
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0, "texCoord": 1, "extensions": {
            "KHR_texture_transform": {"scale": [2, 3], "offset": [0.25, 0.5], "rotation": 0.3}}},
            "metallicRoughnessTexture": {"index": 3}},
         "emissiveTexture": {"index": 2, "texCoord": 2}},
    ]
    m = plane_mesh()
    m["material"] = 0
    write_glb(path, [m], materials=materials, images=images, textures=textures, samplers=samplers)
    return a, b, c


def test_gltf_texture_registration(built, tmp_path):
    a, b, c = _write(tmp_path / "t.glb")
    imp = gltf.load_gltf(tmp_path / "t.glb")
    # registration: A as sRGB, B linear, C linear; A again as sRGB (emissive) is the same texture; the JPEG and the
    # texture-coordinate set 2 view do not bind
    assert len(imp.textures) == 3
    assert [t.color_space for t in imp.textures] == [abi.COLOR_SPACE_SRGB, abi.COLOR_SPACE_LINEAR,
                                                      abi.COLOR_SPACE_LINEAR]
    np.testing.assert_array_equal(imp.textures[0].pixels, a)
    assert imp.textures[1].pixels.dtype == np.uint16
    np.testing.assert_array_equal(imp.textures[1].pixels[..., 0], b[..., 0])
    m0, m1 = imp.materials[0], imp.materials[1]
    assert (m0["baseColorTextureIndex"], m0["metallicRoughnessTextureIndex"], m0["normalTextureIndex"],
            m0["emissiveTextureIndex"]) == (0, 1, 2, 0)
    assert m0["baseColorTextureWrap"] == CLAMP | (MIRROR << 16)
    assert m0["metallicRoughnessTextureWrap"] == REPEAT | (REPEAT << 16)
    assert m0["normalTextureScale"] == 0.5
    assert m1["baseColorTextureIndex"] == 0 and m1["metallicRoughnessTextureIndex"] == INVALID
    assert m1["emissiveTextureIndex"] == INVALID
    assert m1["textureTexcoordSets"] & 0xFF == 1
    np.testing.assert_allclose(m1["baseColorTextureTransform"], [2, 3, 0.25, 0.5])
    np.testing.assert_allclose(m1["textureRotations"], [0.3, 0, 0, 0], rtol=1e-6)
    assert any("JPEG" in w for w in imp.ignored)


def test_scene_file_texture_offsets_and_standalone_textures(built, tmp_path):
    a, b, c = _write(tmp_path / "one.glb", 0)
    a2, _, _ = _write(tmp_path / "two.glb", 1)
    rng = np.random.default_rng(9)
    solo = rng.integers(0, 256, (4, 4, 4))
    (tmp_path / "solo.png").write_bytes(encode_png(solo, 8, 6))
    (tmp_path / "solo.jpg").write_bytes(b"\xff\xd8\xff\xe0" + bytes(32))
    mesh = {"materialIndex": 0, "hasMaterialAssignment": False, "renderBackfaces": False, "opacity": 1}
    doc = {"format": "vkrt.scene", "version": 1, "meshImports": ["one.glb", "two.glb"],
           "textureImports": [{"index": 7, "colorSpace": abi.COLOR_SPACE_SRGB, "path": "solo.png"},
                              {"index": 8, "colorSpace": abi.COLOR_SPACE_SRGB, "path": "solo.jpg"}],
           "materials": [{"index": 5, "name": "saved", "material": {"baseColorTextureIndex": 7,
                                                                    "normalTextureIndex": 8}}],
           "meshes": [dict(mesh, name="a", importIndex=0, importLocalIndex=0),
                      dict(mesh, name="b", importIndex=1, importLocalIndex=0)],
           "sceneObjects": [], "sceneSettings": {"camera": {"position": [0, -5, 0], "target": [0, 0, 0],
                                                             "up": [0, 0, 1], "vfov": 40}}}
    path = tmp_path / "scene.json"
    path.write_text(json.dumps(doc))
    s = scene_file.load_scene_file(path, 32, 32)
    # material 0 is vkrt's default; import one's materials are 1-2 with textures 0-2, import two's 3-4 with 3-5
    assert len(s.textures) == 7
    assert s.materials[1]["baseColorTextureIndex"] == 0 and s.materials[3]["baseColorTextureIndex"] == 3
    assert s.materials[3]["normalTextureIndex"] == 5
    # the saved material's texture 7 is the standalone image (scene index 6); the JPEG is left out
    assert s.materials[5]["baseColorTextureIndex"] == 6
    assert s.materials[5]["normalTextureIndex"] == 8  # unmapped saved index stays as saved
    assert any("solo.jpg" in n for n in s.notes)
    want = texture_texels(decode_image(encode_png(a2, 8, 6), "image/png", abi.COLOR_SPACE_SRGB))
    np.testing.assert_array_equal(s.textures[3], want)
    np.testing.assert_array_equal(s.textures[6][..., 3], (solo[..., 3] / np.float32(255)).astype(np.float32))
