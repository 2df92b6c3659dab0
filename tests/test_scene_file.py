"""glTF import and vkrt scene files (vkrt_gb300.gltf, vkrt_gb300.scene_file) against hand-built GLB files with
known answers: vkrt's Y-up -> Z-up vertex basis, winding alignment, generated normals and tangents, node transforms
B M B^-1, material factors, scene-object hierarchies decomposed into MeshInfo TRS, scene settings into SceneData;
and, where vkrt's own scene files are present, their structure."""
import json
import os
from pathlib import Path

import numpy as np
import pytest

from tests.gltf_writer import icosphere_mesh, plane_mesh, write_glb
from vkrt_gb300 import abi, gltf, scene_file


def _world_of(mesh):
    out = np.zeros(16, np.float32)
    p = np.asarray(mesh["position"], np.float32)
    r = np.asarray(mesh["rotation"], np.float32)
    s = np.asarray(mesh["scale"], np.float32)
    abi.load().vkrt_host_mesh_transform(abi.ptr(p), abi.ptr(r), abi.ptr(s), abi.ptr(out))
    return out.reshape(4, 4).T.astype(np.float64)


def test_glb_vertices_in_vkrt_basis(built, tmp_path):
    m = plane_mesh()
    write_glb(tmp_path / "p.glb", [m])
    imp = gltf.load_gltf(tmp_path / "p.glb")
    assert len(imp.entries) == 1 and len(imp.materials) == 0
    v = imp.entries[0].vertices
    want = np.stack([m["positions"][:, 0], -m["positions"][:, 2], m["positions"][:, 1]], 1)
    np.testing.assert_array_equal(v["position"][:, :3], want)
    np.testing.assert_allclose(v["normal"][:, :3], np.tile([0, 0, 1], (4, 1)), atol=1e-7)
    # tangents from the UV gradient: +u runs along glTF +X = vkrt +X; orthonormal to the normal
    np.testing.assert_allclose(v["tangent"][:, :3], np.tile([1, 0, 0], (4, 1)), atol=1e-6)
    assert np.all(np.abs(v["tangent"][:, 3]) == 1.0)
    np.testing.assert_array_equal(v["color"], 1.0)
    np.testing.assert_array_equal(imp.entries[0].indices, [0, 1, 2, 0, 2, 3])
    np.testing.assert_array_equal(imp.node_world[0], np.eye(4))


def test_winding_follows_vertex_normals(built, tmp_path):
    m = plane_mesh()
    m["normals"] = -m["normals"]  # normals say -Y: both triangles are rewound
    write_glb(tmp_path / "p.glb", [m])
    e = gltf.load_gltf(tmp_path / "p.glb").entries[0]
    np.testing.assert_array_equal(e.indices, [0, 2, 1, 0, 3, 2])


def test_generated_normals_without_normal_attribute(built, tmp_path):
    m = icosphere_mesh(1)
    m["normals"] = None
    write_glb(tmp_path / "s.glb", [m])
    e = gltf.load_gltf(tmp_path / "s.glb").entries[0]
    p = e.vertices["position"][:, :3]
    n = e.vertices["normal"][:, :3]
    # a convex sphere: the area-weighted face normal sum points outward along the position
    cos = (n * p).sum(1) / np.linalg.norm(p, axis=1)
    assert cos.min() > 0.98
    np.testing.assert_allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-6)
    np.testing.assert_array_equal(e.vertices["tangent"], 0.0)


def test_node_transforms_in_vkrt_basis(built, tmp_path):
    s = np.sin(np.pi / 4)
    nodes = [{"name": "parent", "translation": [1, 2, 3], "children": [1]},
             {"name": "child", "mesh": 0, "rotation": [0, s, 0, s], "scale": [2, 2, 2]}]  # 90 deg about glTF +Y
    write_glb(tmp_path / "n.glb", [plane_mesh()], nodes=nodes)
    imp = gltf.load_gltf(tmp_path / "n.glb")
    world = imp.node_world[imp.entries[0].node]
    np.testing.assert_allclose(world[:3, 3], [1, -3, 2], atol=1e-12)  # glTF (x, y, z) -> vkrt (x, -z, y)
    # +90 degrees about glTF +Y takes glTF +X to glTF -Z, which is vkrt +Y; the scale is 2; vkrt +Z (glTF +Y) stays
    np.testing.assert_allclose(world[:3, :3] @ [1, 0, 0], [0, 2, 0], atol=1e-12)
    np.testing.assert_allclose(world[:3, 2], [0, 0, 2], atol=1e-12)


def test_material_factors(built, tmp_path):
    mats = [{"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 0.5], "metallicFactor": 0.25,
                                      "roughnessFactor": 0.75},
             "emissiveFactor": [2.0, 1.0, 0.0], "doubleSided": True, "alphaMode": "MASK", "alphaCutoff": 0.3,
             "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 3.0},
                            "KHR_materials_ior": {"ior": 1.33},
                            "KHR_materials_specular": {"specularFactor": 0.8}}},
            {"name": "no pbr block"}]
    m0, m1 = plane_mesh(), plane_mesh()
    m0["material"], m1["material"] = 0, 1
    write_glb(tmp_path / "m.glb", [m0, m1], materials=mats)
    imp = gltf.load_gltf(tmp_path / "m.glb")
    a, b = imp.materials[0], imp.materials[1]
    np.testing.assert_allclose(a["baseColor"], [0.2, 0.4, 0.6], rtol=1e-6)
    assert a["opacity"] == np.float32(0.5) and a["metallic"] == np.float32(0.25) and a["roughness"] == np.float32(0.75)
    np.testing.assert_allclose(a["emissionColor"], [1.0, 0.5, 0.0])
    assert a["emissionLuminance"] == np.float32(6.0)
    assert a["ior"] == np.float32(1.33) and a["specular"] == np.float32(0.8)
    assert a["alphaMode"] == gltf.ALPHA_MODE_MASK and a["alphaCutoff"] == np.float32(0.3)
    assert imp.entries[0].render_backfaces == 1 and imp.entries[1].render_backfaces == 0
    d = gltf.default_material()[0]
    for f in ("baseColor", "roughness", "metallic", "opacity"):  # no pbrMetallicRoughness: vkrt's defaults stay
        np.testing.assert_array_equal(b[f], d[f])


@pytest.mark.parametrize("seed", range(4))
def test_decompose_recompose(built, seed):
    rng = np.random.default_rng(seed)
    for _ in range(50):
        pos = rng.uniform(-5, 5, 3)
        rot = rng.uniform(-180, 180, 3)
        rot[1] = rng.uniform(-89, 89)
        scl = rng.uniform(0.1, 3, 3) * rng.choice([-1, 1], 3)
        w = scene_file.mesh_transform_matrix(pos, rot, scl)
        p, r, s = scene_file.decompose_mesh_transform(w)
        np.testing.assert_allclose(scene_file.mesh_transform_matrix(p, r, s), w, atol=1e-9)
        np.testing.assert_allclose(_world_of({"position": p, "rotation": r, "scale": s}), w, atol=2e-5)


def _cornell_like(tmp_path, with_missing=False):
    write_glb(tmp_path / "plane.glb", [plane_mesh()])
    write_glb(tmp_path / "sphere.glb", [icosphere_mesh(2)])
    imports = ["plane.glb", "plane.glb", "sphere.glb"] + (["absent.glb"] if with_missing else [])
    doc = {
        "format": "vkrt.scene", "version": 1, "meshImports": imports, "textureImports": [],
        "materials": [{"index": 1, "name": "floor", "material": {"roughness": 1, "baseColor": [0.7, 0.6, 0.5]}},
                      {"index": 3, "name": "light", "material": {"roughness": 1, "emissionLuminance": 20}}],
        "meshes": [{"name": "floor", "materialIndex": 1, "hasMaterialAssignment": True, "renderBackfaces": False,
                    "opacity": 1, "importIndex": 0, "importLocalIndex": 0},
                   {"name": "wall", "materialIndex": 1, "hasMaterialAssignment": False, "renderBackfaces": True,
                    "opacity": 1, "importIndex": 1, "importLocalIndex": 0},
                   {"name": "light", "materialIndex": 3, "hasMaterialAssignment": True, "renderBackfaces": False,
                    "opacity": 1, "importIndex": 2, "importLocalIndex": 0}]
        + ([{"name": "ghost", "materialIndex": 1, "hasMaterialAssignment": True, "renderBackfaces": False,
             "opacity": 1, "importIndex": 3, "importLocalIndex": 0}] if with_missing else []),
        "sceneObjects": [{"name": "floor", "parentIndex": None, "meshIndex": 0, "localPosition": [0, 0, -1],
                          "localRotation": [180, 0, 90], "localScale": [1, 1, 1]},
                         {"name": "room", "parentIndex": None, "meshIndex": None, "localPosition": [0, 0.5, 0],
                          "localRotation": [0, 0, 30], "localScale": [2, 2, 2]},
                         {"name": "wall", "parentIndex": 1, "meshIndex": 1, "localPosition": [0, 1, 0],
                          "localRotation": [90, 90, 0], "localScale": [1, 1, 1]},
                         {"name": "light", "parentIndex": None, "meshIndex": 2, "localPosition": [0, 0, 0.9],
                          "localRotation": [0, 0, 0], "localScale": [0.2, 0.2, 0.05]}]
        + ([{"name": "ghost", "parentIndex": None, "meshIndex": 3, "localPosition": [0, 0, 0],
             "localRotation": [0, 0, 0], "localScale": [1, 1, 1]}] if with_missing else []),
        "sceneSettings": {"camera": {"position": [0, -5, 0], "target": [0, 0, 0], "up": [0, 0, 1], "vfov": 27},
                          "rrMinDepth": 3, "rrMaxDepth": 7, "toneMappingMode": 1, "renderMode": 0,
                          "spectralSamplingMode": 1, "exposure": 1.5, "environmentColor": [0.5, 0.25, 1.0],
                          "environmentStrength": 0.5, "environmentRotation": 10, "misNeeEnabled": True},
    }
    path = tmp_path / "scene.json"
    path.write_text(json.dumps(doc))
    return path, doc


def test_scene_file_structure(built, tmp_path):
    path, doc = _cornell_like(tmp_path)
    s = scene_file.load_scene_file(path, 96, 64)
    assert s.mesh_names == ["floor", "wall", "light"]
    assert list(s.meshes["materialIndex"]) == [1, 0, 3]  # wall: no assignment -> default material 0
    assert list(s.meshes["renderBackfaces"]) == [0, 1, 0]
    assert len(s.materials) == 4
    np.testing.assert_allclose(s.materials[1]["baseColor"], [0.7, 0.6, 0.5], rtol=1e-6)
    assert s.materials[3]["emissionLuminance"] == 20.0
    np.testing.assert_array_equal(s.materials[2]["baseColor"], gltf.default_material()[0]["baseColor"])
    mt = scene_file.mesh_transform_matrix
    floor = mt([0, 0, -1], [180, 0, 90], [1, 1, 1])
    wall = mt([0, 0.5, 0], [0, 0, 30], [2, 2, 2]) @ mt([0, 1, 0], [90, 90, 0], [1, 1, 1])
    light = mt([0, 0, 0.9], [0, 0, 0], [0.2, 0.2, 0.05])
    for m, want in zip(s.meshes, (floor, wall, light)):
        np.testing.assert_allclose(_world_of(m), want, atol=2e-5)
    sd = s.scene_data[0]
    assert sd["rrMinDepth"] == 3 and sd["rrMaxDepth"] == 7
    assert sd["packedRenderSettings"] == abi.pack_render_settings(1, 0, 1)
    np.testing.assert_allclose(sd["environmentLight"], [0.25, 0.125, 0.5, 0.5])
    assert sd["exposure"] == np.float32(1.5) and sd["environmentRotation"] == np.float32(10)
    np.testing.assert_allclose(sd["viewInverse"][3, :3], [0, -5, 0], atol=1e-6)
    assert list(sd["viewportRect"]) == [0, 0, 96, 64]
    # the emissive sphere feeds the light tables
    assert s.emissive_meshes is not None and len(s.emissive_meshes) >= 1


def test_scene_file_missing_import(built, tmp_path):
    path, _ = _cornell_like(tmp_path, with_missing=True)
    with pytest.raises(scene_file.SceneFileError):
        scene_file.load_scene_file(path, 32, 32)
    s = scene_file.load_scene_file(path, 32, 32, missing="skip")
    assert s.mesh_names == ["floor", "wall", "light"] and any("absent.glb" in n for n in s.notes)


def test_scene_file_rejects_bad_documents(built, tmp_path):
    path, doc = _cornell_like(tmp_path)
    for bad in ({**doc, "format": "other"}, {**doc, "version": 2},
                {**doc, "sceneObjects": [{**doc["sceneObjects"][2], "parentIndex": 3}]}):
        p = tmp_path / "bad.json"
        p.write_text(json.dumps(bad))
        with pytest.raises(scene_file.SceneFileError):
            scene_file.load_scene_file(p, 32, 32)


# vkrt's bundled scene files, read from a vkrt checkout named by VKRT_REFERENCE (the tests skip without one)
_REF_SCENES = Path(os.environ.get("VKRT_REFERENCE", "")) / "assets" / "scenes" if os.environ.get("VKRT_REFERENCE") \
    else None


@pytest.mark.skipif(_REF_SCENES is None or not _REF_SCENES.exists(), reason="no vkrt checkout named by VKRT_REFERENCE")
@pytest.mark.parametrize("name", ["cornell", "prism", "caustics"])
def test_vkrt_scene_files(built, name):
    """vkrt's bundled scene files: every saved mesh whose import exists is loaded with its saved material and the
    world matrix of its scene object."""
    path = _REF_SCENES / f"{name}.json"
    doc = json.loads(path.read_text())
    s = scene_file.load_scene_file(path, 64, 64, missing="skip")
    present = [(path.parent / doc["meshImports"][m["importIndex"]]).resolve().exists() for m in doc["meshes"]]
    assert len(s.meshes) == sum(present)
    kept = [m for m, ok in zip(doc["meshes"], present) if ok]
    assert s.mesh_names == [m["name"] for m in kept]
    assert list(s.meshes["materialIndex"]) == [m["materialIndex"] if m["hasMaterialAssignment"] else 0 for m in kept]
    mt = scene_file.mesh_transform_matrix
    worlds = []
    for so in doc["sceneObjects"]:
        local = mt(so["localPosition"], so["localRotation"], so["localScale"])
        worlds.append(local if so["parentIndex"] is None else worlds[so["parentIndex"]] @ local)
    saved = [k for k, ok in enumerate(present) if ok]
    for so, w in zip(doc["sceneObjects"], worlds):
        if so["meshIndex"] is None or so["meshIndex"] not in saved:
            continue
        m = s.meshes[saved.index(so["meshIndex"])]
        np.testing.assert_allclose(_world_of(m), w, atol=2e-4 * max(1.0, np.abs(w).max()))
