"""A vkrt scene file rendered on the GPU: a Cornell-style room assembled from GLB planes and spheres through
vkrt_gb300.scene_file, rendered by both integrators and checked per sample against the oracle's restatement of
vkrt's integrator on the same loaded records."""
import json

import numpy as np
import pytest

from parity import assert_match

from tests.gltf_writer import icosphere_mesh, plane_mesh, write_glb
from vkrt_gb300 import RenderContext, abi, scene_file

pytestmark = pytest.mark.gpu


def _room(tmp_path):
    write_glb(tmp_path / "plane.glb", [plane_mesh()])
    write_glb(tmp_path / "sphere.glb", [icosphere_mesh(3)])
    walls = [("floor", [0, 0, -1], [180, 0, 90], 1), ("ceiling", [0, 0, 1], [0, 0, -90], 1),
             ("back", [0, 1, 0], [90, 90, 0], 1), ("left", [-1, 0, 0], [-90, 0, -90], 2),
             ("right", [1, 0, 0], [90, 0, -90], 3)]
    meshes, objects = [], []
    for k, (name, pos, rot, mat) in enumerate(walls):
        meshes.append({"name": name, "materialIndex": mat, "hasMaterialAssignment": True, "renderBackfaces": False,
                       "opacity": 1, "importIndex": k, "importLocalIndex": 0})
        objects.append({"name": name, "parentIndex": None, "meshIndex": k, "localPosition": pos,
                        "localRotation": rot, "localScale": [1, 1, 1]})
    meshes.append({"name": "light", "materialIndex": 4, "hasMaterialAssignment": True, "renderBackfaces": False,
                   "opacity": 1, "importIndex": 5, "importLocalIndex": 0})
    objects.append({"name": "light", "parentIndex": None, "meshIndex": 5, "localPosition": [0, 0, 0.98],
                    "localRotation": [0, 0, 0], "localScale": [0.25, 0.25, 0.03]})
    meshes.append({"name": "ball", "materialIndex": 5, "hasMaterialAssignment": True, "renderBackfaces": False,
                   "opacity": 1, "importIndex": 6, "importLocalIndex": 0})
    objects.append({"name": "ball", "parentIndex": None, "meshIndex": 6, "localPosition": [0.3, -0.1, -0.65],
                    "localRotation": [0, 0, 20], "localScale": [0.35, 0.35, 0.35]})
    doc = {"format": "vkrt.scene", "version": 1, "meshImports": ["plane.glb"] * 5 + ["sphere.glb"] * 2,
           "materials": [{"index": 1, "name": "white", "material": {"roughness": 1, "baseColor": [0.73, 0.73, 0.73],
                                                                    "specular": 0}},
                         {"index": 2, "name": "red", "material": {"roughness": 1, "baseColor": [0.65, 0.05, 0.05],
                                                                  "specular": 0}},
                         {"index": 3, "name": "green", "material": {"roughness": 1, "baseColor": [0.12, 0.45, 0.15],
                                                                    "specular": 0}},
                         {"index": 4, "name": "light", "material": {"roughness": 1, "emissionLuminance": 15}},
                         {"index": 5, "name": "ball", "material": {"baseColor": [0.9, 0.8, 0.6], "metallic": 1,
                                                                   "roughness": 0.3}}],
           "meshes": meshes, "sceneObjects": objects,
           "sceneSettings": {"camera": {"position": [0, -5.2, 0], "target": [0, 0, 0], "up": [0, 0, 1], "vfov": 27},
                             "rrMinDepth": 4, "rrMaxDepth": 8, "toneMappingMode": 1, "renderMode": 0,
                             "spectralSamplingMode": 1, "exposure": 1, "environmentColor": [0.25, 0.25, 0.25],
                             "environmentStrength": 1, "environmentRotation": 0, "misNeeEnabled": True}}
    p = tmp_path / "room.json"
    p.write_text(json.dumps(doc))
    return p


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_scene_file_render_matches_oracle(built, tmp_path, integrator):
    from oracle import cpu
    s = scene_file.load_scene_file(_room(tmp_path), 96, 96)
    sd = s.scene_data.copy()
    sd["samplesPerPixel"] = 4
    s.scene_data = sd
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        ctx.upload_scene(s)
        ctx.render_frame(sd)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(sd, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 1e-3, 1e-3, max_outside=2)
    np.testing.assert_array_equal(gpu[..., 3], 4.0)
    # the light and the coloured walls are in view
    assert gpu[..., 0].max() > 1.0 and (gpu[..., 0] > 1.5 * gpu[..., 1]).mean() > 0.05


def _dispersion_room(tmp_path, abbe):
    """A glass prism (Abbe number `abbe`) between a bright bar light and a white corner, like vkrt's prism scene:
    floor, back wall, left wall, hero-spectral mode."""
    from tests.gltf_writer import prism_mesh
    write_glb(tmp_path / "plane.glb", [plane_mesh()])
    write_glb(tmp_path / "prism.glb", [prism_mesh()])
    walls = [("floor", [0, 0, -1], [180, 0, 90]), ("back", [0, 1, 0], [90, 90, 0]), ("left", [-1, 0, 0], [-90, 0, -90])]
    meshes, objects = [], []
    for k, (name, pos, rot) in enumerate(walls):
        meshes.append({"name": name, "materialIndex": 1, "hasMaterialAssignment": True, "renderBackfaces": False,
                       "opacity": 1, "importIndex": k, "importLocalIndex": 0})
        objects.append({"name": name, "parentIndex": None, "meshIndex": k, "localPosition": pos,
                        "localRotation": rot, "localScale": [1, 1, 1]})
    meshes.append({"name": "bar", "materialIndex": 2, "hasMaterialAssignment": True, "renderBackfaces": True,
                   "opacity": 1, "importIndex": 3, "importLocalIndex": 0})
    objects.append({"name": "bar", "parentIndex": None, "meshIndex": 3, "localPosition": [0.9, 0.0, 0.0],
                    "localRotation": [0, 90, 0], "localScale": [0.6, 0.03, 1]})
    meshes.append({"name": "prism", "materialIndex": 3, "hasMaterialAssignment": True, "renderBackfaces": True,
                   "opacity": 1, "importIndex": 4, "importLocalIndex": 0})
    objects.append({"name": "prism", "parentIndex": None, "meshIndex": 4, "localPosition": [0.2, -0.15, -0.2],
                    "localRotation": [-20, 90, -60], "localScale": [0.8, 0.5, 0.5]})
    doc = {"format": "vkrt.scene", "version": 1, "meshImports": ["plane.glb"] * 4 + ["prism.glb"],
           "materials": [{"index": 1, "name": "white", "material": {"roughness": 1, "baseColor": [0.8, 0.8, 0.8],
                                                                    "specular": 0}},
                         {"index": 2, "name": "bar", "material": {"roughness": 1, "emissionLuminance": 40}},
                         {"index": 3, "name": "prism", "material": {"roughness": 0, "transmission": 1, "ior": 1.5,
                                                                    "abbeNumber": abbe}}],
           "meshes": meshes, "sceneObjects": objects,
           "sceneSettings": {"camera": {"position": [4.2, -3.8, 4.9], "target": [0, 0, 0], "up": [0, 0, 1],
                                        "vfov": 27}, "rrMinDepth": 4, "rrMaxDepth": 8, "toneMappingMode": 1,
                             "renderMode": 1, "spectralSamplingMode": 1, "exposure": 1,
                             "environmentColor": [0.25, 0.25, 0.25], "environmentStrength": 0.16,
                             "environmentRotation": 0, "misNeeEnabled": True}}
    p = tmp_path / f"prism{int(abbe)}.json"
    p.write_text(json.dumps(doc))
    return p


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_dispersive_prism_scene_matches_oracle(built, tmp_path, integrator):
    """Hero-spectral transport through a dispersive prism loaded from a scene file: refracted paths collapse to one
    wavelength; per-sample parity with the oracle."""
    from oracle import cpu
    s = scene_file.load_scene_file(_dispersion_room(tmp_path, 25.2), 64, 64)
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        table, info = ctx.generate_rgb2spec(32)
        s.rgb2spec = table
        s.scene_data["rgb2specSRGB"] = info
        s.scene_data["samplesPerPixel"] = 4
        ctx.upload_scene(s)
        ctx.render_frame(s.scene_data)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 2e-3, 2e-3, max_outside=2)
    # the same scene without dispersion renders differently where light went through the prism
    s0 = scene_file.load_scene_file(_dispersion_room(tmp_path, 0.0), 64, 64)
    s0.rgb2spec, s0.scene_data = s.rgb2spec, s.scene_data.copy()
    ref0, _ = cpu.OracleScene(s0).render(s0.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert (np.abs(ref0[..., :3] - ref[..., :3]).max(-1) > 1e-3).mean() > 0.01


def _textured_room(tmp_path):
    """A floor imported with a textured glTF material (8-bit sRGB base-colour checker, 16-bit metallic-roughness
    with roughness in G and metallic in B, normal map, clamp / mirror samplers), a metal ball and a light."""
    from png_writer import encode_png
    yy, xx = np.mgrid[0:32, 0:32]
    checker = np.where(((yy // 4) + (xx // 4)) % 2 == 0, 220, 40)
    base = np.stack([checker, checker // 2 + 60, 255 - checker, np.full_like(checker, 255)], -1)
    mr = np.zeros((16, 16, 3), np.int64)
    mr[..., 1] = (np.linspace(0.2, 1.0, 16)[None, :] * 65535).astype(np.int64)   # roughness
    mr[..., 2] = np.where(np.arange(16)[:, None] < 8, 0, 65535)                   # metallic bands
    nrm = np.zeros((8, 8, 3), np.int64)
    nrm[..., 0] = 128 + (np.arange(8)[None, :] - 4) * 12
    nrm[..., 1] = 128
    nrm[..., 2] = 240
    images = [(encode_png(base, 8, 6), "image/png"), (encode_png(mr, 16, 2), "image/png"),
              (encode_png(nrm, 8, 2), "image/png")]
    material = {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicRoughnessTexture": {"index": 1},
                                         "metallicFactor": 1.0, "roughnessFactor": 1.0},
                "normalTexture": {"index": 2, "scale": 0.8}}
    floor = plane_mesh()
    floor["material"] = 0
    write_glb(tmp_path / "floor.glb", [floor], materials=[material], images=images,
              textures=[{"source": 0, "sampler": 0}, {"source": 1, "sampler": 1}, {"source": 2}],
              samplers=[{"wrapS": abi.WRAP_MIRROR, "wrapT": abi.WRAP_CLAMP}, {"wrapS": abi.WRAP_CLAMP}])
    write_glb(tmp_path / "sphere.glb", [icosphere_mesh(3)])
    write_glb(tmp_path / "plane.glb", [plane_mesh()])
    mesh = {"renderBackfaces": False, "opacity": 1, "importLocalIndex": 0}
    doc = {"format": "vkrt.scene", "version": 1, "meshImports": ["floor.glb", "sphere.glb", "plane.glb"],
           "materials": [{"index": 2, "name": "ball", "material": {"baseColor": [0.9, 0.8, 0.6], "metallic": 1,
                                                                   "roughness": 0.2}},
                         {"index": 3, "name": "light", "material": {"roughness": 1, "emissionLuminance": 12}}],
           "meshes": [dict(mesh, name="floor", materialIndex=1, hasMaterialAssignment=True, importIndex=0),
                      dict(mesh, name="ball", materialIndex=2, hasMaterialAssignment=True, importIndex=1),
                      dict(mesh, name="light", materialIndex=3, hasMaterialAssignment=True, importIndex=2)],
           "sceneObjects": [{"name": "floor", "parentIndex": None, "meshIndex": 0, "localPosition": [0, 0, -0.5],
                             "localRotation": [0, 0, 15], "localScale": [1.5, 1.5, 1.5]},
                            {"name": "ball", "parentIndex": None, "meshIndex": 1, "localPosition": [0.2, 0.1, -0.1],
                             "localRotation": [0, 0, 0], "localScale": [0.4, 0.4, 0.4]},
                            {"name": "light", "parentIndex": None, "meshIndex": 2, "localPosition": [0, 0, 1.2],
                             "localRotation": [180, 0, 0], "localScale": [0.4, 0.4, 0.4]}],
           "sceneSettings": {"camera": {"position": [0, -3.2, 1.4], "target": [0, 0, -0.4], "up": [0, 0, 1],
                                        "vfov": 40},
                             "rrMinDepth": 4, "rrMaxDepth": 8, "toneMappingMode": 1, "renderMode": 0,
                             "spectralSamplingMode": 1, "exposure": 1, "environmentColor": [0.3, 0.35, 0.4],
                             "environmentStrength": 1, "environmentRotation": 0, "misNeeEnabled": True}}
    p = tmp_path / "textured.json"
    p.write_text(json.dumps(doc))
    return p


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_textured_scene_file_matches_oracle(built, tmp_path, integrator):
    """Decoded PNG textures (base colour, metallic-roughness, normal map) render per sample as the oracle renders
    the same texels."""
    from oracle import cpu
    s = scene_file.load_scene_file(_textured_room(tmp_path), 96, 80)
    assert len(s.textures) == 3 and s.materials[1]["baseColorTextureIndex"] == 0
    sd = s.scene_data.copy()
    sd["samplesPerPixel"] = 4
    s.scene_data = sd
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        ctx.upload_scene(s)
        ctx.render_frame(sd)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(sd, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 1e-3, 1e-3, max_outside=4)
    # the checker shows: the floor's pixels spread over a wide range of blue / red ratios
    floor = gpu[60:, :, :3]
    ratio = (floor[..., 2] + 1e-3) / (floor[..., 0] + 1e-3)
    assert np.percentile(ratio, 90) > 2.0 * np.percentile(ratio, 10)
