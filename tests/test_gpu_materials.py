"""vkrt's material stack beyond the glTF subset on the GPU against the oracle's restatement, per sample, for both
integrators in RGB and hero-spectral mode:
* the reflection layers: clearcoat, Oren-Nayar diffuse, fake subsurface (principled/eval_rgb.slang,
  lobes/clearcoat.slang, diffuse.slang, subsurface.slang);
* the transmissive interface: smooth and rough dielectric refraction (lobes/dielectric/**), Beer-Lambert absorption
  inside (bsdf/base/medium.slang), Abbe-number dispersion that collapses a hero path to one wavelength
  (spectral_hero/transport.slang), and NEE marked unsupported by transmissive occluders."""
import numpy as np
import pytest

from parity import assert_match

from vkrt_gb300 import RenderContext, abi, scenes

pytestmark = pytest.mark.gpu


def extended_cornell(width=64, height=64, spp=4):
    s = scenes.cornell(width, height, spp=spp)
    base = s.materials[0].copy()
    coat = base.copy()  # red clear-coated box
    coat["baseColor"] = [0.7, 0.15, 0.1]
    coat["clearcoat"] = 1.0
    coat["clearcoatGloss"] = 0.8
    sss = base.copy()  # soft subsurface box with a rough diffuse base
    sss["baseColor"] = [0.8, 0.7, 0.5]
    sss["subsurface"] = 0.7
    sss["diffuseRoughness"] = 0.5
    floor = base.copy()  # Oren-Nayar floor
    floor["diffuseRoughness"] = 1.0
    first = len(s.materials)
    s.materials = np.concatenate([s.materials, coat.reshape(1), sss.reshape(1), floor.reshape(1)])
    meshes = s.meshes.copy()
    meshes["materialIndex"][-2] = first
    meshes["materialIndex"][-1] = first + 1
    meshes["materialIndex"][0] = first + 2  # the first wall mesh carries the floor
    s.meshes = meshes
    return s


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_extended_stack_rgb_parity(built, integrator):
    from oracle import cpu
    s = extended_cornell()
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        ctx.upload_scene(s)
        ctx.render_frame(s.scene_data)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 1e-3, 1e-3, max_outside=2)
    # the coat adds a grey specular on the red box: some pixels are brighter in blue than the base would give
    assert float(gpu[..., :3].mean()) > 0.05


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_extended_stack_spectral_parity(built, integrator):
    from oracle import cpu
    s = extended_cornell(48, 48, spp=2)
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=integrator) as ctx:
        table, info = ctx.generate_rgb2spec(32)
        s.rgb2spec = table
        s.scene_data["rgb2specSRGB"] = info
        s.scene_data["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES,
                                                                         abi.RENDER_MODE_SPECTRAL, abi.SPECTRAL_HERO)
        sd = s.scene_data.copy()
        ctx.upload_scene(s)
        ctx.render_frame(sd)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(sd, rng_mode=abi.RNG_PCG32)
    assert_match(None, gpu, ref, 2e-3, 2e-3, max_outside=2)


def test_extended_materials_rejected_by_the_adjoint(built):
    s = extended_cornell(32, 32, spp=1)
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(s)
        with pytest.raises(Exception):
            ctx.render_adjoint(s.scene_data, np.ones((32, 32, 3), np.float32))


def glass_cornell(width=64, height=64, spp=4, rough=0.0, abbe=0.0, absorb=0.0):
    """Both boxes are glass (IOR 1.5) with the given roughness, Abbe number and absorption (tint (0.6, 0.8, 0.9))."""
    s = scenes.cornell(width, height, spp=spp)
    g = s.materials[0].copy()
    g["baseColor"] = [1.0, 1.0, 1.0]
    g["metallic"] = 0.0
    g["roughness"] = rough
    g["specular"] = 0.5
    g["transmission"] = 1.0
    g["ior"] = 1.5
    g["abbeNumber"] = abbe
    g["absorptionCoefficient"] = absorb
    g["attenuationColor"] = [0.6, 0.8, 0.9]
    first = len(s.materials)
    s.materials = np.concatenate([s.materials, g.reshape(1)])
    meshes = s.meshes.copy()
    meshes["materialIndex"][-1] = first
    meshes["materialIndex"][-2] = first
    meshes["position"][-2:, 2] += 2e-3  # off the floor plane: no coplanar glass / floor faces
    s.meshes = meshes
    return s


GLASS = {"smooth": {}, "rough": {"rough": 0.3}, "dispersive": {"abbe": 30.0, "absorb": 2.0}}


@pytest.mark.parametrize("variant", sorted(GLASS))
@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_transmission_rgb_parity(built, integrator, variant):
    from oracle import cpu
    s = glass_cornell(**GLASS[variant])
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        ctx.upload_scene(s)
        ctx.render_frame(s.scene_data)
        gpu = ctx.read_accumulation()
        st = ctx.stats()
    ref, ost = cpu.OracleScene(s).render(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 1e-3, 1e-3, max_outside=2)
    assert np.isfinite(gpu).all()
    # shadow rays of the device and the oracle agree to the share of diverged paths
    assert abs(st["shadowRays"] - ost["shadowRays"]) <= 0.05 * ost["shadowRays"]


@pytest.mark.parametrize("variant", ["smooth", "dispersive"])
@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_transmission_spectral_parity(built, integrator, variant):
    """Hero-wavelength transport through glass; with dispersion refracted paths collapse to their first lane."""
    from oracle import cpu
    s = glass_cornell(48, 48, spp=4, **GLASS[variant])
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        table, info = ctx.generate_rgb2spec(32)
        s.rgb2spec = table
        s.scene_data["rgb2specSRGB"] = info
        s.scene_data["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES,
                                                                         abi.RENDER_MODE_SPECTRAL, abi.SPECTRAL_HERO)
        ctx.upload_scene(s)
        ctx.render_frame(s.scene_data)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 2e-3, 2e-3, max_outside=2)
    assert np.isfinite(gpu).all()


def test_transmissive_materials_rejected_by_the_adjoint_and_the_cache(built):
    s = glass_cornell(32, 32, spp=1)
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(s)
        with pytest.raises(Exception):
            ctx.render_adjoint(s.scene_data, np.ones((32, 32, 3), np.float32))
        ctx.nrc_configure(seed=3, enabled=1)
        with pytest.raises(Exception):
            ctx.render_frame(s.scene_data)


def synthetic_sheen_table():
    """A smooth stand-in for vkrt's sheen LTC table with the same layout and value ranges ([layer][roughness][cos]):
    parity does not depend on the table's values, since the device and the oracle read the same table."""
    c = np.linspace(0.0, 1.0, 32, dtype=np.float32)[None, :]
    r = np.linspace(0.0, 1.0, 32, dtype=np.float32)[:, None]
    a = 0.25 + 0.6 * r + 0.1 * c
    b = 0.2 * (c - 0.5) * (1.0 - r)
    albedo = 0.05 + 0.3 * r * (1.0 - 0.5 * c)
    return np.stack([a + 0 * c, b + 0 * r, albedo]).astype(np.float32).reshape(-1)


def sheen_cornell(width=64, height=64, spp=4, table=True):
    s = scenes.cornell(width, height, spp=spp)
    velvet = s.materials[0].copy()  # red velvet: diffuse base under a bright sheen layer
    velvet["baseColor"] = [0.5, 0.05, 0.05]
    velvet["sheenTintWeight"] = [1.0, 0.9, 0.8, 1.0]
    velvet["sheenRoughness"] = 0.5
    satin = s.materials[0].copy()  # sheen over clear coat over a metal
    satin["metallic"] = 1.0
    satin["roughness"] = 0.4
    satin["baseColor"] = [0.8, 0.7, 0.3]
    satin["sheenTintWeight"] = [0.6, 0.7, 1.0, 0.7]
    satin["sheenRoughness"] = 0.2
    satin["clearcoat"] = 0.5
    first = len(s.materials)
    s.materials = np.concatenate([s.materials, velvet.reshape(1), satin.reshape(1)])
    meshes = s.meshes.copy()
    meshes["materialIndex"][-1] = first
    meshes["materialIndex"][-2] = first + 1
    s.meshes = meshes
    if table:
        s.sheen_table = synthetic_sheen_table()
    return s


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_sheen_rgb_parity(built, integrator):
    from oracle import cpu
    s = sheen_cornell()
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        ctx.upload_scene(s)
        ctx.render_frame(s.scene_data)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 1e-3, 1e-3, max_outside=2)
    # the sheen layer changes the image against the same scene without it
    plain = sheen_cornell(table=False)
    plain.materials["sheenTintWeight"] = 0.0
    ref0, _ = cpu.OracleScene(plain).render(plain.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert np.abs(ref0[..., :3] - ref[..., :3]).max(-1).mean() > 1e-3


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_sheen_spectral_parity(built, integrator):
    from oracle import cpu
    s = sheen_cornell(48, 48, spp=2)
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        table, info = ctx.generate_rgb2spec(32)
        s.rgb2spec = table
        s.scene_data["rgb2specSRGB"] = info
        s.scene_data["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES,
                                                                         abi.RENDER_MODE_SPECTRAL, abi.SPECTRAL_HERO)
        ctx.upload_scene(s)
        ctx.render_frame(s.scene_data)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 2e-3, 2e-3, max_outside=2)


def test_sheen_needs_the_table(built):
    s = sheen_cornell(32, 32, spp=1, table=False)
    with RenderContext(rng_mode=abi.RNG_PCG32) as ctx:
        ctx.upload_scene(s)
        with pytest.raises(Exception):
            ctx.render_frame(s.scene_data)
        with pytest.raises(Exception):
            ctx.upload_sheen_table(np.zeros(100, np.float32))
        ctx.upload_sheen_table(synthetic_sheen_table())
        ctx.render_frame(s.scene_data)


def alpha_cornell(width=64, height=64, spp=4):
    """The tall box is cut out by an alpha-mask checker texture, the short box is half transparent (material
    opacity 0.5, stochastic) and the left wall's mesh opacity is 0.7."""
    s = scenes.cornell(width, height, spp=spp)
    # 8 x 8 cells of 8 x 8 texels: bilinear alpha crosses the cutoff within 1/8 of a cell, so few pixels sit where
    # FP32 rounding of the interpolated uv can flip the cut
    cells = (np.add.outer(np.arange(64) // 8, np.arange(64) // 8) % 2).astype(np.float32)
    checker = np.ones((64, 64, 4), np.float32)
    checker[..., :3] = 0.73
    checker[..., 3] = cells
    s.textures = dict(s.textures)
    s.textures[0] = checker
    cut = s.materials[0].copy()
    cut["baseColorTextureIndex"] = 0
    cut["alphaMode"] = 1
    cut["alphaCutoff"] = 0.5
    veil = s.materials[0].copy()
    veil["baseColor"] = [0.2, 0.3, 0.8]
    veil["opacity"] = 0.5
    first = len(s.materials)
    s.materials = np.concatenate([s.materials, cut.reshape(1), veil.reshape(1)])
    meshes = s.meshes.copy()
    meshes["materialIndex"][-1] = first
    meshes["materialIndex"][-2] = first + 1
    meshes["opacity"][3] = 0.7
    # the boxes' bottoms lie in the floor plane; lifted a little, so that no ray meets an alpha-tested face and the
    # floor at the same distance (which of two coplanar faces is nearer is decided by rounding)
    meshes["position"][-2:, 2] += 2e-3
    s.meshes = meshes
    return s


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_alpha_parity(built, integrator):
    """Alpha mask and blend any-hit tests (rt/alpha_test.slang) on path and shadow rays."""
    from oracle import cpu
    s = alpha_cornell()
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        ctx.upload_scene(s)
        ctx.render_frame(s.scene_data)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 1e-3, 1e-3, max_outside=2)
    opaque = scenes.cornell(64, 64, spp=4)
    ref0, _ = cpu.OracleScene(opaque).render(opaque.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert (np.abs(ref0[..., :3] - ref[..., :3]).max(-1) > 1e-2).mean() > 0.05


def test_alpha_decisions_are_schedule_independent(built):
    """The stochastic alpha decisions hash the ray seed and the triangle: the wavefront render is the same image
    for different slot counts (refill orders)."""
    s = alpha_cornell(48, 48, spp=2)
    imgs = []
    for q in (0, 997):
        with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
            ctx.upload_scene(s)
            ctx.set_wavefront_config(queueCapacity=q)
            ctx.render_frame(s.scene_data)
            imgs.append(ctx.read_accumulation())
    np.testing.assert_array_equal(imgs[0], imgs[1])


@pytest.mark.parametrize("scene", ["cornell", "glass"])
@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_single_wavelength_parity(built, integrator, scene):
    """Single-wavelength spectral mode (raygen_spectral_single.slang, spectral_single/*.slang): one wavelength per
    path, scalar NEE and power-heuristic MIS, dispersive refraction at that wavelength."""
    from oracle import cpu
    s = scenes.cornell(48, 48, spp=4) if scene == "cornell" else glass_cornell(48, 48, spp=4, abbe=30.0, absorb=2.0)
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        table, info = ctx.generate_rgb2spec(32)
        s.rgb2spec = table
        s.scene_data["rgb2specSRGB"] = info
        s.scene_data["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES,
                                                                         abi.RENDER_MODE_SPECTRAL, abi.SPECTRAL_SINGLE)
        ctx.upload_scene(s)
        ctx.render_frame(s.scene_data)
        gpu = ctx.read_accumulation()
    ref, _ = cpu.OracleScene(s).render(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match(None, gpu, ref, 2e-3, 2e-3, max_outside=2)
    assert np.isfinite(gpu).all()
