"""The extended reflection stack (clearcoat, Oren-Nayar diffuse, fake subsurface; principled/eval_rgb.slang and
lobes/clearcoat.slang, diffuse.slang, subsurface.slang) on the GPU against the oracle's restatement: per-sample
parity on a Cornell box whose boxes and floor use those lobes, for both integrators, in RGB and hero-spectral mode."""
import numpy as np
import pytest

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
    close = (np.abs(gpu[..., :3] - ref[..., :3]) <= 1e-3 + 1e-3 * np.abs(ref[..., :3])).all(-1)
    assert close.mean() > 0.97, close.mean()
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
    close = (np.abs(gpu[..., :3] - ref[..., :3]) <= 2e-3 + 2e-3 * np.abs(ref[..., :3])).all(-1)
    assert close.mean() > 0.95, close.mean()


def test_extended_materials_rejected_by_the_adjoint(built):
    s = extended_cornell(32, 32, spp=1)
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(s)
        with pytest.raises(Exception):
            ctx.render_adjoint(s.scene_data, np.ones((32, 32, 3), np.float32))
