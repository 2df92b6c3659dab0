"""Denoiser features (albedo / shading normal films) on the GPU against the oracle's restatement of vkrt's feature
rules (bsdf/principled/denoiser.slang, integrator/path/loop.slang:83-111): per-sample parity on a Cornell box with
a mirror box (features followed through the sharp specular hit), for both integrators; running-mean weights over
frames; features off leave the frame untouched."""
import numpy as np
import pytest

from parity import assert_match

from vkrt_gb300 import RenderContext, abi, scenes

pytestmark = pytest.mark.gpu


def _mirror_cornell(coat=False):
    """With `coat`, the mirror box wears a clear coat (a visible layer: features stop there) and the short box is a
    subsurface material with an Oren-Nayar base."""
    s = scenes.cornell(64, 64, spp=4)
    mirror = s.materials[int(s.meshes["materialIndex"][-1])].copy()  # the last box gets its own smooth mirror
    mirror["metallic"] = 1.0
    mirror["roughness"] = 0.0
    mirror["baseColor"] = [0.9, 0.9, 0.9]
    mats = [mirror]
    if coat:
        mirror["clearcoat"] = 1.0
        mirror["clearcoatGloss"] = 1.0
        sss = s.materials[0].copy()
        sss["baseColor"] = [0.8, 0.6, 0.4]
        sss["subsurface"] = 0.8
        sss["diffuseRoughness"] = 0.6
        mats.append(sss)
    first = len(s.materials)
    s.materials = np.concatenate([s.materials] + [m.reshape(1) for m in mats])
    meshes = s.meshes.copy()
    meshes["materialIndex"][-1] = first
    if coat:
        meshes["materialIndex"][-2] = first + 1
    s.meshes = meshes
    return s


@pytest.mark.parametrize("coat", [False, True])
@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_features_match_oracle(built, integrator, coat):
    from oracle import cpu
    s = _mirror_cornell(coat)
    sd = s.scene_data
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        ctx.upload_scene(s)
        ctx.set_denoiser_features(True)
        ctx.render_frame(sd)
        acc = ctx.read_accumulation()
        alb, nrm = ctx.read_denoiser_features()
    ref_acc, ref_alb, ref_nrm = cpu.OracleScene(s).render_features(sd, rng_mode=abi.RNG_REFERENCE)
    assert_match("features mirror: radiance", acc, ref_acc, 1e-3, 1e-3, max_outside=20)
    np.testing.assert_array_equal(alb[..., 3], ref_alb[..., 3])  # resolved-sample counts
    assert_match("features mirror: albedo", alb, ref_alb, 1e-4, 0.0, max_outside=2)
    assert_match("features mirror: normal", nrm, ref_nrm, 1e-4, 0.0, max_outside=2)
    # pixels that see the mirror carry the albedo of what it reflects, not the mirror's 0.9 grey
    assert (alb[..., 3] > 0).mean() > 0.9
    assert np.all(alb[..., 3] <= 4.0)
    # a clear-coated mirror is a visible layer: its pixels keep the mirror's own F0 (0.9) instead of following it
    mirror_albedo = (np.abs(alb[..., :3] - 0.9) < 1e-4).all(-1).mean()
    assert (mirror_albedo > 0.05) if coat else (mirror_albedo == 0.0), mirror_albedo


def test_features_accumulate_over_frames(built):
    s = _mirror_cornell()
    sd = s.scene_data.copy()
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(s)
        ctx.set_denoiser_features(True)
        ws = []
        for f in range(3):
            sd["frameNumber"] = f
            ctx.render_frame(sd)
            ws.append(ctx.read_denoiser_features()[0][..., 3].copy())
        assert np.all(ws[1] >= ws[0]) and np.all(ws[2] >= ws[1])
        assert ws[2].max() <= 12.0 and ws[2].mean() > 8.0
        n = ctx.read_denoiser_features()[1]
        covered = n[..., 3] > 0
        assert np.all(np.linalg.norm(n[..., :3][covered], axis=-1) <= 1.0 + 1e-5)
        ctx.reset_accumulation()
        assert ctx.read_denoiser_features()[0][..., 3].max() == 0.0
        acc_on = ctx.read_accumulation()
        ctx.set_denoiser_features(False)
        with pytest.raises(Exception):
            ctx.read_denoiser_features()
    # features do not change the image: same frame with features off (the feature frame runs the full-stack kernel,
    # whose arithmetic is ordered differently, so equal to float rounding)
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as a, \
            RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as b:
        a.upload_scene(s)
        b.upload_scene(s)
        b.set_denoiser_features(True)
        a.render_frame(s.scene_data)
        b.render_frame(s.scene_data)
        np.testing.assert_allclose(a.read_accumulation(), b.read_accumulation(), rtol=1e-5, atol=1e-7)
    del acc_on


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_features_through_glass_match_oracle(built, integrator):
    """Smooth glass is followed through (denoiser.slang:13-21): the albedo behind it is taken."""
    from oracle import cpu
    from tests.test_gpu_materials import glass_cornell
    s = glass_cornell()
    with RenderContext(rng_mode=abi.RNG_REFERENCE, integrator=integrator) as ctx:
        ctx.upload_scene(s)
        ctx.set_denoiser_features(True)
        ctx.render_frame(s.scene_data)
        alb, nrm = ctx.read_denoiser_features()
    _, ref_alb, ref_nrm = cpu.OracleScene(s).render_features(s.scene_data, rng_mode=abi.RNG_REFERENCE)
    assert_match("features glass: albedo", alb, ref_alb, 1e-4, 0.0, max_outside=2)
    assert_match("features glass: normal", nrm, ref_nrm, 1e-4, 0.0, max_outside=2)
