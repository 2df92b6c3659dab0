"""Render parity of the megakernel (render.cu) against the oracle's restatement of vkrt's integrators.

Per-sample parity: with vkrt's own random stream (seed = f(pixel, frame, sample)) both renders follow the same paths,
so pixels agree to FP32 rounding except where a rounding difference flips a branch; the share of matching pixels is
bounded from below. Precision: relative MSE of the FP32 device render against the oracle's FP64 render of the same
seeds is <= 1e-3. Statistics: 16 x 16 tile means of independent device and oracle renders agree within a 99%
confidence interval."""
import numpy as np
import pytest

from parity import assert_match

from vkrt_gb300 import RenderContext, abi, scenes

pytestmark = pytest.mark.gpu


def relmse(x, ref):
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))


def _render_gpu(scene, frames=1, **ctx_kw):
    with RenderContext(**ctx_kw) as ctx:
        ctx.upload_scene(scene)
        sd = scene.scene_data.copy()
        for f in range(frames):
            sd["frameNumber"] = f
            ctx.render_frame(sd)
        return ctx.read_accumulation(), ctx.stats()


@pytest.mark.parametrize("rng_mode", [abi.RNG_REFERENCE, abi.RNG_PCG32])
def test_cornell_per_sample_parity(built, rng_mode):
    from oracle import cpu
    scene = scenes.cornell(96, 96, spp=4)
    gpu, st = _render_gpu(scene, rng_mode=rng_mode)
    ref, ost = cpu.OracleScene(scene).render(scene.scene_data, rng_mode=rng_mode)
    assert_match(None, gpu, ref, 1e-3, 1e-3, max_outside=2)
    np.testing.assert_array_equal(gpu[..., 3], 4.0)
    assert st["primaryRays"] == ost["primaryRays"] == 96 * 96 * 4
    # ray counts agree to the share of diverged paths
    assert abs(st["extensionRays"] - ost["extensionRays"]) <= 0.03 * ost["extensionRays"]
    assert abs(st["shadowRays"] - ost["shadowRays"]) <= 0.03 * ost["shadowRays"]


def test_cornell_fp64_relmse(built):
    from oracle import cpu
    scene = scenes.cornell(64, 64, spp=8)
    gpu, _ = _render_gpu(scene)
    ref64, _ = cpu.OracleScene(scene).render(scene.scene_data, precision=64)
    assert relmse(gpu[..., :3], ref64[..., :3]) <= 1e-3


def test_cornell_tile_means_ci(built):
    from oracle import cpu
    scene = scenes.cornell(128, 128, spp=16)
    gpu, _ = _render_gpu(scene, rng_mode=abi.RNG_PCG32)
    ref, _ = cpu.OracleScene(scene).render(scene.scene_data, rng_mode=abi.RNG_REFERENCE)
    # 16x16 tiles: independent estimators (different streams); z-test on the tile means with the pooled variance
    t = 16
    g = gpu[..., :3].reshape(128 // t, t, 128 // t, t, 3)
    r = ref[..., :3].reshape(128 // t, t, 128 // t, t, 3)
    gm, rm = g.mean((1, 3)), r.mean((1, 3))
    gv, rv = g.var((1, 3), ddof=1) / (t * t), r.var((1, 3), ddof=1) / (t * t)
    z = np.abs(gm - rm) / np.sqrt(gv + rv + 1e-12)
    # 99% two-sided per tile; allow the expected 1% of tiles (plus slack) to fall outside
    assert (z > 2.576).mean() <= 0.03, (z > 2.576).mean()


def test_hero_spectral_parity(built):
    from oracle import cpu
    scene = scenes.cornell(64, 64, spp=4)
    with RenderContext() as ctx:
        table, info = ctx.generate_rgb2spec(32)
    scene.rgb2spec = table
    scene.scene_data["rgb2specSRGB"] = info
    scene.scene_data["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES,
                                                                        abi.RENDER_MODE_SPECTRAL, abi.SPECTRAL_HERO)
    gpu, _ = _render_gpu(scene)
    ref, _ = cpu.OracleScene(scene).render(scene.scene_data)
    assert_match(None, gpu, ref, 2e-3, 2e-3, max_outside=2)


def test_environment_importance_sampling_unbiased(built):
    """Env NEE + MIS (new estimator) and vkrt's BSDF-only estimator converge to the same image."""
    scene = scenes.icosphere_field(n_spheres=30, width=64, height=48, spp=64, max_depth=4, seed=3, spectral=False,
                                   env_size=(128, 64))
    a, _ = _render_gpu(scene, rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_BSDF_ONLY)
    b, _ = _render_gpu(scene, rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_IMPORTANCE)
    am, bm = a[..., :3].mean(), b[..., :3].mean()
    assert abs(am - bm) <= 0.05 * am, (am, bm)


def test_accumulation_running_mean(built):
    scene = scenes.cornell(32, 32, spp=2)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        sd = scene.scene_data.copy()
        ctx.render_frame(sd)
        first = ctx.read_accumulation().copy()
        sd["frameNumber"] = 1
        ctx.render_frame(sd)
        second = ctx.read_accumulation()
    np.testing.assert_array_equal(first[..., 3], 2.0)
    np.testing.assert_array_equal(second[..., 3], 4.0)
    assert not np.array_equal(first[..., :3], second[..., :3])


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
def test_pipelined_readback_matches_synchronous(built, integrator):
    """vkrt_cuda_read_accumulation_async: each frame's accumulation, copied on the context's copy stream while the
    following frames render (the next one blending from it, the one after overwriting its buffer), equals the
    synchronous read of the same frame in a second context; a film reset and a resize wait for copies in flight."""
    torch = pytest.importorskip("torch")
    scene = scenes.cornell(96, 64, spp=2)
    frames = 5
    expected = []
    with RenderContext(integrator=integrator) as ctx:
        ctx.upload_scene(scene)
        sd = scene.scene_data.copy()
        for f in range(frames):
            sd["frameNumber"] = f
            ctx.render_frame(sd)
            expected.append(ctx.read_accumulation().copy())
    pinned = [torch.empty((64, 96, 4), dtype=torch.float32, pin_memory=True) for _ in range(frames)]
    with RenderContext(integrator=integrator) as ctx:
        ctx.upload_scene(scene)
        sd = scene.scene_data.copy()
        for f in range(frames):
            sd["frameNumber"] = f
            ctx.render_frame(sd)
            ctx.read_accumulation_async(pinned[f].numpy())
        ctx.reset_accumulation()
        ctx.render_frame(sd)
        ctx.wait_readback()
        for f in range(frames):
            np.testing.assert_array_equal(pinned[f].numpy(), expected[f])
        ctx.read_accumulation_async(pinned[0].numpy())
        ctx.resize(48, 32)
        ctx.wait_readback()
        np.testing.assert_array_equal(pinned[0].numpy()[..., 3], 2.0)  # the frame after the reset


def test_frame_validation(built):
    """Frames the backend cannot render as vkrt would are refused, not rendered differently: debug views, unknown
    spectral modes, spectral frames without an rgb2spec table; the context stays usable."""
    scene = scenes.cornell(16, 16, spp=1)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        for field, value in (("debugMode", 3), ("debugMode", 16)):
            sd = scene.scene_data.copy()
            sd[field] = value
            with pytest.raises(Exception):
                ctx.render_frame(sd)
        sd = scene.scene_data.copy()
        sd["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES, abi.RENDER_MODE_SPECTRAL, 7)
        with pytest.raises(Exception):
            ctx.render_frame(sd)
        ctx.render_frame(scene.scene_data)
        assert np.isfinite(ctx.read_accumulation()).all()
