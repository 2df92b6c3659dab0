"""Wavefront integrator (wavefront.cu): same estimator, same random streams and same per-vertex arithmetic as the
megakernel, so images agree with the megakernel's to float rounding; material sorting, graph capture and tile
order change only the schedule, never the result; a batch of uneven scenes renders each scene as if alone."""
import numpy as np
import pytest

from vkrt_gb300 import RenderContext, abi, scenes
from vkrt_gb300.context import autotune_batch, render_batch

pytestmark = pytest.mark.gpu


def _render(scene, integrator, frames=1, wf=None, viewport=None, **kw):
    with RenderContext(integrator=integrator, **kw) as ctx:
        ctx.upload_scene(scene)
        if wf:
            ctx.set_wavefront_config(**wf)
        sd = scene.scene_data.copy()
        if viewport is not None:
            sd["viewportRect"] = viewport
        for f in range(frames):
            sd["frameNumber"] = f
            ctx.render_frame(sd)
        return ctx.read_accumulation(), ctx.stats()


def _assert_same(a, b, rtol=2e-5):
    np.testing.assert_array_equal(a[..., 3], b[..., 3])
    np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=rtol, atol=1e-6)


@pytest.mark.parametrize("spectral", [False, True])
def test_wavefront_matches_megakernel(built, spectral):
    scene = scenes.cornell(96, 80, spp=3)
    if spectral:
        with RenderContext() as ctx:
            table, info = ctx.generate_rgb2spec(24)
        scene.rgb2spec = table
        scene.scene_data["rgb2specSRGB"] = info
        scene.scene_data["packedRenderSettings"] = abi.pack_render_settings(1, abi.RENDER_MODE_SPECTRAL, 1)
    mega, ms = _render(scene, abi.INTEGRATOR_MEGAKERNEL, frames=2)
    wave, ws = _render(scene, abi.INTEGRATOR_WAVEFRONT, frames=2, wf={"queueCapacity": 4096})
    _assert_same(wave, mega)
    for k in ("primaryRays", "extensionRays", "shadowRays", "pathSamples"):
        assert ws[k] == ms[k], k


def test_wavefront_schedule_independence(built):
    scene = scenes.icosphere_field(n_spheres=40, width=72, height=40, spp=4, max_depth=6, seed=5, spectral=False,
                                   env_size=(64, 32))
    kw = dict(rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_IMPORTANCE)
    base, _ = _render(scene, abi.INTEGRATOR_WAVEFRONT, wf={"queueCapacity": 0}, **kw)
    for wf in ({"sortByMaterial": 1}, {"sortByMaterial": 2}, {"useGraph": 0},
               {"tileWidth": 4, "tileHeight": 4, "queueCapacity": 300, "sortByMaterial": 2},
               {"queueCapacity": 97, "sortByMaterial": 1, "intersectBlocksPerSM": 2},
               {"rayOrder": 1}, {"rayOrder": 1, "sortByMaterial": 0}, {"rayOrder": 1, "sortByMaterial": 1},
               {"rayOrder": 1, "queueCapacity": 300, "useGraph": 0}, {"sortByMaterial": 3},
               {"sortByMaterial": 3, "queueCapacity": 300}):
        got, _ = _render(scene, abi.INTEGRATOR_WAVEFRONT, wf=wf, **kw)
        np.testing.assert_array_equal(got, base, err_msg=str(wf))
    # another shade residency is another compiled kernel (its register budget changes inlining and so which
    # multiply-adds fuse): equal to float rounding, not bit for bit
    for blocks in (3, 6, 8):
        got, _ = _render(scene, abi.INTEGRATOR_WAVEFRONT, wf={"shadeBlocksPerSM": blocks, "queueCapacity": 97}, **kw)
        _assert_same(got, base, rtol=1e-5)
    mega, _ = _render(scene, abi.INTEGRATOR_MEGAKERNEL, **kw)
    _assert_same(base, mega)


def test_wavefront_viewport_subrect(built):
    scene = scenes.cornell(64, 48, spp=2)
    mega, _ = _render(scene, abi.INTEGRATOR_MEGAKERNEL, viewport=(8, 4, 40, 30))
    wave, _ = _render(scene, abi.INTEGRATOR_WAVEFRONT, viewport=(8, 4, 40, 30))
    _assert_same(wave, mega)
    assert (wave[:4] == 0).all() and (wave[:, :8] == 0).all()


def test_batch_pipelined_readback(built):
    """vkrt_cuda_read_accumulation_async on every context of a batch: the batch leader's stream waits for each
    context's copy in flight before a batched frame overwrites that context's buffer, so every copy equals the
    synchronous read of the same frame in a second batch."""
    torch = pytest.importorskip("torch")
    specs = [dict(n_spheres=20, width=48, height=32, seed=1), dict(n_spheres=30, width=64, height=40, seed=2)]
    ss = [scenes.icosphere_field(spp=2, max_depth=5, spectral=False, env_size=(64, 32), **p) for p in specs]
    kw = dict(rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_IMPORTANCE)
    frames = 4

    def run(pipelined):
        ctxs = [RenderContext(integrator=abi.INTEGRATOR_WAVEFRONT, **kw) for _ in ss]
        try:
            for c, s in zip(ctxs, ss):
                c.upload_scene(s)
            out = [[torch.empty((c.height, c.width, 4), dtype=torch.float32, pin_memory=True).numpy() for c in ctxs]
                   for _ in range(frames)]
            sds = np.concatenate([s.scene_data for s in ss])
            for f in range(frames):
                sds["frameNumber"] = f
                render_batch(ctxs, sds)
                for c, o in zip(ctxs, out[f]):
                    if pipelined:
                        c.read_accumulation_async(o)
                    else:
                        o[:] = c.read_accumulation()
            for c in ctxs:
                c.wait_readback()
            return out
        finally:
            for c in ctxs:
                c.close()

    want, got = run(False), run(True)
    for f in range(frames):
        for g, w in zip(got[f], want[f]):
            np.testing.assert_array_equal(g, w)


def test_batch_of_uneven_scenes(built):
    specs = [dict(n_spheres=20, width=48, height=32, seed=1), dict(n_spheres=60, width=80, height=64, seed=2),
             dict(n_spheres=8, width=32, height=32, seed=3)]
    ss = [scenes.icosphere_field(spp=2, max_depth=5, spectral=False, env_size=(64, 32), **p) for p in specs]
    kw = dict(rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_IMPORTANCE)
    alone = [_render(s, abi.INTEGRATOR_MEGAKERNEL, **kw)[0] for s in ss]
    ctxs = [RenderContext(integrator=abi.INTEGRATOR_WAVEFRONT, **kw) for _ in ss]
    try:
        for c, s in zip(ctxs, ss):
            c.upload_scene(s)
        sds = np.concatenate([s.scene_data for s in ss])
        render_batch(ctxs, sds)
        got = [c.read_accumulation() for c in ctxs]
        for g, a in zip(got, alone):
            _assert_same(g, a)
        best, ms = autotune_batch(ctxs, sds, frames_per_trial=1)
        assert ms > 0 and best["tileWidth"][0] >= 1 and best["intersectBlocksPerSM"][0] >= 1
        # after tuning (which clears the films) the batch still reproduces the single-scene renders
        render_batch(ctxs, sds)
        for c, a in zip(ctxs, alone):
            _assert_same(c.read_accumulation(), a)
    finally:
        for c in ctxs:
            c.close()


def test_batch_of_mixed_material_scenes(built):
    """A batch holding a glass scene, an alpha-tested scene and a reflection-only scene runs the full-stack, alpha
    and transmissive-shadow kernels for all three; each scene's image equals its single-scene wavefront render
    (the reflection-only scene's to float rounding: it is shaded by the full-stack kernel in the batch)."""
    from tests.test_gpu_materials import alpha_cornell, glass_cornell
    ss = [glass_cornell(48, 40, spp=2, abbe=30.0, absorb=2.0), alpha_cornell(40, 48, spp=2), scenes.cornell(32, 32, spp=2)]
    kw = dict(rng_mode=abi.RNG_PCG32)
    alone = [_render(s, abi.INTEGRATOR_WAVEFRONT, **kw)[0] for s in ss]
    ctxs = [RenderContext(integrator=abi.INTEGRATOR_WAVEFRONT, **kw) for _ in ss]
    try:
        for c, s in zip(ctxs, ss):
            c.upload_scene(s)
        render_batch(ctxs, np.concatenate([s.scene_data for s in ss]))
        for c, a in zip(ctxs, alone):
            g = c.read_accumulation()
            np.testing.assert_array_equal(g[..., 3], a[..., 3])
            close = (np.abs(g[..., :3] - a[..., :3]) <= 1e-5 + 1e-4 * np.abs(a[..., :3])).all(-1)
            assert close.mean() > 0.99, close.mean()
    finally:
        for c in ctxs:
            c.close()


def test_ray_order_with_alpha_and_glass(built):
    """Direction-octant queue bins and the material-ordered shade queue feed the alpha-tested traversal and the
    full-stack kernels the same paths: the images equal the default order's bit for bit."""
    from tests.test_gpu_materials import alpha_cornell, glass_cornell
    for s in (alpha_cornell(40, 48, spp=2), glass_cornell(48, 40, spp=2, abbe=30.0, absorb=2.0)):
        base, _ = _render(s, abi.INTEGRATOR_WAVEFRONT, rng_mode=abi.RNG_PCG32)
        for wf in ({"rayOrder": 1}, {"sortByMaterial": 3}):
            got, _ = _render(s, abi.INTEGRATOR_WAVEFRONT, wf=wf, rng_mode=abi.RNG_PCG32)
            np.testing.assert_array_equal(got, base, err_msg=str(wf))
