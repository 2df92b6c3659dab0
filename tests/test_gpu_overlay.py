"""Selection passes and frame timing through the C ABI on the GPU: the selection mask against the oracle's FP64
brute force over the selected mesh alone, the outline pass bit-exact against the oracle restatement, pick queries
against the FP64 closest hit, and the auto-SPP loop driven by the device frame time."""
import numpy as np
import pytest

from oracle import overlay
from vkrt_gb300 import AutoSpp, RenderContext, abi, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def field(built):
    s = scenes.icosphere_field(n_spheres=60, width=240, height=136, spp=1, max_depth=4, seed=5, spectral=False,
                               env_size=(64, 32))
    ctx = RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT)
    ctx.upload_scene(s)
    yield s, ctx
    ctx.close()


def _visible_meshes(s, ctx, n):
    """Meshes under a grid of pixels, most covered first."""
    sd = s.scene_data
    got = {}
    for y in range(4, s.height, 12):
        for x in range(4, s.width, 12):
            m = ctx.pick_mesh(sd, x, y)
            if m != abi.INVALID_INDEX:
                got[m] = got.get(m, 0) + 1
    return [m for m, _ in sorted(got.items(), key=lambda kv: -kv[1])][:n]


def test_pick_matches_fp64_closest_hit(field):
    from oracle import cpu
    s, ctx = field
    rng = np.random.default_rng(3)
    agree = amb = 0
    orc = cpu.OracleScene(s)
    for _ in range(48):
        x, y = int(rng.integers(0, s.width)), int(rng.integers(0, s.height))
        want, ambiguous = overlay.pick_mesh(s, s.scene_data, x, y, orc)
        got = ctx.pick_mesh(s.scene_data, x, y)
        if ambiguous:
            amb += 1
            continue
        assert got == want, (x, y, got, want)
        agree += 1
    orc.close()
    assert agree >= 40


def test_selection_mask_and_outline(field):
    s, ctx = field
    for mesh in _visible_meshes(s, ctx, 3):
        sd = s.scene_data.copy()
        sd["selectionEnabled"] = 1
        sd["selectedMeshIndex"] = mesh
        ctx.render_frame(sd)
        before = ctx.read_output()
        ctx.render_selection_overlay(sd)
        mask = ctx.read_selection_mask()
        after = ctx.read_output()
        want, amb = overlay.selection_mask(s, sd, s.width, s.height)
        assert want.sum() > 5
        diff = (mask != want) & ~amb
        assert diff.sum() <= 2, (mesh, int(diff.sum()), int(want.sum()))
        # the outline of the device mask, bit-exact
        np.testing.assert_array_equal(after, overlay.outline(mask, before))
        assert (after != before).any()


def test_selection_disabled_clears_mask(field):
    s, ctx = field
    sd = s.scene_data.copy()
    sd["selectionEnabled"] = 1
    sd["selectedMeshIndex"] = _visible_meshes(s, ctx, 1)[0]
    ctx.render_selection_overlay(sd)
    assert ctx.read_selection_mask().sum() > 0
    sd["selectionEnabled"] = 0
    ctx.render_frame(sd)
    before = ctx.read_output()
    ctx.render_selection_overlay(sd)
    assert ctx.read_selection_mask().sum() == 0
    np.testing.assert_array_equal(ctx.read_output(), before)


def test_selection_rejects_bad_mesh(field):
    s, ctx = field
    sd = s.scene_data.copy()
    sd["selectionEnabled"] = 1
    sd["selectedMeshIndex"] = 10_000
    with pytest.raises(Exception):
        ctx.render_selection_overlay(sd)


def test_auto_spp_follows_the_frame_budget(built):
    """Cornell box frames whose spp the controller sets from vkrt_cuda_last_frame_ms: spp grows from 1 and the frame
    time settles under the 240 FPS budget."""
    s = scenes.cornell(256, 256, spp=1, max_depth=8)
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(s)
        sd = s.scene_data.copy()
        c = AutoSpp(240)
        spp, times = 1, []
        for f in range(48):
            sd["samplesPerPixel"] = spp
            sd["frameNumber"] = f
            ctx.render_frame(sd)
            ms = ctx.last_frame_ms()
            times.append((spp, ms))
            spp = c.update(ms, spp)
    last_spp, last_ms = times[-1]
    assert last_spp > 4, times[-8:]
    assert last_ms < 1.1 * c.target_ms, times[-8:]


def test_selection_and_pick_drop_mask_cut_outs(built):
    """A mesh with an alpha-mask checker: its selection mask has the cut-outs as holes, and picks through a hole
    name what lies behind (selectionAlphaHitAccepted, rt/alpha_test.slang:68-76)."""
    from oracle import cpu
    from tests.test_gpu_materials import alpha_cornell
    s = alpha_cornell(96, 96, spp=1)
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(s)
        sd = s.scene_data.copy()
        sd["selectionEnabled"] = 1
        sd["selectedMeshIndex"] = 7  # the cut-out box
        ctx.render_frame(sd)
        ctx.render_selection_overlay(sd)
        mask = ctx.read_selection_mask()
        want, _ = overlay.selection_mask(s, sd, 96, 96)
        assert want.sum() > 50
        assert (mask != want).mean() <= 0.002, int((mask != want).sum())
        orc = cpu.OracleScene(s)
        picks = [(x, y) for y in range(8, 96, 6) for x in range(8, 96, 6)]
        same = sum(ctx.pick_mesh(sd, x, y) == overlay.pick_mesh(s, sd, x, y, orc)[0] for x, y in picks)
        assert same >= len(picks) - 1, (same, len(picks))
    # the same box without the cut-out covers more pixels
    opaque = alpha_cornell(96, 96, spp=1)
    opaque.materials["alphaMode"][-2] = 0
    full, _ = overlay.selection_mask(opaque, sd, 96, 96)
    assert full.sum() > want.sum()
