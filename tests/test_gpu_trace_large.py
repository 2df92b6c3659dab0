"""Closest-hit parity at the benchmarked scene sizes: the full seeded 1,024,000-triangle icosphere field of the
headline frame and the largest scene of the 64-scene uneven batch (465,920 triangles), where the BVH is deepest and
the traversal stack's spill to local memory actually runs.

For each scene, 100,000 seeded camera rays plus secondary rays from their hits in uniform random directions are
traced by both device traversals (one ray per thread, and the wavefront's persistent vote-scheduled traversal) and
must equal the oracle's FP32 BVH2 traversal with the same watertight test bit for bit: mesh and primitive ids, t and
both barycentrics; any-hit answers must agree on occlusion. 2,000 primary and 2,000 secondary rays are also checked
against the FP64 brute-force all-triangle intersector on every ray it does not mark as a near-edge or near-tie case.
The device's error word must stay clear (no traversal stack overflow). Semantics: vkrt's scene query
(rt/queries/scene_query.slang:10-42), no culling, tMin 1e-3, tMax 1e4."""
import numpy as np
import pytest

from test_gpu_trace import _rays_from_camera, _secondary
from vkrt_gb300 import RenderContext, abi, scenes

pytestmark = pytest.mark.gpu

N_RAYS = 100_000
N_FP64 = 2_000
# near-edge / near-tie band of the FP64 classifier, relative to the triangle: FP32 rounding of the watertight test
# on the field's smallest triangles seen from 30 units away reaches about 4e-5 of their size
FP64_EPS = 1e-4


def _largest_batch_scene():
    spec = max(scenes.batch_specs(), key=lambda p: p["n_spheres"])
    return scenes.icosphere_field(**spec)


SCENES = {
    "field-1M": lambda: scenes.icosphere_field(n_spheres=800, width=1920, height=1080, seed=1, spectral=False),
    "batch-466k": _largest_batch_scene,
}


def _assert_bit_exact(g, o, what):
    for k in ("instanceIndex", "primitiveIndex", "t", "u", "v"):
        bad = np.flatnonzero(g[k] != o[k])
        assert len(bad) == 0, f"{what}: {k} differs on {len(bad)} rays (first {bad[:5].tolist()})"


@pytest.mark.parametrize("name", list(SCENES))
def test_large_scene_closest_hit_bit_exact(built, name):
    from oracle import cpu
    scene = SCENES[name]()
    orc = cpu.OracleScene(scene)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        st = ctx.stats()
        assert st["bvhTriangleCount"] == scene.triangle_count
        rays = _rays_from_camera(scene, N_RAYS, 21)
        ref = orc.trace_fp32(rays)
        assert (ref["instanceIndex"] != abi.INVALID_INDEX).mean() > 0.2  # the rays do meet the field
        sec = _secondary(scene, ref, rays, 22)
        ref_sec = orc.trace_fp32(sec)
        ref_any = orc.trace_fp32(sec, any_hit=True)
        for persistent in (False, True):
            tag = f"{name} {'persistent' if persistent else 'per-thread'}"
            g = ctx.trace_rays(rays, persistent=persistent)
            assert ctx.stats()["errorFlags"] == 0, tag
            _assert_bit_exact(g, ref, f"{tag} primary")
            g = ctx.trace_rays(sec, persistent=persistent)
            assert ctx.stats()["errorFlags"] == 0, tag
            _assert_bit_exact(g, ref_sec, f"{tag} secondary")
            g = ctx.trace_rays(sec, any_hit=True, persistent=persistent)
            assert ctx.stats()["errorFlags"] == 0, tag
            np.testing.assert_array_equal(g["instanceIndex"] != abi.INVALID_INDEX,
                                          ref_any["instanceIndex"] != abi.INVALID_INDEX, err_msg=f"{tag} any-hit")


@pytest.mark.parametrize("name", list(SCENES))
def test_large_scene_fp64_bruteforce(built, name):
    from oracle import cpu
    scene = SCENES[name]()
    orc = cpu.OracleScene(scene)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        rays = _rays_from_camera(scene, N_FP64, 31)
        g = ctx.trace_rays(rays, persistent=True)
        sec = _secondary(scene, g, rays, 32)[:N_FP64]
        g2 = ctx.trace_rays(sec, persistent=True)
    for rr, gg, what in ((rays, g, "primary"), (sec, g2, "secondary")):
        f, amb = orc.trace_fp64(rr, eps=FP64_EPS)
        ok = ~amb
        # secondary rays start 1e-3 from the surface they left, inside the tMin band, so more of them are ambiguous
        assert amb.mean() < (0.01 if what == "primary" else 0.15), f"{what}: ambiguous share {amb.mean():.4f}"
        assert ok.sum() > 0.5 * len(rr)
        np.testing.assert_array_equal(gg["instanceIndex"][ok], f["instanceIndex"][ok], err_msg=f"{name} {what}")
        np.testing.assert_array_equal(gg["primitiveIndex"][ok], f["primitiveIndex"][ok], err_msg=f"{name} {what}")
