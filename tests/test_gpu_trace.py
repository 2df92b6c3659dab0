"""Closest-hit / any-hit parity of the device BVH traversal (bvh_build.cu + traverse.cuh) through the C ABI.

Two oracles: the oracle's FP32 BVH2 traversal with the same watertight test (must agree bit for bit on every ray,
ids and t), and the FP64 brute-force all-triangle intersector (must agree on every ray it does not mark as a
near-tie / near-edge case; the ambiguous share is reported and bounded)."""
import numpy as np
import pytest

from vkrt_gb300 import RenderContext, abi, scenes

pytestmark = pytest.mark.gpu


def _rays_from_camera(scene, n, seed, bounce=False):
    rng = np.random.default_rng(seed)
    sd = scene.scene_data[0]
    vi = sd["viewInverse"]
    pi = sd["projInverse"]
    ndc = rng.uniform(-1, 1, size=(n, 2))
    v4 = np.stack([ndc[:, 0], ndc[:, 1], np.ones(n), np.ones(n)], 1) @ pi.astype(np.float64)
    d = v4[:, :3] @ vi[:3, :3].astype(np.float64)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, dtype=abi.RAY)
    rays["origin"] = vi[3, :3]
    rays["direction"] = d
    rays["tMin"] = 1e-3
    rays["tMax"] = 1e4
    return rays


def _secondary(scene, hits, rays, seed):
    """Secondary rays from the primary hit points in random directions (cosine-free uniform sphere)."""
    rng = np.random.default_rng(seed)
    ok = hits["instanceIndex"] != abi.INVALID_INDEX
    p = rays["origin"][ok] + rays["direction"][ok] * hits["t"][ok][:, None]
    d = rng.normal(size=(ok.sum(), 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.zeros(ok.sum(), dtype=abi.RAY)
    out["origin"] = p - 1e-3 * rays["direction"][ok]
    out["direction"] = d
    out["tMin"] = 1e-3
    out["tMax"] = 1e4
    return out


def _check(scene, ctx, rays, any_hit=False):
    from oracle import cpu
    orc = cpu.OracleScene(scene)
    g = ctx.trace_rays(rays, any_hit=any_hit)
    o = orc.trace_fp32(rays, any_hit=any_hit)
    if any_hit:
        np.testing.assert_array_equal(g["instanceIndex"] != abi.INVALID_INDEX, o["instanceIndex"] != abi.INVALID_INDEX)
        return g
    np.testing.assert_array_equal(g["instanceIndex"], o["instanceIndex"])
    np.testing.assert_array_equal(g["primitiveIndex"], o["primitiveIndex"])
    np.testing.assert_array_equal(g["t"], o["t"])
    np.testing.assert_array_equal(g["u"], o["u"])
    np.testing.assert_array_equal(g["v"], o["v"])
    return g


@pytest.mark.parametrize("seed", [1, 2])
def test_cornell_primary_and_secondary_bit_exact(built, seed):
    scene = scenes.cornell(64, 64)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        rays = _rays_from_camera(scene, 20000, seed)
        hits = _check(scene, ctx, rays)
        sec = _secondary(scene, hits, rays, seed + 100)
        _check(scene, ctx, sec)
        _check(scene, ctx, sec, any_hit=True)


def test_cornell_fp64_bruteforce(built):
    from oracle import cpu
    scene = scenes.cornell(64, 64)
    orc = cpu.OracleScene(scene)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        rays = _rays_from_camera(scene, 20000, 3)
        g = ctx.trace_rays(rays)
        sec = _secondary(scene, g, rays, 5)
        g2 = ctx.trace_rays(sec)
    for rr, gg in ((rays, g), (sec, g2)):
        f, amb = orc.trace_fp64(rr)
        ok = ~amb
        assert amb.mean() < 0.01, f"ambiguous share {amb.mean():.4f}"
        np.testing.assert_array_equal(gg["instanceIndex"][ok], f["instanceIndex"][ok])
        np.testing.assert_array_equal(gg["primitiveIndex"][ok], f["primitiveIndex"][ok])


def test_icosphere_field_bit_exact(built):
    scene = scenes.icosphere_field(n_spheres=60, width=320, height=180, seed=4, spectral=False, env_size=(64, 32))
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        st = ctx.stats()
        assert st["bvhTriangleCount"] == scene.triangle_count
        rays = _rays_from_camera(scene, 30000, 9)
        hits = _check(scene, ctx, rays)
        sec = _secondary(scene, hits, rays, 11)
        _check(scene, ctx, sec)
        _check(scene, ctx, sec, any_hit=True)


def test_bvh_build_options(built):
    """Treelet restructuring runs from treeletMinTriangles up (default 65,536), treeletPasses times, and, after
    mesh-transform edits, only when treeletsOnUpdate asks; every variant of the tree traces bit for bit like the
    oracle."""
    scene = scenes.icosphere_field(n_spheres=60, width=64, height=48, seed=4, spectral=False, env_size=(64, 32))
    rays = _rays_from_camera(scene, 20000, 13)
    with RenderContext() as ctx:  # 76,800 triangles: restructured
        ctx.upload_scene(scene)
        st = ctx.stats()
        assert st["bvhSahTreelets"] < st["bvhSahLbvh"]
        _check(scene, ctx, rays)
        moved = scene.meshes.copy()
        moved["position"][::7] += np.float32(0.5)  # a transform edit: rebuilt as the plain LBVH
        ctx.update_meshes(moved)
        st = ctx.stats()
        assert st["bvhSahTreelets"] == st["bvhSahLbvh"]
        edited = scenes.icosphere_field(n_spheres=60, width=64, height=48, seed=4, spectral=False, env_size=(64, 32))
        edited.meshes = moved
        _check(edited, ctx, rays)
    with RenderContext(treelet_min_triangles=0xFFFFFFFF) as ctx:
        ctx.upload_scene(scene)
        st = ctx.stats()
        assert st["bvhSahTreelets"] == st["bvhSahLbvh"]
        _check(scene, ctx, rays)
    with RenderContext(treelets_on_update=True) as ctx:
        ctx.upload_scene(scene)
        ctx.update_meshes(moved)
        st = ctx.stats()
        assert st["bvhSahTreelets"] < st["bvhSahLbvh"]
        _check(edited, ctx, rays)
    sah = {}
    for passes in (1, 3):  # repeated bottom-up passes (default 2) never raise the cost and trace the same hits
        with RenderContext(treelet_passes=passes) as ctx:
            ctx.upload_scene(scene)
            sah[passes] = ctx.stats()["bvhSahTreelets"]
            _check(scene, ctx, rays)
    assert sah[3] <= sah[1] * (1.0 + 1e-6)
    small = scenes.cornell(32, 32)
    with RenderContext() as ctx:  # 36 triangles: no restructuring
        ctx.upload_scene(small)
        st = ctx.stats()
        assert st["bvhSahTreelets"] == st["bvhSahLbvh"]
    small_rays = _rays_from_camera(small, 4096, 17)
    with RenderContext(treelet_min_triangles=1, treelet_passes=8) as ctx:  # forced: one block, most lanes idle
        ctx.upload_scene(small)
        st = ctx.stats()
        assert st["bvhSahTreelets"] <= st["bvhSahLbvh"]
        _check(small, ctx, small_rays)
