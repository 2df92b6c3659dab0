"""vkrt_cuda_trace_rays_noalloc: the allocation-free trace entry point.

Callers on a real-time frame thread or under a fixed device-memory budget cannot let the backend call cudaMalloc /
cudaFree per trace (cudaFree synchronises the whole device). This entry point stages rays and hits in fixed device
arrays instead. Here it is called through the C ABI exactly as such a caller would, twice in a row on different ray
sets, and must return the same hit records as the allocating entry point vkrt_cuda_trace_rays (both run the same
traversal kernel, so the comparison is exact). The file name sorts last so that a run stopping at the first failure
has already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from vkrt_gb300 import RenderContext, abi, scenes

pytestmark = pytest.mark.gpu

MAX_RAYS = 65536


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, dtype=abi.RAY)
    r["origin"] = rng.uniform(0.05, 0.95, size=(n, 3))
    d = rng.normal(size=(n, 3))
    r["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r["tMin"] = 1e-3
    r["tMax"] = 1e4
    return r


def _noalloc(ctx, rays, any_hit=0):
    hits = np.zeros(len(rays), dtype=abi.HIT)
    rc = ctx.lib.vkrt_cuda_trace_rays_noalloc(ctx.handle, abi.ptr(rays), len(rays), any_hit, abi.ptr(hits))
    return rc, hits


def test_noalloc_trace_matches_allocating_trace(built):
    scene = scenes.cornell(32, 32)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        # two calls in a row: the second uses fewer rays, so stale hits from the first call must not leak through
        for n, seed, any_hit in ((MAX_RAYS, 1, 0), (5000, 2, 0), (3000, 3, 1)):
            rays = _rays(n, seed)
            rc, got = _noalloc(ctx, rays, any_hit)
            assert rc == abi.SUCCESS, ctx.lib.vkrt_cuda_last_error(ctx.handle)
            want = ctx.trace_rays(rays, any_hit=bool(any_hit))
            for f in ("instanceIndex", "primitiveIndex", "t", "u", "v"):
                np.testing.assert_array_equal(got[f], want[f], err_msg=f)
            assert (got["instanceIndex"] != abi.INVALID_INDEX).mean() > 0.5


def test_noalloc_rejects_more_than_the_scratch_holds(built):
    scene = scenes.cornell(16, 16)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        rays = _rays(MAX_RAYS + 1, 4)
        rc, _ = _noalloc(ctx, rays)
        assert rc == abi.ERROR_INVALID_ARGUMENT
        assert b"65536" in ctx.lib.vkrt_cuda_last_error(ctx.handle)
        # the context stays usable
        rc, got = _noalloc(ctx, rays[:100])
        assert rc == abi.SUCCESS
        np.testing.assert_array_equal(got["primitiveIndex"], ctx.trace_rays(rays[:100])["primitiveIndex"])


def test_noalloc_makes_no_device_allocation(built):
    """After one warm-up call (the driver may size the kernel's local-memory reservation on its first launch), the
    entry point leaves the device's free memory unchanged across calls of every size up to the cap."""
    torch = pytest.importorskip("torch")
    scene = scenes.cornell(32, 32)
    with RenderContext() as ctx:
        ctx.upload_scene(scene)
        rays = _rays(MAX_RAYS, 5)
        torch.cuda.mem_get_info()
        rc, _ = _noalloc(ctx, rays)
        assert rc == abi.SUCCESS
        ctx.sync()
        free0, _ = torch.cuda.mem_get_info()
        for n, any_hit in ((MAX_RAYS, 0), (1000, 1), (MAX_RAYS, 1), (17, 0)):
            rc, _ = _noalloc(ctx, rays[:n], any_hit)
            assert rc == abi.SUCCESS
        ctx.sync()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, (free0, free1)
