"""Neural radiance cache kernels (nrc.cu) against the FP64 oracle (oracle/nrc.py): predictions, loss and the gradients
of the FP16 tensor-core forward/backward with respect to the MLP weights and the hash table, on the same FP16
parameters. FP16 activations limit agreement to about a percent, which the tolerances state."""
import numpy as np
import pytest

from oracle.nrc import Cache
from vkrt_gb300 import RenderContext, abi, scenes

pytestmark = pytest.mark.gpu


def _records(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 16), np.float32)
    x[:, 0:3] = rng.uniform(lo, hi, size=(n, 3))
    x[:, 3] = rng.uniform(0.05, 1.0, n)
    d = rng.normal(size=(n, 3))
    x[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    x[:, 7] = (rng.uniform(size=n) < 0.3).astype(np.float32)
    nn = rng.normal(size=(n, 3))
    x[:, 8:11] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    x[:, 12:15] = rng.uniform(0.1, 0.9, size=(n, 3))
    t = rng.uniform(0.0, 2.0, size=(n, 3)).astype(np.float32)
    return x, t


@pytest.fixture(scope="module")
def cache_ctx(built):
    s = scenes.icosphere_field(n_spheres=40, width=64, height=64, spp=1, max_depth=4, seed=3, spectral=False,
                               env_size=(64, 32))
    ctx = RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT)
    ctx.upload_scene(s)
    ctx.nrc_configure(seed=7, learningRate=1e-2)
    yield ctx
    ctx.close()


def _oracle(ctx):
    w, tb = ctx.nrc_parameters(read_table=True)
    lo, hi, res, dense = ctx.nrc_grid()
    return Cache(w, tb, lo, hi, res, dense), lo, hi


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_cache_inference_matches_fp64(cache_ctx):
    # perturb the table so hash features are not negligible next to the other inputs
    w, tb = cache_ctx.nrc_parameters(read_table=True)
    rng = np.random.default_rng(1)
    tbf = rng.uniform(-0.5, 0.5, tb.size).astype(np.float16).view(np.uint16)
    cache_ctx.nrc_parameters(weights=w, table=tbf)
    oc, lo, hi = _oracle(cache_ctx)
    x, _ = _records(4099, lo, hi, seed=2)  # not a multiple of the 16-row tiles
    got = cache_ctx.nrc_infer(x)[:, :3]
    want, _, _ = oc.forward(x)
    assert _rel(got, want[:, :3]) < 2e-2


def test_cache_gradients_match_fp64(cache_ctx):
    oc, lo, hi = _oracle(cache_ctx)
    x, t = _records(3000, lo, hi, seed=3)
    loss = cache_ctx.nrc_train(x, t, apply=False)
    gw, gt = cache_ctx.nrc_gradients(table=True)
    want_loss, _, want_gw, want_gt = oc.loss_and_grads(x, t)
    assert abs(loss - want_loss) <= 1e-2 * want_loss
    assert _rel(gw, want_gw) < 3e-2
    assert float(gw @ want_gw) / (np.linalg.norm(gw) * np.linalg.norm(want_gw)) > 0.999
    nz = np.abs(want_gt) > 0
    assert nz.sum() > 1000
    assert _rel(gt[nz], want_gt[nz]) < 3e-2
    # entries the oracle leaves untouched only receive zero-weight corners of cells chosen differently in FP32
    assert np.linalg.norm(gt[~nz]) < 1e-4 * np.linalg.norm(want_gt)


def test_cache_training_reduces_loss(cache_ctx):
    """Adam steps on a fixed smooth target field lower the relative L2 loss."""
    cache_ctx.nrc_configure(seed=11, learningRate=1e-2)
    _, lo, hi = _oracle(cache_ctx)
    x, _ = _records(16384, lo, hi, seed=5)
    p = (x[:, 0:3] - lo) / (hi - lo)
    t = np.stack([1.0 + np.sin(3 * p[:, 0]), 0.5 + p[:, 1] ** 2, 0.2 + p[:, 2] * x[:, 4] ** 2], 1).astype(np.float32)
    first = cache_ctx.nrc_train(x, t)
    for _ in range(200):
        last = cache_ctx.nrc_train(x, t)
    assert last < 0.05 * first


def test_cache_lowers_error_at_equal_samples(built):
    """Cornell box, 1 spp frames: with the trained cache ending render paths at bounce 2, the running image is closer
    to a 4096-spp reference than the plain tracer's after the same number of samples, and stays unbiased to 1%."""
    s = scenes.cornell(128, 128, spp=1, max_depth=8)
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(s)
        sd = s.scene_data.copy()
        sd["samplesPerPixel"] = 64
        for f in range(64):
            sd["frameNumber"] = 100000 + f
            ctx.render_frame(sd)
        ref = ctx.read_accumulation()[..., :3].copy()
        sd["samplesPerPixel"] = 1

        def run(**cache):
            ctx.nrc_configure(**cache)
            ctx.reset_accumulation()
            for f in range(64):
                sd["frameNumber"] = f
                ctx.render_frame(sd)
            img = ctx.read_accumulation()[..., :3]
            return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2))), float(img.mean() / ref.mean())

        plain, _ = run(enabled=0)
        cached, ratio = run(enabled=1, terminationDepth=2, trainingPaths=65536, trainingSteps=4, seed=3)
    assert cached < 0.9 * plain
    assert abs(ratio - 1.0) < 0.01


@pytest.mark.parametrize("spectral", [False, True])
def test_wavefront_training_paths_match_per_thread_paths(built, spectral):
    """The training paths traced through the wavefront stages (a pass of their own before the frame) give the same
    training records as one thread per path: the same pixels, random streams, closest hits and shadow answers, so
    the same vertices. The two tracers are different compiled kernels, whose inlining fuses different multiply-adds
    (as between the wavefront and the megakernel), so continuation directions and radiance sums differ in the last
    bits: most records are equal bit for bit and all agree to float rounding. The order the records are written in
    differs, so both sets are matched on their positions rounded to 1e-3."""
    s = scenes.icosphere_field(n_spheres=400, width=48, height=32, spp=1, max_depth=6, seed=9, spectral=spectral,
                               env_size=(64, 32))
    with RenderContext(rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_IMPORTANCE,
                       integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        if spectral:
            s.rgb2spec, info = ctx.generate_rgb2spec(16)
            s.scene_data["rgb2specSRGB"] = info
        ctx.upload_scene(s)
        sets = []
        for tracer in (0, 1):
            ctx.nrc_configure(enabled=1, trainingPaths=4096, trainingSteps=1, seed=21, trainingTracer=tracer)
            sd = s.scene_data.copy()
            sd["frameNumber"] = 3
            ctx.render_frame(sd)
            x, t = ctx.nrc_training_records()
            assert ctx.stats()["cacheTrainingRecords"] == len(x)
            key = np.round(x[:, :3].astype(np.float64), 3)
            order = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
            sets.append((x[order], t[order]))
    assert len(sets[0][0]) > 1000 and len(sets[1][0]) == len(sets[0][0]), (len(sets[0][0]), len(sets[1][0]))
    np.testing.assert_allclose(sets[1][0], sets[0][0], rtol=1e-3, atol=1e-4)
    np.testing.assert_allclose(sets[1][1], sets[0][1], rtol=2e-3, atol=1e-4)
    assert (sets[1][0] == sets[0][0]).all(axis=1).mean() > 0.9


def test_spread_termination_limits(built):
    """Area-spread termination (Mueller et al. 2021, section 3.3) at its two limits, with an untrained cache (no
    training paths, so every frame is deterministic): a constant no spread exceeds ends every path at
    terminationDepth, bit for bit the fixed-depth image; a constant every spread exceeds ends every path at its first
    secondary vertex, bit for bit the image of terminationDepth 1. The paper's c = 0.01 ends some paths at each and
    gives an image unlike both."""
    s = scenes.icosphere_field(n_spheres=40, width=64, height=48, spp=4, max_depth=8, seed=7, spectral=True,
                               env_size=(128, 64))
    with RenderContext(rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_IMPORTANCE,
                       integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        s.rgb2spec, info = ctx.generate_rgb2spec(16)
        s.scene_data["rgb2specSRGB"] = info
        ctx.upload_scene(s)

        def render(**cache):
            ctx.nrc_configure(enabled=1, trainingPaths=0, trainingSteps=0, seed=5, **cache)
            ctx.reset_accumulation()
            sd = s.scene_data.copy()
            for f in range(2):
                sd["frameNumber"] = f
                ctx.render_frame(sd)
            assert ctx.stats()["errorFlags"] == 0
            return ctx.read_accumulation()[..., :3].copy()

        depth3 = render(terminationDepth=3)
        depth1 = render(terminationDepth=1)
        never = render(terminationDepth=3, terminationSpread=3.0e38)
        always = render(terminationDepth=3, terminationSpread=1.0e-38)
        paper = render(terminationDepth=3, terminationSpread=0.01)
    assert np.array_equal(never, depth3)
    assert np.array_equal(always, depth1)
    assert not np.array_equal(paper, depth3) and not np.array_equal(paper, depth1)
    assert np.isfinite(paper).all()


def test_spread_constant_validated(built):
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(scenes.cornell(32, 32, 1, 2))
        for bad in (-1.0, float("nan"), float("inf")):
            with pytest.raises(RuntimeError):
                ctx.nrc_configure(terminationSpread=bad)


@pytest.mark.parametrize("n", [1, 127, 128, 129, 4099, 70001])
def test_tcgen05_inference_matches_mma_sync_and_fp64(built, n):
    """Cache inference on the tcgen05 path (128-row tiles, FP32 accumulators in tensor memory) against the mma.sync
    path on the same FP16 parameters and inputs, and both against the FP64 oracle. The two paths round the same FP32
    sums to FP16 between layers but may accumulate in another order, so they agree to about 1e-3, not bit for bit."""
    s = scenes.icosphere_field(n_spheres=20, width=32, height=32, spp=1, max_depth=3, seed=5, spectral=False,
                               env_size=(64, 32))
    with RenderContext(rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT) as ctx:
        ctx.upload_scene(s)
        ctx.nrc_configure(seed=11, inferenceTensorPath=abi.NRC_MMA_SYNC)
        w, tb = ctx.nrc_parameters(read_table=True)
        rng = np.random.default_rng(n)
        tbf = rng.uniform(-0.5, 0.5, tb.size).astype(np.float16).view(np.uint16)
        ctx.nrc_parameters(weights=w, table=tbf)
        oc, lo, hi = _oracle(ctx)
        x, _ = _records(n, lo, hi, seed=n + 1)
        outs = {}
        for path in (abi.NRC_MMA_SYNC, abi.NRC_TCGEN05, abi.NRC_TCGEN05):  # the tcgen05 path twice in a row
            ctx.nrc_configure(seed=11, inferenceTensorPath=path)
            ctx.nrc_parameters(weights=w, table=tbf)
            got = ctx.nrc_infer(x)
            assert np.isfinite(got).all()
            if path in outs:
                np.testing.assert_array_equal(got, outs[path])  # deterministic
            outs[path] = got
    ref = outs[abi.NRC_MMA_SYNC][:, :4]
    assert _rel(outs[abi.NRC_TCGEN05][:, :4], ref) < 5e-3
    want, _, _ = oc.forward(x)
    assert _rel(outs[abi.NRC_TCGEN05][:, :3], want[:, :3]) < 2e-2
