"""Parity of the benchmarked frame's path with the oracle: the seeded 1,024,000-triangle icosphere field (glTF
metallic-roughness spheres: base colour U[0.1, 0.9]^3, roughness U[0.05, 1], metallic Bernoulli(0.3), specular 0.5)
under the 1024 x 512 sky with a 5e3-radiance sun, at 96 x 64 and 4 samples per pixel, depth 12, PCG32 seed 1.

* Environment lookup on miss (light/environment.slang:9-27: lat-long UV with rotation, repeat-U / clamp-V bilinear,
  times environmentLight.w) and this backend's environment importance sampling (FP64-summed 2D CDF, sampling, pdf and
  power-heuristic MIS against the BSDF, no counterpart in vkrt): per sample against the oracle's restatement, in RGB
  and hero-spectral transport, with environment NEE on and off, through both integrators.
* The device's environment distribution against the oracle's FP64 tables, entry by entry.
* Precision: relative MSE of the FP32 device frame against the oracle's FP64 render of the same seeds."""
import numpy as np
import pytest

from parity import assert_match, relmse
from vkrt_gb300 import RenderContext, abi, scenes

pytestmark = pytest.mark.gpu

WIDTH, HEIGHT, SPP = 96, 64, 4


@pytest.fixture(scope="module")
def rgb2spec(built):
    with RenderContext() as ctx:
        return ctx.generate_rgb2spec(64)


@pytest.fixture(scope="module")
def field(built):
    return scenes.icosphere_field(n_spheres=800, width=WIDTH, height=HEIGHT, spp=SPP, max_depth=12, seed=1,
                                  spectral=False)


def _scene(field, rgb2spec, spectral):
    import copy
    s = copy.copy(field)
    s.scene_data = field.scene_data.copy()
    if spectral:
        s.rgb2spec, info = rgb2spec
        s.scene_data["rgb2specSRGB"] = info
        s.scene_data["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES,
                                                                        abi.RENDER_MODE_SPECTRAL, abi.SPECTRAL_HERO)
    return s


def _render(scene, integrator, env):
    with RenderContext(rng_mode=abi.RNG_PCG32, rng_seed=1, environment_sampling=env, integrator=integrator) as ctx:
        ctx.upload_scene(scene)
        ctx.render_frame(scene.scene_data)
        return ctx.read_accumulation(), ctx.stats()


_oracles = {}


def _oracle(scene, spectral, env):
    """One oracle scene per (transport, environment mode); the BVH2 build over a million triangles takes a second."""
    from oracle import cpu
    key = (spectral, env)
    if key not in _oracles:
        _oracles[key] = cpu.OracleScene(scene, environment_sampling=env)
    return _oracles[key]


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT],
                         ids=["megakernel", "wavefront"])
@pytest.mark.parametrize("spectral", [False, True], ids=["rgb", "hero"])
@pytest.mark.parametrize("env", [abi.ENV_IMPORTANCE, abi.ENV_BSDF_ONLY], ids=["env-nee", "bsdf-only"])
def test_headline_per_sample_parity(field, rgb2spec, integrator, spectral, env):
    s = _scene(field, rgb2spec, spectral)
    gpu, st = _render(s, integrator, env)
    ref, ost = _oracle(s, spectral, env).render(s.scene_data, rng_mode=abi.RNG_PCG32, rng_seed=1)
    label = f"headline {'hero' if spectral else 'rgb'} env={env} integrator={integrator}"
    # hero transport runs exp / sqrt / division chains through the rgb2spec sigmoid on every lane: a looser band
    tol = 2e-3 if spectral else 1e-3
    # 7-13 of the 6,144 pixels hold a sample whose path took another branch after an FP32 rounding difference
    assert_match(label, gpu, ref, tol, tol, max_outside=20)
    np.testing.assert_array_equal(gpu[..., 3], float(SPP))
    assert st["primaryRays"] == ost["primaryRays"] == WIDTH * HEIGHT * SPP
    assert abs(st["extensionRays"] - ost["extensionRays"]) <= 0.002 * ost["extensionRays"] + 4
    assert abs(st["shadowRays"] - ost["shadowRays"]) <= 0.002 * ost["shadowRays"] + 4
    if env == abi.ENV_IMPORTANCE:
        assert st["shadowRays"] > 0  # environment NEE ran (the field has no emissive triangles)
    else:
        assert st["shadowRays"] == 0
    assert st["errorFlags"] == 0


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT],
                         ids=["megakernel", "wavefront"])
def test_headline_fp64_relmse(field, rgb2spec, integrator):
    """The FP32 device frame against the oracle's FP64 render of the same seeds (hero spectral, environment NEE)."""
    s = _scene(field, rgb2spec, True)
    gpu, _ = _render(s, integrator, abi.ENV_IMPORTANCE)
    ref64 = _oracle(s, True, abi.ENV_IMPORTANCE).render_f64(s.scene_data, rng_mode=abi.RNG_PCG32, rng_seed=1)
    err = relmse(gpu, ref64)
    assert err <= 1e-3, err


def test_environment_distribution_matches_oracle(field):
    """Marginal and conditional CDFs and texel weights of the 1024 x 512 sky: FP64 prefix sums on the device (tree
    order) and in the oracle (sequential) rounded to FP32 agree to within 2 ulp; sampling searches these tables, so
    equal tables mean the same texel for the same random numbers."""
    from oracle import cpu
    env = field.textures[field.env_texture]
    h, w = env.shape[:2]
    with RenderContext(environment_sampling=abi.ENV_IMPORTANCE) as ctx:
        ctx.upload_scene(field)
        marg, cond, pdf = ctx.read_environment_distribution(w, h)
    omarg, ocond, _, opdf = cpu.env_cdf(env, texel_pdf=True)
    np.testing.assert_array_max_ulp(marg, omarg, maxulp=2)
    np.testing.assert_array_max_ulp(cond, ocond, maxulp=2)
    np.testing.assert_array_max_ulp(pdf, opdf, maxulp=2)
    assert marg[0] == 0.0 and marg[-1] == 1.0 and (np.diff(marg) >= 0).all()
    # the sun's texels carry most of the marginal mass
    assert float(pdf.max()) > 1e3 * float(np.median(pdf))
