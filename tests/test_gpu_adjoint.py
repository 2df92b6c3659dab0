"""Path-replay adjoint (adjoint.cu) through the torch.autograd wrapper, checked against FP64 central finite
differences with common random numbers: the oracle renders the same seeds and sample indices in double precision at
theta +- h, and the L2 loss against the same target gives (L+ - L-) / 2h. The workload is the inverse-rendering Cornell
box: Lambertian walls with albedo and roughness textures, Russian roulette off, so the fixed-seed estimator is smooth in
every parameter and the adjoint is its exact derivative."""
import numpy as np
import pytest
import torch

from oracle.cpu import OracleScene
from vkrt_gb300 import RenderContext, abi, build_light_tables, scenes
from vkrt_gb300.autograd import TextureRenderer, render

pytestmark = pytest.mark.gpu

H_FD = 1e-3
ALBEDO_SLOTS = [0, 2, 4, 6, 8]
ROUGH_SLOTS = [1, 3, 5, 7, 9]
LIGHT_MATERIAL = 3


def _problem(width, height, spp, depth, tex, integrator):
    target = scenes.inverse_rendering_cornell(width, height, spp, depth, tex_size=tex, target=True)
    scene = scenes.inverse_rendering_cornell(width, height, spp, depth, tex_size=tex, target=False)
    ctx = RenderContext(rng_mode=abi.RNG_PCG32, rng_seed=1, integrator=integrator)
    ctx.upload_scene(target)
    ctx.render_frame(target.scene_data)
    t_img = ctx.read_accumulation()[..., :3].copy()
    ctx.upload_scene(scene)
    renderer = TextureRenderer(ctx, scene, ALBEDO_SLOTS, ROUGH_SLOTS, [LIGHT_MATERIAL])
    return ctx, scene, renderer, t_img


def _fd_loss(scene, t_img, edit):
    """FP64 oracle loss of the scene with `edit` applied to copies of its textures / materials."""
    s = scenes.Scene(**{k: getattr(scene, k) for k in scene.__dataclass_fields__})
    s.textures = {k: v.copy() for k, v in scene.textures.items()}
    s.materials = scene.materials.copy()
    s.meshes = scene.meshes.copy()
    s.scene_data = scene.scene_data.copy()
    edit(s)
    build_light_tables(s)
    o = OracleScene(s)
    img = o.render_f64(s.scene_data, rng_mode=abi.RNG_PCG32, rng_seed=1, precision=64)[..., :3]
    o.close()
    return float(np.mean((img - t_img.astype(np.float64)) ** 2))


def _central(scene, t_img, edit_plus, edit_minus):
    return (_fd_loss(scene, t_img, edit_plus) - _fd_loss(scene, t_img, edit_minus)) / (2 * H_FD)


def _pick(grad, k, rng, frac=0.05):
    """k random entries among those whose gradient magnitude is at least frac of the largest."""
    g = np.abs(grad).reshape(-1)
    cand = np.nonzero(g >= frac * g.max())[0]
    return rng.choice(cand, size=min(k, len(cand)), replace=False)


def _check(name, got, want, rel=1e-2):
    got, want = np.asarray(got), np.asarray(want)
    err = np.abs(got - want) / np.maximum(np.abs(want), 1e-12)
    assert (err <= rel).all(), f"{name}: worst relative error {err.max():.3e}\nadjoint {got}\nfd      {want}"


def _run_check(width, height, spp, depth, tex, n_albedo, n_rough, seed, integrator):
    ctx, scene, renderer, t_img = _problem(width, height, spp, depth, tex, integrator)
    try:
        params = [p.clone().requires_grad_() for p in renderer.parameters()]
        img = render(renderer, *params)
        loss = ((img - torch.from_numpy(t_img)) ** 2).mean()
        loss.backward()
        grads = [p.grad.numpy() for p in params]
    finally:
        ctx.close()
    rng = np.random.default_rng(seed)
    # albedo texels: random (wall, texel, channel)
    alb = np.stack(grads[:5])  # (5, tex, tex, 3)
    got, want = [], []
    for flat in _pick(alb, n_albedo, rng):
        w, y, x, c = np.unravel_index(flat, alb.shape)
        slot = ALBEDO_SLOTS[w]

        def edit(s, d, slot=slot, y=y, x=x, c=c):
            s.textures[slot][y, x, c] += d
        got.append(alb[w, y, x, c])
        want.append(_central(scene, t_img, lambda s: edit(s, H_FD), lambda s: edit(s, -H_FD)))
    _check("albedo", got, want)
    rough = np.stack(grads[5:10])  # (5, tex, tex)
    got, want = [], []
    for flat in _pick(rough, n_rough, rng):
        w, y, x = np.unravel_index(flat, rough.shape)
        slot = ROUGH_SLOTS[w]

        def edit(s, d, slot=slot, y=y, x=x):
            s.textures[slot][y, x, 1] += d
        got.append(rough[w, y, x])
        want.append(_central(scene, t_img, lambda s: edit(s, H_FD), lambda s: edit(s, -H_FD)))
    _check("roughness", got, want)
    em = grads[10]
    got, want = [], []
    base = scene.materials[LIGHT_MATERIAL]["emissionColor"] * scene.materials[LIGHT_MATERIAL]["emissionLuminance"]
    for c in range(3):
        def edit(s, d, c=c):
            e = base.copy()
            e[c] += d
            s.materials[LIGHT_MATERIAL]["emissionColor"] = e
            s.materials[LIGHT_MATERIAL]["emissionLuminance"] = 1.0
        got.append(em[c])
        want.append(_central(scene, t_img, lambda s: edit(s, H_FD), lambda s: edit(s, -H_FD)))
    _check("emission", got, want)
    return alb, rough, em


INTEGRATORS = [pytest.param(abi.INTEGRATOR_MEGAKERNEL, id="per-path"),
               pytest.param(abi.INTEGRATOR_WAVEFRONT, id="wavefront")]


@pytest.mark.parametrize("integrator", INTEGRATORS)
def test_adjoint_matches_central_differences_small(built, integrator):
    _run_check(48, 48, spp=4, depth=4, tex=16, n_albedo=12, n_rough=8, seed=7, integrator=integrator)


@pytest.mark.parametrize("integrator", INTEGRATORS)
def test_adjoint_matches_central_differences_inverse_rendering_workload(built, integrator):
    # 128 x 128, 16 spp, depth 6, five 64 x 64 albedo + roughness textures; 32 random texels (20 albedo, 12 roughness)
    _run_check(128, 128, spp=16, depth=6, tex=64, n_albedo=20, n_rough=12, seed=11, integrator=integrator)


def test_wavefront_adjoint_equals_per_path_adjoint(built):
    """Both adjoint implementations replay the same paths: their gradients agree to float summation order."""
    s = scenes.inverse_rendering_cornell(64, 48, 4, 5, tex_size=16, target=False)
    d = np.random.default_rng(1).normal(size=(48, 64, 3)).astype(np.float32)
    out = []
    for integ in (abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT):
        with RenderContext(rng_mode=abi.RNG_PCG32, integrator=integ) as ctx:
            ctx.upload_scene(s)
            if integ == abi.INTEGRATOR_WAVEFRONT:
                ctx.set_wavefront_config(queueCapacity=1000)  # slots reused across many items
            ctx.render_adjoint(s.scene_data, d)
            tex = np.stack([ctx.read_texture_gradient(k, (16, 16)) for k in range(10)])
            mat = ctx.read_material_gradients(len(s.materials))
            out.append((tex, np.concatenate([mat["baseColor"], mat["roughness"][:, None], mat["emission"]], 1)))
    scale = np.abs(out[0][0]).max()
    np.testing.assert_allclose(out[1][0], out[0][0], rtol=1e-3, atol=1e-5 * scale)
    np.testing.assert_allclose(out[1][1], out[0][1], rtol=1e-3, atol=1e-5 * np.abs(out[0][1]).max())


def test_adjoint_gradient_linear_in_dimage(built):
    """The adjoint is linear in d(loss)/d(image): two half-weighted accumulating calls equal one full call."""
    s = scenes.inverse_rendering_cornell(32, 32, 2, 3, tex_size=8, target=False)
    with RenderContext(rng_mode=abi.RNG_PCG32) as ctx:
        ctx.upload_scene(s)
        d = np.random.default_rng(0).normal(size=(32, 32, 3)).astype(np.float32)
        ctx.render_adjoint(s.scene_data, d)
        full = ctx.read_texture_gradient(0, (8, 8))
        ctx.render_adjoint(s.scene_data, 0.5 * d)
        ctx.render_adjoint(s.scene_data, 0.5 * d, accumulate=True)
        half = ctx.read_texture_gradient(0, (8, 8))
        np.testing.assert_allclose(half, full, rtol=1e-4, atol=1e-7)
        assert np.abs(full[..., :3]).max() > 0


def test_adjoint_rejects_unsupported(built):
    s = scenes.inverse_rendering_cornell(16, 16, 1, 2, tex_size=4)
    with RenderContext(rng_mode=abi.RNG_PCG32) as ctx:
        ctx.upload_scene(s)
        sd = s.scene_data.copy()
        sd["packedRenderSettings"] = abi.pack_render_settings(1, abi.RENDER_MODE_SPECTRAL, 1)
        with pytest.raises(Exception):
            ctx.render_adjoint(sd, np.zeros((16, 16, 3), np.float32))
