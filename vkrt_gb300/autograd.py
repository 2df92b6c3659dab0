"""torch.autograd bridge over the path-replay adjoint (vkrt_cuda_render_adjoint), used to check its gradients
against finite differences and to drive inverse rendering from PyTorch.

`TextureRenderer` binds torch parameters to a scene: base-colour textures (RGB), metallic-roughness textures (the
roughness in G) and material emission radiance. `render(renderer, *params)` returns the accumulated image of one
frame (H, W, 3) as a differentiable torch tensor; its backward calls the adjoint with d(loss)/d(image) and reads the
texel and material gradients back. Parameters live on the host: every forward uploads them through the C ABI.
"""
from __future__ import annotations

import numpy as np
import torch

from . import abi
from .context import RenderContext, Scene, build_light_tables
from .scenes import albedo_texture, roughness_texture


class TextureRenderer:
    """Forward and adjoint passes over one scene whose listed texture slots and material emissions are parameters.

    albedo_slots     texture slots bound as baseColor textures; parameter shape (H, W, 3)
    roughness_slots  texture slots bound as metallic-roughness textures; parameter shape (H, W) (G channel)
    emission_materials  material indices whose emission radiance (emissionColor x emissionLuminance) is a
                        parameter of shape (3,)
    """

    def __init__(self, ctx: RenderContext, scene: Scene, albedo_slots=(), roughness_slots=(), emission_materials=(),
                 frame: int = 0):
        self.ctx, self.scene = ctx, scene
        self.albedo_slots = list(albedo_slots)
        self.roughness_slots = list(roughness_slots)
        self.emission_materials = list(emission_materials)
        self.scene_data = scene.scene_data.copy()
        self.scene_data["frameNumber"] = frame

    def parameters(self) -> list[torch.Tensor]:
        """Current values as float32 tensors (albedos, then roughnesses, then emissions)."""
        out = [torch.from_numpy(self.scene.textures[s][..., :3].copy()) for s in self.albedo_slots]
        out += [torch.from_numpy(self.scene.textures[s][..., 1].copy()) for s in self.roughness_slots]
        for m in self.emission_materials:
            mat = self.scene.materials[m]
            out.append(torch.from_numpy((mat["emissionColor"] * mat["emissionLuminance"]).astype(np.float32)))
        return out

    def _bind(self, params) -> None:
        na, nr = len(self.albedo_slots), len(self.roughness_slots)
        if len(params) != na + nr + len(self.emission_materials):
            raise ValueError("one tensor per albedo slot, roughness slot and emission material")
        for slot, p in zip(self.albedo_slots, params[:na]):
            t = albedo_texture(p.detach().cpu().numpy())
            self.scene.textures[slot] = t
            self.ctx.upload_texture(slot, t)
        for slot, p in zip(self.roughness_slots, params[na:na + nr]):
            t = roughness_texture(p.detach().cpu().numpy())
            self.scene.textures[slot] = t
            self.ctx.upload_texture(slot, t)
        if self.emission_materials:
            for m, p in zip(self.emission_materials, params[na + nr:]):
                self.scene.materials[m]["emissionColor"] = p.detach().cpu().numpy().astype(np.float32)
                self.scene.materials[m]["emissionLuminance"] = 1.0
            build_light_tables(self.scene)
            self.ctx.upload_scene_materials(self.scene)

    def render_image(self, params) -> np.ndarray:
        self._bind(params)
        self.ctx.reset_accumulation()
        self.ctx.render_frame(self.scene_data)
        return self.ctx.read_accumulation()[..., :3].copy()

    def adjoint(self, d_image: np.ndarray) -> list[np.ndarray]:
        self.ctx.render_adjoint(self.scene_data, np.ascontiguousarray(d_image, dtype=np.float32))
        grads = []
        for slot in self.albedo_slots:
            t = self.scene.textures[slot]
            grads.append(self.ctx.read_texture_gradient(slot, t.shape[:2])[..., :3].copy())
        for slot in self.roughness_slots:
            t = self.scene.textures[slot]
            grads.append(self.ctx.read_texture_gradient(slot, t.shape[:2])[..., 1].copy())
        if self.emission_materials:
            mg = self.ctx.read_material_gradients(len(self.scene.materials))
            for m in self.emission_materials:
                grads.append(mg[m]["emission"].astype(np.float32).copy())
        return grads


class _RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, renderer: TextureRenderer, *params):
        ctx.renderer = renderer
        return torch.from_numpy(renderer.render_image(params))

    @staticmethod
    def backward(ctx, grad_image):
        grads = ctx.renderer.adjoint(grad_image.detach().cpu().numpy())
        return (None,) + tuple(torch.from_numpy(g) for g in grads)


def render(renderer: TextureRenderer, *params: torch.Tensor) -> torch.Tensor:
    """Differentiable accumulated image (H, W, 3) of one frame from a cleared film."""
    return _RenderFunction.apply(renderer, *params)
