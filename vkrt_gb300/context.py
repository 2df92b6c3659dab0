"""Python host mirror of the backend's C ABI: one RenderContext per CUDA context.

This is the operator interface a Python caller (tests, bench, tools) uses; every call goes straight to
libvkrt_gb300.so. There is no CPU path: a missing or failing library raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi


class VkrtError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"VKRT_Result {code}: {message}")
        self.code = code


@dataclass
class Scene:
    """All host arrays of one scene, in vkrt's record layouts (see abi.py)."""
    vertices: np.ndarray                  # VERTEX (authoring vertices)
    indices: np.ndarray                   # uint32, mesh-relative
    meshes: np.ndarray                    # MESH_INFO
    materials: np.ndarray                 # MATERIAL
    scene_data: np.ndarray                # SCENE_DATA, shape (1,)
    textures: dict = field(default_factory=dict)   # slot -> float32 (H, W, 4) linear RGBA
    env_texture: int = abi.INVALID_INDEX  # slot used for importance sampling
    shader_vertices: np.ndarray | None = None
    emissive_meshes: np.ndarray | None = None
    emissive_triangles: np.ndarray | None = None
    mesh_alias_q: np.ndarray | None = None
    mesh_alias_idx: np.ndarray | None = None
    tri_alias_q: np.ndarray | None = None
    tri_alias_idx: np.ndarray | None = None
    rgb2spec: np.ndarray | None = None    # float32 table in vkrt's layout
    sheen_table: np.ndarray | None = None  # float32 [3][32][32] sheen LTC table (vkrt's SHEEN_LTC_TABLE layout)
    emissive_mesh_materials: np.ndarray | None = None  # uint32, material of each emissive-mesh entry
    name: str = ""
    mesh_names: list = field(default_factory=list)  # per MeshInfo (scene files)
    notes: list = field(default_factory=list)       # what a loader dropped or ignored

    @property
    def triangle_count(self) -> int:
        return int(self.meshes["indexCount"].sum() // 3)

    @property
    def width(self) -> int:
        return int(self.scene_data["viewportRect"][0][2])

    @property
    def height(self) -> int:
        return int(self.scene_data["viewportRect"][0][3])


def pack_vertices(vertices: np.ndarray) -> np.ndarray:
    lib = abi.load()
    v = np.ascontiguousarray(vertices, dtype=abi.VERTEX)
    out = np.zeros(len(v), dtype=abi.SHADER_VERTEX)
    lib.vkrt_host_pack_shader_vertices(abi.ptr(v), len(v), abi.ptr(out))
    return out


def build_light_tables(scene: Scene) -> None:
    """Fills the emissive-light tables and MeshInfo.lightPdfArea with the host library (vkrt's lighting.c rules)."""
    lib = abi.load()
    tri_cap = max(1, scene.triangle_count)
    mesh_cap = max(1, len(scene.meshes))
    em = np.zeros(mesh_cap, dtype=abi.EMISSIVE_MESH)
    et = np.zeros(tri_cap, dtype=abi.EMISSIVE_TRIANGLE)
    mq = np.zeros(mesh_cap, dtype=np.float32)
    mi = np.zeros(mesh_cap, dtype=np.uint32)
    tq = np.zeros(tri_cap, dtype=np.float32)
    ti = np.zeros(tri_cap, dtype=np.uint32)
    nm = C.c_uint32(0)
    nt = C.c_uint32(0)
    r = lib.vkrt_host_build_light_tables(
        abi.ptr(scene.meshes), len(scene.meshes), abi.ptr(scene.materials), len(scene.materials),
        abi.ptr(scene.vertices), abi.ptr(scene.indices), abi.ptr(em), mesh_cap, abi.ptr(et), tri_cap, abi.ptr(mq),
        abi.ptr(mi), abi.ptr(tq), abi.ptr(ti), C.byref(nm), C.byref(nt))
    if r != 0:
        raise VkrtError(r, "building light tables")
    scene.emissive_meshes = em[: nm.value].copy()
    scene.emissive_triangles = et[: nt.value].copy()
    scene.mesh_alias_q, scene.mesh_alias_idx = mq[: nm.value].copy(), mi[: nm.value].copy()
    scene.tri_alias_q, scene.tri_alias_idx = tq[: nt.value].copy(), ti[: nt.value].copy()
    # entries follow mesh order and every entry's mesh gets lightPdfArea > 0
    lit = np.nonzero(scene.meshes["lightPdfArea"] > 0.0)[0]
    scene.emissive_mesh_materials = np.ascontiguousarray(scene.meshes["materialIndex"][lit][: nm.value],
                                                         dtype=np.uint32)
    scene.scene_data["emissiveMeshCount"] = nm.value
    scene.scene_data["emissiveTriangleCount"] = nt.value


class RenderContext:
    """A CUDA context of the backend: scene buffers, BVH, film and one stream."""

    def __init__(self, device: int = 0, rng_mode: int = abi.RNG_REFERENCE, rng_seed: int = 1,
                 environment_sampling: int = abi.ENV_BSDF_ONLY, count_rays: bool = False,
                 integrator: int = abi.INTEGRATOR_MEGAKERNEL, treelet_min_triangles: int = 0,
                 treelets_on_update: bool = False, treelet_passes: int = 0):
        self.lib = abi.load()
        cfg = np.zeros(1, dtype=abi.CONFIG)
        self.lib.vkrt_cuda_default_config(abi.ptr(cfg))
        cfg["treeletMinTriangles"] = treelet_min_triangles
        cfg["treeletsOnUpdate"] = 1 if treelets_on_update else 0
        cfg["treeletPasses"] = treelet_passes
        cfg["deviceIndex"] = device
        cfg["rngMode"] = rng_mode
        cfg["rngSeed"] = rng_seed
        cfg["environmentSampling"] = environment_sampling
        cfg["countRays"] = 1 if count_rays else 0
        cfg["integrator"] = integrator
        handle = C.c_void_p()
        r = self.lib.vkrt_cuda_create(abi.ptr(cfg), C.byref(handle))
        if r != abi.SUCCESS:
            raise VkrtError(r, "vkrt_cuda_create (is a CUDA device visible?)")
        self.handle = handle
        self.width = 0
        self.height = 0
        self.scene: Scene | None = None

    # -- plumbing ----------------------------------------------------------------------------------------------
    def _check(self, r: int, what: str) -> None:
        if r != abi.SUCCESS:
            msg = self.lib.vkrt_cuda_last_error(self.handle)
            raise VkrtError(r, f"{what}: {msg.decode() if msg else ''}")

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.vkrt_cuda_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self.lib.vkrt_cuda_stream(self.handle) or 0)

    # -- scene -------------------------------------------------------------------------------------------------
    def upload_scene(self, scene: Scene, generate_rgb2spec_res: int | None = None) -> None:
        if scene.shader_vertices is None:
            scene.shader_vertices = pack_vertices(scene.vertices)
        sv, idx = scene.shader_vertices, np.ascontiguousarray(scene.indices, dtype=np.uint32)
        self._check(self.lib.vkrt_cuda_upload_materials(self.handle, abi.ptr(scene.materials), len(scene.materials)),
                    "upload materials")
        self._check(self.lib.vkrt_cuda_upload_geometry(self.handle, abi.ptr(sv), len(sv), abi.ptr(idx), len(idx),
                                                       abi.ptr(scene.meshes), len(scene.meshes)), "upload geometry")
        self._upload_lights(scene)
        for slot, tex in scene.textures.items():
            self.upload_texture(slot, tex)
        if scene.env_texture != abi.INVALID_INDEX:
            self._check(self.lib.vkrt_cuda_set_environment(self.handle, scene.env_texture), "set environment")
        if scene.sheen_table is not None:
            self.upload_sheen_table(scene.sheen_table)
        if scene.rgb2spec is not None:
            info = np.array([scene.scene_data["rgb2specSRGB"][0]], dtype=np.uint32).reshape(3)
            self._check(self.lib.vkrt_cuda_upload_rgb2spec(self.handle, abi.ptr(scene.rgb2spec), len(scene.rgb2spec),
                                                           abi.ptr(info)), "upload rgb2spec")
        elif generate_rgb2spec_res:
            info = np.zeros(3, dtype=np.uint32)
            self._check(self.lib.vkrt_cuda_generate_rgb2spec(self.handle, generate_rgb2spec_res, abi.ptr(info)),
                        "generate rgb2spec")
            scene.scene_data["rgb2specSRGB"] = info
        self.resize(scene.width, scene.height)
        self.scene = scene

    def _upload_lights(self, scene: Scene) -> None:
        if scene.emissive_meshes is None or not len(scene.emissive_meshes):
            return
        self._check(self.lib.vkrt_cuda_upload_lights(
            self.handle, abi.ptr(scene.emissive_meshes), len(scene.emissive_meshes),
            abi.ptr(scene.emissive_triangles), len(scene.emissive_triangles), abi.ptr(scene.mesh_alias_q),
            abi.ptr(scene.mesh_alias_idx), abi.ptr(scene.tri_alias_q), abi.ptr(scene.tri_alias_idx)),
            "upload lights")
        if scene.emissive_mesh_materials is not None:
            m = np.ascontiguousarray(scene.emissive_mesh_materials, dtype=np.uint32)
            self._check(self.lib.vkrt_cuda_set_emissive_mesh_materials(self.handle, abi.ptr(m), len(m)),
                        "set emissive mesh materials")

    def upload_scene_materials(self, scene: Scene) -> None:
        """Re-uploads materials, mesh records (lightPdfArea) and light tables after material edits; call
        build_light_tables(scene) first when emission changed."""
        self._check(self.lib.vkrt_cuda_upload_materials(self.handle, abi.ptr(scene.materials), len(scene.materials)),
                    "upload materials")
        self.update_meshes(scene.meshes)
        self._upload_lights(scene)

    def upload_texture(self, slot: int, rgba: np.ndarray, fmt: int = abi.TEXTURE_FORMAT_RGBA32_SFLOAT,
                       color_space: int = abi.COLOR_SPACE_LINEAR) -> None:
        a = np.ascontiguousarray(rgba)
        h, w = a.shape[0], a.shape[1]
        self._check(self.lib.vkrt_cuda_upload_texture(self.handle, slot, abi.ptr(a), w, h, fmt, color_space),
                    "upload texture")

    def update_meshes(self, meshes: np.ndarray) -> None:
        self._check(self.lib.vkrt_cuda_update_meshes(self.handle, abi.ptr(meshes), len(meshes)), "update meshes")

    def upload_sheen_table(self, table: np.ndarray) -> None:
        """vkrt's sheen LTC table: 3 x 32 x 32 float32 (transform a, transform b, albedo over cos theta, roughness)."""
        t = np.ascontiguousarray(table, dtype=np.float32).reshape(-1)
        self._check(self.lib.vkrt_cuda_upload_sheen_table(self.handle, abi.ptr(t), len(t)), "upload sheen table")

    def generate_rgb2spec(self, res: int) -> tuple[np.ndarray, np.ndarray]:
        info = np.zeros(3, dtype=np.uint32)
        self._check(self.lib.vkrt_cuda_generate_rgb2spec(self.handle, res, abi.ptr(info)), "generate rgb2spec")
        table = np.zeros(res + 9 * res ** 3, dtype=np.float32)
        self._check(self.lib.vkrt_cuda_download_rgb2spec(self.handle, abi.ptr(table), len(table)), "download rgb2spec")
        return table, info

    # -- wavefront integrator --------------------------------------------------------------------------------
    def set_integrator(self, integrator: int) -> None:
        self._check(self.lib.vkrt_cuda_set_integrator(self.handle, integrator), "set integrator")

    def wavefront_config(self) -> np.ndarray:
        w = np.zeros(1, dtype=abi.WAVEFRONT_CONFIG)
        self._check(self.lib.vkrt_cuda_get_wavefront_config(self.handle, abi.ptr(w)), "get wavefront config")
        return w

    def set_wavefront_config(self, w: np.ndarray | None = None, **fields) -> None:
        if w is None:
            w = self.wavefront_config()
        w = np.ascontiguousarray(w, dtype=abi.WAVEFRONT_CONFIG).copy()
        for k, v in fields.items():
            w[k] = v
        self._check(self.lib.vkrt_cuda_set_wavefront_config(self.handle, abi.ptr(w)), "set wavefront config")

    # -- film / frames -----------------------------------------------------------------------------------------
    def resize(self, width: int, height: int) -> None:
        self._check(self.lib.vkrt_cuda_resize(self.handle, width, height), "resize")
        self.width, self.height = width, height

    def reset_accumulation(self) -> None:
        self._check(self.lib.vkrt_cuda_reset_accumulation(self.handle), "reset accumulation")

    def render_frame(self, scene_data: np.ndarray) -> None:
        sd = np.ascontiguousarray(scene_data, dtype=abi.SCENE_DATA)
        self._check(self.lib.vkrt_cuda_render_frame(self.handle, abi.ptr(sd)), "render frame")

    def sync(self, timeout_ms: int = 0) -> None:
        self._check(self.lib.vkrt_cuda_sync(self.handle, timeout_ms), "sync")

    def read_accumulation(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width, 4), dtype=np.float32)
        self._check(self.lib.vkrt_cuda_read_accumulation(self.handle, abi.ptr(out), out.nbytes), "read accumulation")
        return out

    def read_accumulation_async(self, out: np.ndarray) -> None:
        """Starts the pipelined readback of the latest accumulation into `out` (pinned host memory overlaps the copy
        with the next frame); `out` is complete after wait_readback()."""
        if out.dtype != np.float32 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("read_accumulation_async needs a C-contiguous float32 array")
        self._check(self.lib.vkrt_cuda_read_accumulation_async(self.handle, abi.ptr(out), out.nbytes),
                    "read accumulation async")

    def wait_readback(self, timeout_ms: int = 0) -> None:
        self._check(self.lib.vkrt_cuda_wait_readback(self.handle, timeout_ms), "wait readback")

    def read_output(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), dtype=np.uint16)
        self._check(self.lib.vkrt_cuda_read_output(self.handle, abi.ptr(out), out.nbytes), "read output")
        return out

    # ---- denoiser features --------------------------------------------------------------------------------------
    def set_denoiser_features(self, enabled: bool = True) -> None:
        self._check(self.lib.vkrt_cuda_set_denoiser_features(self.handle, 1 if enabled else 0), "denoiser features")

    def read_denoiser_features(self):
        """(albedo, normal), each (height, width, 4) float32 with .w = resolved samples."""
        a = np.empty((self.height, self.width, 4), np.float32)
        n = np.empty_like(a)
        self._check(self.lib.vkrt_cuda_read_denoiser_features(self.handle, abi.ptr(a), abi.ptr(n), a.nbytes),
                    "read features")
        return a, n

    # ---- selection passes and frame timing ---------------------------------------------------------------------
    def render_selection_overlay(self, scene_data: np.ndarray) -> None:
        """Selection mask of scene_data's selectedMeshIndex and its outline drawn into the output image."""
        sd = np.ascontiguousarray(scene_data, dtype=abi.SCENE_DATA).reshape(1)
        self._check(self.lib.vkrt_cuda_render_selection_overlay(self.handle, abi.ptr(sd)), "selection overlay")

    def read_selection_mask(self) -> np.ndarray:
        out = np.empty((self.height, self.width), dtype=np.uint32)
        self._check(self.lib.vkrt_cuda_read_selection_mask(self.handle, abi.ptr(out), out.nbytes), "selection mask")
        return out

    def pick_mesh(self, scene_data: np.ndarray, x: int, y: int) -> int:
        sd = np.ascontiguousarray(scene_data, dtype=abi.SCENE_DATA).reshape(1)
        out = np.zeros(1, np.uint32)
        self._check(self.lib.vkrt_cuda_pick_mesh(self.handle, abi.ptr(sd), x, y, abi.ptr(out)), "pick")
        return int(out[0])

    def last_frame_ms(self) -> float:
        out = np.zeros(1, np.float32)
        self._check(self.lib.vkrt_cuda_last_frame_ms(self.handle, abi.ptr(out)), "frame time")
        return float(out[0])

    # ---- path-replay adjoint -----------------------------------------------------------------------------------
    def render_adjoint(self, scene_data: np.ndarray, d_image: np.ndarray, sample_base: int = 0, gradients: int = 0,
                       accumulate: bool = False) -> None:
        """Adds d(loss)/d(parameters) for the frame `scene_data` renders, given d_image = d(loss)/d(accumulation)
        as (height, width, 3 or 4) float32 (vkrt_cuda_render_adjoint)."""
        d = np.zeros((self.height, self.width, 4), dtype=np.float32)
        d[..., : d_image.shape[-1]] = d_image
        cfg = np.zeros(1, dtype=abi.ADJOINT_CONFIG)
        cfg["sampleBase"] = sample_base
        cfg["gradients"] = gradients
        cfg["accumulate"] = 1 if accumulate else 0
        sd = np.ascontiguousarray(scene_data, dtype=abi.SCENE_DATA)
        self._check(self.lib.vkrt_cuda_render_adjoint(self.handle, abi.ptr(sd), abi.ptr(d), abi.ptr(cfg)),
                    "render adjoint")

    def render_adjoint_device(self, scene_data: np.ndarray, d_image_ptr: int, sample_base: int = 0,
                              gradients: int = 0, accumulate: bool = False) -> None:
        """Same with d(loss)/d(accumulation) in device memory (height*width RGBA32F at d_image_ptr)."""
        cfg = np.zeros(1, dtype=abi.ADJOINT_CONFIG)
        cfg["sampleBase"] = sample_base
        cfg["gradients"] = gradients
        cfg["accumulate"] = 1 if accumulate else 0
        sd = np.ascontiguousarray(scene_data, dtype=abi.SCENE_DATA)
        self._check(self.lib.vkrt_cuda_render_adjoint_device(self.handle, abi.ptr(sd), C.c_void_p(d_image_ptr),
                                                             abi.ptr(cfg)), "render adjoint")

    def read_texture_gradient(self, slot: int, shape: tuple[int, int]) -> np.ndarray:
        out = np.empty((shape[0], shape[1], 4), dtype=np.float32)
        self._check(self.lib.vkrt_cuda_read_texture_gradient(self.handle, slot, abi.ptr(out), out.nbytes),
                    "read texture gradient")
        return out

    def read_material_gradients(self, count: int) -> np.ndarray:
        out = np.zeros(count, dtype=abi.MATERIAL_GRADIENT)
        self._check(self.lib.vkrt_cuda_read_material_gradients(self.handle, abi.ptr(out), count),
                    "read material gradients")
        return out

    # ---- neural radiance cache ---------------------------------------------------------------------------------
    def nrc_configure(self, **fields) -> None:
        cfg = np.zeros(1, dtype=abi.NRC_CONFIG)
        self.lib.vkrt_cuda_default_nrc_config(abi.ptr(cfg))
        for k, v in fields.items():
            cfg[k] = v
        self._check(self.lib.vkrt_cuda_nrc_configure(self.handle, abi.ptr(cfg)), "configure radiance cache")

    def nrc_training_records(self, capacity: int = 1 << 20) -> tuple[np.ndarray, np.ndarray]:
        """The last cache frame's training records: inputs (n, 16) and targets (n, 4), in write order."""
        x = np.zeros((capacity, abi.NRC_INPUT_FLOATS), np.float32)
        t = np.zeros((capacity, 4), np.float32)
        n = np.zeros(1, np.uint32)
        self._check(self.lib.vkrt_cuda_nrc_read_training_records(self.handle, abi.ptr(x), abi.ptr(t), capacity,
                                                                 abi.ptr(n)), "read training records")
        k = min(int(n[0]), capacity)
        return x[:k], t[:k]

    def nrc_infer(self, inputs: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(inputs, dtype=np.float32).reshape(-1, abi.NRC_INPUT_FLOATS)
        out = np.zeros((len(x), 4), np.float32)
        self._check(self.lib.vkrt_cuda_nrc_infer(self.handle, abi.ptr(x), len(x), abi.ptr(out)), "cache inference")
        return out

    def nrc_train(self, inputs: np.ndarray, targets: np.ndarray, apply: bool = True) -> float:
        x = np.ascontiguousarray(inputs, dtype=np.float32).reshape(-1, abi.NRC_INPUT_FLOATS)
        t = np.zeros((len(x), 4), np.float32)
        t[:, : targets.shape[1]] = targets
        loss = np.zeros(1, np.float32)
        self._check(self.lib.vkrt_cuda_nrc_train(self.handle, abi.ptr(x), abi.ptr(t), len(x), 1 if apply else 0,
                                                 abi.ptr(loss)), "cache training")
        return float(loss[0])

    def nrc_parameters(self, weights: np.ndarray | None = None, table: np.ndarray | None = None,
                       read_table: bool = False):
        """Writes the given FP16 parameters (uint16 views), or reads them when none are given."""
        if weights is None and table is None:
            w = np.zeros(abi.NRC_WEIGHTS, np.uint16)
            tb = np.zeros(abi.NRC_TABLE_HALVES, np.uint16) if read_table else None
            self._check(self.lib.vkrt_cuda_nrc_parameters(self.handle, abi.ptr(w), abi.ptr(tb), 0), "cache parameters")
            return w, tb
        w = None if weights is None else np.ascontiguousarray(weights, np.uint16)
        tb = None if table is None else np.ascontiguousarray(table, np.uint16)
        self._check(self.lib.vkrt_cuda_nrc_parameters(self.handle, abi.ptr(w), abi.ptr(tb), 1), "cache parameters")
        return None

    def nrc_gradients(self, table: bool = False):
        w = np.zeros(abi.NRC_WEIGHTS, np.float32)
        tb = np.zeros(abi.NRC_TABLE_HALVES, np.float32) if table else None
        self._check(self.lib.vkrt_cuda_nrc_gradients(self.handle, abi.ptr(w), abi.ptr(tb)), "cache gradients")
        return w, tb

    def nrc_grid(self):
        lo, hi = np.zeros(3, np.float32), np.zeros(3, np.float32)
        res, dense = np.zeros(16, np.uint32), np.zeros(16, np.uint32)
        self._check(self.lib.vkrt_cuda_nrc_grid(self.handle, abi.ptr(lo), abi.ptr(hi), abi.ptr(res), abi.ptr(dense)),
                    "cache grid")
        return lo, hi, res, dense

    def stats(self) -> dict:
        st = np.zeros(1, dtype=abi.STATS)
        self._check(self.lib.vkrt_cuda_get_stats(self.handle, abi.ptr(st)), "stats")
        return {k: st[k][0].tolist() for k in abi.STATS.names}

    def trace_rays(self, rays: np.ndarray, any_hit: bool = False, persistent: bool = False) -> np.ndarray:
        """Closest (or, with any_hit, first accepted) hits of `rays`; persistent runs them through the wavefront's
        persistent vote-scheduled traversal instead of one ray per thread."""
        r = np.ascontiguousarray(rays, dtype=abi.RAY)
        hits = np.zeros(len(r), dtype=abi.HIT)
        flags = (abi.TRACE_ANY_HIT if any_hit else 0) | (abi.TRACE_PERSISTENT if persistent else 0)
        self._check(self.lib.vkrt_cuda_trace_rays(self.handle, abi.ptr(r), len(r), flags, abi.ptr(hits)),
                    "trace rays")
        return hits

    def read_environment_distribution(self, width: int, height: int):
        """(marginal CDF (H + 1), conditional CDFs (H, W + 1), texel weights (H, W)) of the environment importance
        distribution built at upload, float32."""
        marg = np.zeros(height + 1, np.float32)
        cond = np.zeros((height, width + 1), np.float32)
        pdf = np.zeros((height, width), np.float32)
        self._check(self.lib.vkrt_cuda_read_environment_distribution(self.handle, width, height, abi.ptr(marg),
                                                                     abi.ptr(cond), abi.ptr(pdf)),
                    "read environment distribution")
        return marg, cond, pdf

    def trace_rays_device(self, rays_ptr: int, count: int, hits_ptr: int, any_hit: bool = False) -> None:
        self._check(self.lib.vkrt_cuda_trace_rays_device(self.handle, C.c_void_p(rays_ptr), count,
                                                         1 if any_hit else 0, C.c_void_p(hits_ptr)),
                    "trace rays (device)")


def _handles(contexts):
    arr = (C.c_void_p * len(contexts))(*[c.handle.value for c in contexts])
    return arr


def render_batch(contexts: list, scene_datas: np.ndarray) -> None:
    """One batched wavefront frame over several contexts (vkrt_cuda_render_batch)."""
    sds = np.ascontiguousarray(scene_datas, dtype=abi.SCENE_DATA)
    arr = _handles(contexts)
    r = contexts[0].lib.vkrt_cuda_render_batch(C.cast(arr, C.c_void_p), abi.ptr(sds), len(contexts))
    contexts[0]._check(r, "render batch")


def autotune_batch(contexts: list, scene_datas: np.ndarray, frames_per_trial: int = 1):
    """Autotunes the wavefront configuration of a batch; returns (config, frame ms)."""
    sds = np.ascontiguousarray(scene_datas, dtype=abi.SCENE_DATA)
    arr = _handles(contexts)
    best = np.zeros(1, dtype=abi.WAVEFRONT_CONFIG)
    ms = C.c_float(0.0)
    r = contexts[0].lib.vkrt_cuda_autotune_batch(C.cast(arr, C.c_void_p), abi.ptr(sds), len(contexts),
                                                 frames_per_trial, abi.ptr(best), C.byref(ms))
    contexts[0]._check(r, "autotune batch")
    return best, ms.value


class AutoSpp:
    """vkrt's auto-SPP controller (vkrt_host_auto_spp_*): feed it each frame's render milliseconds and the spp the
    frame used; it returns the spp for the next frame."""

    def __init__(self, target_fps: int = 60):
        self.lib = abi.load()
        self.state = np.zeros(1, dtype=abi.AUTO_SPP)
        self.lib.vkrt_host_auto_spp_init(abi.ptr(self.state), int(target_fps))

    @property
    def target_ms(self) -> float:
        return float(self.state["targetFrameMs"][0])

    def update(self, render_ms: float, spp: int) -> int:
        s = np.array([spp], np.uint32)
        if self.lib.vkrt_host_auto_spp_update(abi.ptr(self.state), float(render_ms), abi.ptr(s)) < 0:
            raise VkrtError("auto-SPP update: invalid arguments")
        return int(s[0])
