"""TEST INFRASTRUCTURE ONLY. ctypes wrapper of liboracle.so, the CPU restatement of vkrt's path tracer and the FP64
intersector. Only tests, __graft_entry__.smoke() and bench.py's CPU baseline use it, as the checker."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libvkrt_ref.so"

_V, _I32, _U32, _U64, _F, _D = C.c_void_p, C.c_int32, C.c_uint32, C.c_uint64, C.c_float, C.c_double


class OracleTexture(C.Structure):
    _fields_ = [("rgba", _V), ("width", _U32), ("height", _U32)]


class OracleSceneDesc(C.Structure):
    _fields_ = [("vertices", _V), ("vertexCount", _U32), ("indices", _V), ("indexCount", _U32), ("meshes", _V),
                ("meshCount", _U32), ("materials", _V), ("materialCount", _U32), ("emissiveMeshes", _V),
                ("emissiveMeshCount", _U32), ("emissiveTriangles", _V), ("emissiveTriangleCount", _U32),
                ("meshAliasQ", _V), ("meshAliasIdx", _V), ("triAliasQ", _V), ("triAliasIdx", _V),
                ("textures", C.POINTER(OracleTexture)), ("textureCount", _U32), ("rgb2spec", _V),
                ("rgb2specFloatCount", _U32), ("environmentSampling", _U32), ("envTextureIndex", _U32),
                ("sheenLtc", _V), ("sheenLtcFloatCount", _U32)]


class OracleRenderParams(C.Structure):
    _fields_ = [("rngMode", _U32), ("rngSeed", _U64), ("precision", _U32), ("threads", _U32), ("rowBegin", _U32),
                ("rowEnd", _U32), ("useBruteForce", _U32), ("rowStep", _U32)]


class OracleRenderStats(C.Structure):
    _fields_ = [("primaryRays", _U64), ("extensionRays", _U64), ("shadowRays", _U64), ("pathSamples", _U64)]


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        from . import build
        build.build_oracle()
    lib = C.CDLL(str(LIB))
    sig = {
        "oracle_scene_create": (_V, [_V]), "oracle_scene_destroy": (None, [_V]),
        "oracle_trace_fp32": (_I32, [_V, _V, _U32, _U32, _V, _U32]),
        "oracle_trace_fp64_bruteforce": (_I32, [_V, _V, _U32, _V, _V, _D, _U32]),
        "oracle_render": (_I32, [_V, _V, _V, _V, _V, _V, _V]),
        "oracle_render_f64": (_I32, [_V, _V, _V, _V, _V]),
        "oracle_render_features": (_I32, [_V, _V, _V, _V, _V, _V, _V]),
        "oracle_hash": (_U32, [_U32]), "oracle_init_pixel_seed": (_U32, [C.c_int32, C.c_int32, _U32, _U32]),
        "oracle_rand": (_F, [_V]), "oracle_pcg32": (_U32, [_V, _U64]),
        "oracle_world_triangles": (_U32, [_V, _V, _U32]),
        "oracle_env_cdf": (_I32, [_V, _U32, _U32, _V, _V, _V, _V]),
        "oracle_env_pdf": (_F, [_V, _V, _F]), "oracle_env_sample": (_I32, [_V, _F, _F, _F, _V, _V]),
        "oracle_rgb2spec_generate": (_I32, [_U32, _V, _U32, _U32]),
        "oracle_rgb2spec_fetch": (None, [_V, _U32, _V, _V]), "oracle_rgb2spec_eval": (_F, [_V, _F]),
        "oracle_spectral_to_xyz": (None, [_F, _V]), "oracle_xyz_to_linear_srgb": (None, [_V, _V]),
        "oracle_bsdf_eval_rgb": (_I32, [_V, _V, _V, _U32, _V, _V]),
        "oracle_bsdf_sample_rgb": (_I32, [_V, _V, _U32, _U32, _V, _V, _V]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class OracleScene:
    """The oracle's copy of a vkrt_gb300.Scene (world triangles, BVH2, environment distribution)."""

    def __init__(self, scene, environment_sampling: int = 0):
        from .host import pack_vertices  # the oracle's own restatement of vkrt's packing
        self.lib = load()
        if scene.shader_vertices is None:
            scene.shader_vertices = pack_vertices(scene.vertices)
        self._keep = []
        tex_count = (max(scene.textures) + 1) if scene.textures else 0
        texs = (OracleTexture * max(1, tex_count))()
        for slot, img in scene.textures.items():
            a = np.ascontiguousarray(img, dtype=np.float32)
            self._keep.append(a)
            texs[slot] = OracleTexture(C.c_void_p(a.ctypes.data), a.shape[1], a.shape[0])
        self._keep.append(texs)
        d = OracleSceneDesc()
        d.vertices, d.vertexCount = _p(scene.shader_vertices), len(scene.shader_vertices)
        d.indices, d.indexCount = _p(scene.indices), len(scene.indices)
        d.meshes, d.meshCount = _p(scene.meshes), len(scene.meshes)
        d.materials, d.materialCount = _p(scene.materials), len(scene.materials)
        n_em = 0 if scene.emissive_meshes is None else len(scene.emissive_meshes)
        n_et = 0 if scene.emissive_triangles is None else len(scene.emissive_triangles)
        d.emissiveMeshes, d.emissiveMeshCount = _p(scene.emissive_meshes), n_em
        d.emissiveTriangles, d.emissiveTriangleCount = _p(scene.emissive_triangles), n_et
        d.meshAliasQ, d.meshAliasIdx = _p(scene.mesh_alias_q), _p(scene.mesh_alias_idx)
        d.triAliasQ, d.triAliasIdx = _p(scene.tri_alias_q), _p(scene.tri_alias_idx)
        d.textures, d.textureCount = texs, tex_count
        if scene.rgb2spec is not None:
            d.rgb2spec, d.rgb2specFloatCount = _p(scene.rgb2spec), len(scene.rgb2spec)
        d.environmentSampling = environment_sampling
        d.envTextureIndex = scene.env_texture
        if scene.sheen_table is not None:
            d.sheenLtc, d.sheenLtcFloatCount = _p(scene.sheen_table), len(scene.sheen_table)
        self.handle = self.lib.oracle_scene_create(C.byref(d))
        self.scene = scene

    def close(self):
        if self.handle:
            self.lib.oracle_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace_fp32(self, rays, any_hit=False, threads=0, selection_alpha=False):
        """FP32 traversal; selection_alpha drops mask cut-outs as vkrt's selection rays do."""
        from vkrt_gb300 import abi
        r = np.ascontiguousarray(rays, dtype=abi.RAY)
        hits = np.zeros(len(r), dtype=abi.HIT)
        flags = (1 if any_hit else 0) | (2 if selection_alpha else 0)
        self.lib.oracle_trace_fp32(self.handle, _p(r), len(r), flags, _p(hits), threads)
        return hits

    def trace_fp64(self, rays, eps=1e-5, threads=0):
        from vkrt_gb300 import abi
        r = np.ascontiguousarray(rays, dtype=abi.RAY)
        hits = np.zeros(len(r), dtype=abi.HIT)
        amb = np.zeros(len(r), dtype=np.uint8)
        self.lib.oracle_trace_fp64_bruteforce(self.handle, _p(r), len(r), _p(hits), _p(amb), eps, threads)
        return hits, amb.astype(bool)

    def world_triangles(self):
        n = self.lib.oracle_world_triangles(self.handle, None, 0)
        out = np.zeros((n, 9), dtype=np.float32)
        self.lib.oracle_world_triangles(self.handle, _p(out), n)
        return out.reshape(n, 3, 3)

    def render(self, scene_data, accum_in=None, rng_mode=0, rng_seed=1, precision=32, threads=0, rows=None,
               brute_force=False, want_output=False, row_step=1):
        """One frame; rows = (begin, end) and row_step render every row_step-th row of that range only."""
        from vkrt_gb300 import abi
        sd = np.ascontiguousarray(scene_data, dtype=abi.SCENE_DATA)
        w = int(sd["viewportRect"][0][0] + sd["viewportRect"][0][2])
        h = int(sd["viewportRect"][0][1] + sd["viewportRect"][0][3])
        acc_in = np.zeros((h, w, 4), np.float32) if accum_in is None else np.ascontiguousarray(accum_in, np.float32)
        acc_out = acc_in.copy()
        out = np.zeros((h, w, 4), np.uint16) if want_output else None
        p = OracleRenderParams(rng_mode, rng_seed, precision, threads, rows[0] if rows else 0, rows[1] if rows else 0,
                               1 if brute_force else 0, row_step)
        st = OracleRenderStats()
        r = self.lib.oracle_render(self.handle, _p(sd), C.byref(p), _p(acc_in), _p(acc_out), _p(out), C.byref(st))
        if r != 0:
            raise RuntimeError(f"oracle_render failed ({r})")
        stats = {k: getattr(st, k) for k, _ in OracleRenderStats._fields_}
        return (acc_out, out, stats) if want_output else (acc_out, stats)

    def render_features(self, scene_data, rng_mode=0, rng_seed=1, precision=32, threads=0):
        """One frame from a cleared film: (accumulation, albedo, normal), each (H, W, 4) float32; the feature
        images hold the frame's per-pixel means with .w = resolved samples."""
        from vkrt_gb300 import abi
        sd = np.ascontiguousarray(scene_data, dtype=abi.SCENE_DATA)
        w = int(sd["viewportRect"][0][0] + sd["viewportRect"][0][2])
        h = int(sd["viewportRect"][0][1] + sd["viewportRect"][0][3])
        acc_in = np.zeros((h, w, 4), np.float32)
        acc_out, alb, nrm = (np.zeros((h, w, 4), np.float32) for _ in range(3))
        p = OracleRenderParams(rng_mode, rng_seed, precision, threads, 0, 0, 0, 1)
        r = self.lib.oracle_render_features(self.handle, _p(sd), C.byref(p), _p(acc_in), _p(acc_out), _p(alb),
                                            _p(nrm))
        if r != 0:
            raise RuntimeError(f"oracle_render_features failed ({r})")
        return acc_out, alb, nrm

    def render_f64(self, scene_data, rng_mode=0, rng_seed=1, precision=64, threads=0):
        """One frame from a cleared film, the accumulation returned in float64 (H, W, 4)."""
        from vkrt_gb300 import abi
        sd = np.ascontiguousarray(scene_data, dtype=abi.SCENE_DATA)
        w = int(sd["viewportRect"][0][0] + sd["viewportRect"][0][2])
        h = int(sd["viewportRect"][0][1] + sd["viewportRect"][0][3])
        acc_in = np.zeros((h, w, 4), np.float32)
        acc_out = np.zeros((h, w, 4), np.float64)
        p = OracleRenderParams(rng_mode, rng_seed, precision, threads, 0, 0, 0, 1)
        r = self.lib.oracle_render_f64(self.handle, _p(sd), C.byref(p), _p(acc_in), _p(acc_out))
        if r != 0:
            raise RuntimeError(f"oracle_render_f64 failed ({r})")
        return acc_out

    def env_pdf(self, direction, rotation=0.0):
        d = np.ascontiguousarray(direction, np.float32)
        return float(self.lib.oracle_env_pdf(self.handle, _p(d), rotation))

    def env_sample(self, u1, u2, rotation=0.0):
        d = np.zeros(3, np.float32)
        pdf = np.zeros(1, np.float32)
        ok = self.lib.oracle_env_sample(self.handle, u1, u2, rotation, _p(d), _p(pdf))
        return (d, float(pdf[0])) if ok == 0 else (None, 0.0)


def rgb2spec_generate(res: int, threads: int = 0) -> np.ndarray:
    lib = load()
    out = np.zeros(res + 9 * res ** 3, dtype=np.float32)
    if lib.oracle_rgb2spec_generate(res, _p(out), len(out), threads) != 0:
        raise RuntimeError("rgb2spec fit failed")
    return out


def env_cdf(rgba: np.ndarray, texel_pdf: bool = False):
    """(marginal CDF, conditional CDFs (H, W + 1), FP64 total[, texel weights (H, W)]) of the environment
    importance distribution."""
    lib = load()
    a = np.ascontiguousarray(rgba, np.float32)
    h, w = a.shape[:2]
    marg = np.zeros(h + 1, np.float32)
    cond = np.zeros(h * (w + 1), np.float32)
    tot = np.zeros(1, np.float64)
    pdf = np.zeros((h, w), np.float32)
    lib.oracle_env_cdf(_p(a), w, h, _p(marg), _p(cond), _p(tot), _p(pdf))
    if texel_pdf:
        return marg, cond.reshape(h, w + 1), float(tot[0]), pdf
    return marg, cond.reshape(h, w + 1), float(tot[0])
