"""ctypes view of the C ABI in include/vkrt_cuda.h and include/vkrt_cuda_host.h.

Records are numpy structured dtypes with the exact offsets of vkrt's shared layouts (src/shared/types.h:25-159), so
arrays built here are handed to the library as plain pointers, the way a vkrt host hands over its own arrays.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

INVALID_INDEX = 0xFFFFFFFF

# ---- record layouts ---------------------------------------------------------------------------------------------
VERTEX = np.dtype({
    "names": ["position", "normal", "tangent", "color", "texcoord0", "texcoord1"],
    "formats": [("<f4", 4), ("<f4", 4), ("<f4", 4), ("<f4", 4), ("<f4", 2), ("<f4", 2)],
    "offsets": [0, 16, 32, 48, 64, 72], "itemsize": 80})

SHADER_VERTEX = np.dtype({
    "names": ["position", "texcoord0", "texcoord1", "packedNormal", "packedTangent", "packedColor"],
    "formats": [("<f4", 4), ("<f4", 2), ("<f4", 2), "<u4", "<u4", "<u4"],
    "offsets": [0, 16, 24, 32, 36, 40], "itemsize": 48})

MESH_INFO = np.dtype({
    "names": ["position", "vertexBase", "rotation", "vertexCount", "scale", "indexBase", "indexCount",
              "materialIndex", "renderBackfaces", "lightPdfArea", "opacity", "reserved0", "reserved1", "reserved2"],
    "formats": [("<f4", 3), "<u4", ("<f4", 3), "<u4", ("<f4", 3), "<u4", "<u4", "<u4", "<u4", "<f4", "<f4", "<u4",
                "<u4", "<u4"],
    "offsets": [0, 12, 16, 28, 32, 44, 48, 52, 56, 60, 64, 68, 72, 76], "itemsize": 80})

_MAT_FIELDS = [
    ("baseColor", ("<f4", 3), 0), ("roughness", "<f4", 12), ("emissionColor", ("<f4", 3), 16),
    ("emissionLuminance", "<f4", 28), ("eta", ("<f4", 3), 32), ("metallic", "<f4", 44), ("k", ("<f4", 3), 48),
    ("anisotropic", "<f4", 60), ("specular", "<f4", 64), ("specularTint", "<f4", 68), ("abbeNumber", "<f4", 72),
    ("reserved0", "<f4", 76), ("sheenTintWeight", ("<f4", 4), 80), ("clearcoat", "<f4", 96),
    ("clearcoatGloss", "<f4", 100), ("ior", "<f4", 104), ("diffuseRoughness", "<f4", 108),
    ("transmission", "<f4", 112), ("subsurface", "<f4", 116), ("sheenRoughness", "<f4", 120),
    ("absorptionCoefficient", "<f4", 124), ("attenuationColor", ("<f4", 3), 128), ("normalTextureScale", "<f4", 140),
    ("baseColorTextureIndex", "<u4", 144), ("metallicRoughnessTextureIndex", "<u4", 148),
    ("normalTextureIndex", "<u4", 152), ("emissiveTextureIndex", "<u4", 156), ("baseColorTextureWrap", "<u4", 160),
    ("metallicRoughnessTextureWrap", "<u4", 164), ("normalTextureWrap", "<u4", 168),
    ("emissiveTextureWrap", "<u4", 172), ("opacity", "<f4", 176), ("alphaCutoff", "<f4", 180),
    ("alphaMode", "<u4", 184), ("textureTexcoordSets", "<u4", 188), ("baseColorTextureTransform", ("<f4", 4), 192),
    ("metallicRoughnessTextureTransform", ("<f4", 4), 208), ("normalTextureTransform", ("<f4", 4), 224),
    ("emissiveTextureTransform", ("<f4", 4), 240), ("textureRotations", ("<f4", 4), 256)]
MATERIAL = np.dtype({"names": [f[0] for f in _MAT_FIELDS], "formats": [f[1] for f in _MAT_FIELDS],
                     "offsets": [f[2] for f in _MAT_FIELDS], "itemsize": 272})

EMISSIVE_MESH = np.dtype({
    "names": ["triOffset", "triCount", "pmfMesh", "invTotalArea", "emission", "reserved0"],
    "formats": ["<u4", "<u4", "<f4", "<f4", ("<f4", 3), "<f4"], "offsets": [0, 4, 8, 12, 16, 28], "itemsize": 32})

EMISSIVE_TRIANGLE = np.dtype({"names": ["v0Area", "e1Pad", "e2Pad"],
                              "formats": [("<f4", 4), ("<f4", 4), ("<f4", 4)], "offsets": [0, 16, 32],
                              "itemsize": 48})

SCENE_DATA = np.dtype({
    "names": ["viewInverse", "projInverse", "frameNumber", "samplesPerPixel", "rrMaxDepth", "rrMinDepth",
              "viewportRect", "packedRenderSettings", "exposure", "timeBase", "timeStep", "environmentLight",
              "environmentTextureIndex", "environmentRotation", "debugMode", "misNeeEnabled", "emissiveMeshCount",
              "emissiveTriangleCount", "selectionEnabled", "selectedMeshIndex", "rgb2specSRGB"],
    "formats": [("<f4", (4, 4)), ("<f4", (4, 4)), "<u4", "<u4", "<u4", "<u4", ("<u4", 4), "<u4", "<f4", "<f4",
                "<f4", ("<f4", 4), "<u4", "<f4", "<u4", "<u4", "<u4", "<u4", "<u4", "<u4", ("<u4", 3)],
    "offsets": [0, 64, 128, 132, 136, 140, 144, 160, 164, 168, 172, 176, 192, 196, 200, 204, 208, 212, 216, 220, 224],
    "itemsize": 240})

RAY = np.dtype({"names": ["origin", "tMin", "direction", "tMax"], "formats": [("<f4", 3), "<f4", ("<f4", 3), "<f4"],
                "offsets": [0, 12, 16, 28], "itemsize": 32})

HIT = np.dtype({"names": ["instanceIndex", "primitiveIndex", "t", "u", "v", "reserved"],
                "formats": ["<u4", "<u4", "<f4", "<f4", "<f4", ("<u4", 3)], "offsets": [0, 4, 8, 12, 16, 20],
                "itemsize": 32})

CONFIG = np.dtype({"names": ["deviceIndex", "rngMode", "rngSeed", "environmentSampling", "countRays",
                             "threadsPerBlock", "blocksPerSM", "integrator", "treeletMinTriangles",
                             "treeletsOnUpdate", "treeletPasses", "reserved"],
                   "formats": ["<i4", "<u4", "<u8", "<u4", "<u4", "<u4", "<u4", "<u4", "<u4", "<u4", "<u4",
                               ("<u4", 4)],
                   "offsets": [0, 4, 8, 16, 20, 24, 28, 32, 36, 40, 44, 48], "itemsize": 64})

WAVEFRONT_CONFIG = np.dtype({"names": ["queueCapacity", "tileWidth", "tileHeight", "sortByMaterial",
                                       "intersectBlocksPerSM", "shadeBlocksPerSM", "useGraph", "profileStages",
                                       "refillLanes", "rayOrder", "reserved"],
                             "formats": ["<u4"] * 10 + [("<u4", 6)],
                             "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40], "itemsize": 64})

STATS = np.dtype({"names": ["primaryRays", "extensionRays", "shadowRays", "pathSamples", "nodeFetchBytes",
                            "triFetchBytes", "bvhNodeCount", "bvhTriangleCount", "bvhBytes", "bvhBuildMs",
                            "errorFlags", "wavefrontBodies", "cacheTrainingRecords", "shadowNodeFetchBytes",
                            "shadowTriFetchBytes", "kernelLaunches", "stageMs", "bvhSahLbvh", "bvhSahTreelets"],
                  "formats": ["<u8", "<u8", "<u8", "<u8", "<u8", "<u8", "<u4", "<u4", "<u8", "<f4", "<u4", "<u4",
                              "<u4", "<u8", "<u8", "<u8", ("<f4", 8), "<f4", "<f4"],
                  "offsets": [0, 8, 16, 24, 32, 40, 48, 52, 56, 64, 68, 72, 76, 80, 88, 96, 104, 136, 140],
                  "itemsize": 144})

WAVEFRONT_STAGES = ("prologue", "begin", "intersect", "sort", "shade", "shadow", "finalize", "resolve")

ADJOINT_CONFIG = np.dtype({"names": ["sampleBase", "gradients", "accumulate", "reserved"],
                           "formats": ["<u4", "<u4", "<u4", ("<u4", 5)], "offsets": [0, 4, 8, 12], "itemsize": 32})

MATERIAL_GRADIENT = np.dtype({"names": ["baseColor", "roughness", "emission", "reserved"],
                              "formats": [("<f4", 3), "<f4", ("<f4", 3), "<f4"], "offsets": [0, 12, 16, 28],
                              "itemsize": 32})

GRADIENT_BASE_COLOR, GRADIENT_ROUGHNESS, GRADIENT_EMISSION = 1, 2, 4

NRC_CONFIG = np.dtype({"names": ["enabled", "terminationDepth", "trainingPaths", "trainingSteps", "learningRate", "seed",
                                 "inferenceTensorPath", "inferenceAverage", "terminationSpread", "trainingTracer",
                                 "reserved"],
                       "formats": ["<u4", "<u4", "<u4", "<u4", "<f4", "<u4", "<u4", "<f4", "<f4", "<u4", ("<u4", 6)],
                       "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40], "itemsize": 64})
NRC_TCGEN05, NRC_MMA_SYNC = 0, 1
NRC_INPUT_FLOATS, NRC_WEIGHTS, NRC_TABLE_HALVES = 16, 21504, 16777216

# constants (src/shared/constants.h)
TONE_MAPPING_NONE, TONE_MAPPING_ACES = 0, 1
RENDER_MODE_RGB, RENDER_MODE_SPECTRAL = 0, 1
SPECTRAL_SINGLE, SPECTRAL_HERO = 0, 1
RNG_REFERENCE, RNG_PCG32 = 0, 1
ENV_BSDF_ONLY, ENV_IMPORTANCE = 0, 1
INTEGRATOR_MEGAKERNEL, INTEGRATOR_WAVEFRONT = 0, 1
TRACE_ANY_HIT, TRACE_PERSISTENT = 1, 2
TEXTURE_FORMAT_RGBA8_UNORM, TEXTURE_FORMAT_RGBA16_UNORM, TEXTURE_FORMAT_RGBA16_SFLOAT, TEXTURE_FORMAT_RGBA32_SFLOAT = 0, 1, 2, 3
COLOR_SPACE_SRGB, COLOR_SPACE_LINEAR = 0, 1
WRAP_REPEAT, WRAP_CLAMP, WRAP_MIRROR = 10497, 33071, 33648

SUCCESS = 0
ERROR_INVALID_ARGUMENT = -1
ERROR_OPERATION_FAILED = -2
ERROR_OUT_OF_MEMORY = -3
ERROR_DEVICE_LOST = -4
ERROR_INITIALIZATION_FAILED = -5


def pack_render_settings(tone: int, mode: int, spectral: int) -> int:
    return (tone & 0xFFFF) | ((mode & 0xFF) << 16) | ((spectral & 0xFF) << 24)


def unpack_render_settings(packed: int) -> tuple[int, int, int]:
    """(tone mapping mode, render mode, spectral sampling mode)"""
    return packed & 0xFFFF, (packed >> 16) & 0xFF, (packed >> 24) & 0xFF


def ptr(a: np.ndarray | None) -> C.c_void_p:
    if a is None:
        return C.c_void_p(None)
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("arrays passed to the C ABI must be C-contiguous")
    return C.c_void_p(a.ctypes.data)


# ---- library loading ------------------------------------------------------------------------------------------------
_LIB_PATH = Path(__file__).resolve().parent / "libvkrt_gb300.so"

# name -> (restype, argtypes); every pointer is passed as c_void_p
_V, _I32, _U32, _U64, _SZ, _F = C.c_void_p, C.c_int32, C.c_uint32, C.c_uint64, C.c_size_t, C.c_float
EXPORTS = {
    "vkrt_cuda_default_config": (None, [_V]),
    "vkrt_cuda_create": (_I32, [_V, _V]),
    "vkrt_cuda_destroy": (None, [_V]),
    "vkrt_cuda_upload_geometry": (_I32, [_V, _V, _U32, _V, _U32, _V, _U32]),
    "vkrt_cuda_update_meshes": (_I32, [_V, _V, _U32]),
    "vkrt_cuda_upload_materials": (_I32, [_V, _V, _U32]),
    "vkrt_cuda_upload_lights": (_I32, [_V, _V, _U32, _V, _U32, _V, _V, _V, _V]),
    "vkrt_cuda_upload_texture": (_I32, [_V, _U32, _V, _U32, _U32, _U32, _U32]),
    "vkrt_cuda_set_environment": (_I32, [_V, _U32]),
    "vkrt_cuda_read_environment_distribution": (_I32, [_V, _U32, _U32, _V, _V, _V]),
    "vkrt_cuda_upload_rgb2spec": (_I32, [_V, _V, _U32, _V]),
    "vkrt_cuda_upload_sheen_table": (_I32, [_V, _V, _U32]),
    "vkrt_cuda_generate_rgb2spec": (_I32, [_V, _U32, _V]),
    "vkrt_cuda_download_rgb2spec": (_I32, [_V, _V, _U32]),
    "vkrt_cuda_resize": (_I32, [_V, _U32, _U32]),
    "vkrt_cuda_reset_accumulation": (_I32, [_V]),
    "vkrt_cuda_render_frame": (_I32, [_V, _V]),
    "vkrt_cuda_sync": (_I32, [_V, _U32]),
    "vkrt_cuda_read_accumulation": (_I32, [_V, _V, _SZ]),
    "vkrt_cuda_read_accumulation_async": (_I32, [_V, _V, _SZ]),
    "vkrt_cuda_wait_readback": (_I32, [_V, _U32]),
    "vkrt_cuda_read_output": (_I32, [_V, _V, _SZ]),
    "vkrt_cuda_get_stats": (_I32, [_V, _V]),
    "vkrt_cuda_stream": (_V, [_V]),
    "vkrt_cuda_trace_rays": (_I32, [_V, _V, _U32, _U32, _V]),
    "vkrt_cuda_trace_rays_device": (_I32, [_V, _V, _U32, _U32, _V]),
    "vkrt_cuda_trace_rays_noalloc": (_I32, [_V, _V, _U32, _U32, _V]),
    "vkrt_cuda_last_error": (C.c_char_p, [_V]),
    "vkrt_cuda_set_integrator": (_I32, [_V, _U32]),
    "vkrt_cuda_default_wavefront_config": (None, [_V]),
    "vkrt_cuda_set_wavefront_config": (_I32, [_V, _V]),
    "vkrt_cuda_get_wavefront_config": (_I32, [_V, _V]),
    "vkrt_cuda_render_batch": (_I32, [_V, _V, _U32]),
    "vkrt_cuda_autotune_batch": (_I32, [_V, _V, _U32, _U32, _V, _V]),
    "vkrt_cuda_default_adjoint_config": (None, [_V]),
    "vkrt_cuda_set_emissive_mesh_materials": (_I32, [_V, _V, _U32]),
    "vkrt_cuda_render_adjoint": (_I32, [_V, _V, _V, _V]),
    "vkrt_cuda_render_adjoint_device": (_I32, [_V, _V, _V, _V]),
    "vkrt_cuda_read_texture_gradient": (_I32, [_V, _U32, _V, _SZ]),
    "vkrt_cuda_read_material_gradients": (_I32, [_V, _V, _U32]),
    "vkrt_cuda_default_nrc_config": (None, [_V]),
    "vkrt_cuda_nrc_configure": (_I32, [_V, _V]),
    "vkrt_cuda_nrc_infer": (_I32, [_V, _V, _U32, _V]),
    "vkrt_cuda_nrc_read_training_records": (_I32, [_V, _V, _V, _U32, _V]),
    "vkrt_cuda_nrc_train": (_I32, [_V, _V, _V, _U32, _U32, _V]),
    "vkrt_cuda_nrc_parameters": (_I32, [_V, _V, _V, _U32]),
    "vkrt_cuda_nrc_gradients": (_I32, [_V, _V, _V]),
    "vkrt_cuda_nrc_grid": (_I32, [_V, _V, _V, _V, _V]),
    "vkrt_cuda_render_selection_overlay": (_I32, [_V, _V]),
    "vkrt_cuda_read_selection_mask": (_I32, [_V, _V, _SZ]),
    "vkrt_cuda_pick_mesh": (_I32, [_V, _V, _U32, _U32, _V]),
    "vkrt_cuda_last_frame_ms": (_I32, [_V, _V]),
    "vkrt_cuda_set_denoiser_features": (_I32, [_V, _U32]),
    "vkrt_cuda_read_denoiser_features": (_I32, [_V, _V, _V, _SZ]),
    "vkrt_host_pack_shader_vertices": (None, [_V, _U32, _V]),
    "vkrt_host_mesh_transform": (None, [_V, _V, _V, _V]),
    "vkrt_host_camera_matrices": (None, [_V, _V, _V, _F, _F, _F, _U32, _U32, _V]),
    "vkrt_host_default_scene_data": (None, [_U32, _U32, _V]),
    "vkrt_host_build_light_tables": (_I32, [_V, _U32, _V, _U32, _V, _V, _V, _U32, _V, _U32, _V, _V, _V, _V, _V, _V]),
    "vkrt_host_build_alias_table": (None, [_V, _U32, _V, _V]),
    "vkrt_host_default_material": (None, [_V]),
    "vkrt_host_auto_spp_init": (None, [_V, _U32]),
    "vkrt_host_auto_spp_update": (_I32, [_V, _F, _V]),
    "vkrt_host_png_unfilter": (_I32, [_V, _U32, _U64, _U32, _V]),
}

# VKRT_CudaAutoSpp
AUTO_SPP = np.dtype([("targetFrameMs", "<f4"), ("controlMs", "<f4")])

_lib: C.CDLL | None = None


def library_path() -> Path:
    return _LIB_PATH


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads libvkrt_gb300.so (building it first when absent). Raises when it cannot be loaded: there is no
    fallback implementation."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists() and build_if_missing:
        from . import build as _build
        _build.build()
    if not _LIB_PATH.exists():
        raise RuntimeError(f"{_LIB_PATH} is missing: build it with python -m vkrt_gb300.build")
    lib = C.CDLL(str(_LIB_PATH))
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
