"""vkrt_gb300 — GB300 (sm_103a) path-tracing backend for vkrt behind a C ABI.

The product is libvkrt_gb300.so (CUDA kernels + C host layer, see include/vkrt_cuda.h). This package holds its build
script, the ctypes view of the ABI (abi.py), a thin Python host mirror (context.py) and seeded scene generators
(scenes.py). Nothing here renders on the CPU.
"""
from . import abi
from .context import AutoSpp, RenderContext, Scene, VkrtError, build_light_tables, pack_vertices

__all__ = ["abi", "RenderContext", "Scene", "VkrtError", "build_light_tables", "pack_vertices"]
