"""The C-ABI library loads and exports every entry point include/*.h declares; record layouts match vkrt's."""
import json
import re
from pathlib import Path

import numpy as np

from vkrt_gb300 import abi

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(vkrt_(?:cuda|host)_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(built):
    lib = abi.load(build_if_missing=False)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert names <= set(abi.EXPORTS), sorted(names - set(abi.EXPORTS))


def test_record_sizes_match_vkrt():
    ref = json.loads((ROOT / "tests/golden/layouts.json").read_text())
    assert abi.VERTEX.itemsize == ref["Vertex"]
    assert abi.SHADER_VERTEX.itemsize == ref["ShaderVertex"]
    assert abi.MESH_INFO.itemsize == ref["MeshInfo"]
    assert abi.MATERIAL.itemsize == ref["Material"]
    assert abi.EMISSIVE_MESH.itemsize == ref["EmissiveMesh"]
    assert abi.EMISSIVE_TRIANGLE.itemsize == ref["EmissiveTriangle"]
    assert abi.SCENE_DATA.itemsize == ref["SceneData"]


def test_host_defaults_read_through_the_layouts(built):
    """vkrt defaults written by the C host library land on the numpy field offsets (vkrt_types.h:79-121,
    uniform.c:93-174)."""
    lib = abi.load()
    m = np.zeros(1, abi.MATERIAL)
    lib.vkrt_host_default_material(abi.ptr(m))
    assert np.allclose(m["baseColor"], 0.8) and m["roughness"] == np.float32(0.5) and m["ior"] == np.float32(1.5)
    assert m["baseColorTextureIndex"] == abi.INVALID_INDEX and m["emissiveTextureIndex"] == abi.INVALID_INDEX
    assert np.allclose(m["baseColorTextureTransform"], [1, 1, 0, 0]) and m["opacity"] == 1.0
    sd = np.zeros(1, abi.SCENE_DATA)
    lib.vkrt_host_default_scene_data(640, 480, abi.ptr(sd))
    assert sd["samplesPerPixel"] == 8 and sd["rrMaxDepth"] == 8 and sd["rrMinDepth"] == 4
    assert list(sd["viewportRect"][0]) == [0, 0, 640, 480]
    assert sd["environmentTextureIndex"] == abi.INVALID_INDEX and sd["misNeeEnabled"] == 1
    assert np.allclose(sd["environmentLight"][0], [0.25, 0.25, 0.25, 1.0])
    assert sd["packedRenderSettings"] == abi.pack_render_settings(1, 0, 1)
    # camera at (-0.5, 0.2, -0.2): the inverse view's translation column is the eye position
    assert np.allclose(sd["viewInverse"][0][3, :3], [-0.5, 0.2, -0.2], atol=1e-6)


def test_context_config_is_validated_before_any_device_call(built):
    """vkrt_cuda_create refuses out-of-range configuration fields with VKRT_ERROR_INVALID_ARGUMENT before it looks
    for a device, so this runs without a GPU."""
    import ctypes as C
    lib = abi.load()
    cfg = np.zeros(1, abi.CONFIG)
    lib.vkrt_cuda_default_config(abi.ptr(cfg))
    assert cfg["treeletPasses"] == 0 and cfg["treeletMinTriangles"] == 0 and cfg["treeletsOnUpdate"] == 0
    for field, bad in (("treeletPasses", 9), ("treeletsOnUpdate", 2), ("rngMode", 7), ("environmentSampling", 5)):
        c = cfg.copy()
        c[field] = bad
        handle = C.c_void_p()
        assert lib.vkrt_cuda_create(abi.ptr(c), C.byref(handle)) == abi.ERROR_INVALID_ARGUMENT, field
        assert not handle.value


def test_backend_records_match_the_header(tmp_path):
    """The numpy layouts of the backend's own records (configuration, statistics, rays, hits, gradients) have the
    field offsets and sizes the C header gives them: a probe compiled against include/vkrt_cuda.h prints offsetof
    and sizeof for every field abi.py declares."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    records = {"VKRT_CudaConfig": abi.CONFIG, "VKRT_CudaWavefrontConfig": abi.WAVEFRONT_CONFIG,
               "VKRT_CudaStats": abi.STATS, "VKRT_CudaRay": abi.RAY, "VKRT_CudaHit": abi.HIT,
               "VKRT_CudaAdjointConfig": abi.ADJOINT_CONFIG, "VKRT_CudaMaterialGradient": abi.MATERIAL_GRADIENT,
               "VKRT_CudaNrcConfig": abi.NRC_CONFIG}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "vkrt_cuda.h"', "int main(void) {"]
    for rec, dt in records.items():
        lines.append(f'printf("{rec} size %zu\\n", sizeof({rec}));')
        for name in dt.names:
            lines.append(f'printf("{rec} {name} %zu %zu\\n", offsetof({rec}, {name}), sizeof((({rec}*)0)->{name}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in filter(None, out):
        parts = line.split()
        if parts[1] == "size":
            got[(parts[0], None)] = int(parts[2])
        else:
            got[(parts[0], parts[1])] = (int(parts[2]), int(parts[3]))
    for rec, dt in records.items():
        assert got[(rec, None)] == dt.itemsize, rec
        for name in dt.names:
            off, size = got[(rec, name)]
            assert (dt.fields[name][1], dt.fields[name][0].itemsize) == (off, size), (rec, name)
