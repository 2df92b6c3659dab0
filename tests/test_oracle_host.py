"""The oracle's numpy restatement of vkrt's host scene layer (oracle/host.py), which the CPU reference run builds its
scenes with: against the vectors vkrt's own packing.c and cglm produced (tests/golden) and against the backend's
host library, record by record, on the benchmark's scenes."""
from pathlib import Path

import numpy as np
import pytest

from oracle import host
from vkrt_gb300 import abi, context, scenes

GOLD = Path(__file__).resolve().parent / "golden"


def test_pack_vertices_bit_exact_vs_vkrt():
    g = np.load(GOLD / "packing.npz")
    v = g["vertices"].view(abi.VERTEX).reshape(-1)
    want = g["packed"].view(abi.SHADER_VERTEX).reshape(-1)
    got = host.pack_vertices(v)
    for f in ("position", "texcoord0", "texcoord1", "packedNormal", "packedTangent", "packedColor"):
        np.testing.assert_array_equal(got[f], want[f], err_msg=f)


def test_camera_matrices_vs_cglm():
    g = np.load(GOLD / "camera.npz")
    for k in range(len(g["pos"])):
        sd = np.zeros(1, abi.SCENE_DATA)
        sd["viewportRect"] = (0, 0, int(g["wh"][k, 0]), int(g["wh"][k, 1]))
        host.camera_matrices(sd, g["pos"][k], g["target"][k], (0.0, 0.0, 1.0), float(g["vfov"][k]))
        np.testing.assert_allclose(sd["viewInverse"][0].reshape(16), g["viewInverse"][k], rtol=2e-5, atol=2e-5)
        np.testing.assert_allclose(sd["projInverse"][0].reshape(16), g["projInverse"][k], rtol=2e-5, atol=1e-6)


def test_mesh_transform_vs_cglm():
    g = np.load(GOLD / "transform.npz")
    for k in range(len(g["position"])):
        m = host.mesh_transform(g["position"][k], g["rotation"][k], g["scale"][k])
        np.testing.assert_allclose(m.T.reshape(16), g["matrix"][k], rtol=1e-5, atol=2e-6)


@pytest.mark.parametrize("n", [1, 2, 7, 64, 1000])
def test_alias_table_same_as_host_library(built, n):
    rng = np.random.default_rng(n)
    pmf = rng.exponential(size=n).astype(np.float32)
    pmf /= pmf.sum()
    q = np.zeros(n, np.float32)
    idx = np.zeros(n, np.uint32)
    abi.load().vkrt_host_build_alias_table(abi.ptr(pmf), n, abi.ptr(q), abi.ptr(idx))
    oq, oidx = host.build_alias_table(pmf)
    np.testing.assert_array_equal(oq, q)
    np.testing.assert_array_equal(oidx, idx)


def test_default_records_same_as_host_library(built):
    np.testing.assert_array_equal(host.default_material().view(np.uint8),
                                  scenes.ProductHost.default_material().view(np.uint8))
    a, b = host.default_scene_data(320, 200), scenes.ProductHost.default_scene_data(320, 200)
    for f in abi.SCENE_DATA.names:
        if f in ("viewInverse", "projInverse"):
            np.testing.assert_allclose(a[f], b[f], rtol=2e-6, atol=2e-7, err_msg=f)
        else:
            np.testing.assert_array_equal(a[f], b[f], err_msg=f)


@pytest.mark.parametrize("which", ["cornell", "field"])
def test_benchmark_scenes_same_through_either_host(built, which):
    """The oracle-built scene is the product-built one: identical geometry, materials, packing and light tables;
    camera matrices within FP32 rounding of the two inverse computations."""
    if which == "cornell":
        a, b = scenes.cornell(64, 64, host=host.OracleHost), scenes.cornell(64, 64)
    else:
        kw = dict(n_spheres=40, width=64, height=48, seed=3, spectral=True, env_size=(64, 32))
        a, b = scenes.icosphere_field(host=host.OracleHost, **kw), scenes.icosphere_field(**kw)
    for f in ("vertices", "indices", "meshes", "materials"):
        np.testing.assert_array_equal(getattr(a, f).view(np.uint8), getattr(b, f).view(np.uint8), err_msg=f)
    np.testing.assert_array_equal(a.shader_vertices.view(np.uint8),
                                  context.pack_vertices(b.vertices).view(np.uint8))
    for f in ("emissive_meshes", "emissive_triangles", "mesh_alias_q", "mesh_alias_idx", "tri_alias_q",
              "tri_alias_idx", "emissive_mesh_materials"):
        np.testing.assert_array_equal(np.asarray(getattr(a, f)).view(np.uint8),
                                      np.asarray(getattr(b, f)).view(np.uint8), err_msg=f)
    for f in abi.SCENE_DATA.names:
        if f in ("viewInverse", "projInverse"):
            np.testing.assert_allclose(a.scene_data[f], b.scene_data[f], rtol=2e-6, atol=2e-7, err_msg=f)
        else:
            np.testing.assert_array_equal(a.scene_data[f], b.scene_data[f], err_msg=f)
