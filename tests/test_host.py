"""Host scene preparation (vkrt_gb300/csrc/host/scene_host.c) against vkrt's own compiled code: golden fixtures
generated by tests/golden/make_golden.py from vkrt's packing.c and vendored cglm."""
from pathlib import Path

import numpy as np
import pytest

from vkrt_gb300 import abi, context, scenes

GOLD = Path(__file__).resolve().parent / "golden"


def test_pack_shader_vertex_bit_exact_vs_vkrt(built):
    g = np.load(GOLD / "packing.npz")
    v = g["vertices"].view(abi.VERTEX).reshape(-1)
    want = g["packed"].view(abi.SHADER_VERTEX).reshape(-1)
    got = context.pack_vertices(v)
    for f in ("position", "texcoord0", "texcoord1", "packedNormal", "packedTangent", "packedColor"):
        np.testing.assert_array_equal(got[f], want[f], err_msg=f)


def test_camera_matrices_vs_cglm(built):
    g = np.load(GOLD / "camera.npz")
    lib = abi.load()
    up = np.array([0, 0, 1], np.float32)
    for k in range(len(g["pos"])):
        sd = np.zeros(1, abi.SCENE_DATA)
        pos = np.ascontiguousarray(g["pos"][k])
        tgt = np.ascontiguousarray(g["target"][k])
        lib.vkrt_host_camera_matrices(abi.ptr(pos), abi.ptr(tgt), abi.ptr(up),
                                      float(g["vfov"][k]), 0.001, 10000.0, int(g["wh"][k, 0]), int(g["wh"][k, 1]),
                                      abi.ptr(sd))
        np.testing.assert_allclose(sd["viewInverse"][0].reshape(16), g["viewInverse"][k], rtol=2e-5, atol=2e-5)
        np.testing.assert_allclose(sd["projInverse"][0].reshape(16), g["projInverse"][k], rtol=2e-5, atol=1e-6)


def test_mesh_transform_vs_cglm(built):
    g = np.load(GOLD / "transform.npz")
    lib = abi.load()
    for k in range(len(g["position"])):
        out = np.zeros(16, np.float32)
        p, r, sc = (np.ascontiguousarray(g[f][k]) for f in ("position", "rotation", "scale"))
        lib.vkrt_host_mesh_transform(abi.ptr(p), abi.ptr(r), abi.ptr(sc), abi.ptr(out))
        np.testing.assert_allclose(out, g["matrix"][k], rtol=1e-5, atol=2e-6)


@pytest.mark.parametrize("n", [1, 2, 7, 64, 1000])
def test_alias_table_reproduces_pmf(built, n):
    rng = np.random.default_rng(n)
    pmf = rng.exponential(size=n).astype(np.float32)
    pmf /= pmf.sum()
    q = np.zeros(n, np.float32)
    idx = np.zeros(n, np.uint32)
    abi.load().vkrt_host_build_alias_table(abi.ptr(pmf), n, abi.ptr(q), abi.ptr(idx))
    # exact probability mass implied by the table (sampleAlias, sampling/discrete.slang:13-18)
    mass = q.astype(np.float64) / n
    np.add.at(mass, idx, (1.0 - q.astype(np.float64)) / n)
    np.testing.assert_allclose(mass, pmf, atol=2e-6)
    assert (idx < n).all() and (q >= 0).all() and (q <= 1.0).all()


def test_light_tables_cornell(built):
    s = scenes.cornell(32, 32)
    assert s.scene_data["emissiveMeshCount"][0] == 1 and s.scene_data["emissiveTriangleCount"][0] == 2
    em = s.emissive_meshes[0]
    assert em["triCount"] == 2 and em["pmfMesh"] == 1.0
    np.testing.assert_allclose(em["invTotalArea"], 1 / 0.0625, rtol=1e-5)
    np.testing.assert_allclose(em["emission"], [15, 15, 15])
    np.testing.assert_allclose(s.emissive_triangles["v0Area"][:, 3], [0.03125, 0.03125], rtol=1e-5)
    light = int(np.nonzero(s.meshes["lightPdfArea"])[0][0])
    assert s.materials[s.meshes[light]["materialIndex"]]["emissionLuminance"] == 15.0
    np.testing.assert_allclose(s.meshes[light]["lightPdfArea"], 16.0, rtol=1e-5)
