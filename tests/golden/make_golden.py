"""Generates the golden fixtures in this directory from vkrt's own compiled code.

Run in a checkout that has the vkrt sources (oracle/build.py compiles vkrt's src/core/utility/packing.c and a driver
around vkrt's vendored cglm into oracle/_ref/libvkrt_ref.so):

    python tests/golden/make_golden.py

Fixtures:
  packing.npz   — vkrt packShaderVertex outputs for 512 seeded vertices plus edge cases
  camera.npz    — syncCameraMatrices (cglm lookat / perspective / inverse, Vulkan Y flip) for seeded poses
  transform.npz — VKRT_buildMeshTransformMatrix (cglm translate / rotate / scale) for seeded TRS triples
  layouts.json  — sizeof of vkrt's shared records as compiled by gcc from src/shared/types.h
  rng.npz       — Wellons-hash stream values (sampling/random.slang:7-27) from an independent numpy restatement
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def _ref():
    from oracle import build
    lib_path = build.build_reference()
    if lib_path is None:
        raise SystemExit("vkrt sources not found: set VKRT_REFERENCE to a vkrt checkout")
    lib = C.CDLL(str(lib_path))
    lib.ref_sizeof.restype = C.c_int32
    lib.ref_sizeof.argtypes = [C.c_char_p]
    lib.ref_pack_vertices.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
    lib.ref_camera_matrices.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_float,
                                        C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    lib.ref_mesh_transform.argtypes = [C.c_void_p] * 4
    return lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


def vertices(n: int, seed: int):
    from vkrt_gb300 import abi
    rng = np.random.default_rng(seed)
    v = np.zeros(n, dtype=abi.VERTEX)
    v["position"] = rng.normal(size=(n, 4)).astype(np.float32)
    v["normal"][:, :3] = rng.normal(size=(n, 3)).astype(np.float32)
    v["tangent"] = rng.normal(size=(n, 4)).astype(np.float32)
    v["color"] = rng.uniform(-0.2, 1.2, size=(n, 4)).astype(np.float32)
    v["texcoord0"] = rng.uniform(-2, 2, size=(n, 2)).astype(np.float32)
    v["texcoord1"] = rng.uniform(-2, 2, size=(n, 2)).astype(np.float32)
    # edge cases: zero-length normal/tangent, poles, octahedral folds, exact axes
    edge = [(0, 0, 0), (0, 0, 1), (0, 0, -1), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (1, 1, -1),
            (-1, 1, -1e-7), (1e-30, 0, -1)]
    for k, e in enumerate(edge):
        v["normal"][k, :3] = e
        v["tangent"][k, :3] = e
        v["tangent"][k, 3] = -1.0 if k % 2 else 1.0
    return v


def hash32(x):
    x = np.asarray(x, dtype=np.uint64) & 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7feb352d) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846ca68b) & 0xFFFFFFFF
    x ^= x >> 16
    return x.astype(np.uint32)


def pixel_seed(x, y, frame, s):
    m = 0xFFFFFFFF
    v = (np.uint64(x) * 73856093) & m
    v ^= (np.uint64(y) * 19349663) & m
    v ^= (np.uint64(frame) * 83492791) & m
    v ^= (np.uint64(s) * 2654435761) & m
    return hash32(v)


def main():
    from vkrt_gb300 import abi
    lib = _ref()
    layouts = {n: lib.ref_sizeof(n.encode()) for n in
               ["Vertex", "ShaderVertex", "MeshInfo", "Material", "EmissiveMesh", "EmissiveTriangle", "SceneData"]}
    (HERE / "layouts.json").write_text(json.dumps(layouts, indent=1) + "\n")

    v = vertices(512, 11)
    packed = np.zeros(len(v), dtype=abi.SHADER_VERTEX)
    lib.ref_pack_vertices(_p(v), len(v), _p(packed))
    np.savez_compressed(HERE / "packing.npz", vertices=v.view(np.uint8).reshape(len(v), -1),
                        packed=packed.view(np.uint8).reshape(len(v), -1))

    rng = np.random.default_rng(5)
    n = 64
    pos = rng.uniform(-20, 20, size=(n, 3)).astype(np.float32)
    tgt = rng.uniform(-5, 5, size=(n, 3)).astype(np.float32)
    fov = rng.uniform(20, 90, size=n).astype(np.float32)
    wh = rng.integers(16, 4096, size=(n, 2)).astype(np.uint32)
    vi = np.zeros((n, 16), np.float32)
    pi = np.zeros((n, 16), np.float32)
    up = np.array([0, 0, 1], np.float32)
    for k in range(n):
        lib.ref_camera_matrices(_p(pos[k]), _p(tgt[k]), _p(up), float(fov[k]), 0.001, 10000.0, int(wh[k, 0]),
                                int(wh[k, 1]), _p(vi[k]), _p(pi[k]))
    np.savez_compressed(HERE / "camera.npz", pos=pos, target=tgt, vfov=fov, wh=wh, viewInverse=vi, projInverse=pi)

    tp = rng.uniform(-10, 10, size=(n, 3)).astype(np.float32)
    tr = rng.uniform(-180, 180, size=(n, 3)).astype(np.float32)
    ts = rng.uniform(0.2, 3, size=(n, 3)).astype(np.float32) * rng.choice([-1, 1], size=(n, 3)).astype(np.float32)
    tm = np.zeros((n, 16), np.float32)
    for k in range(n):
        lib.ref_mesh_transform(_p(tp[k]), _p(tr[k]), _p(ts[k]), _p(tm[k]))
    np.savez_compressed(HERE / "transform.npz", position=tp, rotation=tr, scale=ts, matrix=tm)

    inputs = np.arange(0, 1 << 20, 4099, dtype=np.uint32)
    seeds = pixel_seed(17, 29, 3, 5)
    stream = []
    h = np.uint32(seeds)
    for _ in range(64):
        h = hash32(np.uint64(h) + 0x9e3779b9)
        stream.append(h)
    np.savez_compressed(HERE / "rng.npz", inputs=inputs, hashes=hash32(inputs),
                        seed_xyfs=np.array([17, 29, 3, 5], np.uint32), seed=np.array([seeds], np.uint32),
                        stream=np.array(stream, np.uint32))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
