"""Minimal GLB writer for the scene-file tests: triangle meshes (positions, optional normals / texture coordinates /
tangents, uint32 indices) on nodes with TRS transforms and metallic-roughness materials. glTF 2.0, Y-up."""
from __future__ import annotations

import json
import struct

import numpy as np


def write_glb(path, meshes, nodes=None, materials=None, images=None, textures=None, samplers=None):
    """meshes: list of dicts with 'positions' (n, 3) and optional 'normals', 'uv', 'tangents' (n, 4), 'indices',
    'material'. nodes: list of dicts (glTF node fields: 'mesh', 'translation', 'rotation', 'scale', 'children',
    'name'); default one node per mesh. materials: list of glTF material dicts. images: list of (bytes, MIME type)
    stored in buffer views, or {'uri': ...} dicts; textures and samplers: glTF dicts."""
    blob = bytearray()
    views, accessors = [], []

    def add(array, target, kind, comp):
        nonlocal blob
        while len(blob) % 4:
            blob += b"\0"
        data = np.ascontiguousarray(array).tobytes()
        views.append({"buffer": 0, "byteOffset": len(blob), "byteLength": len(data), "target": target})
        blob += data
        acc = {"bufferView": len(views) - 1, "componentType": comp, "count": int(len(array)), "type": kind}
        if kind == "VEC3" and comp == 5126:
            acc["min"] = np.asarray(array).min(0).tolist()
            acc["max"] = np.asarray(array).max(0).tolist()
        accessors.append(acc)
        return len(accessors) - 1

    gl_meshes = []
    for m in meshes:
        attrs = {"POSITION": add(np.asarray(m["positions"], np.float32), 34962, "VEC3", 5126)}
        if m.get("normals") is not None:
            attrs["NORMAL"] = add(np.asarray(m["normals"], np.float32), 34962, "VEC3", 5126)
        if m.get("uv") is not None:
            attrs["TEXCOORD_0"] = add(np.asarray(m["uv"], np.float32), 34962, "VEC2", 5126)
        if m.get("tangents") is not None:
            attrs["TANGENT"] = add(np.asarray(m["tangents"], np.float32), 34962, "VEC4", 5126)
        prim = {"attributes": attrs, "mode": 4,
                "indices": add(np.asarray(m["indices"], np.uint32).reshape(-1), 34963, "SCALAR", 5125)}
        if m.get("material") is not None:
            prim["material"] = m["material"]
        gl_meshes.append({"name": m.get("name", f"mesh{len(gl_meshes)}"), "primitives": [prim]})
    if nodes is None:
        nodes = [{"mesh": i, "name": gl_meshes[i]["name"]} for i in range(len(gl_meshes))]
    children = {c for nd in nodes for c in nd.get("children", [])}
    doc = {"asset": {"version": "2.0"}, "scene": 0,
           "scenes": [{"nodes": [i for i in range(len(nodes)) if i not in children]}],
           "nodes": nodes, "meshes": gl_meshes, "accessors": accessors, "bufferViews": views,
           "buffers": [{"byteLength": len(blob)}]}
    if materials:
        doc["materials"] = materials
    if images:
        gl_images = []
        for im in images:
            if isinstance(im, dict):
                gl_images.append(im)
                continue
            data, mime = im
            while len(blob) % 4:
                blob += b"\0"
            views.append({"buffer": 0, "byteOffset": len(blob), "byteLength": len(data)})
            blob += data
            gl_images.append({"bufferView": len(views) - 1, "mimeType": mime})
        doc["images"] = gl_images
        doc["buffers"][0]["byteLength"] = len(blob)
    if textures:
        doc["textures"] = textures
    if samplers:
        doc["samplers"] = samplers
    js = json.dumps(doc).encode()
    js += b" " * (-len(js) % 4)
    while len(blob) % 4:
        blob += b"\0"
    out = struct.pack("<III", 0x46546C67, 2, 12 + 8 + len(js) + 8 + len(blob))
    out += struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(blob), 0x004E4942) + bytes(blob)
    with open(path, "wb") as f:
        f.write(out)


def plane_mesh():
    """2 x 2 quad in glTF's XZ plane facing +Y (vkrt: the XY plane facing +Z), two triangles."""
    p = np.array([[-1, 0, 1], [1, 0, 1], [1, 0, -1], [-1, 0, -1]], np.float32)
    n = np.tile(np.array([[0, 1, 0]], np.float32), (4, 1))
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    return {"positions": p, "normals": n, "uv": uv, "indices": [0, 1, 2, 0, 2, 3], "name": "Plane"}


def icosphere_mesh(subdivisions=2):
    """Unit icosphere with smooth normals and no texture coordinates."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6],
         [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
         [8, 6, 7], [9, 8, 1]]
    verts = [np.array(p, float) / np.linalg.norm(p) for p in v]
    for _ in range(subdivisions):
        cache, nf = {}, []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        f = nf
    p = np.array(verts, np.float32)
    return {"positions": p, "normals": p.copy(), "indices": np.array(f, np.uint32).reshape(-1), "name": "Sphere"}


def prism_mesh():
    """Triangular prism with flat faces: an equilateral cross-section (unit circumradius) in glTF's XY plane, extruded
    from z = -1 to z = 1; faces carry their own vertices so normals stay flat."""
    ang = np.deg2rad([90.0, 210.0, 330.0])
    tri = np.stack([np.cos(ang), np.sin(ang)], 1).astype(np.float32)
    pos, nrm, idx = [], [], []

    def face(pts, n):
        b = len(pos)
        pos.extend(pts)
        nrm.extend([n] * len(pts))
        idx.extend([b + 0, b + 1, b + 2] if len(pts) == 3 else [b + 0, b + 1, b + 2, b + 0, b + 2, b + 3])

    face([[*tri[0], 1], [*tri[1], 1], [*tri[2], 1]], [0, 0, 1])
    face([[*tri[0], -1], [*tri[2], -1], [*tri[1], -1]], [0, 0, -1])
    for k in range(3):
        a, b = tri[k], tri[(k + 1) % 3]
        n = np.array([b[1] - a[1], a[0] - b[0], 0.0])  # outward for the counter-clockwise section
        n = n / np.linalg.norm(n)
        face([[*a, -1], [*b, -1], [*b, 1], [*a, 1]], n.tolist())
    return {"positions": np.asarray(pos, np.float32), "normals": np.asarray(nrm, np.float32), "indices": idx,
            "name": "Prism"}
