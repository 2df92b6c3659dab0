"""TEST INFRASTRUCTURE ONLY (the oracle): CPU restatements of vkrt's selection passes and auto-SPP controller, used by
tests as the checker of vkrt_gb300/csrc/overlay.cu and the host auto-SPP code.

* selection_mask  src/shaders/entry/select/raygen.slang:5-14 with rt/queries/selection_query.slang:7-11: pixel-centre
                  camera rays (camera/ray.slang:15-30, zero jitter) against the selected mesh alone, first-hit
                  termination; FP64 brute force, with the near-edge flags of the FP64 intersector.
* outline         src/shaders/entry/post/outline.slang:9-60 and scene/constants.slang:17-18.
* pick_mesh       src/shaders/integrator/path/debug.slang:21-29: closest-hit mesh of a pixel-centre ray.
* auto_spp_update src/core/scene/timing.c:121-178 (and settings.c:68-79 for the target), in float32 arithmetic.
"""
from __future__ import annotations

import numpy as np

OUTLINE_GROUP, OUTLINE_MAX_RADIUS = 16, 5
OUTLINE_RGBA16 = (65535, 36044, 6554)  # (1, 0.55, 0.1) as RGBA16 UNORM


def camera_rays(scene_data, width: int, height: int):
    """Pixel-centre camera rays of every film pixel (FP64 arithmetic), as the C ABI's ray records; mask of pixels
    inside the viewport."""
    from vkrt_gb300 import abi
    sd = np.asarray(scene_data).reshape(-1)[0]
    vx0, vy0, vw, vh = (int(v) for v in sd["viewportRect"])
    ys, xs = np.mgrid[0:height, 0:width]
    vx = (xs - vx0).astype(np.float64) + 0.5
    vy = (ys - vy0).astype(np.float64) + 0.5
    ndcx = vx / max(vw, 1) * 2.0 - 1.0
    ndcy = vy / max(vh, 1) * 2.0 - 1.0
    pi = sd["projInverse"].astype(np.float64)  # [column][row]
    vi = sd["viewInverse"].astype(np.float64)
    v4 = ndcx[..., None] * pi[0] + ndcy[..., None] * pi[1] + pi[2] + pi[3]
    d = v4[..., 0:1] * vi[0, :3] + v4[..., 1:2] * vi[1, :3] + v4[..., 2:3] * vi[2, :3]
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    rays = np.zeros((height, width), dtype=abi.RAY)
    rays["origin"] = vi[3, :3]
    rays["direction"] = d
    rays["tMin"] = 1e-3
    rays["tMax"] = 1e4
    inside = (vw > 0) & (vh > 0) & (xs >= vx0) & (ys >= vy0) & (xs < vx0 + vw) & (ys < vy0 + vh)
    return rays, inside


def single_mesh_scene(scene, mesh_index: int):
    """The scene reduced to one mesh (the selection TLAS of vkrt holds the selected mesh alone)."""
    from vkrt_gb300.context import Scene
    m = scene.meshes[mesh_index]
    vb, vc, ib, ic = int(m["vertexBase"]), int(m["vertexCount"]), int(m["indexBase"]), int(m["indexCount"])
    meshes = scene.meshes[mesh_index:mesh_index + 1].copy()
    meshes["vertexBase"] = 0
    meshes["indexBase"] = 0
    meshes["materialIndex"] = 0
    mat = scene.materials[int(m["materialIndex"]):int(m["materialIndex"]) + 1].copy()
    return Scene(vertices=scene.vertices[vb:vb + vc].copy(), indices=scene.indices[ib:ib + ic].copy(), meshes=meshes,
                 materials=mat, scene_data=scene.scene_data.copy(), name=scene.name + f"[mesh {mesh_index}]")


def selection_mask(scene, scene_data, width: int, height: int):
    """(mask uint32 (H, W), ambiguous bool (H, W)) for scene_data's selectedMeshIndex."""
    from oracle import cpu
    from vkrt_gb300 import abi
    sd = np.asarray(scene_data).reshape(-1)[0]
    mask = np.zeros((height, width), np.uint32)
    amb = np.zeros((height, width), bool)
    sel = int(sd["selectedMeshIndex"])
    if int(sd["selectionEnabled"]) == 0 or sel == abi.INVALID_INDEX:
        return mask, amb
    rays, inside = camera_rays(scene_data, width, height)
    sub = single_mesh_scene(scene, sel)
    sub.textures = scene.textures
    orc = cpu.OracleScene(sub)
    try:
        if int(sub.materials["alphaMode"][0]) == 1:  # mask cut-outs: the FP32 traversal with the selection alpha test
            hits = orc.trace_fp32(rays.reshape(-1), any_hit=True, selection_alpha=True)
            ambiguous = np.zeros(len(hits), bool)
        else:
            hits, ambiguous = orc.trace_fp64(rays.reshape(-1))
    finally:
        orc.close()
    hit = (hits["instanceIndex"] != abi.INVALID_INDEX).reshape(height, width)
    mask[hit & inside] = 1
    amb[:] = ambiguous.reshape(height, width) & inside
    return mask, amb


def outline_radius(width: int, height: int) -> int:
    # round half to even, as the kernel does
    return int(min(max(int(np.rint(np.float32(min(width, height)) * np.float32(2.0 / 1080.0))), 1),
                   OUTLINE_MAX_RADIUS))


def outline(mask, output):
    """The display image after the outline pass: output (H, W, 4) uint16, mask (H, W)."""
    h, w = mask.shape
    r = outline_radius(w, h)
    m = np.zeros((h + 2 * r, w + 2 * r), bool)
    m[r:r + h, r:r + w] = mask != 0
    near = np.zeros((h, w), bool)
    for dy in range(-r, r + 1):
        for dx in range(-r, r + 1):
            if dx or dy:
                near |= m[r + dy:r + dy + h, r + dx:r + dx + w]
    paint = near & (mask == 0)
    out = output.copy()
    out[paint, 0], out[paint, 1], out[paint, 2] = OUTLINE_RGBA16
    return out


def pick_mesh(scene, scene_data, x: int, y: int, oracle_scene=None):
    """(mesh index or INVALID_INDEX, ambiguous) of the closest hit of pixel (x, y)'s centre ray; `oracle_scene`
    (an oracle.cpu.OracleScene of `scene`) may be passed to reuse it across queries."""
    from oracle import cpu
    from vkrt_gb300 import abi
    rays, inside = camera_rays(scene_data, x + 1, y + 1)
    if not inside[y, x]:
        return abi.INVALID_INDEX, False
    orc = oracle_scene if oracle_scene is not None else cpu.OracleScene(scene)
    try:
        if (scene.materials["alphaMode"] == 1).any():  # mask cut-outs: FP32 traversal with the selection alpha test
            hits = orc.trace_fp32(rays[y:y + 1, x], selection_alpha=True)
            amb = np.zeros(1, bool)
        else:
            hits, amb = orc.trace_fp64(rays[y:y + 1, x])
    finally:
        if oracle_scene is None:
            orc.close()
    return int(hits["instanceIndex"][0]), bool(amb[0])


def auto_spp_init(target_fps: int):
    fps = target_fps if target_fps else 60
    fps = min(max(fps, 30), 360)
    return {"targetFrameMs": np.float32(1000.0) / np.float32(fps), "controlMs": np.float32(0.0)}


def auto_spp_update(state, render_ms: float, spp: int) -> int:
    """The next samples-per-pixel; updates state in place. float32 throughout, as the C controller."""
    f = np.float32
    smoothing, budget = f(0.35), f(0.90)
    up_band, down_band, up_step, down_step = f(0.18), f(0.08), f(1.25), f(0.60)
    target = f(state["targetFrameMs"])
    ms = f(render_ms)
    if not (target > 0) or not (ms > 0):
        return spp
    cur = spp if spp else 1
    sppf = f(cur)
    per = f(ms / sppf)
    if not (per > 0):
        return spp
    c = f(state["controlMs"])
    c = per if c <= 0 else f(f(c * f(f(1) - smoothing)) + f(per * smoothing))
    state["controlMs"] = c
    desired = f(f(target * budget) / c)
    desired = min(max(desired, f(1)), f(2048))
    delta = f(desired - sppf)
    band = max(f(sppf * (up_band if delta > 0 else down_band)), f(1))
    if abs(delta) <= band:
        return spp
    if delta > 0:
        nxt = int(np.floor(min(desired, f(np.ceil(f(sppf * up_step))))))
        if nxt <= cur and cur < 2048:
            nxt = cur + 1
    else:
        nxt = int(np.ceil(max(desired, f(np.floor(f(sppf * down_step))))))
        if nxt >= cur and cur > 1:
            nxt = cur - 1
    nxt = min(max(nxt, 1), 2048)
    return spp if nxt == cur else nxt
