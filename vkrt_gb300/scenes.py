"""Seeded synthetic scenes for the benchmark configurations (no dataset or asset is needed).

* cornell(...)          — the Cornell box: unit cube open at the front (10 wall triangles), a 0.25 x 0.25 ceiling
                          light (2 triangles, own mesh for alias-table NEE) and two boxes rotated +-18 degrees about
                          Z (24 triangles, placed through MeshInfo position/rotation so the instance transform path
                          is exercised). Lambertian materials (metallic 0, roughness 1, specular 0).
* icosphere_field(...)  — N icospheres of 1,280 triangles (three subdivisions of the icosahedron), centres uniform
                          in [-10, 10]^3, radii log-uniform in [0.1, 1], vertices flattened to world space, one mesh
                          record per sphere so each keeps its own material; glTF metallic-roughness materials.
* sky_environment(...)  — 1024 x 512 FP32 lat-long map: grey sky gradient 0.2-1.0 plus a 0.5-degree sun disc of
                          radiance 5e3 at a seeded direction.
All scenes are Z-up like vkrt's default camera (src/core/scene/uniform.c:133-138).

Records (default material and SceneData, camera matrices, vertex packing, light tables) come from a host layer:
the backend's own host library by default (ProductHost), or any object with the same five methods passed as
`host=` — the CPU reference run of the benchmark passes the oracle's independent restatement, so it loads no product
code.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from . import context
from .context import Scene


class ProductHost:
    """The backend's host library (vkrt_host_* in libvkrt_gb300.so)."""

    @staticmethod
    def default_material() -> np.ndarray:
        m = np.zeros(1, dtype=abi.MATERIAL)
        abi.load().vkrt_host_default_material(abi.ptr(m))
        return m

    @staticmethod
    def default_scene_data(width: int, height: int) -> np.ndarray:
        sd = np.zeros(1, dtype=abi.SCENE_DATA)
        abi.load().vkrt_host_default_scene_data(width, height, abi.ptr(sd))
        return sd

    @staticmethod
    def camera_matrices(sd: np.ndarray, pos, target, up, vfov: float) -> None:
        p = np.array(pos, dtype=np.float32)
        t = np.array(target, dtype=np.float32)
        u = np.array(up, dtype=np.float32)
        w, h = int(sd["viewportRect"][0][2]), int(sd["viewportRect"][0][3])
        abi.load().vkrt_host_camera_matrices(abi.ptr(p), abi.ptr(t), abi.ptr(u), vfov, 0.001, 10000.0, w, h,
                                             abi.ptr(sd))

    pack_vertices = staticmethod(context.pack_vertices)
    build_light_tables = staticmethod(context.build_light_tables)


def default_material(host=None, **overrides) -> np.ndarray:
    m = (host or ProductHost).default_material()
    for k, v in overrides.items():
        m[k] = v
    return m


def default_scene_data(width: int, height: int, host=None) -> np.ndarray:
    return (host or ProductHost).default_scene_data(width, height)


def set_camera(sd: np.ndarray, pos, target, up=(0.0, 0.0, 1.0), vfov: float = 40.0, host=None) -> None:
    (host or ProductHost).camera_matrices(sd, pos, target, up, vfov)


def _quad(p0, p1, p2, p3, normal):
    """Two triangles (p0,p1,p2), (p0,p2,p3) with a flat normal and unit UVs."""
    verts = np.zeros(4, dtype=abi.VERTEX)
    pts = np.array([p0, p1, p2, p3], dtype=np.float32)
    verts["position"][:, :3] = pts
    verts["position"][:, 3] = 1.0
    n = np.asarray(normal, dtype=np.float32)
    verts["normal"][:, :3] = n
    t = pts[1] - pts[0]
    t = t / max(np.linalg.norm(t), 1e-12)
    verts["tangent"][:, :3] = t
    verts["tangent"][:, 3] = 1.0
    verts["color"] = 1.0
    verts["texcoord0"] = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], dtype=np.uint32)
    return verts, idx


def _box(sx, sy, sz):
    """Axis-aligned box [-sx/2, sx/2] x [-sy/2, sy/2] x [0, sz], 6 faces, outward normals."""
    x0, x1, y0, y1, z0, z1 = -sx / 2, sx / 2, -sy / 2, sy / 2, 0.0, sz
    faces = [
        ((x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0), (0, 0, -1)),
        ((x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1), (0, 0, 1)),
        ((x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1), (0, -1, 0)),
        ((x1, y1, z0), (x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (0, 1, 0)),
        ((x0, y1, z0), (x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (-1, 0, 0)),
        ((x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1), (1, 0, 0)),
    ]
    vs, ids = [], []
    for f in faces:
        v, i = _quad(*f)
        ids.append(i + 4 * len(vs))
        vs.append(v)
    return np.concatenate(vs), np.concatenate(ids)


def _assemble(parts, materials, scene_data, name, host=None) -> Scene:
    """parts: list of (vertices, mesh-relative indices, material index, position, rotation, scale)."""
    verts, idxs = [], []
    meshes = np.zeros(len(parts), dtype=abi.MESH_INFO)
    vb = ib = 0
    for k, (v, i, mat, pos, rot, scl) in enumerate(parts):
        meshes[k]["position"] = pos
        meshes[k]["rotation"] = rot
        meshes[k]["scale"] = scl
        meshes[k]["vertexBase"] = vb
        meshes[k]["vertexCount"] = len(v)
        meshes[k]["indexBase"] = ib
        meshes[k]["indexCount"] = len(i)
        meshes[k]["materialIndex"] = mat
        meshes[k]["opacity"] = 1.0
        verts.append(v)
        idxs.append(i.astype(np.uint32))
        vb += len(v)
        ib += len(i)
    s = Scene(vertices=np.concatenate(verts), indices=np.concatenate(idxs), meshes=meshes,
              materials=np.concatenate(materials), scene_data=scene_data, name=name)
    _finish(s, host)
    return s


def _finish(s: Scene, host) -> None:
    """Light tables, and with a host other than the product library the packed vertices too (so that nothing
    downstream packs them through the product library)."""
    host = host or ProductHost
    host.build_light_tables(s)
    if host is not ProductHost:
        s.shader_vertices = host.pack_vertices(s.vertices)


def cornell(width: int = 256, height: int = 256, spp: int = 1, max_depth: int = 8,
            wall_textures: list | None = None, host=None) -> Scene:
    """The Cornell box. With `wall_textures` (five (albedo, roughness) pairs of float32 (H, W) or (H, W, 3)
    arrays, for floor, ceiling, back, left, right), each wall gets its own material whose base colour (1, 1, 1) is
    multiplied by the albedo texture (slot 2k) and whose roughness 1 by the G channel of a metallic-roughness
    texture (slot 2k + 1); walls stay Lambertian (specular 0), so roughness acts through the dielectric
    directional-albedo attenuation of the Lambert lobe."""
    lamb = dict(metallic=0.0, roughness=1.0, specular=0.0, diffuseRoughness=0.0)
    mats = [default_material(host, baseColor=(0.73, 0.73, 0.73), **lamb),
            default_material(host, baseColor=(0.65, 0.05, 0.05), **lamb),
            default_material(host, baseColor=(0.12, 0.45, 0.15), **lamb),
            default_material(host, baseColor=(0.0, 0.0, 0.0), emissionColor=(1.0, 1.0, 1.0), emissionLuminance=15.0,
                             **lamb)]
    WHITE, RED, GREEN, LIGHT = 0, 1, 2, 3
    textures = {}
    wall_mats = [WHITE, WHITE, WHITE, RED, GREEN]
    if wall_textures is not None:
        if len(wall_textures) != 5:
            raise ValueError("five (albedo, roughness) texture pairs: floor, ceiling, back, left, right")
        for k, (alb, rough) in enumerate(wall_textures):
            textures[2 * k] = albedo_texture(alb)
            textures[2 * k + 1] = roughness_texture(rough)
            mats.append(default_material(host, baseColor=(1.0, 1.0, 1.0), baseColorTextureIndex=2 * k,
                                         metallicRoughnessTextureIndex=2 * k + 1, **lamb))
            wall_mats[k] = len(mats) - 1
    ident = ((0, 0, 0), (0, 0, 0), (1, 1, 1))
    parts = []
    # walls: x = left/right, y = depth (open at y = 0), z = up; normals point into the box
    walls = [
        (((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1)), WHITE),   # floor
        (((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, -1)), WHITE),  # ceiling
        (((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1), (0, -1, 0)), WHITE),  # back
        (((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (1, 0, 0)), RED),     # left
        (((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0), (-1, 0, 0)), GREEN),  # right
    ]
    for k, (q, _) in enumerate(walls):
        v, i = _quad(*q)
        parts.append((v, i, wall_mats[k]) + ident)
    h = 1.0 - 1e-3
    v, i = _quad((0.375, 0.375, h), (0.375, 0.625, h), (0.625, 0.625, h), (0.625, 0.375, h), (0, 0, -1))
    parts.append((v, i, LIGHT) + ident)
    sv, si = _box(0.3, 0.3, 0.3)
    parts.append((sv, si, WHITE, (0.68, 0.32, 0.0), (0.0, 0.0, -18.0), (1, 1, 1)))
    tv, ti = _box(0.3, 0.3, 0.6)
    parts.append((tv, ti, WHITE, (0.32, 0.65, 0.0), (0.0, 0.0, 18.0), (1, 1, 1)))
    sd = default_scene_data(width, height, host)
    set_camera(sd, (0.5, -1.35, 0.5), (0.5, 0.5, 0.5), host=host)
    sd["samplesPerPixel"] = spp
    sd["rrMaxDepth"] = max_depth
    sd["environmentLight"] = (0.0, 0.0, 0.0, 0.0)
    sd["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES, abi.RENDER_MODE_RGB, abi.SPECTRAL_HERO)
    scene = _assemble(parts, mats, sd, "cornell", host)
    scene.textures = textures
    return scene


def albedo_texture(albedo: np.ndarray) -> np.ndarray:
    """RGBA32F base-colour texture from (H, W) grey or (H, W, 3) RGB albedo."""
    a = np.asarray(albedo, dtype=np.float32)
    if a.ndim == 2:
        a = np.repeat(a[..., None], 3, axis=2)
    t = np.ones(a.shape[:2] + (4,), dtype=np.float32)
    t[..., :3] = a
    return t


def roughness_texture(roughness: np.ndarray) -> np.ndarray:
    """RGBA32F glTF metallic-roughness texture: roughness in G, metallic factor B = 1 (the material's metallic 0
    keeps the surface dielectric)."""
    r = np.asarray(roughness, dtype=np.float32)
    t = np.ones(r.shape[:2] + (4,), dtype=np.float32)
    t[..., 1] = r
    return t


def inverse_rendering_cornell(width: int = 128, height: int = 128, spp: int = 16, max_depth: int = 6,
                              tex_size: int = 64, seed: int = 3, target: bool = False) -> Scene:
    """Differentiable-rendering workload on the Cornell geometry: five 64 x 64 FP32 wall textures, albedo 0.5 and
    roughness 0.5 (target=False), or seeded albedo uniform in [0.05, 0.95]^3 and roughness uniform in [0.1, 0.9]
    (target=True). Russian roulette is off (rrMinDepth > rrMaxDepth) so the fixed-seed estimator is smooth in the
    texture values."""
    rng = np.random.default_rng(seed)
    pairs = []
    for _ in range(5):
        if target:
            alb = rng.uniform(0.05, 0.95, (tex_size, tex_size, 3)).astype(np.float32)
            rough = rng.uniform(0.1, 0.9, (tex_size, tex_size)).astype(np.float32)
        else:
            alb = np.full((tex_size, tex_size, 3), 0.5, np.float32)
            rough = np.full((tex_size, tex_size), 0.5, np.float32)
        pairs.append((alb, rough))
    s = cornell(width, height, spp=spp, max_depth=max_depth, wall_textures=pairs)
    s.scene_data["rrMinDepth"] = max_depth + 1
    s.name = "cornell-inverse"
    return s


def batch_specs(count: int = 64, seed: int = 2, spp: int = 8, max_depth: int = 10,
                tri_range=(10_000, 500_000), resolutions=(256, 512, 768, 1024)) -> list[dict]:
    """icosphere_field arguments of the uneven batch's scenes: triangle counts log-uniform over tri_range (1,280
    triangles per sphere), square resolutions drawn uniformly from `resolutions`, RGB transport."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        tris = math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))
        res = int(rng.choice(resolutions))
        out.append(dict(n_spheres=max(1, int(round(tris / 1280))), width=res, height=res, spp=spp,
                        max_depth=max_depth, seed=int(seed * 1000 + k), spectral=False))
    return out


def batch_workload(count: int = 64, seed: int = 2, spp: int = 8, max_depth: int = 10,
                   tri_range=(10_000, 500_000), resolutions=(256, 512, 768, 1024)) -> list[Scene]:
    """Uneven batch: `count` icosphere fields built as icosphere_field from batch_specs."""
    return [icosphere_field(**p) for p in batch_specs(count, seed, spp, max_depth, tri_range, resolutions)]


def unit_icosphere(subdivisions: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """Icosahedron refined `subdivisions` times (20 * 4^s triangles); vertices on the unit sphere."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts, dtype=np.float64), np.array(faces, dtype=np.uint32).reshape(-1)


def sky_environment(width: int = 1024, height: int = 512, seed: int = 1, sun_radiance: float = 5e3,
                    sun_diameter_deg: float = 0.5) -> tuple[np.ndarray, np.ndarray]:
    """Returns (rgba float32 (H, W, 4), unit sun direction)."""
    rng = np.random.default_rng(seed + 1000)
    elev = math.radians(rng.uniform(20.0, 70.0))
    azim = rng.uniform(0.0, 2.0 * math.pi)
    sun = np.array([math.cos(elev) * math.cos(azim), math.cos(elev) * math.sin(azim), math.sin(elev)])
    j = (np.arange(height) + 0.5) / height
    theta = j * math.pi
    grad = 0.2 + 0.8 * np.clip(np.cos(theta), 0.0, 1.0)
    img = np.zeros((height, width, 4), dtype=np.float32)
    img[..., :3] = grad[:, None, None].astype(np.float32)
    img[..., 3] = 1.0
    # sun disc with 8x8 supersampled coverage near the sun's texels (lookup: u = frac(phi/2pi + 0.5), v = theta/pi)
    cos_r = math.cos(math.radians(sun_diameter_deg * 0.5))
    sun_theta = math.acos(sun[2])
    sun_phi = math.atan2(sun[1], sun[0])
    jc = int(sun_theta / math.pi * height)
    ic = int(((sun_phi / (2 * math.pi) + 0.5) % 1.0) * width)
    ss = 8
    offs = (np.arange(ss) + 0.5) / ss
    for jj in range(max(0, jc - 4), min(height, jc + 5)):
        for ii0 in range(ic - 4, ic + 5):
            ii = ii0 % width
            u = (ii + offs[None, :]) / width
            v = (jj + offs[:, None]) / height
            th = v * math.pi
            ph = (u - 0.5) * 2 * math.pi
            d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th) * np.ones_like(ph)], -1)
            cover = float(((d @ sun) >= cos_r).mean())
            if cover > 0:
                img[jj, ii, :3] += np.float32(sun_radiance * cover)
    return img, sun


def icosphere_field(n_spheres: int = 800, width: int = 1920, height: int = 1080, spp: int = 16, max_depth: int = 12,
                    seed: int = 1, spectral: bool = True, env_size=(1024, 512), subdivisions: int = 3,
                    extent: float = 10.0, host=None) -> Scene:
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-extent, extent, size=(n_spheres, 3))
    radii = np.exp(rng.uniform(math.log(0.1), math.log(1.0), size=n_spheres))
    base_color = rng.uniform(0.1, 0.9, size=(n_spheres, 3))
    roughness = rng.uniform(0.05, 1.0, size=n_spheres)
    metallic = (rng.uniform(0.0, 1.0, size=n_spheres) < 0.3).astype(np.float32)
    uv, uf = unit_icosphere(subdivisions)
    nv, nt = len(uv), len(uf) // 3
    verts = np.zeros(n_spheres * nv, dtype=abi.VERTEX)
    pos = (centers[:, None, :] + radii[:, None, None] * uv[None, :, :]).reshape(-1, 3)
    nrm = np.broadcast_to(uv[None], (n_spheres, nv, 3)).reshape(-1, 3)
    verts["position"][:, :3] = pos.astype(np.float32)
    verts["position"][:, 3] = 1.0
    verts["normal"][:, :3] = nrm.astype(np.float32)
    up = np.where(np.abs(nrm[:, 2:3]) < 0.999, np.array([[0.0, 0.0, 1.0]]), np.array([[1.0, 0.0, 0.0]]))
    tan = np.cross(up, nrm)
    tan /= np.linalg.norm(tan, axis=1, keepdims=True)
    verts["tangent"][:, :3] = tan.astype(np.float32)
    verts["tangent"][:, 3] = 1.0
    verts["color"] = 1.0
    verts["texcoord0"][:, 0] = (np.arctan2(nrm[:, 1], nrm[:, 0]) / (2 * math.pi) + 0.5).astype(np.float32)
    verts["texcoord0"][:, 1] = (np.arccos(np.clip(nrm[:, 2], -1, 1)) / math.pi).astype(np.float32)
    indices = np.tile(uf, n_spheres).astype(np.uint32)
    meshes = np.zeros(n_spheres, dtype=abi.MESH_INFO)
    meshes["vertexBase"] = np.arange(n_spheres, dtype=np.uint32) * nv
    meshes["vertexCount"] = nv
    meshes["indexBase"] = np.arange(n_spheres, dtype=np.uint32) * (3 * nt)
    meshes["indexCount"] = 3 * nt
    meshes["materialIndex"] = np.arange(n_spheres, dtype=np.uint32)
    meshes["scale"] = 1.0
    meshes["opacity"] = 1.0
    mats = np.repeat(default_material(host), n_spheres)
    mats["baseColor"] = base_color.astype(np.float32)
    mats["roughness"] = roughness.astype(np.float32)
    mats["metallic"] = metallic
    mats["specular"] = 0.5
    mats["ior"] = 1.5
    sd = default_scene_data(width, height, host)
    set_camera(sd, (0.0, -30.0, 6.0), (0.0, 0.0, 0.0), host=host)
    sd["samplesPerPixel"] = spp
    sd["rrMaxDepth"] = max_depth
    mode = abi.RENDER_MODE_SPECTRAL if spectral else abi.RENDER_MODE_RGB
    sd["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES, mode, abi.SPECTRAL_HERO)
    env, _sun = sky_environment(env_size[0], env_size[1], seed)
    sd["environmentTextureIndex"] = 0
    sd["environmentLight"] = (1.0, 1.0, 1.0, 1.0)
    s = Scene(vertices=verts, indices=indices, meshes=meshes, materials=mats, scene_data=sd,
              textures={0: env}, env_texture=0, name=f"icospheres{n_spheres}")
    _finish(s, host)
    return s
