"""Seeded synthetic scenes for the render core (host-side input generation, numpy).

Every scene is a plain description -- meshes of ``lh2g_core_tri`` records (the CoreTri layout of
lib/RenderSystem/common_classes.h:57-97), instances with 4x4 object-to-world transforms, materials,
textures, lights and a camera -- that is handed unchanged to the GPU core and to the CPU oracle.

Triangle records follow the reference's host conventions:
  * quads as in HostScene::AddQuad (lib/RenderSystem/host_scene.cpp:401-440): two triangles, face normal,
    tangent/bitangent of the quad frame;
  * smooth meshes as in HostMesh (lib/RenderSystem/host_mesh.cpp:167-210, 280-318): per-vertex normals,
    consistent-normal alphas acos(min dot) * (1 + 0.03632 (1 - min dot)^2), texture LOD
    0.5 log2(texel area / primitive area);
  * area lights as HostTriLight (lib/RenderSystem/host_light.cpp:25-62): Heron area, energy = sum(radiance*area);
  * textures with a 5-level box-filtered MIP chain stored back to back (host_texture.cpp:128-150);
  * the camera as Camera::GetView (lib/RenderSystem/camera.cpp:107-128).

Workloads (sizes as named by the benchmark configurations):
  * ``cornell_sphere``: Cornell-style room of 12 axis-aligned quads (24 triangles) plus a noise-displaced
    icosphere of subdivision 6 (20 * 4^6 = 81,920 triangles; "50k" in the workload name is not reachable
    with an icosphere, so the subdivision level is kept), 8 diffuse/specular materials, one quad light of
    emission 10, 512x512.
  * ``spheres_2m``: 64 distinct 32,000-triangle noise-displaced UV spheres with random affine transforms over a
    2-triangle 1000x1000 ground (2,048,002 triangles), 16 quad lights + 4 point lights, 20 materials (4 with
    1024^2 RGBA8 value-noise textures), a sky dome, 1920x1080.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

CORE_TRI_DTYPE = np.dtype([
    ("u", "<f4", 3), ("ltriIdx", "<i4"), ("v", "<f4", 3), ("material", "<u4"),
    ("vN0", "<f4", 3), ("Nx", "<f4"), ("vN1", "<f4", 3), ("Ny", "<f4"), ("vN2", "<f4", 3), ("Nz", "<f4"),
    ("T", "<f4", 3), ("area", "<f4"), ("B", "<f4", 3), ("invArea", "<f4"),
    ("alpha", "<f4", 3), ("LOD", "<f4"),
    ("vertex0", "<f4", 3), ("dummy0", "<f4"), ("vertex1", "<f4", 3), ("dummy1", "<f4"),
    ("vertex2", "<f4", 3), ("dummy2", "<f4"),
    ("u1", "<f4", 3), ("dummy3", "<f4"), ("v1", "<f4", 3), ("dummy4", "<f4"),
])
assert CORE_TRI_DTYPE.itemsize == 208

MAP_DTYPE = np.dtype([("texture", "<i4"), ("uvscale", "<f4", 2), ("uvoffset", "<f4", 2)])
MATERIAL_DTYPE = np.dtype([
    ("color", "<f4", 3), ("absorption", "<f4", 3),
    ("metallic", "<f4"), ("subsurface", "<f4"), ("specular", "<f4"), ("roughness", "<f4"),
    ("specularTint", "<f4"), ("anisotropic", "<f4"), ("sheen", "<f4"), ("sheenTint", "<f4"),
    ("clearcoat", "<f4"), ("clearcoatGloss", "<f4"), ("transmission", "<f4"), ("eta", "<f4"),
    ("flags", "<u4"),
    ("color_map", MAP_DTYPE), ("detail_color_map", MAP_DTYPE), ("normal_map", MAP_DTYPE),
    ("detail_normal_map", MAP_DTYPE), ("specular_map", MAP_DTYPE), ("roughness_map", MAP_DTYPE),
])
LIGHT_TRI_DTYPE = np.dtype([
    ("centre", "<f4", 3), ("energy", "<f4"), ("N", "<f4", 3), ("area", "<f4"),
    ("radiance", "<f4", 3), ("dummy2", "<i4"), ("vertex0", "<f4", 3), ("triIdx", "<i4"),
    ("vertex1", "<f4", 3), ("instIdx", "<i4"), ("vertex2", "<f4", 3), ("dummy1", "<i4"),
])
POINT_LIGHT_DTYPE = np.dtype([("position", "<f4", 3), ("energy", "<f4"), ("radiance", "<f4", 3), ("dummy", "<i4")])
SPOT_LIGHT_DTYPE = np.dtype([("position", "<f4", 3), ("cosInner", "<f4"), ("radiance", "<f4", 3), ("cosOuter", "<f4"),
                             ("direction", "<f4", 3), ("dummy", "<i4")])
DIR_LIGHT_DTYPE = np.dtype([("direction", "<f4", 3), ("energy", "<f4"), ("radiance", "<f4", 3), ("dummy", "<i4")])
VIEW_DTYPE = np.dtype([("pos", "<f4", 3), ("p1", "<f4", 3), ("p2", "<f4", 3), ("p3", "<f4", 3),
                       ("aperture", "<f4"), ("spreadAngle", "<f4"), ("imagePlane", "<f4"),
                       ("focalDistance", "<f4"), ("distortion", "<f4")])
RAY_DTYPE = np.dtype([("o", "<f4", 3), ("tmin", "<f4"), ("d", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("bary", "<u4"), ("inst", "<i4"), ("prim", "<i4"), ("t", "<f4")])
assert MATERIAL_DTYPE.itemsize == 4 * (6 + 12 + 1) + 6 * 20 and LIGHT_TRI_DTYPE.itemsize == 96


@dataclass
class Mesh:
    vertices: np.ndarray  # (3*T, 4) float32, three per triangle (the SetGeometry vertex buffer)
    tris: np.ndarray      # (T,) CORE_TRI_DTYPE


@dataclass
class Texture:
    width: int
    height: int
    texels: np.ndarray    # uint32 ARGB32 words, all MIP levels back to back


@dataclass
class Scene:
    meshes: list = field(default_factory=list)
    instances: list = field(default_factory=list)     # (mesh index, 4x4 float32 row-major object->world)
    materials: np.ndarray = None
    textures: list = field(default_factory=list)
    tri_lights: np.ndarray = None
    point_lights: np.ndarray = None
    spot_lights: np.ndarray = None
    dir_lights: np.ndarray = None
    sky: tuple | None = None                           # (rgb float32 (h*w*3), w, h)
    bounds: tuple = None                               # (min3, max3) world bounds
    blue_noise: tuple | None = None                    # (sobol 65536, scrambling 131072, ranking 131072) uint8 tables

    @property
    def triangle_count(self):
        return sum(len(m.tris) for m in self.meshes)


# ----------------------------------------------------------------------------------------------------
# basic geometry helpers
# ----------------------------------------------------------------------------------------------------
def _normalize(v):
    v = np.asarray(v, dtype=np.float32)
    n = np.sqrt(np.sum(v * v, axis=-1, keepdims=True, dtype=np.float32)).astype(np.float32)
    n = np.where(n == 0, np.float32(1), n)
    return (v / n).astype(np.float32)


def empty_material():
    m = np.zeros((), dtype=MATERIAL_DTYPE)
    m["eta"] = 1.0
    m["roughness"] = 1.0
    for key in ("color_map", "detail_color_map", "normal_map", "detail_normal_map", "specular_map", "roughness_map"):
        m[key]["texture"] = -1
        m[key]["uvscale"] = (1.0, 1.0)
    return m


def _tris_from_vertices(v0, v1, v2, material, n0=None, n1=None, n2=None, alpha=None, uv=None, tex_wh=None):
    """CoreTri records for a batch of triangles (HostScene::AddTriToMesh / HostMesh conventions)."""
    t = v0.shape[0]
    tris = np.zeros(t, dtype=CORE_TRI_DTYPE)
    e1, e2 = (v1 - v0).astype(np.float32), (v2 - v0).astype(np.float32)
    N = _normalize(np.cross(e1, e2))
    tris["Nx"], tris["Ny"], tris["Nz"] = N[:, 0], N[:, 1], N[:, 2]
    tris["vN0"] = N if n0 is None else n0
    tris["vN1"] = N if n1 is None else n1
    tris["vN2"] = N if n2 is None else n2
    tris["vertex0"], tris["vertex1"], tris["vertex2"] = v0, v1, v2
    tris["material"] = material
    tris["ltriIdx"] = -1
    T = _normalize(e1)
    tris["T"] = T
    tris["B"] = _normalize(np.cross(N, T))
    tris["alpha"] = 0.0 if alpha is None else alpha
    if uv is not None:
        (u0, w0), (u1, w1), (u2, w2) = uv
        tris["u"] = np.stack([u0, u1, u2], -1)
        tris["v"] = np.stack([w0, w1, w2], -1)
        if tex_wh is not None:
            Ta = (tex_wh[0] * tex_wh[1]) * np.abs((u1 - u0) * (w2 - w0) - (u2 - u0) * (w1 - w0))
            Pa = np.sqrt(np.sum(np.cross(e1, e2) ** 2, -1))
            with np.errstate(divide="ignore", invalid="ignore"):
                lod = 0.5 * np.log2(np.maximum(Ta, 1e-30) / np.maximum(Pa, 1e-30))
            tris["LOD"] = np.where(tex_wh is None, 0, lod).astype(np.float32)
    return tris


def _mesh(v0, v1, v2, tris):
    verts = np.zeros((3 * len(tris), 4), dtype=np.float32)
    verts[0::3, :3], verts[1::3, :3], verts[2::3, :3] = v0, v1, v2
    verts[:, 3] = 1.0
    return Mesh(verts, tris)


def add_quad(N, pos, width, height, mat):
    """Two triangles of a quad (HostScene::AddQuad, host_scene.cpp:401-440)."""
    N = _normalize(np.asarray(N, np.float32))
    pos = np.asarray(pos, np.float32)
    tmp = np.array([0, 1, 0], np.float32) if abs(N[0]) > 0.9 else np.array([1, 0, 0], np.float32)
    T = np.float32(0.5 * width) * _normalize(np.cross(N, tmp))
    B = np.float32(0.5 * height) * _normalize(np.cross(_normalize(T), N))
    c = [pos - B - T, pos + B - T, pos - B + T, pos + B - T, pos + B + T, pos - B + T]
    v0 = np.stack([c[0], c[3]]); v1 = np.stack([c[1], c[4]]); v2 = np.stack([c[2], c[5]])
    tris = _tris_from_vertices(v0, v1, v2, mat)
    tris["vN0"] = tris["vN1"] = tris["vN2"] = N
    tris["Nx"], tris["Ny"], tris["Nz"] = N
    tris["T"] = T / np.float32(0.5 * height)
    tris["B"] = B / np.float32(0.5 * width)
    return v0, v1, v2, tris


def _concat(parts):
    v0 = np.concatenate([p[0] for p in parts]); v1 = np.concatenate([p[1] for p in parts])
    v2 = np.concatenate([p[2] for p in parts]); tris = np.concatenate([p[3] for p in parts])
    return v0, v1, v2, tris


def _value_noise3(p, seed, freq):
    """Seeded 3-D value noise in [0,1]: random lattice values, smoothstep-trilinear interpolation."""
    rng = np.random.default_rng(seed)
    lat = rng.random((freq + 2, freq + 2, freq + 2)).astype(np.float32)
    q = (p * 0.5 + 0.5) * freq
    i = np.clip(np.floor(q).astype(np.int64), 0, freq)
    f = q - i
    f = f * f * (3 - 2 * f)
    out = 0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * (f[:, 2] if dz else 1 - f[:, 2])
                out = out + w * lat[i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz]
    return out.astype(np.float32)


def _smooth_mesh(verts, faces, seed, radius, center, mat, uv=None, tex_wh=None, amp=0.1):
    """Noise-displaced smooth mesh from unit-sphere vertices and an index list."""
    n = _value_noise3(verts, seed, 6) * 0.7 + _value_noise3(verts, seed + 1, 13) * 0.3
    r = radius * (1.0 + amp * (2.0 * n - 1.0))
    P = (verts * r[:, None] + center).astype(np.float32)
    f0, f1, f2 = faces[:, 0], faces[:, 1], faces[:, 2]
    fn = np.cross(P[f1] - P[f0], P[f2] - P[f0])              # area-weighted face normals
    vn = np.zeros_like(P)
    for k in (f0, f1, f2):
        np.add.at(vn, k, fn)
    vn = _normalize(vn)
    fnu = _normalize(fn)
    # consistent normal interpolation alphas (host_mesh.cpp:167-210)
    dmin = np.ones(len(P), np.float32)
    for k in (f0, f1, f2):
        np.minimum.at(dmin, k, np.maximum(0.7, np.sum(vn[k] * fnu, -1)).astype(np.float32))
    alpha = (np.arccos(np.clip(dmin, -1, 1)) * (1 + 0.03632 * (1 - dmin) * (1 - dmin))).astype(np.float32)
    uvs = None
    if uv is not None:
        uvs = ((uv[f0, 0], uv[f0, 1]), (uv[f1, 0], uv[f1, 1]), (uv[f2, 0], uv[f2, 1]))
    tris = _tris_from_vertices(P[f0], P[f1], P[f2], mat, vn[f0], vn[f1], vn[f2],
                               np.stack([alpha[f0], alpha[f1], alpha[f2]], -1), uvs, tex_wh)
    return P[f0], P[f1], P[f2], tris


def icosphere(subdiv):
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = _normalize(np.array(v, np.float64)).astype(np.float64)
    faces = np.array(f, np.int64)
    for _ in range(subdiv):
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        mids = verts[uniq[:, 0]] + verts[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = len(verts)
        verts = np.concatenate([verts, mids])
        nf = len(faces)
        a, b, c = inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base
        faces = np.concatenate([np.stack([faces[:, 0], a, c], 1), np.stack([faces[:, 1], b, a], 1),
                                np.stack([faces[:, 2], c, b], 1), np.stack([a, b, c], 1)])
    return verts.astype(np.float32), faces


def uv_sphere(slices, stacks):
    """UV sphere with 2*slices*(stacks-1) triangles and (u, v) texture coordinates."""
    th = np.linspace(0, math.pi, stacks + 1)
    ph = np.linspace(0, 2 * math.pi, slices + 1)
    TH, PH = np.meshgrid(th, ph, indexing="ij")
    verts = np.stack([np.sin(TH) * np.cos(PH), np.cos(TH), np.sin(TH) * np.sin(PH)], -1).reshape(-1, 3)
    uv = np.stack([PH / (2 * math.pi), TH / math.pi], -1).reshape(-1, 2).astype(np.float32)
    idx = lambda i, j: i * (slices + 1) + j
    faces = []
    for i in range(stacks):
        j = np.arange(slices)
        a, b, c, d = idx(i, j), idx(i, j + 1), idx(i + 1, j), idx(i + 1, j + 1)
        if i > 0:
            faces.append(np.stack([a, b, c], 1))
        if i < stacks - 1:
            faces.append(np.stack([b, d, c], 1))
    return verts.astype(np.float32), np.concatenate(faces), uv


def make_light_tris(v0, v1, v2, tris, radiance, inst_idx, tri_offset=0):
    lt = np.zeros(len(tris), dtype=LIGHT_TRI_DTYPE)
    a = np.linalg.norm(v1 - v0, axis=1).astype(np.float32)
    b = np.linalg.norm(v2 - v1, axis=1).astype(np.float32)
    c = np.linalg.norm(v0 - v2, axis=1).astype(np.float32)
    s = (a + b + c) * np.float32(0.5)
    area = np.sqrt(s * (s - a) * (s - b) * (s - c)).astype(np.float32)
    lt["vertex0"], lt["vertex1"], lt["vertex2"] = v0, v1, v2
    lt["centre"] = np.float32(0.333333) * (v0 + v1 + v2)
    lt["N"] = np.stack([tris["Nx"], tris["Ny"], tris["Nz"]], -1)
    lt["area"] = area
    lt["radiance"] = radiance
    E = np.asarray(radiance, np.float32)[None, :] * area[:, None]
    lt["energy"] = E.sum(1)
    lt["triIdx"] = np.arange(len(tris)) + tri_offset
    lt["instIdx"] = inst_idx
    return lt


def make_view(pos, target, fov_deg, width, height, up=(0, 1, 0), focal=1.0):
    """ViewPyramid as Camera::GetView builds it (camera.cpp:107-128); p1 top-left, p2 top-right, p3 bottom-left."""
    pos = np.asarray(pos, np.float32)
    fwd = _normalize(np.asarray(target, np.float32) - pos)
    right = _normalize(np.cross(fwd, np.asarray(up, np.float32)))
    upv = _normalize(np.cross(right, fwd))
    aspect = width / height
    screen = math.tan(math.radians(fov_deg) / 2)
    C = pos + focal * fwd
    v = np.zeros((), dtype=VIEW_DTYPE)
    v["pos"] = pos
    v["p1"] = C - screen * right * focal * aspect + screen * focal * upv
    v["p2"] = C + screen * right * focal * aspect + screen * focal * upv
    v["p3"] = C - screen * right * focal * aspect - screen * focal * upv
    v["spreadAngle"] = math.radians(fov_deg) / height
    v["focalDistance"] = focal
    v["imagePlane"] = 1.0
    return v


def make_texture(seed, size=1024, levels=5):
    """RGBA8 value-noise texture with a box-filtered MIP chain (host_texture.cpp:128-150)."""
    rng = np.random.default_rng(seed)
    img = np.zeros((size, size, 3), np.float32)
    for octave, w in ((8, 0.5), (32, 0.3), (128, 0.2)):
        lat = rng.random((octave + 1, octave + 1, 3)).astype(np.float32)
        x = np.linspace(0, octave, size, endpoint=False)
        i = np.floor(x).astype(int)
        f = (x - i).astype(np.float32)
        f = f * f * (3 - 2 * f)
        a = lat[i][:, i] * (1 - f)[:, None, None] * (1 - f)[None, :, None]
        b = lat[i + 1][:, i] * f[:, None, None] * (1 - f)[None, :, None]
        c = lat[i][:, i + 1] * (1 - f)[:, None, None] * f[None, :, None]
        d = lat[i + 1][:, i + 1] * f[:, None, None] * f[None, :, None]
        img += w * (a + b + c + d)
    rgb = np.clip(img * 255.0, 0, 255).astype(np.uint32)
    level = np.concatenate([rgb, np.full((size, size, 1), 255, np.uint32)], -1)
    chain = []
    for _ in range(levels):
        chain.append(level[..., 0] | (level[..., 1] << 8) | (level[..., 2] << 16) | (level[..., 3] << 24))
        h = level.shape[0] // 2
        if h == 0:
            break
        level = ((level[0::2, 0::2] + level[1::2, 0::2] + level[0::2, 1::2] + level[1::2, 1::2]) >> 2)
    return Texture(size, size, np.concatenate([c.reshape(-1) for c in chain]).astype(np.uint32))


# ----------------------------------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------------------------------
def cornell_sphere(seed=1, subdiv=6):
    """Cornell-style room (12 quads) + noise-displaced icosphere; materials 0..7 diffuse/specular, 8 light."""
    rng = np.random.default_rng(seed)
    mats = np.zeros(9, dtype=MATERIAL_DTYPE)
    for i in range(8):
        m = empty_material()
        m["color"] = rng.uniform(0.1, 0.9, 3)
        m["roughness"] = 0.75          # Lambert pReflect = 1 - roughness: 25% specular
        mats[i] = m
    light = empty_material()
    light["color"] = (10.0, 10.0, 10.0)
    mats[8] = light
    q = []
    q.append(add_quad((0, 1, 0), (0, 0, 0), 2, 2, 0))        # floor
    q.append(add_quad((0, -1, 0), (0, 2, 0), 2, 2, 1))       # ceiling
    q.append(add_quad((0, 0, 1), (0, 1, -1), 2, 2, 2))       # back
    q.append(add_quad((0, 0, -1), (0, 1, 1), 2, 2, 3))       # front (behind the camera)
    q.append(add_quad((1, 0, 0), (-1, 1, 0), 2, 2, 4))       # left
    q.append(add_quad((-1, 0, 0), (1, 1, 0), 2, 2, 5))       # right
    q.append(add_quad((0, -1, 0), (0, 1.98, -0.1), 0.6, 0.6, 8))  # light
    bx, bz, hs, hh = -0.45, -0.35, 0.25, 0.6                  # box of 5 visible faces
    q.append(add_quad((0, 1, 0), (bx, hh, bz), 2 * hs, 2 * hs, 6))
    q.append(add_quad((1, 0, 0), (bx + hs, hh / 2, bz), 2 * hs, hh, 6))
    q.append(add_quad((-1, 0, 0), (bx - hs, hh / 2, bz), 2 * hs, hh, 6))
    q.append(add_quad((0, 0, 1), (bx, hh / 2, bz + hs), 2 * hs, hh, 7))
    q.append(add_quad((0, 0, -1), (bx, hh / 2, bz - hs), 2 * hs, hh, 7))
    room = _concat(q)
    light_first = 12
    room[3]["ltriIdx"][light_first:light_first + 2] = [0, 1]
    verts, faces = icosphere(subdiv)
    sph = _smooth_mesh(verts, faces, seed + 100, 0.35, np.array([0.35, 0.45, -0.2], np.float32), 0)
    mat_ids = rng.integers(0, 8, len(sph[3]))
    sph[3]["material"] = mat_ids
    s = Scene()
    s.meshes = [_mesh(*room), _mesh(*sph)]
    smooth = empty_material()
    for i in range(8):
        mats[i]["flags"] = 1   # smooth normals (only the sphere carries per-vertex normals; quads have N everywhere)
    s.materials = mats
    ident = np.eye(4, dtype=np.float32)
    s.instances = [(0, ident), (1, ident)]
    lv0, lv1, lv2 = room[0][12:14], room[1][12:14], room[2][12:14]
    s.tri_lights = make_light_tris(lv0, lv1, lv2, room[3][12:14], (10.0, 10.0, 10.0), 0, 12)
    s.point_lights = np.zeros(0, POINT_LIGHT_DTYPE)
    s.spot_lights = np.zeros(0, SPOT_LIGHT_DTYPE)
    s.dir_lights = np.zeros(0, DIR_LIGHT_DTYPE)
    s.bounds = (np.array([-1, 0, -1], np.float32), np.array([1, 2, 1], np.float32))
    return s


def lit_room(seed=11, grid=8, n_points=24, n_spots=12, subdiv=3):
    """The Cornell room and displaced icosphere lit by many lights (for the light tree): a grid x grid array of
    small ceiling quads (2 grid^2 area lights, seeded colours), n_points point lights and n_spots downward spot
    lights at seeded positions. The defaults give 164 lights, beyond the 64 that selection by potentials takes."""
    rng = np.random.default_rng(seed)
    mats = np.zeros(8 + grid * grid, dtype=MATERIAL_DTYPE)
    for i in range(8):
        m = empty_material()
        m["color"] = rng.uniform(0.1, 0.9, 3)
        m["roughness"] = 0.75
        m["flags"] = 1
        mats[i] = m
    radiance = rng.uniform(2.0, 12.0, (grid * grid, 3)).astype(np.float32)
    for k in range(grid * grid):
        lm = empty_material()
        lm["color"] = radiance[k]
        mats[8 + k] = lm
    q = [add_quad((0, 1, 0), (0, 0, 0), 2, 2, 0), add_quad((0, -1, 0), (0, 2, 0), 2, 2, 1), add_quad((0, 0, 1), (0, 1, -1), 2, 2, 2),
         add_quad((0, 0, -1), (0, 1, 1), 2, 2, 3), add_quad((1, 0, 0), (-1, 1, 0), 2, 2, 4), add_quad((-1, 0, 0), (1, 1, 0), 2, 2, 5)]
    cell = 1.6 / grid
    for gz in range(grid):
        for gx in range(grid):
            q.append(add_quad((0, -1, 0), (-0.8 + (gx + 0.5) * cell, 1.98, -0.8 + (gz + 0.5) * cell), 0.5 * cell, 0.5 * cell, 8 + gz * grid + gx))
    room = _concat(q)
    first = 12
    nl = 2 * grid * grid
    room[3]["ltriIdx"][first:first + nl] = np.arange(nl)
    verts, faces = icosphere(subdiv)
    sph = _smooth_mesh(verts, faces, seed + 100, 0.35, np.array([0.3, 0.45, -0.25], np.float32), 0)
    sph[3]["material"] = rng.integers(0, 8, len(sph[3]))
    sc = Scene()
    sc.meshes = [_mesh(*room), _mesh(*sph)]
    sc.materials = mats
    ident = np.eye(4, dtype=np.float32)
    sc.instances = [(0, ident), (1, ident)]
    lt = make_light_tris(room[0][first:first + nl], room[1][first:first + nl], room[2][first:first + nl], room[3][first:first + nl],
                         (1.0, 1.0, 1.0), 0, first)
    lt["radiance"] = np.repeat(radiance, 2, axis=0)
    lt["energy"] = (lt["radiance"] * lt["area"][:, None]).sum(1)
    sc.tri_lights = lt
    pl = np.zeros(n_points, POINT_LIGHT_DTYPE)
    pl["position"] = rng.uniform((-0.9, 0.2, -0.9), (0.9, 1.8, 0.9), (n_points, 3))
    pl["radiance"] = rng.uniform(0.05, 0.4, (n_points, 3))
    pl["energy"] = pl["radiance"].sum(1)
    sc.point_lights = pl
    sp = np.zeros(n_spots, SPOT_LIGHT_DTYPE)
    sp["position"] = rng.uniform((-0.8, 1.5, -0.8), (0.8, 1.9, 0.8), (n_spots, 3))
    sp["radiance"] = rng.uniform(0.5, 3.0, (n_spots, 3))
    sp["direction"] = (0.0, -1.0, 0.0)
    sp["cosInner"], sp["cosOuter"] = 0.95, 0.8
    sc.spot_lights = sp
    sc.dir_lights = np.zeros(0, DIR_LIGHT_DTYPE)
    sc.bounds = (np.array([-1, 0, -1], np.float32), np.array([1, 2, 1], np.float32))
    return sc


def cornell_view(width=512, height=512, frame=0):
    """Camera in the open side of the room; frame > 0 moves it along a short seeded-free dolly (for the filter)."""
    return make_view((0.02 * frame, 1.0 - 0.01 * frame, 0.95), (0.0, 0.9, -1.0), 65.0, width, height)


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]], np.float64)


def spheres_2m(seed=7, n_spheres=64, slices=160, stacks=101, tex_size=1024, with_textures=True, sky_size=(64, 32)):
    """64 distinct noise-displaced UV spheres (32,000 tris each) over a 1000x1000 ground."""
    rng = np.random.default_rng(seed)
    s = Scene()
    n_mats = 20
    mats = np.zeros(n_mats + 2, dtype=MATERIAL_DTYPE)
    textured = [0, 5, 10, 15] if with_textures else []
    for i in range(n_mats):
        m = empty_material()
        m["color"] = rng.uniform(0.1, 0.9, 3)
        m["roughness"] = rng.choice([0.75, 0.9, 1.0])
        m["flags"] = 1
        if i in textured:
            m["color"] = (1.0, 1.0, 1.0)
            m["color_map"]["texture"] = textured.index(i)
            m["color_map"]["uvscale"] = (4.0, 2.0)
        mats[i] = m
    ground = empty_material()
    ground["color"] = (0.6, 0.6, 0.55)
    ground["roughness"] = 1.0
    mats[n_mats] = ground
    lightm = empty_material()
    lightm["color"] = (12.0, 12.0, 11.0)
    mats[n_mats + 1] = lightm
    s.materials = mats
    if with_textures:
        s.textures = [make_texture(seed * 31 + k, tex_size) for k in range(4)]
    verts, faces, uv = uv_sphere(slices, stacks)
    area = 400.0
    for k in range(n_spheres):
        mat = int(rng.integers(0, n_mats))
        tw = (tex_size, tex_size) if mat in textured else None
        m = _smooth_mesh(verts, faces, seed * 1000 + k, 1.0, np.zeros(3, np.float32), mat, uv=uv, tex_wh=tw)
        s.meshes.append(_mesh(*m))
        sc = rng.uniform(0.5, 3.0)
        R = _rotation(rng) * sc
        T = np.eye(4, dtype=np.float64)
        T[:3, :3] = R
        T[:3, 3] = (rng.uniform(-area / 2, area / 2) * 0.2, sc * 1.1, rng.uniform(-area / 2, area / 2) * 0.2)
        s.instances.append((k, T.astype(np.float32)))
    # ground plane: two triangles, uv tiling
    g = add_quad((0, 1, 0), (0, 0, 0), 1000, 1000, n_mats)
    s.meshes.append(_mesh(*g))
    s.instances.append((n_spheres, np.eye(4, dtype=np.float32)))
    # 16 quad lights (32 triangles) in one mesh
    parts = []
    for k in range(16):
        pos = (rng.uniform(-40, 40), rng.uniform(15, 25), rng.uniform(-40, 40))
        parts.append(add_quad((0, -1, 0), pos, 4.0, 4.0, n_mats + 1))
    L = _concat(parts)
    L[3]["ltriIdx"] = np.arange(len(L[3]))
    s.meshes.append(_mesh(*L))
    s.instances.append((n_spheres + 1, np.eye(4, dtype=np.float32)))
    s.tri_lights = make_light_tris(L[0], L[1], L[2], L[3], (12.0, 12.0, 11.0), len(s.instances) - 1)
    pl = np.zeros(4, POINT_LIGHT_DTYPE)
    for k in range(4):
        pl[k]["position"] = (rng.uniform(-30, 30), rng.uniform(5, 12), rng.uniform(-30, 30))
        pl[k]["radiance"] = (300.0, 280.0, 250.0)
        pl[k]["energy"] = 830.0
    s.point_lights = pl
    s.spot_lights = np.zeros(0, SPOT_LIGHT_DTYPE)
    s.dir_lights = np.zeros(0, DIR_LIGHT_DTYPE)
    sw, sh = sky_size
    yy = (np.arange(sh) + 0.5) / sh
    sky = np.zeros((sh, sw, 3), np.float32)
    sky[..., 0] = (0.25 + 0.5 * (1 - yy))[:, None]
    sky[..., 1] = (0.35 + 0.5 * (1 - yy))[:, None]
    sky[..., 2] = (0.55 + 0.45 * (1 - yy))[:, None]
    s.sky = (sky.reshape(-1), sw, sh)
    s.bounds = (np.array([-500, 0, -500], np.float32), np.array([500, 30, 500], np.float32))
    return s


def spheres_view(width=1920, height=1080, frame=0, seed=7):
    """Seeded camera path over the sphere field (frame index selects the pose)."""
    rng = np.random.default_rng(seed * 7919 + 13)
    base_angle = rng.uniform(0, 2 * math.pi)
    a = base_angle + 0.01 * frame
    pos = (70 * math.cos(a), 18.0, 70 * math.sin(a))
    return make_view(pos, (0.0, 2.0, 0.0), 55.0, width, height)


def random_rays(scene, n, seed, kind="incoherent"):
    """Ray-query workloads: 'incoherent' = origins uniform in the scene box, directions uniform on the sphere;
    'secondary' = origins on area-weighted random surface points (offset along the normal), cosine-weighted
    hemisphere directions. tmax ~ U[0.1, scene diagonal]."""
    rng = np.random.default_rng(seed)
    lo, hi = scene.bounds
    diag = float(np.linalg.norm(hi - lo))
    rays = np.zeros(n, dtype=RAY_DTYPE)
    if kind == "incoherent":
        rays["o"] = rng.uniform(lo, hi, (n, 3))
        d = rng.normal(size=(n, 3))
    else:
        mesh_tris = []
        for mi, T in scene.instances:
            m = scene.meshes[mi]
            v = m.vertices[:, :3].reshape(-1, 3, 3) @ T[:3, :3].T + T[:3, 3]
            mesh_tris.append(v)
        V = np.concatenate(mesh_tris).astype(np.float64)
        areas = 0.5 * np.linalg.norm(np.cross(V[:, 1] - V[:, 0], V[:, 2] - V[:, 0]), axis=1)
        idx = rng.choice(len(V), size=n, p=areas / areas.sum())
        r1, r2 = rng.random(n), rng.random(n)
        su = np.sqrt(r1)
        b0, b1, b2 = 1 - su, su * (1 - r2), su * r2
        P = b0[:, None] * V[idx, 0] + b1[:, None] * V[idx, 1] + b2[:, None] * V[idx, 2]
        N = np.cross(V[idx, 1] - V[idx, 0], V[idx, 2] - V[idx, 0])
        N /= np.linalg.norm(N, axis=1, keepdims=True)
        flip = np.where(rng.random(n) < 0.5, -1.0, 1.0)[:, None]
        N = N * flip
        phi = 2 * math.pi * rng.random(n)
        r = rng.random(n)
        local = np.stack([np.cos(phi) * np.sqrt(1 - r), np.sin(phi) * np.sqrt(1 - r), np.sqrt(r)], -1)
        t = np.where(np.abs(N[:, :1]) > 0.9, np.array([[0, 1, 0]]), np.array([[1, 0, 0]]))
        Tg = np.cross(N, t); Tg /= np.linalg.norm(Tg, axis=1, keepdims=True)
        Bg = np.cross(N, Tg)
        d = local[:, :1] * Tg + local[:, 1:2] * Bg + local[:, 2:] * N
        rays["o"] = P + N * 1e-3 * max(1.0, diag * 1e-3)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["d"] = d
    rays["tmin"] = 0.0
    rays["tmax"] = rng.uniform(0.1, diag, n)
    return rays


def synthetic_blue_noise(seed=5):
    """Blue-noise tables in the layout of the OptiX 7 core's (a 256 x 256 Sobol table of 8-bit values and two
    128 x 128 x 8 tiles of scrambling and ranking keys), filled with seeded uniform bytes. The sampler maps any such
    bytes to numbers in (0, 1); the reference's published tables are the user's to upload."""
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 256, 65536, dtype=np.uint8), rng.integers(0, 256, 131072, dtype=np.uint8),
            rng.integers(0, 256, 131072, dtype=np.uint8))
