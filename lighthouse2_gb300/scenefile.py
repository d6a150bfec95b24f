"""Scene and frame-sequence files for the headless application (harness/headless_app.cpp).

The application drives a render core through the Lighthouse 2 plugin interface exactly as the reference's
RenderSystem does (lib/RenderSystem/rendersystem.cpp:50-211), so it needs the scene as the RenderSystem holds it:
meshes as unindexed float4 vertex triplets plus CoreTri records, instances with 4x4 transforms, materials,
ARGB32 textures with their MIP chains, lights and sky. This module writes them in a flat little-endian format:

  scene file   "LH2GSCN1", u32 counts [meshes, instances, materials, textures, tri lights, point lights,
               spot lights, directional lights, sky width, sky height], then per mesh u32 triangle count,
               float32 vertices (3 x 4 per triangle), CoreTri (208 B) per triangle; per instance i32 mesh and
               float32 4x4 row-major object-to-world; materials (lh2g_material, 196 B); per texture u32 width,
               height, texel count and the texels (u32); the four light arrays; sky rgb float32
  frames file  "LH2GFRM1", u32 frame count, then per frame the camera view (68 B), i32 converge (1 = Restart,
               0 = Converge) and an instance change applied before the frame (i32 instance, -1 for none,
               i32 mesh, float32 4x4 transform)
"""
from __future__ import annotations

import struct

import numpy as np

from . import scenes as S


def write_scene(path, sc: S.Scene):
    empty = lambda a, dt: np.zeros(0, dt) if a is None else np.ascontiguousarray(a, dt)
    tri, pt, spot, dirl = (empty(sc.tri_lights, S.LIGHT_TRI_DTYPE), empty(sc.point_lights, S.POINT_LIGHT_DTYPE),
                           empty(sc.spot_lights, S.SPOT_LIGHT_DTYPE), empty(sc.dir_lights, S.DIR_LIGHT_DTYPE))
    sky_rgb, sky_w, sky_h = sc.sky if sc.sky is not None else (np.zeros(0, np.float32), 0, 0)
    mats = np.ascontiguousarray(sc.materials, S.MATERIAL_DTYPE)
    with open(path, "wb") as f:
        f.write(b"LH2GSCN1")
        f.write(struct.pack("<10I", len(sc.meshes), len(sc.instances), len(mats), len(sc.textures), len(tri), len(pt), len(spot),
                            len(dirl), sky_w, sky_h))
        for m in sc.meshes:
            tris = np.ascontiguousarray(m.tris, S.CORE_TRI_DTYPE)
            verts = np.ascontiguousarray(m.vertices, np.float32).reshape(-1)
            assert verts.size == 12 * len(tris)
            f.write(struct.pack("<I", len(tris)))
            f.write(verts.tobytes())
            f.write(tris.tobytes())
        for mi, T in sc.instances:
            f.write(struct.pack("<i", int(mi)))
            f.write(np.ascontiguousarray(T, np.float32).reshape(16).tobytes())
        f.write(mats.tobytes())
        for t in sc.textures:
            texels = np.ascontiguousarray(t.texels, np.uint32)
            f.write(struct.pack("<3I", t.width, t.height, texels.size))
            f.write(texels.tobytes())
        for a in (tri, pt, spot, dirl):
            f.write(a.tobytes())
        f.write(np.ascontiguousarray(sky_rgb, np.float32).reshape(-1).tobytes())


def write_frames(path, frames):
    """frames: list of (view (VIEW_DTYPE), converge (1 Restart / 0 Converge), change) where change is None or
    (instance index, mesh index, 4x4 transform)."""
    with open(path, "wb") as f:
        f.write(b"LH2GFRM1")
        f.write(struct.pack("<I", len(frames)))
        for view, converge, change in frames:
            v = np.ascontiguousarray(view, S.VIEW_DTYPE).reshape(1)
            f.write(v.tobytes())
            f.write(struct.pack("<i", int(converge)))
            if change is None:
                f.write(struct.pack("<ii", -1, -1))
                f.write(np.eye(4, dtype=np.float32).tobytes())
            else:
                inst, mesh, T = change
                f.write(struct.pack("<ii", int(inst), int(mesh)))
                f.write(np.ascontiguousarray(T, np.float32).reshape(16).tobytes())


def read_frames_output(path, width, height):
    """The application's output: per frame a line of statistics in the log and W*H float4 in this file."""
    data = np.fromfile(path, np.float32)
    return data.reshape(-1, width * height, 4)
