"""Generates tests/golden/raster_vectors.npz from the reference's own SoftRasterizer core (TEST INFRASTRUCTURE).

Runs where the reference tree is given (LH2_REFERENCE): oracle/ref compiles, by path,
lib/RenderCore_SoftRasterizer/rasterizer.cpp and rendercore.cpp for the host, and this script renders the cases
below through that core's own RenderCore methods, keeping its uploaded pixels and its z-buffer.

    LH2_REFERENCE=<lighthouse2 tree> python tests/golden/make_golden_raster.py

The cases cover what the rasterizer's arithmetic branches on: triangles crossing the near and left clipping planes
(camera inside the room), a rolled camera, a camera facing away (mesh culling), texture coordinates far outside
[0, 1] in both signs on a non-square texture, instances that share a mesh (the reference's scene graph gives them
the transform set last), emitters whose colour exceeds 1 (the packed colour overflows into the next channel), odd
and minimal target sizes.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lighthouse2_gb300 import scenes as S  # noqa: E402


def raster_scene(seed=3):
    """The Cornell room (subdivision 3 sphere) plus a textured quad mesh with texture coordinates in [-2.3, 3.7],
    instanced twice, and the sphere instanced a second time (both shared meshes end with the transform set last)."""
    sc = S.cornell_sphere(subdiv=3)
    rng = np.random.default_rng(seed)
    tw, th = 64, 32
    sc.textures = [S.Texture(tw, th, rng.integers(0, 2 ** 32, tw * th + (tw // 2) * (th // 2), dtype=np.uint64).astype(np.uint32))]
    mats = np.zeros(len(sc.materials) + 1, sc.materials.dtype)
    mats[:-1] = sc.materials
    m = S.empty_material()
    m["color"] = (0.6, 0.5, 0.4)
    m["color_map"]["texture"] = 0
    mats[-1] = m
    sc.materials = mats
    v0, v1, v2, tris = S.add_quad((0.3, 0.2, 1.0), (0.0, 0.0, 0.0), 0.8, 0.5, len(mats) - 1)
    tris["u"] = np.array([[-2.3, 3.7, 0.4], [1.9, -1.1, 3.3]], np.float32)
    tris["v"] = np.array([[3.1, -2.2, 0.7], [-0.6, 2.8, -1.9]], np.float32)
    sc.meshes.append(S._mesh(v0, v1, v2, tris))
    quad = len(sc.meshes) - 1

    def T(tx, ty, tz, a=0.0):
        c, s = np.cos(a), np.sin(a)
        return np.array([[c, 0, s, tx], [0, 1, 0, ty], [-s, 0, c, tz], [0, 0, 0, 1]], np.float32)

    sc.instances = list(sc.instances) + [(quad, T(0.2, 1.2, -0.6, 0.3)), (quad, T(-0.3, 0.8, -0.2, -0.5)), (1, T(0.05, 0.1, 0.0))]
    return sc


def views():
    """name -> (scene builder, view, W, H)"""
    small_spheres = lambda: S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=64, sky_size=(64, 32))  # noqa: E731
    return {
        "cornell_64x48": (lambda: S.cornell_sphere(subdiv=3), S.cornell_view(64, 48), 64, 48),
        "inside_80x60": (raster_scene, S.make_view((-0.85, 0.5, 0.6), (0.6, 1.1, -0.9), 95.0, 80, 60), 80, 60),
        "rolled_37x23": (raster_scene, S.make_view((0.1, 1.0, 0.9), (0.0, 0.8, -1.0), 70.0, 37, 23, up=(0.35, 1.0, 0.1)), 37, 23),
        "close_45x31": (raster_scene, S.make_view((0.3, 0.5, 0.2), (0.35, 0.45, -0.2), 80.0, 45, 31), 45, 31),
        "away_16x12": (raster_scene, S.make_view((0.0, 1.0, 0.9), (0.0, 1.0, 5.0), 60.0, 16, 12), 16, 12),
        "tiny_3x3": (raster_scene, S.cornell_view(3, 3), 3, 3),
        "tiny_5x4": (raster_scene, S.cornell_view(5, 4), 5, 4),
        "spheres_96x64": (small_spheres, S.spheres_view(96, 64, frame=1), 96, 64),
    }


def main():
    from oracle import bind as B
    ref = B.RefRaster()
    out = {}
    for name, (build, view, W, H) in views().items():
        r = ref.raster(build(), view, W, H)
        out[name + "/pixels"] = r["pixels"]
        out[name + "/zbuffer"] = r["zbuffer"]
        print(name, np.count_nonzero(r["pixels"]), "pixels drawn")
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "raster_vectors.npz"), **out)


if __name__ == "__main__":
    main()
