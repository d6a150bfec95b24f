"""Shapes of the seeded workloads."""
import numpy as np

from lighthouse2_gb300 import scenes as S


def test_cornell_shape():
    sc = S.cornell_sphere(subdiv=6)
    assert len(sc.meshes[0].tris) == 24                      # 12 quads
    assert len(sc.meshes[1].tris) == 20 * 4 ** 6             # icosphere, subdivision 6
    assert len(sc.materials) == 9 and len(sc.tri_lights) == 2
    assert all(len(m.vertices) == 3 * len(m.tris) for m in sc.meshes)
    m = sc.materials[:8]
    assert np.all((m["color"] >= 0.1) & (m["color"] <= 0.9)) and np.all(m["roughness"] == np.float32(0.75))


def test_spheres_small_shape():
    sc = S.spheres_2m(n_spheres=4, slices=20, stacks=11, tex_size=64)
    assert [len(m.tris) for m in sc.meshes[:4]] == [2 * 20 * 10] * 4
    assert len(sc.tri_lights) + len(sc.point_lights) == 36 <= 64
    t = sc.textures[0]
    assert len(t.texels) == sum((64 >> k) ** 2 for k in range(5))   # 5 MIP levels back to back


def test_uv_sphere_count_for_2m():
    v, f, uv = S.uv_sphere(160, 101)
    assert len(f) == 32000                                   # 64 of these + 2 ground triangles = 2,048,002
