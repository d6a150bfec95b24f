"""The oracle's BVH traversal returns exactly the brute-force closest and any hit (ties: lowest instance, primitive)."""
import numpy as np

from lighthouse2_gb300 import scenes as S


def _same(a, b):
    assert np.array_equal(a["prim"], b["prim"])
    h = a["prim"] >= 0
    assert np.array_equal(a["inst"][h], b["inst"][h]) and np.array_equal(a["t"][h], b["t"][h]) and np.array_equal(a["bary"][h], b["bary"][h])


def test_bvh_equals_brute_force(oracle_lib):
    for sc in (S.cornell_sphere(subdiv=3), S.spheres_2m(n_spheres=5, slices=16, stacks=10, tex_size=32)):
        o = oracle_lib.Oracle()
        o.set_scene(sc)
        for kind, seed in (("incoherent", 1), ("secondary", 2)):
            rays = S.random_rays(sc, 3000, seed, kind)
            _same(o.trace(rays, 0), o.trace(rays, 0, brute=True))
            assert np.array_equal(o.trace(rays, 1), o.trace(rays, 1, brute=True))
