"""Generates tests/golden/lighttree_vectors.npz from the reference's own code (TEST INFRASTRUCTURE).

Runs where the reference tree is given (LH2_REFERENCE): oracle/ref compiles the OptiX 7 core's light-tree build
(RenderCore::UpdateLightTree and its helpers, lib/rendercore_optix7/rendercore.cpp:571-680) and its shading kernel with
the light-tree calls in place and LIGHTTREE defined (lib/CUDA/shared_kernel_code/lights_shared.h:120-395). This script
stores the trees the reference builds for several light sets and renders frames of a many-light room through that
core's wave loop, with the oracle answering the ray queries.

    LH2_REFERENCE=<lighthouse2 tree> python tests/golden/make_golden_lighttree.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lighthouse2_gb300 import scenes as S  # noqa: E402

# name, W, H, spp, depth, samplesTaken (>= 64: xorshift numbers), shift
FRAMES = [("t_a", 48, 40, 1, 4, 0, 0x91331445), ("t_b", 32, 24, 2, 6, 3, 0x11331445), ("t_c", 40, 32, 1, 5, 70, 7)]


def tree_light_sets():
    """(name, area lights, point lights, spot lights): the many-light room's, subsets of it, a single light, ties"""
    sc = S.lit_room()
    tri, pt, sp = sc.tri_lights, sc.point_lights, sc.spot_lights
    twins = np.concatenate([tri[:4], tri[:4]])   # equal clusters: the first index wins the ties
    return [("room", tri, pt, sp), ("tri_only", tri[:37], pt[:0], sp[:0]), ("points_spots", tri[:0], pt, sp),
            ("one", tri[:1], pt[:0], sp[:0]), ("two", tri[:1], pt[:1], sp[:0]), ("twins", twins, pt[:3], sp[:0])]


def scene():
    sc = S.lit_room()
    sc.blue_noise = S.synthetic_blue_noise(17)
    return sc


# name, scene variant, W, H, depth, samplesTaken, shift
MIX_FRAMES = [("m_points_spots", "points_spots", 48, 40, 6, 3, 0x5151), ("m_with_directional", "with_directional", 48, 40, 6, 3, 0x5151)]


def mix_scene(kind):
    """An 88-light room (a 3x3 ceiling grid, 40 point and 30 spot lights) in two variants. "points_spots": no area
    lights, the ceiling tiles no longer emit, so the tree holds only point and spot lights and no path hits an
    emitter. "with_directional": two directional lights as well, which the tree leaves out (with LIGHTTREE defined
    the reference never picks a directional light)."""
    sc = S.lit_room(seed=31, grid=3, n_points=40, n_spots=30)
    if kind == "points_spots":
        sc.tri_lights = sc.tri_lights[:0]
        sc.materials["color"][8:] = (0.5, 0.5, 0.5)
    else:
        d = np.zeros(2, S.DIR_LIGHT_DTYPE)
        d["direction"] = ((0.3, -1.0, 0.2), (-0.5, -0.7, 0.1))
        d["direction"] /= np.linalg.norm(d["direction"], axis=1, keepdims=True)
        d["radiance"] = (0.4, 0.4, 0.35)
        d["energy"] = 1.15
        sc.dir_lights = d
    sc.blue_noise = S.synthetic_blue_noise(23)
    return sc


def main():
    from oracle import bind as B
    out = {}
    ref = B.RefOptix7(light_tree=True)
    for name, tri, pt, sp in tree_light_sets():
        t = B.ref_light_tree(ref.lib, tri, pt, sp)
        out["tree_" + name] = t.view(np.uint32).reshape(len(t), 16) if len(t) else np.zeros((0, 16), np.uint32)
    sc = scene()
    o = B.Oracle()
    o.set_scene(sc)
    for name, W, H, spp, depth, st, shift in FRAMES:
        p = B.make_params(W, H, spp, max_depth=depth, samples_taken=st, camera_r0=B.camera_r0(st),
                          flags=B.RP_NEE | B.RP_OPTIX7 | B.RP_LIGHTTREE, shift=shift)
        r = ref.render(o, sc, S.cornell_view(W, H), p)
        assert not r["flushed"]
        out[name + "/accum"] = r["accum"]
        out[name + "/counters"] = r["counters"]
        print(name, r["counters"][:, 0].tolist(), r["counters"][:, 1].tolist())
    for name, kind, W, H, depth, st, shift in MIX_FRAMES:
        sc = mix_scene(kind)
        o = B.Oracle()
        o.set_scene(sc)
        p = B.make_params(W, H, 1, max_depth=depth, samples_taken=st, camera_r0=B.camera_r0(st), flags=B.RP_NEE | B.RP_OPTIX7 | B.RP_LIGHTTREE, shift=shift)
        r = ref.render(o, sc, S.cornell_view(W, H), p)
        assert not r["flushed"]
        out[name + "/accum"] = r["accum"]
        out[name + "/counters"] = r["counters"]
        print(name, r["counters"][:, 0].tolist(), r["counters"][:, 1].tolist())
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "lighttree_vectors.npz"), **out)


if __name__ == "__main__":
    main()
