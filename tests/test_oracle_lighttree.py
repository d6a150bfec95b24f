"""The stochastic-lightcuts light tree (LH2G_RP_LIGHTTREE) of the oracle and of the core's host build, against the
reference's own code.

Golden vectors (tests/golden/make_golden_lighttree.py, committed) come from the OptiX 7 core's UpdateLightTree
(lib/rendercore_optix7/rendercore.cpp:571-680) and its shading kernel with the light-tree calls in place and
LIGHTTREE defined (lib/CUDA/shared_kernel_code/lights_shared.h:120-395), compiled for the host from the reference tree.
Trees must match record for record, bit for bit (the core's host build through lh2g_build_light_tree, which needs no
GPU, and the oracle's own restatement); frames of a 164-light room: per path length the extension and connection
counts exactly, radiance within 1e-5 relative (the reference adds a pixel's connections after its wave loop; only the
rounding of the sums differs). Where the reference tree is given (LH2_REFERENCE), the same comparisons run live."""
import ctypes as C
import os

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lighttree_vectors.npz")
REF = os.environ.get("LH2_REFERENCE", "")
live = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "lib", "rendercore_optix7")),
                          reason="reference tree not given (LH2_REFERENCE)")


def _close(a, b, tol=1e-5):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-30)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def oracle_tree(B, tri, pt, sp):
    o = B.Oracle()
    vp = C.c_void_p
    p = lambda a: a.ctypes.data_as(vp) if len(a) else None
    dirs = np.zeros(0, S.DIR_LIGHT_DTYPE)
    assert o.lib.lh2o_set_lights(o.s, p(tri), len(tri), p(pt), len(pt), p(sp), len(sp), None, 0) == 0
    return o.light_tree()


def _words(t):
    return t.view(np.uint32).reshape(len(t), 16) if len(t) else np.zeros((0, 16), np.uint32)


def test_oracle_trees_match_reference(gold, oracle_lib):
    from tests.golden import make_golden_lighttree as G
    for name, tri, pt, sp in G.tree_light_sets():
        t = oracle_tree(oracle_lib, tri, pt, sp)
        assert np.array_equal(_words(t), gold["tree_" + name]), name
        assert len(t) == 2 * (len(tri) + len(pt) + len(sp))


def test_core_host_build_matches_reference(gold, core_lib):
    """lh2g_build_light_tree: the tree lh2g_set_lights uploads, built on the host (no GPU)."""
    from lighthouse2_gb300.core import build_light_tree
    from tests.golden import make_golden_lighttree as G
    for name, tri, pt, sp in G.tree_light_sets():
        t = build_light_tree(tri, pt, sp)
        assert np.array_equal(_words(t), gold["tree_" + name]), name
    assert len(build_light_tree(np.zeros(0, S.LIGHT_TRI_DTYPE), np.zeros(0, S.POINT_LIGHT_DTYPE), np.zeros(0, S.SPOT_LIGHT_DTYPE))) == 0


def test_tree_shape(gold):
    """Structure of the room's tree: record 0 the root, every leaf reached once, parents consistent."""
    t = gold["tree_room"].view(np.int32)
    light, left, right, parent = t[:, 0], t[:, 1], t[:, 2], t[:, 15]
    seen, stack = [], [0]
    while stack:
        n = stack.pop()
        if left[n] == -1:
            seen.append(light[n])
            continue
        assert parent[left[n]] == n and parent[right[n]] == n
        stack += [left[n], right[n]]
    n_tri = 128
    expect = list(range(n_tri)) + [(1 << 30) | k for k in range(24)] + [(1 << 29) | k for k in range(12)]
    assert sorted(seen) == sorted(expect)


def test_lighttree_frames(gold, oracle_lib):
    from tests.golden import make_golden_lighttree as G
    B = oracle_lib
    sc = G.scene()
    o = B.Oracle()
    o.set_scene(sc)
    for name, W, H, spp, D, st, shift in G.FRAMES:
        p = B.make_params(W, H, spp, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st),
                          flags=B.RP_NEE | B.RP_OPTIX7 | B.RP_LIGHTTREE, shift=shift)
        r = o.render(S.cornell_view(W, H), p)
        assert np.array_equal(r["counters"], gold[name + "/counters"]), name
        assert _close(r["accum"], gold[name + "/accum"]), name
        assert r["counters"][:, 1].sum() > 0


def test_lighttree_light_mixes(gold, oracle_lib):
    """A tree of point and spot lights only, and a room whose directional lights the tree leaves out."""
    from tests.golden import make_golden_lighttree as G
    B = oracle_lib
    for name, kind, W, H, D, st, shift in G.MIX_FRAMES:
        o = B.Oracle()
        o.set_scene(G.mix_scene(kind))
        p = B.make_params(W, H, 1, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st),
                          flags=B.RP_NEE | B.RP_OPTIX7 | B.RP_LIGHTTREE, shift=shift)
        r = o.render(S.cornell_view(W, H), p)
        assert np.array_equal(r["counters"], gold[name + "/counters"]), name
        assert _close(r["accum"], gold[name + "/accum"]), name


def test_many_lights_need_the_tree(oracle_lib):
    """More than 64 lights: selection by potentials is refused (its arrays hold 64), the light tree renders."""
    B = oracle_lib
    sc = S.lit_room()
    o = B.Oracle()
    o.set_scene(sc)
    W, H = 16, 12
    p = B.make_params(W, H, 1, max_depth=3, flags=B.RP_NEE | B.RP_OPTIX7)
    with pytest.raises(AssertionError):
        o.render(S.cornell_view(W, H), p)
    p["flags"] = B.RP_NEE | B.RP_OPTIX7 | B.RP_LIGHTTREE
    assert o.render(S.cornell_view(W, H), p)["accum"][:, :3].sum() > 0


@live
def test_live_lighttree(oracle_lib):
    B = oracle_lib
    from tests.golden import make_golden_lighttree as G
    ref = B.RefOptix7(light_tree=True)
    for name, tri, pt, sp in G.tree_light_sets():
        assert np.array_equal(_words(oracle_tree(B, tri, pt, sp)), _words(B.ref_light_tree(ref.lib, tri, pt, sp))), name
    sc = S.lit_room(seed=23, grid=6, n_points=9, n_spots=5)
    sc.blue_noise = B.reference_blue_noise()
    o = B.Oracle()
    o.set_scene(sc)
    for W, H, spp, D, st in ((40, 32, 1, 4, 0), (24, 20, 2, 6, 70)):
        p = B.make_params(W, H, spp, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st),
                          flags=B.RP_NEE | B.RP_OPTIX7 | B.RP_LIGHTTREE, shift=0x91331445)
        a = o.render(S.cornell_view(W, H), p)
        r = ref.render(o, sc, S.cornell_view(W, H), p)
        assert not r["flushed"]
        assert np.array_equal(a["counters"], r["counters"])
        assert _close(a["accum"], r["accum"])


def test_core_host_build_errors(core_lib):
    """lh2g_build_light_tree returns minus an error code: -LH2G_ERR_OVERFLOW when the output holds too few records,
    -LH2G_ERR_INVALID for negative counts."""
    import ctypes as C
    from lighthouse2_gb300.core import load_library, LIGHT_TREE_DTYPE
    lib = load_library()
    sc = S.lit_room(grid=2, n_points=1, n_spots=1)
    tri = np.ascontiguousarray(sc.tri_lights)
    out = np.zeros(4, LIGHT_TREE_DTYPE)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    assert lib.lh2g_build_light_tree(p(tri), len(tri), None, 0, None, 0, p(out), 4) == -5       # needs 16 records
    assert lib.lh2g_build_light_tree(p(tri), -1, None, 0, None, 0, p(out), 4) == -1
    n = 2 * len(tri)
    big = np.zeros(n, LIGHT_TREE_DTYPE)
    assert lib.lh2g_build_light_tree(p(tri), len(tri), None, 0, None, 0, p(big), n) == n
