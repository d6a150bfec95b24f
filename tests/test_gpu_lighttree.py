"""The OptiX 7 estimator with its stochastic-lightcuts light tree (LH2G_RP_LIGHTTREE) on the CUDA core against the
oracle.

The oracle's light tree and light-tree frames are pinned to the reference's own code (tests/test_oracle_lighttree.py).
Here the GPU must match the oracle on a 164-light room (beyond the 64 lights selection by potentials takes) and on
the two-light Cornell room, and on two light mixes of an 88-light room (point and spot lights only; with directional
lights): per path and depth the hit record and the RNG state after shading bit-exact (each level
of the tree draws six numbers from the path's seed, so the states also check the walks), per path length the
extension and connection counts exact, per-pixel radiance within 1e-4 relative (the arithmetic and the summation
order are the same, so it is expected to be identical). Frames of more than 64 lights without the tree, and the
tree outside the OptiX 7 estimator, are refused."""
import ctypes as C

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300.core import RenderCore, CoreError, make_params, camera_r0, RP_NEE, RP_OPTIX7, RP_LIGHTTREE, RP_DEPTH_W, RP_DISNEY

pytestmark = pytest.mark.gpu

SCENES = {"lit_room": lambda: S.lit_room(), "cornell": lambda: S.cornell_sphere(subdiv=4)}


@pytest.fixture(scope="module", params=list(SCENES))
def pair(request, core_lib, oracle_lib):
    sc = SCENES[request.param]()
    sc.blue_noise = S.synthetic_blue_noise(19)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    yield request.param, core, o
    core.close()


def _compare(g, c, ga, ca):
    assert np.array_equal(g["counters"], c["counters"]), (g["counters"].tolist(), c["counters"].tolist())
    gh, ch = g["hits"], c["hits"]
    assert np.array_equal(gh["prim"], ch["prim"]), f"prim mismatch {np.count_nonzero(gh['prim'] != ch['prim'])}"
    live = ch["prim"] >= 0
    assert np.array_equal(gh["inst"][live], ch["inst"][live]) and np.array_equal(gh["bary"][live], ch["bary"][live])
    assert np.array_equal(gh["t"][live], ch["t"][live])
    assert np.array_equal(g["seeds"], c["seeds"])
    rel = np.abs(ga - ca) / np.maximum(np.abs(ca), 1e-6)
    assert rel.max() <= 1e-4, f"max rel {rel.max()}"


@pytest.mark.parametrize("W,H,spp,depth,st,tail", [(64, 48, 1, 4, 0, 5), (40, 32, 2, 6, 3, 0), (48, 40, 1, 8, 70, 2)])
def test_lighttree_frames(pair, W, H, spp, depth, st, tail):
    name, core, o = pair
    core.SetTarget(W, H, spp)
    core.Setting("waveTail", tail)
    try:
        p = make_params(W, H, spp, max_depth=depth, samples_taken=st, camera_r0=camera_r0(st), flags=RP_NEE | RP_OPTIX7 | RP_LIGHTTREE,
                        shift=0x91331445 + st)
        g = core.render_ex(S.cornell_view(W, H), p, capture=True)
        c = o.render(S.cornell_view(W, H), p, capture=True)
        _compare(g, c, core.read_accumulator(), c["accum"])
        assert g["counters"][:, 1].sum() > 0 and core.read_accumulator()[:, 3].sum() > 0
        assert core.GetCoreStats()["deviceStatus"] == 0
    finally:
        core.Setting("waveTail", 5)


def test_lighttree_with_disney(pair):
    """The light tree combines with the Disney BSDF (one oracle frame)."""
    name, core, o = pair
    W, H = 40, 32
    core.SetTarget(W, H, 1)
    p = make_params(W, H, 1, max_depth=5, camera_r0=camera_r0(0), flags=RP_NEE | RP_OPTIX7 | RP_LIGHTTREE | RP_DISNEY, shift=0x11331445)
    g = core.render_ex(S.cornell_view(W, H), p, capture=True)
    c = o.render(S.cornell_view(W, H), p, capture=True)
    _compare(g, c, core.read_accumulator(), c["accum"])


def test_plugin_setting_and_refusals(core_lib):
    """Render with settings estimator 1 + lightTree 1 renders the 164-light room; the PrimeRef estimator, the OptiX 7
    one without the tree, the tree without the OptiX 7 estimator, the serving loop and the allocation-free entry
    point refuse it (they select lights by potentials, 64 at most)."""
    import torch
    from lighthouse2_gb300.server import RenderServer
    sc = S.lit_room()
    core = RenderCore()
    core.set_scene(sc)
    W, H = 32, 24
    core.SetTarget(W, H, 1)
    view = S.cornell_view(W, H)
    with pytest.raises(CoreError):
        core.Render(view, 1)                      # PrimeRef, 164 lights
    core.Setting("estimator", 1)
    with pytest.raises(CoreError):
        core.Render(view, 1)                      # OptiX 7 by potentials
    core.Setting("lightTree", 1)
    for k in range(3):
        core.Render(view, 1 if k == 0 else 0)
    core.WaitForRender()
    img = core.read_accumulator()
    assert np.isfinite(img).all() and img[:, :3].sum() > 0
    with pytest.raises(CoreError):
        core.render_ex(view, make_params(W, H, 1, max_depth=3, flags=RP_NEE | RP_DEPTH_W | RP_LIGHTTREE))
    srv = RenderServer(path_capacity=1 << 16)
    with pytest.raises(CoreError):
        srv.add_scene(core)
    srv.close()
    acc = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda:0")
    p = make_params(W, H, 1, max_depth=3, flags=RP_NEE | RP_DEPTH_W)
    status = C.c_uint32(0)
    fn = core.lib.lh2g_render_noalloc
    rc = fn(core.ctx, view.ctypes.data_as(C.c_void_p), p.ctypes.data_as(C.c_void_p), C.c_void_p(acc.data_ptr()), None, C.byref(status))
    assert rc == 1   # LH2G_ERR_INVALID
    core.close()


@pytest.mark.parametrize("frame", range(2))
def test_lighttree_light_mixes(core_lib, oracle_lib, frame):
    """A tree of point and spot lights only (no path hits an emitter), and a room with two directional lights that
    the tree leaves out: GPU frames equal the oracle's (the oracle's are pinned to the reference's)."""
    from tests.golden import make_golden_lighttree as G
    name, kind, W, H, D, st, shift = G.MIX_FRAMES[frame]
    sc = G.mix_scene(kind)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    core.SetTarget(W, H, 1)
    p = make_params(W, H, 1, max_depth=D, samples_taken=st, camera_r0=camera_r0(st), flags=RP_NEE | RP_OPTIX7 | RP_LIGHTTREE, shift=shift)
    g = core.render_ex(S.cornell_view(W, H), p, capture=True)
    c = o.render(S.cornell_view(W, H), p, capture=True)
    _compare(g, c, core.read_accumulator(), c["accum"])
    assert g["counters"][:, 1].sum() > 0 and core.GetCoreStats()["deviceStatus"] == 0
    core.close()
