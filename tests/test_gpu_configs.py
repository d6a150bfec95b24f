"""Parity at the benchmark configurations' own sizes, not shrunken stand-ins.

* Small scene: the Cornell room with the subdivision-6 displaced icosphere (81,944 triangles), 512 x 512, 1 spp,
  max depth 3, next-event estimation, Russian roulette from the first bounce (the PrimeRef estimator).
* Large scene: one full frame of the 2,048,002-triangle sphere field (64 distinct 32k-triangle meshes, 1024^2
  textures with 5 MIP levels, 36 lights, sky), 1920 x 1080, 1 spp, max depth 8, Russian roulette after depth 3,
  next-event estimation.
* Ray queries: 2^22 incoherent and 2^22 secondary-like rays on both scenes' BVHs, closest and any hit.

The wave loop is the one of lib/RenderCore_PrimeRef/rendercore.cpp:551-611 that the oracle restates. Per path and
depth the hit record (instance, primitive, quantised barycentrics, t) and the RNG state after shading are
bit-exact, per path length the extension and connection counts are exact, and per-pixel radiance is within 1e-4
relative; ray queries match IDs exactly and t within 1e-5 relative.
"""
import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300.core import RenderCore, make_params, camera_r0, RP_NEE, RP_DEPTH_W

pytestmark = pytest.mark.gpu


def _frame_parity(core, o, view, p):
    g = core.render_ex(view, p, capture=True)
    c = o.render(view, p, capture=True)
    assert np.array_equal(g["counters"], c["counters"]), (g["counters"].tolist(), c["counters"].tolist())
    gh, ch = g["hits"], c["hits"]
    bad = np.count_nonzero(gh["prim"] != ch["prim"])
    assert bad == 0, f"primitive ids differ on {bad} path vertices"
    live = ch["prim"] >= 0
    assert np.array_equal(gh["inst"][live], ch["inst"][live])
    assert np.array_equal(gh["bary"][live], ch["bary"][live])
    rel_t = np.abs(gh["t"][live] - ch["t"][live]) / np.maximum(np.abs(ch["t"][live]), 1e-30)
    assert rel_t.max(initial=0) <= 1e-5
    assert np.array_equal(g["seeds"], c["seeds"])
    ga, ca = core.read_accumulator(), c["accum"]
    rel = np.abs(ga - ca) / np.maximum(np.abs(ca), 1e-6)
    assert rel.max() <= 1e-4, f"max relative radiance difference {rel.max()}"
    return g["counters"]


def test_small_scene_config(core_lib, oracle_lib):
    sc = S.cornell_sphere(subdiv=6)
    assert sc.triangle_count == 81944
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    W = H = 512
    core.SetTarget(W, H, 1)
    p = make_params(W, H, 1, max_depth=3, rr_start=1, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
    c = _frame_parity(core, o, S.cornell_view(W, H), p)
    assert c[0, 0] > 0.3 * W * H   # most primary paths hit the room and bounce on
    core.close()


def test_large_scene_full_frame(core_lib, oracle_lib):
    sc = S.spheres_2m(seed=7)
    assert sc.triangle_count == 2048002 + 32   # with the 16 quad lights
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    W, H = 1920, 1080
    core.SetTarget(W, H, 1)
    for pose in (0, 5):
        p = make_params(W, H, 1, max_depth=8, rr_start=4, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
        c = _frame_parity(core, o, S.spheres_view(W, H, frame=pose), p)
        assert c[:, 1].sum() > 1_000_000   # next-event connections over the 36 lights at scale
    core.close()


@pytest.mark.parametrize("scene", ["cornell", "spheres"])
def test_ray_queries_at_scale(core_lib, oracle_lib, scene):
    sc = S.cornell_sphere(subdiv=6) if scene == "cornell" else S.spheres_2m(seed=7)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    n = 1 << 22
    for kind, seed in (("incoherent", 21), ("secondary", 22)):
        rays = S.random_rays(sc, n, seed=seed, kind=kind)
        g, c = core.trace_host(rays, mode=0), o.trace(rays, mode=0)
        bad = np.count_nonzero(g["prim"] != c["prim"])
        assert bad == 0, f"{kind}: primitive ids differ on {bad} rays"
        hit = c["prim"] >= 0
        assert np.array_equal(g["inst"][hit], c["inst"][hit])
        assert np.array_equal(g["bary"][hit], c["bary"][hit])
        rel = np.abs(g["t"][hit] - c["t"][hit]) / np.maximum(np.abs(c["t"][hit]), 1e-30)
        assert rel.max(initial=0) <= 1e-5
        assert np.array_equal(core.trace_host(rays, mode=1), o.trace(rays, mode=1))
        if scene == "cornell":
            assert hit.mean() > 0.3   # the room is open on the camera side only
    core.close()
