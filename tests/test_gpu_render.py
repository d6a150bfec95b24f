"""Frame parity of the CUDA wavefront path tracer against the CPU oracle.

Per path and per depth the hit record (instance, primitive, quantised barycentrics, distance) and the RNG
state after shading must match bit-exactly; per path length the extension-ray and connection counts must
match exactly; per-pixel radiance within 1e-4 relative (the arithmetic is the same, so it is expected to be
identical)."""
import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300.core import RenderCore, make_params, camera_r0, RP_NEE, RP_DEPTH_W

pytestmark = pytest.mark.gpu


def _check_frame(core, o, view, p, accumulate=False):
    g = core.render_ex(view, p, accumulate=accumulate, capture=True)
    c = o.render(view, p, capture=True)
    assert np.array_equal(g["counters"], c["counters"]), (g["counters"].tolist(), c["counters"].tolist())
    gh, ch = g["hits"], c["hits"]
    assert np.array_equal(gh["prim"], ch["prim"]), f"prim mismatch {np.count_nonzero(gh['prim'] != ch['prim'])}"
    live = ch["prim"] >= 0
    assert np.array_equal(gh["inst"][live], ch["inst"][live])
    assert np.array_equal(gh["bary"][live], ch["bary"][live])
    assert np.array_equal(gh["t"][live], ch["t"][live])
    assert np.array_equal(g["seeds"], c["seeds"])
    ga = core.read_accumulator()
    ca = c["accum"]
    denom = np.maximum(np.abs(ca), 1e-6)
    rel = np.abs(ga - ca) / denom
    assert rel.max() <= 1e-4, f"max rel {rel.max()}"
    return ga


@pytest.fixture(scope="module")
def cornell(core_lib, oracle_lib):
    sc = S.cornell_sphere(subdiv=5)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    return sc, core, o


@pytest.mark.parametrize("W,H,spp,depth,rr", [(96, 80, 1, 3, 1), (64, 64, 2, 6, 1), (48, 32, 3, 8, 4)])
def test_cornell_frame(cornell, W, H, spp, depth, rr):
    sc, core, o = cornell
    core.SetTarget(W, H, spp)
    view = S.cornell_view(W, H)
    p = make_params(W, H, spp, max_depth=depth, rr_start=rr, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
    _check_frame(core, o, view, p)


def test_cornell_no_nee_and_converge(cornell):
    sc, core, o = cornell
    W, H = 40, 40
    core.SetTarget(W, H, 1)
    view = S.cornell_view(W, H)
    p = make_params(W, H, 1, max_depth=4, camera_r0=camera_r0(0), flags=RP_DEPTH_W)
    _check_frame(core, o, view, p)
    # second converging frame accumulates: compare against the oracle summing both frames
    p2 = make_params(W, H, 1, max_depth=4, samples_taken=1, camera_r0=camera_r0(1), flags=RP_NEE)
    p1 = make_params(W, H, 1, max_depth=4, camera_r0=camera_r0(0), flags=RP_NEE)
    core.render_ex(view, p1, accumulate=False)
    core.render_ex(view, p2, accumulate=True)
    acc = o.render(view, p1)["accum"]
    acc = o.render(view, p2, accum=acc)["accum"]
    assert np.array_equal(core.read_accumulator(), acc)
    fb = core.read_framebuffer()
    assert np.allclose(fb, acc * np.float32(1.0 / 2.0), rtol=1e-6, atol=0)


def test_spheres_textured_sky(core_lib, oracle_lib):
    sc = S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=128)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    W, H = 80, 48
    core.SetTarget(W, H, 1)
    view = S.spheres_view(W, H)
    p = make_params(W, H, 1, max_depth=8, rr_start=4, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
    img = _check_frame(core, o, view, p)
    assert np.isfinite(img).all() and img[:, :3].sum() > 0


def test_render_api_matches_explicit_parameters(cornell):
    """Render(view, Restart/Converge) follows RenderCore_PrimeRef/rendercore.cpp:535-550 bookkeeping."""
    sc, core, o = cornell
    W, H = 32, 24
    core.SetTarget(W, H, 1)
    core.Setting("maxDepth", 3)
    view = S.cornell_view(W, H)
    core.Render(view, converge=1)
    core.Render(view, converge=0)
    core.Render(view, converge=0)
    stats = core.GetCoreStats()
    assert stats["primaryRayCount"] == W * H
    assert stats["totalRays"] == stats["totalExtensionRays"] + stats["totalShadowRays"]
    # Restart, then a Converge frame also clears (first converging frame), then accumulates
    acc = None
    for k in range(2):
        p = make_params(W, H, 1, max_depth=3, samples_taken=k, camera_r0=camera_r0(k), flags=RP_NEE | RP_DEPTH_W)
        acc = o.render(view, p, accum=acc)["accum"]
    assert np.array_equal(core.read_accumulator(), acc)


@pytest.mark.parametrize("tail", [0, 1, 2, 5])
def test_wave_tail_split_changes_nothing(cornell, tail):
    """Running path lengths >= waveTail in the persistent tail kernel instead of wave by wave gives the same
    hits, RNG states, queue counts and radiance (bit for bit) as the oracle."""
    sc, core, o = cornell
    W, H = 48, 40
    core.SetTarget(W, H, 2)
    core.Setting("waveTail", tail)
    try:
        view = S.cornell_view(W, H)
        p = make_params(W, H, 2, max_depth=7, rr_start=3, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
        acc = _check_frame(core, o, view, p)
        assert np.array_equal(acc, o.render(view, p)["accum"])
    finally:
        core.Setting("waveTail", 5)


def test_pipelined_frames_match_one_at_a_time(core_lib):
    """Consecutive plain frames overlap on two or four lanes (setting "pipelineFrames"); the accumulator, the frame and the
    statistics must equal those of the same frames rendered one at a time, whether frames accumulate, restart or
    converge through Render, and whatever is read between them."""
    sc = S.spheres_2m(seed=5, n_spheres=6, slices=40, stacks=26, tex_size=64)
    W, H = 160, 96
    results = {}
    for pipe in (0, 2, 4):
        core = RenderCore()
        core.set_scene(sc)
        core.SetTarget(W, H, 1)
        core.Setting("pipelineFrames", pipe)
        core.Setting("maxDepth", 6)
        out = []
        for k in range(7):
            view = S.spheres_view(W, H, frame=k % 3)
            p = make_params(W, H, 1, max_depth=6, rr_start=3, samples_taken=k, camera_r0=camera_r0(k), flags=RP_NEE | RP_DEPTH_W)
            core.render_ex(view, p, accumulate=k % 3 != 0, counters=False)
            if k % 2 == 1:
                out.append(core.read_accumulator().copy())
        stats = core.GetCoreStats()
        out.append(core.read_framebuffer().copy())
        for k in range(4):   # Render: restart, then converge
            core.Render(S.spheres_view(W, H, frame=1), converge=1 if k == 0 else 0)
        out.append(core.read_framebuffer().copy())
        out.append(np.array([stats["totalRays"], stats["totalShadowRays"]], np.float32))
        # frames copied to host memory as they finish (lh2g_render_to_host), several in flight
        hosts = [np.full((W * H, 4), np.nan, np.float32) for _ in range(3)]
        for k in range(3):
            p = make_params(W, H, 1, max_depth=6, rr_start=3, samples_taken=k, camera_r0=camera_r0(k), flags=RP_NEE | RP_DEPTH_W)
            core.render_to_host(S.spheres_view(W, H, frame=k), p, hosts[k].ctypes.data, accumulate=k > 0)
        core.WaitForRender()
        out += hosts
        results[pipe] = out
        core.close()
    for lanes in (2, 4):
        for a, b in zip(results[0], results[lanes]):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_material_index_out_of_range_is_refused(core_lib):
    """A triangle naming a material that was never set is refused at render time (the shading kernel would read
    past the material array); the context stays usable once the materials cover the index."""
    from lighthouse2_gb300.core import CoreError
    sc = S.cornell_sphere(subdiv=2)
    core = RenderCore()
    core.set_scene(sc)
    n = len(sc.materials)
    core.SetMaterials(sc.materials[:1])
    W, H = 32, 24
    core.SetTarget(W, H, 1)
    view = S.cornell_view(W, H)
    p = make_params(W, H, 1, max_depth=3, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
    with pytest.raises(CoreError):
        core.render_ex(view, p)
    core.SetMaterials(sc.materials)
    assert n > 1
    core.render_ex(view, p)
    assert core.read_accumulator()[:, :3].sum() > 0
    core.close()


@pytest.mark.parametrize("tail", [0, 5])
def test_connections_grouped_by_light_change_nothing(core_lib, tail):
    """Grouping each wave's connections by light before the any-hit queries (setting "sortConnections") reorders
    work only: accumulator and queue counts equal those of the ungrouped frame, bit for bit, also in filter frames."""
    sc = S.spheres_2m(seed=5, n_spheres=6, slices=40, stacks=26, tex_size=64)
    W, H = 160, 96
    view = S.spheres_view(W, H, frame=1)
    p = make_params(W, H, 2, max_depth=6, rr_start=3, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
    out = []
    for on in (0, 1, 2):        # off, by light over the whole queue, by light within chunks of the queue
        core = RenderCore()     # a core per setting: the filter's temporal history must start empty in both
        core.set_scene(sc)
        core.SetTarget(W, H, 2)
        core.Setting("waveTail", tail)
        core.Setting("sortConnections", on)
        c = core.render_ex(view, p, counters=True)["counters"].copy()
        acc = core.read_accumulator().copy()
        core.Setting("filter", 1)
        core.Render(view, converge=1)
        core.Render(S.spheres_view(W, H, frame=2), converge=1)
        out.append((c, acc, core.read_framebuffer().copy()))
        core.close()
    for k in (1, 2):
        assert np.array_equal(out[0][0], out[k][0])
        assert np.array_equal(out[0][1].view(np.uint32), out[k][1].view(np.uint32))
        assert np.array_equal(out[0][2].view(np.uint32), out[k][2].view(np.uint32))


@pytest.fixture(scope="module")
def spheres_small(core_lib, oracle_lib):
    sc = S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=64)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    return sc, core, o


@pytest.mark.parametrize("W,H,spp", [(1, 1, 1), (7, 5, 3), (33, 31, 1)])
def test_ragged_path_counts(spheres_small, W, H, spp):
    """Path counts that fill no whole tile of the shading partition (512 queue slots) nor a whole warp."""
    sc, core, o = spheres_small
    core.SetTarget(W, H, spp)
    view = S.spheres_view(W, H, frame=3)
    p = make_params(W, H, spp, max_depth=8, rr_start=4, camera_r0=camera_r0(2), flags=RP_NEE | RP_DEPTH_W)
    _check_frame(core, o, view, p)


def test_all_rays_miss(spheres_small):
    """A camera above the lights looking up: every primary ray misses, the waves after the first are empty and the
    frame is the sky alone."""
    sc, core, o = spheres_small
    W, H, spp = 37, 23, 3
    core.SetTarget(W, H, spp)
    view = S.make_view((0.0, 60.0, 0.0), (0.0, 200.0, 0.0), 40.0, W, H, up=(1.0, 0.0, 0.0))
    p = make_params(W, H, spp, max_depth=8, rr_start=4, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
    img = _check_frame(core, o, view, p)
    c = core.render_ex(view, p, counters=True)["counters"]
    assert c.sum() == 0, c.tolist()
    assert np.isfinite(img).all() and img[:, :3].min() > 0


@pytest.mark.parametrize("tail,mode", [(0, 1), (5, 1), (0, 2), (5, 2)])
def test_rays_grouped_by_octant_change_nothing(core_lib, oracle_lib, tail, mode):
    """Regrouping each bounce wave's extension rays by direction octant before the closest-hit queries (setting
    "sortRays": 1 over the whole queue, 2 within chunks of it) reorders work only: hit records, RNG states, queue
    counts and radiance equal the oracle's."""
    sc = S.spheres_2m(seed=5, n_spheres=6, slices=40, stacks=26, tex_size=64)
    W, H = 160, 96
    view = S.spheres_view(W, H, frame=1)
    p = make_params(W, H, 2, max_depth=7, rr_start=3, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
    core = RenderCore()
    core.set_scene(sc)
    core.SetTarget(W, H, 2)
    core.Setting("waveTail", tail)
    core.Setting("sortRays", mode)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    _check_frame(core, o, view, p)
    core.Setting("sortConnections", mode)   # both regroupings share the sort buffers
    _check_frame(core, o, view, p)
    core.close()


@pytest.mark.parametrize("rr,tail", [(64, 5), (20, 0), (64, 0)])
def test_deepest_paths(cornell, rr, tail):
    """maxDepth 64, the largest accepted: without Russian roulette most paths in the closed room live to the last
    path length, so every per-depth counter, the tail kernel's loop to depth 64 (waveTail 5) or 64 separate waves
    (waveTail 0), and the 64-deep capture buffers are used; hit records, seeds, counts and radiance equal the
    oracle's."""
    sc, core, o = cornell
    W, H, spp = 32, 24, 2
    core.SetTarget(W, H, spp)
    core.Setting("waveTail", tail)
    try:
        p = make_params(W, H, spp, max_depth=64, rr_start=rr, samples_taken=5, camera_r0=camera_r0(5), flags=RP_NEE | RP_DEPTH_W)
        _check_frame(core, o, S.cornell_view(W, H), p)
        assert core.GetCoreStats()["deviceStatus"] == 0
    finally:
        core.Setting("waveTail", 5)
