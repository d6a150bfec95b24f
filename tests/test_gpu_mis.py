"""The OptiX 7 estimator (LH2G_RP_OPTIX7) and PrimeAdaptive frames of the CUDA core against the oracle.

The oracle's restatement of these estimators is pinned to the reference's own kernels (tests/test_oracle_mis.py).
Here the GPU must match the oracle: per path and depth the hit record and the RNG state after shading bit-exact,
per path length the extension and connection counts exact, per-pixel radiance within 1e-4 relative (the
arithmetic and the summation order are the same, so it is expected to be identical); for adaptive frames also the
variance estimate's outcome (devScale, the second wave's path count, its counts per path length). Blue-noise tables
are seeded synthetic bytes (the reference's tables are the host's to upload)."""
import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300.core import RenderCore, make_params, camera_r0, RP_NEE, RP_OPTIX7

pytestmark = pytest.mark.gpu


def _alpha_holes(sc):
    """Cut holes into the first texture's alpha channel: shading then continues the ray behind the surface."""
    t = sc.textures[0]
    idx = np.arange(len(t.texels))
    t.texels = np.where(idx % 7 < 3, t.texels & np.uint32(0x00FFFFFF), t.texels).astype(np.uint32)
    return sc


SCENES = {
    "cornell": lambda: S.cornell_sphere(subdiv=4),
    "spheres": lambda: _alpha_holes(S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=64, sky_size=(256, 128))),
}


@pytest.fixture(scope="module", params=list(SCENES))
def pair(request, core_lib, oracle_lib):
    sc = SCENES[request.param]()
    sc.blue_noise = S.synthetic_blue_noise(11)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    view = S.cornell_view if request.param == "cornell" else (lambda W, H: S.spheres_view(W, H, frame=2))
    yield request.param, core, o, view
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
def test_optix7_frames(pair, W, H, spp, depth, st, tail):
    name, core, o, view = pair
    core.SetTarget(W, H, spp)
    core.Setting("waveTail", tail)
    try:
        p = make_params(W, H, spp, max_depth=depth, samples_taken=st, camera_r0=camera_r0(st), flags=RP_NEE | RP_OPTIX7, shift=0x91331445 + st)
        g = core.render_ex(view(W, H), p, capture=True)
        c = o.render(view(W, H), p, capture=True)
        _compare(g, c, core.read_accumulator(), c["accum"])
        assert core.read_accumulator()[:, 3].sum() > 0   # unoccluded connections counted in w
    finally:
        core.Setting("waveTail", 5)


@pytest.mark.parametrize("W,H,spp,depth,tail", [(48, 40, 1, 5, 5), (32, 24, 2, 6, 0)])
def test_adaptive_sequence(pair, W, H, spp, depth, tail):
    name, core, o, view = pair
    from tests.golden.make_golden_mis import adaptive_params
    core.SetTarget(W, H, spp)
    core.Setting("waveTail", tail)
    core.set_adaptive_scale(30.0)
    acc = np.zeros((W * H, 4), np.float32)
    ds = 30.0
    try:
        for k in range(3):
            p = adaptive_params(W, H, spp, depth, k)
            g = core.render_adaptive(view(W, H), p, accumulate=k > 0, capture=True)
            c = o.render_adaptive(view(W, H), p, acc, ds, capture=True)
            ds = c["dev_scale"]
            assert g["dev_scale"] == np.float32(ds) and g["adaptive_paths"] == c["adaptive_paths"], (k, g["dev_scale"], ds)
            _compare(g, {"counters": c["counters"], "hits": c["hits"], "seeds": c["seeds"]}, core.read_accumulator(), acc)
            assert np.allclose(core.read_framebuffer(), c["frame"], rtol=1e-4, atol=1e-7)
        assert g["adaptive_paths"] > 0
    finally:
        core.Setting("waveTail", 5)


def test_render_api_estimators(core_lib, oracle_lib):
    """Render with the settings "estimator" 1 and "adaptive" 1 follows the cores' seed bookkeeping
    (rendercore_optix7/rendercore.cpp:855,900; RenderCore_PrimeAdaptive/rendercore.cpp:606-609,749-755)."""
    sc = S.cornell_sphere(subdiv=3)
    sc.blue_noise = S.synthetic_blue_noise(3)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    W, H, D = 40, 32, 4
    core.SetTarget(W, H, 1)
    core.Setting("maxDepth", D)
    view = S.cornell_view(W, H)

    seeds = [0x12345678, 0x11331445]   # camRNGseed (reset by Restart), shiftSeed (never reset)

    def nxt(i):
        x = seeds[i]
        x ^= (x << 13) & 0xFFFFFFFF
        x ^= x >> 17
        x ^= (x << 5) & 0xFFFFFFFF
        seeds[i] = x
        return x

    state = {"first": True, "st": 0}

    def restart_logic(converge):   # RenderCore::Render (rendercore.cpp:535-550 in every core)
        if converge == 1 or state["first"]:
            state["st"], state["first"], seeds[0] = 0, True, 0x12345678
        if converge == 0:
            state["first"] = False
        return state["st"]

    core.Setting("estimator", 1)
    acc = None
    for conv in (1, 0, 0):
        core.Render(view, converge=conv)
        st = restart_logic(conv)
        shift, r0 = nxt(1), nxt(0)
        for _ in range(D - 1):
            nxt(0)
        p = make_params(W, H, 1, max_depth=D, samples_taken=st, camera_r0=r0, flags=RP_NEE | RP_OPTIX7, shift=shift)
        acc = o.render(view, p, accum=acc if st > 0 else None)["accum"]
        state["st"] += 1
    assert np.allclose(core.read_accumulator(), acc, rtol=1e-4, atol=1e-7)
    core.Setting("estimator", 0)
    core.Setting("adaptive", 1)
    ds = 10.0
    for conv in (1, 0, 0):
        core.Render(view, converge=conv)
        st = restart_logic(conv)
        shift, r0, r1 = nxt(1), nxt(0), nxt(0)
        if st == 0:
            acc = np.zeros((W * H, 4), np.float32)
        p = make_params(W, H, 1, max_depth=D, samples_taken=st, camera_r0=r0, frame_seed=r1, flags=RP_NEE, shift=shift)
        ds = o.render_adaptive(view, p, acc, ds)["dev_scale"]
        state["st"] += 1
    assert np.allclose(core.read_accumulator(), acc, rtol=1e-4, atol=1e-7)
    stats = core.GetCoreStats()
    assert stats["primaryRayCount"] >= W * H
    core.close()


# ---- the Disney BSDF (LH2G_RP_DISNEY), pinned in the oracle against the reference kernel built with disney.h ----
@pytest.fixture(scope="module")
def disney_pair(core_lib, oracle_lib):
    from tests.golden.make_golden_disney import disney_scene
    sc = disney_scene()
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    yield core, o
    core.close()


@pytest.mark.parametrize("W,H,spp,depth,st,tail", [(64, 48, 1, 5, 0, 5), (40, 32, 2, 6, 3, 0), (48, 40, 1, 8, 70, 2)])
def test_disney_frames(disney_pair, W, H, spp, depth, st, tail):
    from lighthouse2_gb300.core import RP_DISNEY
    core, o = disney_pair
    core.SetTarget(W, H, spp)
    core.Setting("waveTail", tail)
    try:
        p = make_params(W, H, spp, max_depth=depth, samples_taken=st, camera_r0=camera_r0(st), flags=RP_NEE | RP_OPTIX7 | RP_DISNEY,
                        shift=0x91331445 + st)
        g = core.render_ex(S.cornell_view(W, H), p, capture=True)
        c = o.render(S.cornell_view(W, H), p, capture=True)
        _compare(g, c, core.read_accumulator(), c["accum"])
    finally:
        core.Setting("waveTail", 5)


def test_disney_adaptive_and_render_api(disney_pair, oracle_lib):
    """Adaptive frames with the Disney BSDF, and Render with the settings "adaptive" 1 / "estimator" 1 and "bsdf" 1."""
    from lighthouse2_gb300.core import RP_DISNEY
    from tests.golden.make_golden_mis import adaptive_params
    core, o = disney_pair
    W, H, spp, depth = 40, 32, 1, 5
    core.SetTarget(W, H, spp)
    core.set_adaptive_scale(30.0)
    acc = np.zeros((W * H, 4), np.float32)
    ds = 30.0
    for k in range(2):
        p = adaptive_params(W, H, spp, depth, k)
        p["flags"] = int(p["flags"]) | RP_DISNEY
        g = core.render_adaptive(S.cornell_view(W, H), p, accumulate=k > 0, capture=True)
        c = o.render_adaptive(S.cornell_view(W, H), p, acc, ds, capture=True)
        ds = c["dev_scale"]
        assert g["dev_scale"] == np.float32(ds) and g["adaptive_paths"] == c["adaptive_paths"]
        _compare(g, {"counters": c["counters"], "hits": c["hits"], "seeds": c["seeds"]}, core.read_accumulator(), acc)
    # the plugin-level switch: estimator 1 + bsdf 1 renders the same frame as render_ex with the flags
    core.Setting("maxDepth", depth)
    core.Setting("estimator", 1)
    core.Setting("bsdf", 1)
    try:
        core.Render(S.cornell_view(W, H), converge=1)
        seeds = [0x12345678, 0x11331445]

        def nxt(i):
            x = seeds[i]
            x ^= (x << 13) & 0xFFFFFFFF
            x ^= x >> 17
            x ^= (x << 5) & 0xFFFFFFFF
            seeds[i] = x
            return x
        shift, r0 = nxt(1), nxt(0)
        p = make_params(W, H, spp, max_depth=depth, samples_taken=0, camera_r0=r0, flags=RP_NEE | RP_OPTIX7 | RP_DISNEY, shift=shift)
        ref = o.render(S.cornell_view(W, H), p)["accum"]
        assert np.allclose(core.read_accumulator(), ref, rtol=1e-4, atol=1e-7)
    finally:
        core.Setting("estimator", 0)
        core.Setting("bsdf", 0)
    with pytest.raises(Exception):   # the Disney BSDF belongs to the OptiX 7 / adaptive estimators
        core.render_ex(S.cornell_view(W, H), make_params(W, H, spp, max_depth=depth, flags=RP_NEE | RP_DISNEY))
