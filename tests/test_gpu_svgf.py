"""SVGF on the GPU against the CPU oracle (whose filter chain is pinned bit for bit to the reference's own
kernels in test_oracle_svgf.py).

1. Filter-core frames (LH2G_RP_FILTER): per-path hits and RNG states, queue counts, the direct and indirect
   accumulator halves and the feature buffers (albedo / normal / depth / material, world position, depth
   derivatives) against the oracle.
2. Render with the "filter" setting over a moving camera path and a converging frame, TAA on and off: after every
   frame every filter buffer (features with history counts, world positions, motion, moments, packed light of the
   three a-trous passes, the TAA history) and the presented frame against the oracle, which renders and filters
   the same frame from the parameters the core reports for it. The host bookkeeping (Halton jitter, previous view,
   camera-stationary flag, sample count) is checked against the filter core's Render
   (lib/RenderCore_Optix7Filter/rendercore.cpp:737-797, 897-935).
Bit-exact equality is required throughout: the arithmetic is the same, operation by operation.
"""
import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300.core import RenderCore, make_params, RP_NEE, RP_DEPTH_W, RP_FILTER, FILTER_SLOTS

pytestmark = pytest.mark.gpu

HALTON = ([0.3, 0.7, 0.2, 0.8], [0.2, 0.8, 0.7, 0.3])


def xorshift(s):
    s ^= (s << 13) & 0xFFFFFFFF
    s ^= s >> 17
    s ^= (s << 5) & 0xFFFFFFFF
    return s


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def assert_same(name, got, exp):
    g, e = bits(got), bits(exp)
    bad = np.flatnonzero((g.reshape(len(g), -1) != e.reshape(len(e), -1)).any(axis=1))
    assert len(bad) == 0, f"{name}: {len(bad)} of {len(g)} pixels differ, first {bad[:6].tolist()}: {got[bad[0]]} vs {exp[bad[0]]}"


@pytest.fixture(scope="module")
def scene(core_lib, oracle_lib):
    sc = S.cornell_sphere(subdiv=4)
    core = RenderCore()
    core.set_scene(sc)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    return sc, core, o


@pytest.mark.parametrize("W,H,spp,depth", [(64, 48, 1, 4), (40, 32, 2, 6)])
def test_filter_frame_features_and_halves(scene, oracle_lib, W, H, spp, depth):
    sc, core, o = scene
    core.Setting("filter", 0)
    core.SetTarget(W, H, spp)
    view = S.cornell_view(W, H, frame=1)
    p = make_params(W, H, spp, max_depth=depth, rr_start=2, flags=RP_FILTER | RP_NEE | RP_DEPTH_W, frame_seed=0x9E3779B9)
    g = core.render_ex(view, p, accumulate=False, capture=True)
    st = oracle_lib.SvgfState(o, W, H)
    c = o.render(view, p, capture=True, features=st)
    assert np.array_equal(g["counters"], c["counters"])
    assert np.array_equal(g["hits"]["prim"], c["hits"]["prim"])
    assert np.array_equal(g["seeds"], c["seeds"])
    assert_same("accum (direct, indirect)", core.read_filter_buffer("accum"), c["accum"])
    for name in ("features", "worldPos", "deltaDepth"):
        assert_same(name, core.read_filter_buffer(name), st[name])
    acc = c["accum"].reshape(2, W * H, 4)
    assert acc[0, :, :3].sum() > 0 and acc[1, :, :3].sum() > 0      # both halves carry light
    spec = (st["features"][:, 3] >> 4) & 3
    assert (spec == 0).any() and (spec == 1).any()                   # diffuse and via-specular first vertices


@pytest.mark.parametrize("taa,W,H", [(1, 56, 40), (0, 56, 40), (1, 136, 104)])
def test_filtered_render_sequence(scene, oracle_lib, taa, W, H):
    """56 x 40: every block of the widest a-trous pass reaches past the image (clamped loads); 136 x 104: each pass
    has blocks whose tile lies inside the image as well, and partial blocks at the right edge."""
    sc, _, o = scene
    core = RenderCore()           # a fresh core: jitter cycle, previous jitter and camera seed start from their initial values
    core.set_scene(sc)
    core.SetTarget(W, H, 1)
    core.Setting("maxDepth", 5)
    core.Setting("rrStartDepth", 2)
    core.Setting("filter", 1)
    core.Setting("TAA", taa)
    st = oracle_lib.SvgfState(o, W, H)
    accum = None
    seed = 0x12345678
    prev_view, pj, samples = None, (0.0, 0.0), 0
    cycle = 0
    first_converging = True
    # (camera frame, converge: 1 = Restart); the first Converge frame after a Restart starts over as well
    plan = [(0, 1), (1, 1), (2, 1), (3, 1), (3, 0), (3, 0), (3, 0)]
    for k, (cam, restart) in enumerate(plan):
        view = S.cornell_view(W, H, frame=cam)
        core.Render(view, converge=restart)
        fp, jv, rp = core.last_filter_frame()
        # the filter core's bookkeeping (rendercore.cpp:744-750)
        if restart or first_converging:
            samples, first_converging, accum = 0, True, None
        if not restart:
            first_converging = False
        samples += 1
        j = (HALTON[0][cycle], HALTON[1][cycle]) if taa else (0.0, 0.0)
        cycle = (cycle + 1) & 3
        seed = xorshift(seed)
        assert (float(fp["j0"]), float(fp["j1"])) == (np.float32(j[0]), np.float32(j[1]))
        assert (float(fp["prevj0"]), float(fp["prevj1"])) == (np.float32(pj[0]), np.float32(pj[1]))
        assert int(fp["samplesTaken"]) == samples and int(rp["samplesTaken"]) == samples - 1
        assert int(fp["camIsStationary"]) == (0 if samples == 1 else 1) and int(fp["taa"]) == taa
        assert int(rp["frameSeed"]) == seed and int(rp["flags"]) & RP_FILTER
        assert float(jv["aperture"]) == 0
        expect_prev = prev_view if prev_view is not None else view
        for key in ("pos", "p1", "p2", "p3"):
            assert np.array_equal(fp["prevView"][key], expect_prev[key])
        # the oracle renders and filters the same frame
        if accum is None:
            accum = np.zeros((2 * W * H, 4), np.float32)
        accum = o.render(jv, rp, accum=accum, features=st)["accum"]
        st.frame(accum, fp)
        assert_same(f"frame {k} accum", core.read_filter_buffer("accum"), accum)
        for name in FILTER_SLOTS:
            if name != "accum":
                assert_same(f"frame {k} {name}", core.read_filter_buffer(name), st[name])
        fb = core.read_framebuffer()
        assert_same(f"frame {k} frame buffer", fb, st["target"])
        assert core.GetCoreStats()["deviceStatus"] == 0
        prev_view, pj = view, j
    img = core.read_framebuffer().reshape(H, W, 4)[1:-1, 1:-1, :3]
    assert np.isfinite(img).all() and img.mean() > 0.01
    assert (core.read_filter_buffer("features")[:, 3] & 15).max() >= 3     # history accumulated
    core.close()


def test_filter_requires_a_filter_frame(core_lib):
    """lh2g_filter before any filter-core frame on the target is a state error, not a crash."""
    core = RenderCore()
    sc = S.cornell_sphere(subdiv=2)
    core.set_scene(sc)
    core.SetTarget(16, 16, 1)
    import ctypes as C
    from lighthouse2_gb300.core import FILTER_PARAMS_DTYPE
    fp = np.zeros((), FILTER_PARAMS_DTYPE)
    fp["samplesTaken"] = 1
    rc = core.lib.lh2g_filter(core.ctx, fp.ctypes.data_as(C.c_void_p))
    assert rc == 4   # LH2G_ERR_STATE
    core.close()
