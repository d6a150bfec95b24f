"""The oracle's OptiX 7 estimator and PrimeAdaptive frames against the reference's own kernels.

Golden vectors (tests/golden/make_golden_mis.py, committed) come from the OptiX 7 core's shading kernel and ray
generation and from the PrimeAdaptive core's kernels, compiled for the host from the reference tree and driven
through those cores' wave loops with the oracle answering the ray queries, on seeded synthetic blue-noise tables.
Per path length the extension and connection counts, the variance estimate's sample budget (devScale, second-wave
path count) and the features must match exactly; the blue-noise sampler bit for bit; radiance within 1e-5
relative (the reference adds a pixel's connections after its wave loop and lets the paths of a pixel race on the
accumulator; the oracle sums each path in the order it produces radiance, so only the rounding of the sums differs).
Where the reference tree is given (LH2_REFERENCE), the same comparisons run live on the reference's own blue-noise
tables."""
import ctypes as C
import os

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mis_vectors.npz")
REF = os.environ.get("LH2_REFERENCE", "")
live = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "lib", "RenderCore_PrimeAdaptive")),
                          reason="reference tree not given (LH2_REFERENCE)")


def _close(a, b, tol=1e-5):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-30)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def scene(oracle_lib):
    from tests.golden import make_golden_mis as G
    sc = G.scene()
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    return G, sc, o


def test_blue_noise_sampler(gold, oracle_lib):
    o = oracle_lib.Oracle()
    fn = o.lib.lh2o_bluenoise4
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    bn = oracle_lib.expand_blue_noise(S.synthetic_blue_noise(5))
    out = np.zeros(4, np.float32)
    for q, exp in zip(gold["bn_in"], gold["bn_out"]):
        fn(bn.ctypes.data_as(C.c_void_p), *map(int, q), out.ctypes.data_as(C.c_void_p))
        assert np.array_equal(out, exp), (q, out, exp)


def test_optix7_frames(gold, scene, oracle_lib):
    G, sc, o = scene
    B = oracle_lib
    for name, W, H, spp, D, st, shift in G.OPTIX7_FRAMES:
        p = B.make_params(W, H, spp, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st), flags=B.RP_NEE | B.RP_OPTIX7, shift=shift)
        r = o.render(S.cornell_view(W, H), p)
        assert np.array_equal(r["counters"], gold[name + "_counters"]), name
        assert _close(r["accum"], gold[name + "_accum"]), name


def test_adaptive_sequences(gold, scene, oracle_lib):
    G, sc, o = scene
    for name, W, H, spp, D, frames, ds in G.ADAPTIVE_SEQS:
        acc = np.zeros((W * H, 4), np.float32)
        for k in range(frames):
            r = o.render_adaptive(S.cornell_view(W, H), G.adaptive_params(W, H, spp, D, k), acc, ds)
            ds = r["dev_scale"]
            g = lambda key: gold[f"{name}_{k}_{key}"]
            assert np.array_equal(r["counters"], g("counters")), (name, k)
            assert np.float32(ds) == g("dev_scale") and r["adaptive_paths"] == int(g("adaptive_paths")), (name, k)
            assert np.array_equal(r["features"].view(np.uint32), g("features").view(np.uint32)), (name, k)
            assert _close(r["deviation"], g("deviation"), 1e-4), (name, k)
            assert _close(acc, g("accum")) and _close(r["frame"], g("frame")), (name, k)
        assert r["adaptive_paths"] > 0


@live
def test_live_optix7_on_reference_tables(oracle_lib):
    B = oracle_lib
    ref = B.RefOptix7()
    sc = S.cornell_sphere(subdiv=3)
    sc.blue_noise = B.reference_blue_noise()
    o = B.Oracle()
    o.set_scene(sc)
    for W, H, spp, D, st in ((48, 40, 1, 4, 0), (32, 24, 3, 6, 5), (24, 24, 1, 3, 63)):
        p = B.make_params(W, H, spp, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st), flags=B.RP_NEE | B.RP_OPTIX7, shift=0x91331445)
        a = o.render(S.cornell_view(W, H), p)
        r = ref.render(o, sc, S.cornell_view(W, H), p)
        assert not r["flushed"]
        assert np.array_equal(a["counters"], r["counters"])
        assert _close(a["accum"], r["accum"])


@live
def test_live_adaptive_on_reference_tables(oracle_lib):
    B = oracle_lib
    ref = B.RefAdaptive()
    sc = S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=64, sky_size=(256, 128))
    sc.blue_noise = B.reference_blue_noise()
    o = B.Oracle()
    o.set_scene(sc)
    from tests.golden import make_golden_mis as G
    W, H, spp, D = 48, 32, 1, 6
    acc_o, acc_r = np.zeros((W * H, 4), np.float32), np.zeros((W * H, 4), np.float32)
    ds_o = ds_r = 30.0
    for k in range(3):
        p = G.adaptive_params(W, H, spp, D, k)
        a = o.render_adaptive(S.spheres_view(W, H), p, acc_o, ds_o)
        r = ref.render(o, sc, S.spheres_view(W, H), p, acc_r, ds_r)
        ds_o, ds_r = a["dev_scale"], r["dev_scale"]
        assert not r["flushed"]
        assert np.array_equal(a["counters"], r["counters"]) and ds_o == ds_r and a["adaptive_paths"] == r["adaptive_paths"]
        assert np.array_equal(a["features"].view(np.uint32), r["features"].view(np.uint32))
        assert _close(acc_o, acc_r)


# ---- the Disney BSDF (LH2G_RP_DISNEY): the OptiX 7 kernel built with lib/sharedBSDFs/disney.h ----
DISNEY_GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "disney_vectors.npz")


def test_disney_frames(oracle_lib):
    """Frames of a room whose materials span the Disney parameters (metal with anisotropy, sheen, subsurface,
    clearcoat, rough dielectric, tinted specular) against the reference kernel built with disney.h."""
    from tests.golden import make_golden_disney as G
    B = oracle_lib
    gold = np.load(DISNEY_GOLD)
    sc = G.disney_scene()
    o = B.Oracle()
    o.set_scene(sc)
    for name, W, H, spp, D, st, shift in G.FRAMES:
        p = B.make_params(W, H, spp, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st), flags=B.RP_NEE | B.RP_OPTIX7 | B.RP_DISNEY,
                          shift=shift)
        r = o.render(S.cornell_view(W, H), p)
        assert np.array_equal(r["counters"], gold[name + "/counters"]), name
        assert _close(r["accum"], gold[name + "/accum"]), name
        lam = o.render(S.cornell_view(W, H), B.make_params(W, H, spp, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st),
                                                            flags=B.RP_NEE | B.RP_OPTIX7, shift=shift))
        assert not np.array_equal(lam["accum"], r["accum"])   # the BSDF matters on this scene


def test_own_log_and_pow():
    """The oracle's logf / powf (used by the GTR1 clearcoat distribution and sampler) against numpy in float64."""
    import ctypes as Cc
    from oracle import bind as B
    L = Cc.CDLL(B.LIB)
    L.lh2o_logf.restype, L.lh2o_logf.argtypes = Cc.c_float, [Cc.c_float]
    L.lh2o_powf.restype, L.lh2o_powf.argtypes = Cc.c_float, [Cc.c_float, Cc.c_float]
    rng = np.random.default_rng(4)
    xs = np.concatenate([rng.uniform(1e-6, 1.0, 3000), 10.0 ** rng.uniform(-37, 37, 3000)]).astype(np.float32)
    for x in xs:
        ref = np.log(np.float64(x))
        assert abs(L.lh2o_logf(float(x)) - ref) <= 2.5e-7 * max(abs(ref), 1e-3), x
    a, b = rng.uniform(1e-6, 0.999, 3000).astype(np.float32), rng.uniform(0.0, 1.0, 3000).astype(np.float32)
    for x, y in zip(a, b):
        ref = np.float64(x) ** np.float64(y)
        assert abs(L.lh2o_powf(float(x), float(y)) - ref) <= 1e-6 * ref, (x, y)
    assert L.lh2o_powf(0.0, 0.5) == 0.0 and L.lh2o_powf(0.3, 0.0) == 1.0


@live
def test_live_disney_frames(oracle_lib):
    B = oracle_lib
    from tests.golden import make_golden_disney as G
    ref = B.RefOptix7(disney=True)
    sc = G.disney_scene()
    o = B.Oracle()
    o.set_scene(sc)
    for W, H, spp, D, st in ((40, 32, 1, 5, 0), (32, 24, 2, 6, 66)):
        p = B.make_params(W, H, spp, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st), flags=B.RP_NEE | B.RP_OPTIX7 | B.RP_DISNEY,
                          shift=0x31337)
        a = o.render(S.cornell_view(W, H), p)
        r = ref.render(o, sc, S.cornell_view(W, H), p)
        assert not r["flushed"]
        assert np.array_equal(a["counters"], r["counters"])
        assert _close(a["accum"], r["accum"])
