"""Radiance-cache frames (lh2g_render_nrc) against the plain estimator, both measured against a converged plain render.

The plain estimator (1 spp per frame, accumulated) and the cache estimator (paths end into the cache at their first
diffuse-led vertex from path length 2 on, 1 in 16 trace on and train it online) render the Cornell scene at
512 x 512. After the cache has
been trained for some frames, each gets the same device time (frame counts from measured frame times); the
cached image must have a clearly lower RMSE against a 1024-spp plain render accumulated in FP64. Frames of the
cache estimator must also report their queries and training samples, and with a cache that predicts zero they
must be darker than the plain image (the cache supplies the radiance of the cut paths)."""
import time

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300.core import RenderCore, make_params, camera_r0, RP_NEE, RP_DEPTH_W
from lighthouse2_gb300.nrc import RadianceCache, MLP_PARAMS

pytestmark = pytest.mark.gpu

W = H = 512


def params(k, spp=1):
    return make_params(W, H, spp, max_depth=8, rr_start=4, samples_taken=k, camera_r0=camera_r0(k), flags=RP_NEE | RP_DEPTH_W)


@pytest.fixture(scope="module")
def setup(core_lib):
    sc = S.cornell_sphere(subdiv=5)
    core = RenderCore()
    core.set_scene(sc)
    view = S.cornell_view(W, H)
    core.SetTarget(W, H, 16)
    ref = np.zeros((W * H, 3), np.float64)
    for k in range(64):
        p = params(16 * k, 16)
        p["cameraR0"] = (0x9E3779B9 * (k + 7)) & 0xFFFFFFFF
        core.render_ex(view, p, accumulate=False, counters=False)
        ref += core.read_accumulator()[:, :3]
    core.SetTarget(W, H, 1)
    return sc, core, view, ref / 1024.0


def frame_time(fn, n=12):
    for k in range(3):
        fn(k)
    t = time.perf_counter()
    for k in range(n):
        fn(k)
    return (time.perf_counter() - t) / n


def test_cache_frames_beat_plain_at_equal_time(setup):
    sc, core, view, ref = setup
    cache = RadianceCache(sc.bounds[0], sc.bounds[1], learning_rate=1e-2, seed=5)
    # a cache that predicts zero: the cut paths lose their radiance
    cache.set_params(np.zeros(MLP_PARAMS, np.float32))
    q, n, _ = core.render_nrc(cache, view, params(0), train=False)
    dark = core.read_accumulator()[:, :3].mean()
    core.render_ex(view, params(0), counters=False)
    assert q > 0.5 * W * H and n > 0 and dark < 0.8 * core.read_accumulator()[:, :3].mean()
    cache.close()
    cache = RadianceCache(sc.bounds[0], sc.bounds[1], learning_rate=1e-2, seed=5)
    losses = [core.render_nrc(cache, view, params(100000 + k))[2] for k in range(150)]
    assert np.isfinite(losses).all() and np.mean(losses[-10:]) < np.mean(losses[:10])

    def plain(k):
        core.render_ex(view, params(k), accumulate=k > 0, counters=False)
        core.WaitForRender()

    def cached(k):
        core.render_nrc(cache, view, params(k), accumulate=k > 0)
        core.WaitForRender()

    t_plain, t_cache = frame_time(plain), frame_time(cached)
    n_plain = 24
    n_cache = max(1, int(round(n_plain * t_plain / t_cache)))
    for k in range(n_plain):
        plain(k)
    img_plain = core.read_accumulator()[:, :3] / n_plain
    for k in range(n_cache):
        cached(k)
    img_cache = core.read_accumulator()[:, :3] / n_cache
    rmse_plain = np.sqrt(np.mean((img_plain - ref) ** 2))
    rmse_cache = np.sqrt(np.mean((img_cache - ref) ** 2))
    assert rmse_cache < 0.85 * rmse_plain, (rmse_plain, rmse_cache, t_plain, t_cache, n_cache)
    cache.close()


def test_queued_cache_frames_match_waiting_ones(setup):
    """Cache frames queued without waiting (stats=None: they overlap on the core's lanes, their cache work chained
    in submission order) give what frames that wait for the device give: the first frame (initial weights) bit for
    bit, later ones within the run-to-run noise of the gradient atomics."""
    sc, core, view, ref = setup
    out = []
    for stats in (True, False):
        cache = RadianceCache(sc.bounds[0], sc.bounds[1], learning_rate=1e-2, seed=9)
        core.render_nrc(cache, view, params(300), stats=stats)
        core.WaitForRender()
        first = core.read_accumulator().copy()
        for k in range(1, 8):
            core.render_nrc(cache, view, params(300 + k), accumulate=True, stats=stats)
        core.WaitForRender()
        out.append((first, core.read_accumulator().copy(), cache.params()[0].copy()))
        cache.close()
    (f0, a0, w0), (f1, a1, w1) = out
    assert np.array_equal(f0.view(np.uint32), f1.view(np.uint32))
    assert np.sqrt(np.mean((a0 - a1) ** 2)) <= 1e-3 * np.sqrt(np.mean(a0 ** 2))
    assert np.linalg.norm(w0 - w1) <= 1e-3 * np.linalg.norm(w0)
