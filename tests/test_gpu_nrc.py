"""The radiance cache on the GPU (tcgen05 tensor-core MLP, hash grid, Adam) against the CPU oracle.

Inference and the gradients of the relative L2 loss are compared with the oracle's restatement under the same
rounding points (fp16 grid features, bf16 weights, activations and loss gradients); the tensor cores sum in
fp32 in their own order and an activation can round to the neighbouring bf16 value, hence the tolerances below.
The Adam step must equal the oracle's bit for bit given the same gradients. Training on a synthetic radiance
field must reduce the loss and the prediction error on held-out queries."""
import numpy as np
import pytest

from lighthouse2_gb300.nrc import RadianceCache, grid_spec
from oracle import bind as OB
from tests.test_oracle_nrc import SCENE_MIN, SCENE_MAX, random_queries, random_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair(core_lib, oracle_lib):
    cache = RadianceCache(SCENE_MIN, SCENE_MAX, learning_rate=1e-2, seed=7)
    res, dense, bi = cache.spec()
    ref = grid_spec(SCENE_MIN, SCENE_MAX)
    assert list(res) == ref[0] and list(dense) == ref[1]
    return cache, OB.NrcOracle(list(res), list(dense), list(bi[:3]), list(bi[3:]))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) / max(np.linalg.norm(np.asarray(b, np.float64)), 1e-30))


def test_inference_matches_oracle(pair):
    cache, o = pair
    mlp, grid = random_params(11)
    cache.set_params(mlp, grid)
    q = random_queries(3000, 12)          # 23 full tiles and a partial one
    got = cache.infer(q)
    exp = o.forward(grid, mlp, q, emulate=True)
    assert np.isfinite(got).all() and np.abs(exp[:, :3]).max() > 0.05
    assert rel(got[:, :3], exp[:, :3]) <= 1e-2, rel(got[:, :3], exp[:, :3])
    assert np.percentile(np.abs(got[:, :3] - exp[:, :3]), 99) <= 1e-2 * np.abs(exp[:, :3]).max()
    assert not got[:, 3].any()


def test_gradients_and_adam_match_oracle(pair):
    cache, o = pair
    mlp, grid = random_params(13)
    cache.set_params(mlp, grid)
    q = random_queries(2000, 14)
    t = np.zeros((2000, 4), np.float32)
    t[:, :3] = np.random.default_rng(15).uniform(0, 1, (2000, 3))
    loss = cache.train(q, t, update=False)
    gm, gg = cache.grads()
    em, eg, eloss = o.gradients(grid, mlp, q, t, emulate=True)
    assert abs(loss - eloss) <= 2e-3 * eloss, (loss, eloss)
    for l in range(5):
        rows = 64 if l < 4 else 3
        sl = slice(l * 4096, l * 4096 + rows * 64)
        assert rel(gm[sl], em[sl]) <= 3e-2, (l, rel(gm[sl], em[sl]))
    touched = np.flatnonzero(eg)
    assert len(touched) > 1000 and rel(gg[touched], eg[touched]) <= 3e-2, rel(gg[touched], eg[touched])
    assert not gg[np.setdiff1d(np.arange(0, len(gg), 997), touched)].any()
    # one Adam step on exactly these gradients
    cache.apply_update()
    pm, pg = cache.params()
    for p0, g in ((mlp, gm), (grid, gg)):
        p, m, v = p0.copy(), np.zeros_like(p0), np.zeros_like(p0)
        o.adam(p, m, v, np.ascontiguousarray(g, np.float32), 1e-2, 1)
        got = pm if p0 is mlp else pg
        assert np.array_equal(got.view(np.uint32), p.view(np.uint32))


def synthetic_targets(q):
    """a smooth radiance field of position, direction and albedo"""
    x, y, z = q[:, 0], q[:, 1], q[:, 2]
    s = 0.5 + 0.4 * np.sin(3.0 * x) * np.cos(2.0 * y) + 0.2 * z
    d = 0.5 * (q[:, 6] + 1.0)
    t = np.zeros((len(q), 4), np.float32)
    t[:, :3] = (s * (0.5 + 0.5 * d))[:, None] * q[:, 12:15]
    return t


def test_training_reduces_error(pair):
    cache, o = pair
    cache2 = RadianceCache(SCENE_MIN, SCENE_MAX, learning_rate=1e-2, seed=21)
    held = random_queries(4096, 99)
    ht = synthetic_targets(held)
    err0 = np.sqrt(np.mean((cache2.infer(held)[:, :3] - ht[:, :3]) ** 2))
    losses = []
    for step in range(300):
        q = random_queries(8192, 1000 + step)
        losses.append(cache2.train(q, synthetic_targets(q)))
    err1 = np.sqrt(np.mean((cache2.infer(held)[:, :3] - ht[:, :3]) ** 2))
    assert np.isfinite(losses).all()
    assert np.mean(losses[-20:]) < 0.2 * np.mean(losses[:5]), (losses[:5], losses[-5:])
    assert err1 < 0.3 * err0, (err0, err1)
    cache2.close()


def test_bounded_wait_reports_timeout_and_device_stays_usable(pair):
    """A tensor-core completion wait that never completes gives up after its poll limit and raises the error word
    (no hang, no trap); the cache keeps working afterwards."""
    import ctypes as C
    cache, o = pair
    lib = cache.lib
    lib.lh2g_nrc_wait_selftest.argtypes = [C.c_int, C.c_uint32, C.POINTER(C.c_uint32)]
    status = C.c_uint32(0)
    assert lib.lh2g_nrc_wait_selftest(0, 64, C.byref(status)) == 0
    assert status.value == 1
    mlp, grid = random_params(21)
    cache.set_params(mlp, grid)
    q = random_queries(256, 22)
    got = cache.infer(q)
    exp = o.forward(grid, mlp, q, emulate=True)
    assert rel(got[:, :3], exp[:, :3]) <= 1e-2
