"""The radiance cache's CPU restatement (oracle/lh2o.cpp): its gradients against finite differences, and the
encoding's structure. The GPU kernels are checked against this oracle (tests/test_gpu_nrc.py)."""
import numpy as np
import pytest

from lighthouse2_gb300.nrc import grid_spec, GRID_PARAMS, MLP_PARAMS
from oracle import bind as OB

SCENE_MIN, SCENE_MAX = (-1.0, 0.0, -1.0), (1.0, 2.0, 1.0)


def random_queries(n, seed):
    rng = np.random.default_rng(seed)
    q = np.zeros((n, 16), np.float32)
    q[:, 0:3] = rng.uniform(SCENE_MIN, SCENE_MAX, (n, 3))
    q[:, 3] = rng.uniform(0, 1, n)
    d = rng.normal(size=(n, 3))
    q[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    m = rng.normal(size=(n, 3))
    q[:, 8:11] = m / np.linalg.norm(m, axis=1, keepdims=True)
    q[:, 12:15] = rng.uniform(0, 1, (n, 3))
    return q


def random_params(seed, grid_scale=0.3):
    rng = np.random.default_rng(seed)
    mlp = np.zeros(MLP_PARAMS, np.float32)
    for l in range(5):
        rows = 64 if l < 4 else 3
        mlp[l * 4096:l * 4096 + rows * 64] = rng.uniform(-1, 1, rows * 64) * np.sqrt(6.0 / (64 + rows))
    grid = (rng.uniform(-1, 1, GRID_PARAMS) * grid_scale).astype(np.float32)
    return mlp, grid


@pytest.fixture(scope="module")
def oracle(oracle_lib):
    return OB.NrcOracle(*grid_spec(SCENE_MIN, SCENE_MAX))


def test_encoding_structure(oracle):
    mlp, grid = random_params(1)
    for q in random_queries(20, 2):
        e = oracle.encode(grid, q)
        assert np.isfinite(e).all()
        for a, b in ((24, 28), (28, 32), (32, 36), (36, 40), (40, 44)):
            assert 0.49 <= e[a:b].sum() <= 1.0 + 1e-6 and (e[a:b] >= 0).all()   # one-blob: at most two bins, triangular
        assert np.array_equal(e[44:47], q[12:15]) and e[47] == 1.0 and not e[48:].any()
        assert np.abs(e[:24]).max() <= np.abs(grid).max() * 1.001            # trilinear mix of grid features


def surrogate_loss(oracle, grid, mlp, q, t, den):
    y = oracle.forward64(grid, mlp, q)
    return float((((y - t[:, :3]) ** 2) / den).sum() / (3 * len(q)))


def test_gradients_match_finite_differences(oracle):
    """The relative L2 loss holds y constant in its denominator; the finite differences do the same."""
    mlp, grid = random_params(3)
    q = random_queries(6, 4)
    t = np.zeros((6, 4), np.float32)
    t[:, :3] = np.random.default_rng(5).uniform(0, 1, (6, 3))
    gm, gg, loss = oracle.gradients(grid, mlp, q, t, emulate=False)
    y0 = oracle.forward64(grid, mlp, q)
    den = y0 * y0 + 0.01
    assert abs(surrogate_loss(oracle, grid, mlp, q, t, den) - loss) <= 1e-6 * max(1.0, loss)
    rng = np.random.default_rng(6)

    def fd_mlp(i, h):
        mp, mm = mlp.copy(), mlp.copy()
        mp[i] += h
        mm[i] -= h
        return (surrogate_loss(oracle, grid, mp, q, t, den) - surrogate_loss(oracle, grid, mm, q, t, den)) / (float(mp[i]) - float(mm[i]))

    checked = kinks = 0
    for l in range(5):
        rows = 64 if l < 4 else 3
        for idx in rng.integers(0, rows * 64, 8):
            i = l * 4096 + int(idx)
            h = max(2e-3, 1e-2 * abs(float(mlp[i])))
            fd, fd2 = fd_mlp(i, h), fd_mlp(i, h / 2)
            if abs(fd - fd2) > 2e-2 * max(abs(fd), abs(fd2)) + 1e-9:
                kinks += 1   # a ReLU changes state within the step: the difference quotient is not the derivative
                continue
            if abs(gm[i]) > 1e-7 or abs(fd) > 1e-7:
                assert abs(fd - gm[i]) <= 2e-2 * max(abs(gm[i]), abs(fd)) + 1e-9, (l, i, fd, gm[i])
                checked += 1
    assert kinks <= 10
    def fd_grid(i, h):
        gp, gq = grid.copy(), grid.copy()
        gp[i] += h
        gq[i] -= h
        return (surrogate_loss(oracle, gp, mlp, q, t, den) - surrogate_loss(oracle, gq, mlp, q, t, den)) / (float(gp[i]) - float(gq[i]))

    largest = np.argsort(-np.abs(gg))[:60]   # grid entries the samples depend on most
    for i in rng.choice(largest, 16, replace=False):
        fd, fd2 = fd_grid(i, 1e-2), fd_grid(i, 5e-3)
        if abs(fd - fd2) > 2e-2 * max(abs(fd), abs(fd2)) + 1e-9:
            kinks += 1
            continue
        assert abs(fd - gg[i]) <= 3e-2 * max(abs(gg[i]), abs(fd)) + 1e-9, (i, fd, gg[i])
        checked += 1
    assert checked >= 30 and kinks <= 14
