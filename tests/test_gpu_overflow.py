"""Traversal that runs out of stack reports it.

A variant of the core built with a 3-entry traversal stack (-DLH2G_STACK=3, or 2 group entries, -DLH2G_GSTACK=2, in
its own build directory) cannot
hold the pending children of a two-level traversal through 66 instances (a node a ray crosses often has four or more
hit children, and entering an instance takes a slot for the return marker), so it drops work; every place where a
push is refused (sorted children, an instance leaf's remaining instances, the entry into an instance) sets the
stack-overflow bit of the status word, and the C ABI turns the word into LH2G_ERR_OVERFLOW. No call may return
a truncated traversal as a success. The default build traces the same rays without an error."""
import os

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_stack_lib(core_lib):
    from lighthouse2_gb300 import build
    return build.build(out_dir=os.path.join(build.OUT, "stack3"), defines=["-DLH2G_STACK=3", "-DLH2G_GSTACK=2"])


def _field_rays(scene, n, seed=3):
    """Rays from the camera position towards random points among the spheres: every one crosses the field."""
    rng = np.random.default_rng(seed)
    view = S.spheres_view(64, 48)
    rays = np.zeros(n, S.RAY_DTYPE)
    rays["o"] = view["pos"]
    target = rng.uniform((-40.0, 0.0, -40.0), (40.0, 8.0, 40.0), (n, 3))
    d = target - view["pos"].astype(np.float64)
    rays["d"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"], rays["tmax"] = 0.0, 1e30
    return rays


@pytest.fixture(scope="module")
def scene():
    return S.spheres_2m(slices=24, stacks=16, tex_size=32)


def test_small_stack_reports_overflow(small_stack_lib, scene):
    from lighthouse2_gb300.core import RenderCore, CoreError, make_params, camera_r0, RP_NEE
    core = RenderCore(0, lib_path=small_stack_lib)
    core.set_scene(scene)
    W, H = 64, 48
    core.SetTarget(W, H, 1)
    p = make_params(W, H, 1, max_depth=4, camera_r0=camera_r0(0), flags=RP_NEE)
    with pytest.raises(CoreError, match="overflow"):
        core.render_ex(S.spheres_view(W, H), p, counters=True)
    assert core.GetCoreStats()["deviceStatus"] & 1
    rays = _field_rays(scene, 100_000)
    for mode in (0, 1):
        with pytest.raises(CoreError, match="overflow"):
            core.trace_host(rays, mode=mode)
    core.close()


def test_default_stack_traces_the_same_rays(core_lib, scene, oracle_lib):
    from lighthouse2_gb300.core import RenderCore
    core = RenderCore(0)
    core.set_scene(scene)
    rays = _field_rays(scene, 100_000)
    g = core.trace_host(rays, mode=0)
    o = oracle_lib.Oracle()
    o.set_scene(scene)
    c = o.trace(rays, mode=0)
    assert np.array_equal(g["prim"], c["prim"]) and np.array_equal(g["inst"], c["inst"])
    core.close()
