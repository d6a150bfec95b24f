"""The CUDA SoftRasterizer (lh2g_raster_render, csrc/raster.cu) against the oracle and the reference's vectors.

The oracle (oracle/lh2o.cpp, lh2o_raster) is pinned bit for bit to lib/RenderCore_SoftRasterizer compiled for the
host (tests/test_oracle_raster.py). The GPU must give the same pixels and the same z-buffer bit for bit: on the
fixture cases, on the closed room at 512 x 512 and on the 2M-triangle sphere field at 1920 x 1080 (two poses),
whose 1 spp path-tracing frames are the path tracer's workloads."""
import os

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300.core import RenderCore
from tests.golden.make_golden_raster import views, raster_scene

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "raster_vectors.npz")


def _core(sc):
    core = RenderCore()
    core.set_scene(sc)
    return core


def _same(g, ref_px, ref_z):
    assert np.array_equal(g["pixels"], ref_px), f"{np.count_nonzero(g['pixels'] != ref_px)} pixels differ"
    assert np.array_equal(g["zbuffer"].view(np.uint32), ref_z.view(np.uint32)), "z-buffer differs"


@pytest.mark.parametrize("name", list(views()))
def test_raster_matches_reference_vectors(core_lib, name):
    gold = np.load(GOLDEN)
    build, view, W, H = views()[name]
    core = _core(build())
    core.SetTarget(W, H, 1)
    g = core.raster(view, depth=True, stats=True)
    _same(g, gold[name + "/pixels"], gold[name + "/zbuffer"])
    assert g["stats"]["status"] == 0
    core.close()


@pytest.mark.parametrize("case", ["cornell_512", "spheres_1080p_pose0", "spheres_1080p_pose5"])
def test_raster_full_size(core_lib, oracle_lib, case):
    if case == "cornell_512":
        sc, view, W, H = S.cornell_sphere(subdiv=6), S.cornell_view(512, 512), 512, 512
    else:
        sc, W, H = S.spheres_2m(), 1920, 1080
        view = S.spheres_view(W, H, frame=int(case[-1]))
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    ref = o.raster(view, W, H)
    core = _core(sc)
    core.SetTarget(W, H, 1)
    g = core.raster(view, depth=True, stats=True)
    _same(g, ref["pixels"], ref["zbuffer"])
    st = g["stats"]
    assert st["status"] == 0 and st["triangles"] > 0 and st["fragments"] >= np.count_nonzero(ref["pixels"])
    if case == "cornell_512":
        assert st["bigTriangles"] > 0   # the room's walls take the block path
    # a second frame from the same state is identical (device-side lists and counters are reset per frame)
    g2 = core.raster(view, depth=True)
    _same(g2, ref["pixels"], ref["zbuffer"])
    core.close()


def test_raster_after_instance_update(core_lib, oracle_lib):
    """Moving an instance between frames (SetInstance on an existing index) changes the next frame as the oracle's."""
    sc = raster_scene()
    _, view, W, H = views()["inside_80x60"]
    core = _core(sc)
    core.SetTarget(W, H, 1)
    core.raster(view)
    T = np.array(sc.instances[3][1], np.float32).copy()
    T[0, 3] += 0.15
    sc.instances[3] = (sc.instances[3][0], T)
    core.SetInstance(3, sc.instances[3][0], T)
    g = core.raster(view, depth=True)
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    ref = o.raster(view, W, H)
    _same(g, ref["pixels"], ref["zbuffer"])
    core.close()


def test_raster_device_image_and_rejects(core_lib):
    sc = S.cornell_sphere(subdiv=2)
    core = _core(sc)
    core.SetTarget(2, 2, 1)
    with pytest.raises(RuntimeError):
        core.raster(S.cornell_view(2, 2))
    assert not core.raster_pixels_device()
    core.SetTarget(32, 24, 1)
    core.raster(S.cornell_view(32, 24), pixels=False)
    assert core.raster_pixels_device()
    core.close()
