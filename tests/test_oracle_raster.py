"""The oracle's SoftRasterizer restatement (oracle/lh2o.cpp, lh2o_raster) against the reference core.

Golden vectors (tests/golden/raster_vectors.npz) come from lib/RenderCore_SoftRasterizer compiled for the host and
driven through its own RenderCore methods (tests/golden/make_golden_raster.py); the oracle must reproduce its pixels
and its z-buffer bit for bit. With LH2_REFERENCE set, the same comparison also runs live against the compiled core
at the full sizes of the rasterizer workloads (the closed room at 512 x 512, the 2M-triangle sphere field at
1920 x 1080)."""
import os

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from tests.golden.make_golden_raster import views, raster_scene

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "raster_vectors.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", list(views()))
def test_oracle_matches_reference_vectors(oracle_lib, golden, name):
    build, view, W, H = views()[name]
    o = oracle_lib.Oracle()
    o.set_scene(build())
    r = o.raster(view, W, H)
    assert np.array_equal(r["pixels"], golden[name + "/pixels"]), np.count_nonzero(r["pixels"] != golden[name + "/pixels"])
    assert np.array_equal(r["zbuffer"].view(np.uint32), golden[name + "/zbuffer"].view(np.uint32))


def test_cases_reach_the_branches(oracle_lib, golden):
    """The edge scene's views draw the textured quads (texture coordinates outside [0, 1]), clip at the near and left
    planes, and draw the shared-mesh instances at their last transform."""
    o = oracle_lib.Oracle()
    sc = raster_scene()
    o.set_scene(sc)
    _, view, W, H = views()["inside_80x60"]
    with_quads = o.raster(view, W, H)["pixels"]
    sc.instances = sc.instances[:2]
    o2 = oracle_lib.Oracle()
    o2.set_scene(sc)
    without = o2.raster(view, W, H)["pixels"]
    assert np.count_nonzero(with_quads != without) > 50
    assert np.count_nonzero(golden["inside_80x60/pixels"]) > 0.5 * W * H


def test_shared_mesh_takes_last_transform(oracle_lib):
    """Two instances of one mesh render at the transform set last (rendercore.cpp:118-131)."""
    sc = raster_scene()
    quad = sc.instances[2][0]
    a = oracle_lib.Oracle()
    a.set_scene(sc)
    _, view, W, H = views()["rolled_37x23"]
    both = a.raster(view, W, H)
    sc2 = raster_scene()
    sc2.instances = [inst for k, inst in enumerate(sc2.instances) if k != 2]   # only the last quad instance
    b = oracle_lib.Oracle()
    b.set_scene(sc2)
    assert sc2.instances[2][0] == quad
    assert np.array_equal(both["pixels"], b.raster(view, W, H)["pixels"])


@pytest.mark.skipif(not os.environ.get("LH2_REFERENCE"), reason="needs the reference tree (LH2_REFERENCE)")
@pytest.mark.parametrize("case", ["cornell_512", "spheres_1080p"])
def test_oracle_matches_reference_live_full_size(oracle_lib, case):
    from oracle import bind
    if case == "cornell_512":
        sc, view, W, H = S.cornell_sphere(subdiv=6), S.cornell_view(512, 512), 512, 512
    else:
        sc, view, W, H = S.spheres_2m(), S.spheres_view(1920, 1080, frame=0), 1920, 1080
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    a = o.raster(view, W, H)
    b = bind.RefRaster().raster(sc, view, W, H)
    assert np.array_equal(a["pixels"], b["pixels"])
    assert np.array_equal(a["zbuffer"].view(np.uint32), b["zbuffer"].view(np.uint32))
