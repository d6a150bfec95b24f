"""Bands of rows rendered apart on the GPU equal the frame rendered whole, bit for bit.

lighthouse2_gb300.sharding splits a frame's rows over ranks; each rank's core renders its band (lh2g_render_params
rowBegin / rowCount, the paths keeping their whole-frame seeds). On one GPU the ranks' bands are rendered one after
the other by one core each, then put together; the result must equal the whole frame of the same core and of the
oracle. (The multi-rank gather itself is covered on the CPU by tests/test_sharding.py.)"""
import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300 import sharding
from lighthouse2_gb300.core import RenderCore, make_params, camera_r0, RP_NEE, RP_DEPTH_W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,spp,world", [(96, 61, 1, 2), (64, 40, 3, 3), (160, 90, 1, 8)])
def test_bands_equal_whole_frame(core_lib, oracle_lib, W, H, spp, world):
    sc = S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=64)
    view = S.spheres_view(W, H, frame=4)
    p = make_params(W, H, spp, max_depth=8, rr_start=4, camera_r0=camera_r0(2), flags=RP_NEE | RP_DEPTH_W)
    whole = RenderCore()
    whole.set_scene(sc)
    whole.SetTarget(W, H, spp)
    whole.render_ex(view, p, counters=False)
    ref = whole.read_accumulator()
    whole.close()
    frame = np.zeros((W * H, 4), np.float32)
    for rank in range(world):
        core = RenderCore()
        core.set_scene(sc)
        band = sharding.render_band(core, view, p, rank, world)
        begin, count = sharding.row_bands(H, world)[rank]
        frame[begin * W:(begin + count) * W] = band
        core.close()
    assert np.array_equal(frame.view(np.uint32), ref.view(np.uint32))
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    assert np.allclose(frame, o.render(view, p)["accum"], rtol=1e-4, atol=0)


def test_band_parameters_are_checked(core_lib):
    from lighthouse2_gb300.core import CoreError, RP_OPTIX7
    sc = S.cornell_sphere(subdiv=2)
    core = RenderCore()
    core.set_scene(sc)
    W, H = 32, 24
    core.SetTarget(W, 10, 1)
    p = make_params(W, H, 1, max_depth=3, camera_r0=camera_r0(0), flags=RP_NEE)
    p["rowBegin"], p["rowCount"] = 20, 10           # runs past the frame
    with pytest.raises(CoreError):
        core.render_ex(S.cornell_view(W, H), p)
    p["rowBegin"], p["flags"] = 5, RP_NEE | RP_OPTIX7   # the band is PrimeRef-only
    with pytest.raises(CoreError):
        core.render_ex(S.cornell_view(W, H), p)
    p["flags"] = RP_NEE
    core.render_ex(S.cornell_view(W, H), p)
    assert core.read_accumulator()[:, :3].sum() > 0
    core.close()
