"""The allocation-free frame render (lh2g_render_noalloc) against the allocating one (lh2g_render_ex).

lh2g_render_noalloc exists for callers that cannot allocate device memory when they render (a host with a fixed
memory budget and its own allocator, or a process that must not grow its device footprint after start-up). It
keeps all scratch memory in a static device array of the library, so it must give the same frame as the
allocating path, call after call, and refuse frames larger than the array. The caller's accumulator is the only
device buffer it touches besides the scene; here torch allocates it, as such a caller would from its own pool.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LH2G_ERR_INVALID, LH2G_ERR_OVERFLOW = 1, 5


def test_render_noalloc_matches_render_ex(core_lib):
    import torch
    from lighthouse2_gb300 import scenes as S
    from lighthouse2_gb300.core import RenderCore, make_params, camera_r0, RP_NEE, RP_DEPTH_W

    sc = S.cornell_sphere(subdiv=4)
    core = RenderCore(0)
    core.set_scene(sc)
    W, H, spp = 128, 128, 2                      # 32768 paths: the static capacity
    core.SetTarget(W, H, spp)
    view = S.cornell_view(W, H)                  # 0-d structured records, contiguous
    p = make_params(W, H, spp, max_depth=5, camera_r0=camera_r0(0), flags=RP_NEE | RP_DEPTH_W)
    core.render_ex(view, p, accumulate=False, counters=True)
    expected = core.read_accumulator()
    assert expected[:, :3].sum() > 0

    fn = core.lib.lh2g_render_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    acc = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda:0")
    status = np.full(1, 0xDEAD, np.uint32)
    for call in range(2):                        # two calls in a row share (and must reset) the static scratch
        acc.zero_()
        torch.cuda.synchronize()
        rc = fn(core.ctx, view.ctypes.data, p.ctypes.data, acc.data_ptr(), None, status.ctypes.data)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        assert status[0] == 0, f"call {call}: device status {status[0]}"
        got = acc.cpu().numpy()
        rel = np.abs(got - expected) / np.maximum(np.abs(expected), 1e-6)
        assert rel.max() <= 1e-4, f"call {call}: max relative difference {rel.max()}"

    big = make_params(256, 256, 1, max_depth=3, camera_r0=camera_r0(0), flags=RP_NEE)
    assert fn(core.ctx, view.ctypes.data, big.ctypes.data, acc.data_ptr(), None, None) == LH2G_ERR_OVERFLOW
    assert fn(core.ctx, view.ctypes.data, p.ctypes.data, None, None, None) == LH2G_ERR_INVALID
    core.close()
