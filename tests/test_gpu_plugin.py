"""The core as a Lighthouse 2 plugin: a headless C++ application (lighthouse2_gb300/harness/headless_app.cpp) loads
libRenderCore_GB300.so by name the way lib/RenderSystem/core_api_base.cpp:97-127 does, synchronises a scene through
the CoreAPI_Base setters in RenderSystem order (textures, materials as CoreMaterial, geometry, lights, sky,
instances + truncation, FinalizeInstances), and renders a frame sequence with Restart / Converge and a moved
instance between frames. Every frame must equal, bit for bit, the frame the same calls produce through the C ABI
from Python, and GetCoreStats must report the same ray counts."""
import json
import os
import subprocess

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300 import scenefile
from lighthouse2_gb300.core import RenderCore

pytestmark = pytest.mark.gpu

W, H, SPP = 160, 96, 2
SETTINGS = {"maxDepth": 5, "rrStartDepth": 2}


def test_headless_application_matches_c_abi(core_lib, tmp_path):
    from lighthouse2_gb300 import build as B
    app = B.build_harness()
    sc = S.spheres_2m(seed=5, n_spheres=6, slices=40, stacks=26, tex_size=64)
    moved = sc.instances[2][1].copy()
    moved[0, 3] += 1.5
    frames = [(S.spheres_view(W, H, frame=0), 1, None), (S.spheres_view(W, H, frame=0), 0, None),
              (S.spheres_view(W, H, frame=1), 0, (2, sc.instances[2][0], moved)), (S.spheres_view(W, H, frame=2), 1, None)]
    scenefile.write_scene(tmp_path / "scene.bin", sc)
    scenefile.write_frames(tmp_path / "frames.bin", frames)
    r = subprocess.run([app, core_lib, str(tmp_path / "scene.bin"), str(tmp_path / "frames.bin"), str(tmp_path / "out.bin"), str(W), str(H),
                        str(SPP)] + [f"{k}={v}" for k, v in SETTINGS.items()], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    stats = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    got = scenefile.read_frames_output(tmp_path / "out.bin", W, H)
    assert len(stats) == len(frames) == len(got)

    core = RenderCore()
    core.set_scene(sc)
    for k, v in SETTINGS.items():
        core.Setting(k, v)
    core.SetTarget(W, H, SPP)
    for k, (view, converge, change) in enumerate(frames):
        if change is not None:
            core.SetInstance(change[0], change[1], change[2])
            core.FinalizeInstances()
        core.Render(view, converge=converge)
        expect = core.read_framebuffer()
        st = core.GetCoreStats()
        assert np.array_equal(got[k].view(np.uint32), expect.view(np.uint32)), f"frame {k} differs"
        assert stats[k]["totalRays"] == st["totalRays"] and stats[k]["totalShadowRays"] == st["totalShadowRays"], (stats[k], st)
        assert stats[k]["primaryRayCount"] == W * H * SPP and stats[k]["SMcount"] > 0
        assert expect[:, :3].sum() > 0
    # the move is visible from frame 2's camera: the same view with the instance back in place renders differently
    core.Render(frames[2][0], converge=1)
    moved_img = core.read_framebuffer()
    core.SetInstance(2, sc.instances[2][0], sc.instances[2][1])
    core.FinalizeInstances()
    core.Render(frames[2][0], converge=1)
    assert not np.array_equal(core.read_framebuffer(), moved_img)
    core.close()


def test_headless_application_rasterizer(core_lib, tmp_path):
    """With the setting rasterizer=1 the plugin's Render draws the SoftRasterizer core's frame; every frame equals
    lh2g_raster_render's through the C ABI, a moved instance included."""
    from lighthouse2_gb300 import build as B
    app = B.build_harness()
    W2, H2 = 200, 120
    sc = S.spheres_2m(seed=5, n_spheres=6, slices=40, stacks=26, tex_size=64)
    moved = sc.instances[2][1].copy()
    moved[0, 3] += 1.5
    frames = [(S.spheres_view(W2, H2, frame=0), 1, None), (S.spheres_view(W2, H2, frame=1), 0, (2, sc.instances[2][0], moved))]
    scenefile.write_scene(tmp_path / "scene.bin", sc)
    scenefile.write_frames(tmp_path / "frames.bin", frames)
    r = subprocess.run([app, core_lib, str(tmp_path / "scene.bin"), str(tmp_path / "frames.bin"), str(tmp_path / "out.bin"), str(W2), str(H2),
                        "1", "rasterizer=1"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(tmp_path / "out.bin", np.uint32).reshape(-1, W2 * H2)
    assert len(got) == len(frames)
    core = RenderCore()
    core.set_scene(sc)
    core.SetTarget(W2, H2, 1)
    for k, (view, _, change) in enumerate(frames):
        if change is not None:
            core.SetInstance(change[0], change[1], change[2])
            core.FinalizeInstances()
        expect = core.raster(view)["pixels"]
        assert np.array_equal(got[k], expect), f"frame {k}: {np.count_nonzero(got[k] != expect)} pixels differ"
        assert np.count_nonzero(expect) > W2 * H2 // 10
    core.close()
