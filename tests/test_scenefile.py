"""Host side of the headless application (no GPU): the scene and frame files written by
lighthouse2_gb300/scenefile.py are what harness/headless_app.cpp reads. The application builds with g++, prints its
usage on bad arguments, and reads both files completely before it tries to load a core (exit status 3 = files read,
core not found; 2 = a file could not be read)."""
import os
import struct
import subprocess

import numpy as np

from lighthouse2_gb300 import scenes as S
from lighthouse2_gb300 import scenefile


def _scene():
    return S.spheres_2m(seed=3, n_spheres=3, slices=12, stacks=8, tex_size=32)


def test_scene_file_layout(tmp_path):
    sc = _scene()
    p = tmp_path / "scene.bin"
    scenefile.write_scene(p, sc)
    data = p.read_bytes()
    assert data[:8] == b"LH2GSCN1"
    counts = struct.unpack_from("<10I", data, 8)
    assert counts[:4] == (len(sc.meshes), len(sc.instances), len(sc.materials), len(sc.textures))
    expect = 8 + 40
    expect += sum(4 + 48 * len(m.tris) + 208 * len(m.tris) for m in sc.meshes)
    expect += len(sc.instances) * (4 + 64) + len(sc.materials) * 196
    expect += sum(12 + 4 * len(t.texels) for t in sc.textures)
    expect += 96 * len(sc.tri_lights) + 32 * len(sc.point_lights) + 48 * len(sc.spot_lights) + 32 * len(sc.dir_lights)
    expect += 12 * sc.sky[1] * sc.sky[2]
    assert len(data) == expect


def test_headless_application_reads_the_files(tmp_path):
    from lighthouse2_gb300 import build as B
    app = B.build_harness()
    r = subprocess.run([app], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    sc = _scene()
    scenefile.write_scene(tmp_path / "scene.bin", sc)
    moved = np.eye(4, dtype=np.float32)
    scenefile.write_frames(tmp_path / "frames.bin", [(S.spheres_view(64, 48, frame=0), 1, None), (S.spheres_view(64, 48, frame=1), 0, (1, 1, moved))])
    args = [str(tmp_path / "scene.bin"), str(tmp_path / "frames.bin"), str(tmp_path / "out.bin"), "64", "48", "1"]
    r = subprocess.run([app, str(tmp_path / "no_such_core")] + args, capture_output=True, text=True)
    assert r.returncode == 3 and "cannot load core" in r.stderr, r.stderr
    (tmp_path / "bad.bin").write_bytes(b"LH2GSCN1" + b"\0" * 8)
    r = subprocess.run([app, "x", str(tmp_path / "bad.bin")] + args[1:], capture_output=True, text=True)
    assert r.returncode == 2 and "cannot read scene" in r.stderr
