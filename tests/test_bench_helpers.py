"""Host logic of bench.py that turns the core's per-launch event times into per-stage figures: the launch layout of
a frame (generate, then extend / partition+shade / connect per wave, the tail kernel when the waves stop before the
last path length, finalize) and the algorithmic bytes per stage. CPU only."""
import numpy as np

import bench


def _counts(ext, shadow):
    c = np.zeros((bench.MAX_DEPTH, 2), np.int64)
    c[:len(ext), 0] = ext
    c[:len(shadow), 1] = shadow
    return c


def test_decode_launches_with_tail():
    W, H, waves = 4, 2, 2
    counts = [_counts([5, 3, 2, 1], [6, 4, 2, 1])] * 8
    per_frame = 2 + 3 * waves + 1
    frames = 3
    # per frame: generate 1, (extend 10, shade 20, connect 30) per wave, tail 40, finalize 2
    frame = [1.0, 10.0, 20.0, 30.0, 10.0, 20.0, 30.0, 40.0, 2.0]
    assert len(frame) == per_frame
    k = bench.decode_launches(frame * frames, frames, counts, waves, W, H)
    assert k["generate"][0] == frames * 1.0 and k["finalize"][0] == frames * 2.0
    assert k["extend"][0] == frames * 20.0 and k["extend"][2] == frames * waves
    assert k["shade"][0] == frames * 40.0 and k["connect"][0] == frames * 60.0
    assert k["tail"][0] == frames * 40.0 and k["tail"][2] == frames
    # wave inputs: W*H primary rays, then the extension counts of the previous path lengths
    n_in = [W * H, 5]
    assert k["extend"][1] == frames * sum(bench.algorithmic_bytes("extend", n, 0, 0) for n in n_in)
    assert k["connect"][1] == frames * sum(bench.algorithmic_bytes("connect", s, 0, 0) for s in (6, 4))
    tail = sum(bench.algorithmic_bytes("extend", n, 0, 0) + bench.algorithmic_bytes("shade", n, e, s) +
               bench.algorithmic_bytes("connect", s, 0, 0)
               for n, e, s in zip([3, 2, 1] + [0] * 8, [2, 1, 0, 0, 0, 0], [2, 1, 0, 0, 0, 0]))
    assert k["tail"][1] == frames * tail


def test_decode_launches_without_tail():
    W, H, waves = 2, 2, bench.MAX_DEPTH
    counts = [_counts([3] * bench.MAX_DEPTH, [2] * bench.MAX_DEPTH)] * 8
    per_frame = 2 + 3 * waves
    k = bench.decode_launches([1.0] * per_frame, 1, counts, waves, W, H)
    assert k["tail"] == [0.0, 0, 0]
    assert k["extend"][2] == k["shade"][2] == k["connect"][2] == waves


def test_algorithmic_bytes():
    assert bench.algorithmic_bytes("extend", 10, 0, 0) == 480
    assert bench.algorithmic_bytes("connect", 10, 0, 0) == 480
    # shading: partition (16 + 4), order read back (4), path state, hit, triangle and material reads, written rays
    assert bench.algorithmic_bytes("shade", 10, 3, 2) == 10 * (16 + 4 + 4 + 48 + 16 + 80 + 32) + 48 * 3 + 48 * 2
