"""Generates tests/golden/mis_vectors.npz from the reference's own code (TEST INFRASTRUCTURE).

Runs where the reference tree is given (LH2_REFERENCE): oracle/ref compiles, by path, the OptiX 7 core's shading
kernel and ray generation (lib/rendercore_optix7/kernels/pathtracer.h, optix/.optix.cu) and the PrimeAdaptive core's
kernels (lib/RenderCore_PrimeAdaptive/kernels/*.h with finalize_shared.h's variance and finalize kernels), both with
the Lambert BSDF; this script renders frames through those cores' wave loops with the oracle answering the ray
queries, and evaluates the blue-noise sampler of tools_shared.h. Blue-noise tables are seeded synthetic bytes
(lighthouse2_gb300.scenes.synthetic_blue_noise), so the fixtures pin the oracle without the reference's tables.

    LH2_REFERENCE=<lighthouse2 tree> python tests/golden/make_golden_mis.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lighthouse2_gb300 import scenes as S  # noqa: E402
from oracle import bind as B  # noqa: E402

BN_SEED = 5
# OptiX 7 frames: name, W, H, spp, depth, samplesTaken (>= 64: xorshift numbers), shift
OPTIX7_FRAMES = [("o7_a", 48, 40, 1, 4, 0, 0x91331445), ("o7_b", 32, 24, 2, 5, 3, 0x11331445), ("o7_c", 40, 32, 1, 3, 70, 7)]
# PrimeAdaptive sequences: name, W, H, spp, depth, frames, initial devScale
ADAPTIVE_SEQS = [("ad_a", 40, 32, 1, 4, 3, 60.0), ("ad_b", 32, 24, 2, 5, 2, 40.0)]


def scene():
    sc = S.cornell_sphere(subdiv=3)
    sc.blue_noise = S.synthetic_blue_noise(BN_SEED)
    return sc


def main():
    sc = scene()
    o = B.Oracle()
    o.set_scene(sc)
    out = {}
    o7 = B.RefOptix7()
    for name, W, H, spp, D, st, shift in OPTIX7_FRAMES:
        p = B.make_params(W, H, spp, max_depth=D, samples_taken=st, camera_r0=B.camera_r0(st), flags=B.RP_NEE | B.RP_OPTIX7, shift=shift)
        r = o7.render(o, sc, S.cornell_view(W, H), p)
        assert not r["flushed"]
        out[name + "_accum"], out[name + "_counters"] = r["accum"], r["counters"]
    ad = B.RefAdaptive()
    for name, W, H, spp, D, frames, ds in ADAPTIVE_SEQS:
        acc = np.zeros((W * H, 4), np.float32)
        for k in range(frames):
            p = adaptive_params(W, H, spp, D, k)
            r = ad.render(o, sc, S.cornell_view(W, H), p, acc, ds)
            assert not r["flushed"]
            ds = r["dev_scale"]
            for key in ("counters", "frame", "features", "deviation"):
                out[f"{name}_{k}_{key}"] = r[key]
            out[f"{name}_{k}_dev_scale"] = np.float32(ds)
            out[f"{name}_{k}_adaptive_paths"] = np.uint32(r["adaptive_paths"])
            out[f"{name}_{k}_accum"] = acc.copy()
    bn = B.expand_blue_noise(sc.blue_noise)
    rng = np.random.default_rng(9)
    q = np.stack([rng.integers(0, 128, 4000), rng.integers(0, 128, 4000), rng.integers(0, 64, 4000), 4 * rng.integers(0, 8, 4000)], 1)
    q[:4] = [[127, 127, 63, 28], [0, 0, 0, 0], [127, 0, 5, 24], [0, 127, 63, 4]]
    out["bn_in"] = q.astype(np.int32)
    out["bn_out"] = np.stack([o7.bluenoise4(bn, *map(int, row)) for row in q])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mis_vectors.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def adaptive_params(W, H, spp, D, k):
    """frame k of a converging sequence: the two draws of RandomUInt(camRNGseed) and a shift per frame"""
    return B.make_params(W, H, spp, max_depth=D, samples_taken=k * spp, camera_r0=B.camera_r0(2 * k), frame_seed=B.camera_r0(2 * k + 1),
                         flags=B.RP_NEE, shift=(0x11331445 * (k + 3)) & 0xFFFFFFFF)


if __name__ == "__main__":
    main()
