"""Generates tests/golden/disney_vectors.npz from the reference's own code (TEST INFRASTRUCTURE).

Runs where the reference tree is given (LH2_REFERENCE): oracle/ref compiles the OptiX 7 core's shading kernel with the
Disney BSDF (lib/sharedBSDFs/disney.h, ggxmdf.h, frosted.h: the default branch of lib/rendercore_optix7/kernels/bsdf.h),
and this script renders frames of a Cornell room whose materials span the Disney parameters through that core's wave
loop, with the oracle answering the ray queries.

    LH2_REFERENCE=<lighthouse2 tree> python tests/golden/make_golden_disney.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lighthouse2_gb300 import scenes as S  # noqa: E402

# name, W, H, spp, depth, samplesTaken (>= 64: xorshift numbers), shift
FRAMES = [("d_a", 48, 40, 1, 4, 0, 0x91331445), ("d_b", 32, 24, 2, 6, 3, 0x11331445), ("d_c", 40, 32, 1, 5, 70, 7)]


def disney_scene(seed=9, subdiv=3):
    """The Cornell room with its eight surface materials spread over the Disney BSDF's parameters: metal with
    anisotropy, sheen with subsurface, clearcoat, a rough dielectric with absorption, tinted specular, a near-mirror,
    a mixed one and a plain diffuse one; seeded blue-noise tables."""
    sc = S.cornell_sphere(subdiv=subdiv)
    rng = np.random.default_rng(seed)
    spec = [dict(roughness=0.5),
            dict(metallic=0.9, roughness=0.3, anisotropic=0.6),
            dict(sheen=0.8, sheenTint=0.5, subsurface=0.6, roughness=0.7),
            dict(clearcoat=1.0, clearcoatGloss=0.7, specular=0.5, roughness=0.6),
            dict(transmission=0.9, roughness=0.25, eta=1.5, absorption=(0.3, 0.2, 0.1)),
            dict(specular=0.8, specularTint=0.8, roughness=0.15),
            dict(roughness=0.0, metallic=1.0),
            dict(metallic=0.4, sheen=0.3, clearcoat=0.5, subsurface=0.3, anisotropic=-0.4, roughness=0.45, transmission=0.3, eta=1.3)]
    for i, kv in enumerate(spec):
        m = sc.materials[i]
        for k, v in kv.items():
            m[k] = v
        m["color"] = rng.uniform(0.1, 0.9, 3)
    sc.blue_noise = S.synthetic_blue_noise(13)
    return sc


def main():
    from oracle import bind as B
    sc = disney_scene()
    o = B.Oracle()
    o.set_scene(sc)
    ref = B.RefOptix7(disney=True)
    out = {}
    for name, W, H, spp, depth, st, shift in FRAMES:
        p = B.make_params(W, H, spp, max_depth=depth, samples_taken=st, camera_r0=B.camera_r0(st),
                          flags=B.RP_NEE | B.RP_OPTIX7 | B.RP_DISNEY, shift=shift)
        r = ref.render(o, sc, S.cornell_view(W, H), p)
        assert not r["flushed"]
        out[name + "/accum"] = r["accum"]
        out[name + "/counters"] = r["counters"]
        print(name, r["counters"][:, 0].tolist(), r["counters"][:, 1].tolist())
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "disney_vectors.npz"), **out)


if __name__ == "__main__":
    main()
