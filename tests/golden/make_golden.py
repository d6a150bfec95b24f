"""Generates tests/golden/reference_vectors.npz from the reference's own code (TEST INFRASTRUCTURE).

Runs where the reference tree is mounted: the PrimeRef kernels and shared device headers are compiled for the
host by oracle/ref/Makefile (nothing is copied), then
  * pure functions of lib/CUDA/shared_kernel_code/tools_shared.h and lib/RenderSystem/common_functions.h are
    evaluated on seeded inputs, and
  * whole frames are rendered through the reference's wave loop (lib/RenderCore_PrimeRef/rendercore.cpp:551-611:
    generateEyeRaysKernel, shadeKernel, finalizeConnectionKernel) with the oracle answering the ray queries
    (the reference's traversal is closed OptiX Prime code).
The fixtures pin the oracle on machines without the reference tree.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lighthouse2_gb300 import scenes as S  # noqa: E402
from oracle import bind as B  # noqa: E402

FRAMES = [  # name, scene builder, view builder, W, H, spp, depth, rr, flags
    ("cornell_d3", lambda: S.cornell_sphere(subdiv=4), S.cornell_view, 48, 40, 1, 3, 1, B.RP_NEE | B.RP_DEPTH_W),
    ("cornell_d6_nonee", lambda: S.cornell_sphere(subdiv=4), S.cornell_view, 40, 32, 1, 6, 1, B.RP_DEPTH_W),
    ("spheres_d8", lambda: S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=64, sky_size=(1, 1)), S.spheres_view, 48, 32, 1, 8, 1,
     B.RP_NEE | B.RP_DEPTH_W),
]


def pure_vectors(ref, n=2000, seed=5):
    import ctypes as C
    rng = np.random.default_rng(seed)
    L = ref.lib
    out = {}
    seeds = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    out["wang_in"] = seeds
    out["wang_out"] = np.array([L.ref_wanghash(C.c_uint32(int(s))) for s in seeds], np.uint32)
    rf = np.zeros((n, 4), np.float32)
    st = np.zeros((n, 4), np.uint32)
    for i, s in enumerate(seeds):
        v = C.c_uint32(int(s))
        for k in range(4):
            rf[i, k] = L.ref_random_float(C.byref(v))
            st[i, k] = v.value
    out["rand_float"], out["rand_state"] = rf, st
    r0 = rng.random(n).astype(np.float32)
    r0[:4] = [0.0, 1.0, 0.99999994, 0.5]
    bary = np.zeros((n, 3), np.float32)
    for i in range(n):
        L.ref_random_barycentrics(C.c_float(r0[i]), bary[i].ctypes.data_as(C.c_void_p))
    out["bary_in"], out["bary_out"] = r0, bary
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    pk = np.array([L.ref_pack_normal(nrm[i].ctypes.data_as(C.c_void_p)) for i in range(n)], np.uint32)
    un = np.zeros((n, 3), np.float32)
    for i in range(n):
        L.ref_unpack_normal(C.c_uint32(int(pk[i])), un[i].ctypes.data_as(C.c_void_p))
    out["normal_in"], out["normal_packed"], out["normal_unpacked"] = nrm, pk, un
    q = rng.random((n, 2)).astype(np.float32)
    dc = np.zeros((n, 3), np.float32)
    for i in range(n):
        L.ref_diffuse_cos(C.c_float(q[i, 0]), C.c_float(q[i, 1]), dc[i].ctypes.data_as(C.c_void_p))
    out["diffuse_in"], out["diffuse_out"] = q, dc
    t2w = np.zeros((n, 3), np.float32)
    for i in range(n):
        L.ref_tangent2world(np.ascontiguousarray(dc[i]).ctypes.data_as(C.c_void_p), np.ascontiguousarray(nrm[i]).ctypes.data_as(C.c_void_p),
                            t2w[i].ctypes.data_as(C.c_void_p))
    out["t2w_out"] = t2w
    D = rng.normal(size=(n, 3)).astype(np.float32)
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    iN = np.where((np.sum(D * nrm, 1) < 0)[:, None], nrm, -nrm).astype(np.float32)
    alpha = rng.uniform(0, 0.7, n).astype(np.float32)
    cn = np.zeros((n, 3), np.float32)
    for i in range(n):
        L.ref_consistent_normal(np.ascontiguousarray(-D[i]).ctypes.data_as(C.c_void_p), np.ascontiguousarray(iN[i]).ctypes.data_as(C.c_void_p),
                                C.c_float(alpha[i]), cn[i].ctypes.data_as(C.c_void_p))
    out["cn_D"], out["cn_iN"], out["cn_alpha"], out["cn_out"] = -D, iN, alpha, cn
    M = rng.normal(size=(64, 16)).astype(np.float32)
    M[:, 12:15] = 0
    M[:, 15] = 1
    inv = np.zeros((64, 16), np.float32)
    for i in range(64):
        L.ref_invert4x4(np.ascontiguousarray(M[i]).ctypes.data_as(C.c_void_p), inv[i].ctypes.data_as(C.c_void_p))
    out["inv_in"], out["inv_out"] = M, inv
    return out


def main():
    ref = B.RefKernels()
    o = B.Oracle()
    out = pure_vectors(ref)
    for name, mk, mv, W, H, spp, depth, rr, flags in FRAMES:
        sc = mk()
        o = B.Oracle()
        o.set_scene(sc)
        view = mv(W, H)
        p = B.make_params(W, H, spp, max_depth=depth, rr_start=rr, camera_r0=B.camera_r0(0), flags=flags)
        r = ref.render(o, sc, view, p)
        out[name + "_accum"] = r["accum"]
        out[name + "_counters"] = r["counters"]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
