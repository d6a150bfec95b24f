"""The CPU oracle against golden vectors produced by the reference's own code (tests/golden/make_golden.py).

Pure functions of lib/CUDA/shared_kernel_code/tools_shared.h and lib/RenderSystem/common_functions.h, and whole
frames of the PrimeRef wave loop (generate, shade, connections) compiled from the reference sources, must be
reproduced bit for bit. Runs everywhere; the fixtures are committed."""
import ctypes as C
import os

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_vectors.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def olib(oracle_lib):
    o = oracle_lib.Oracle()
    L = o.lib
    L.lh2o_wanghash.restype = C.c_uint32
    L.lh2o_random_float.restype = C.c_float
    L.lh2o_random_float.argtypes = [C.c_void_p]
    L.lh2o_random_barycentrics.argtypes = [C.c_float, C.c_void_p]
    L.lh2o_pack_normal.restype = C.c_uint32
    L.lh2o_pack_normal.argtypes = [C.c_void_p]
    L.lh2o_unpack_normal.argtypes = [C.c_uint32, C.c_void_p]
    L.lh2o_diffuse_cos.argtypes = [C.c_float, C.c_float, C.c_void_p]
    L.lh2o_tangent2world.argtypes = [C.c_void_p] * 3
    L.lh2o_consistent_normal.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
    L.lh2o_invert4x4.argtypes = [C.c_void_p, C.c_void_p]
    return L


def _v(a):
    return np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)


def test_rng(gold, olib):
    assert all(olib.lh2o_wanghash(C.c_uint32(int(s))) == o for s, o in zip(gold["wang_in"], gold["wang_out"]))
    for s, rf, st in zip(gold["wang_in"][:500], gold["rand_float"], gold["rand_state"]):
        v = C.c_uint32(int(s))
        for k in range(4):
            assert np.float32(olib.lh2o_random_float(C.byref(v))) == rf[k] and v.value == st[k]


def test_barycentrics_normals_sampling(gold, olib):
    out = np.zeros(3, np.float32)
    for r0, ref in zip(gold["bary_in"], gold["bary_out"]):
        if r0 >= 1.0:
            # (uint)(r0 * 2^32) overflows: undefined in C, wraps to 0 in the x86 host build of the reference, saturates
            # to 0xffffffff on the GPU the reference runs on; the oracle follows the GPU (checked below)
            olib.lh2o_random_barycentrics(C.c_float(r0), _v(out))
            assert out[2] > 0.9999 and out[0] < 1e-5 and out[1] < 1e-5
            continue
        olib.lh2o_random_barycentrics(C.c_float(r0), _v(out))
        assert np.array_equal(out, ref)
    for n, pk, un in zip(gold["normal_in"], gold["normal_packed"], gold["normal_unpacked"]):
        assert olib.lh2o_pack_normal(_v(n)) == pk
        olib.lh2o_unpack_normal(C.c_uint32(int(pk)), _v(out))
        assert np.array_equal(out, un)
    for (a, b), dc in zip(gold["diffuse_in"], gold["diffuse_out"]):
        olib.lh2o_diffuse_cos(C.c_float(a), C.c_float(b), _v(out))
        assert np.array_equal(out, dc)
    for dc, n, t in zip(gold["diffuse_out"], gold["normal_in"], gold["t2w_out"]):
        o3 = np.zeros(3, np.float32)
        olib.lh2o_tangent2world(_v(dc), _v(n), _v(o3))
        assert np.array_equal(o3, t)
    for d, n, a, ref in zip(gold["cn_D"], gold["cn_iN"], gold["cn_alpha"], gold["cn_out"]):
        o3 = np.zeros(3, np.float32)
        olib.lh2o_consistent_normal(_v(d), _v(n), C.c_float(a), _v(o3))
        assert np.array_equal(o3, ref)
    for m, ref in zip(gold["inv_in"], gold["inv_out"]):
        o16 = np.zeros(16, np.float32)
        olib.lh2o_invert4x4(_v(m), _v(o16))
        assert np.array_equal(o16, ref)


FRAMES = {
    "cornell_d3": (lambda: S.cornell_sphere(subdiv=4), S.cornell_view, 48, 40, 1, 3, 1, 3),
    "cornell_d6_nonee": (lambda: S.cornell_sphere(subdiv=4), S.cornell_view, 40, 32, 1, 6, 1, 2),
    "spheres_d8": (lambda: S.spheres_2m(n_spheres=6, slices=32, stacks=20, tex_size=64, sky_size=(1, 1)), S.spheres_view, 48, 32, 1, 8, 1, 3),
}


@pytest.mark.parametrize("name", sorted(FRAMES))
def test_frames_match_reference_kernels(gold, oracle_lib, name):
    mk, mv, W, H, spp, depth, rr, flags = FRAMES[name]
    sc = mk()
    o = oracle_lib.Oracle()
    o.set_scene(sc)
    p = oracle_lib.make_params(W, H, spp, max_depth=depth, rr_start=rr, camera_r0=oracle_lib.camera_r0(0), flags=flags)
    r = o.render(mv(W, H), p)
    assert np.array_equal(r["counters"], gold[name + "_counters"])
    assert np.array_equal(r["accum"], gold[name + "_accum"])


def test_transcendentals_close_to_libm(olib):
    """The oracle's own sin/cos/exp/log2/atan2/acos stay within a few ulp of the C library."""
    L = olib
    L.lh2o_sincos.argtypes = [C.c_float, C.c_void_p, C.c_void_p]
    for f in (L.lh2o_expf, L.lh2o_log2f, L.lh2o_acosf):
        f.restype, f.argtypes = C.c_float, [C.c_float]
    L.lh2o_atan2f.restype, L.lh2o_atan2f.argtypes = C.c_float, [C.c_float, C.c_float]
    rng = np.random.default_rng(3)
    s, c = C.c_float(), C.c_float()
    for x in rng.uniform(-20, 20, 2000).astype(np.float32):
        L.lh2o_sincos(C.c_float(x), C.byref(s), C.byref(c))
        assert abs(s.value - np.sin(np.float64(x))) < 4e-7 and abs(c.value - np.cos(np.float64(x))) < 4e-7
    for x in rng.uniform(-80, 80, 2000).astype(np.float32):
        assert abs(L.lh2o_expf(C.c_float(x)) / np.exp(np.float64(x)) - 1) < 5e-7
    for x in np.exp(rng.uniform(-60, 60, 2000)).astype(np.float32):
        assert abs(L.lh2o_log2f(C.c_float(x)) - np.log2(np.float64(x))) < 2e-6 * max(1, abs(np.log2(np.float64(x))))
    for y, x in rng.normal(size=(2000, 2)).astype(np.float32):
        assert abs(L.lh2o_atan2f(C.c_float(y), C.c_float(x)) - np.arctan2(np.float64(y), np.float64(x))) < 5e-7
    for x in rng.uniform(-1, 1, 2000).astype(np.float32):
        assert abs(L.lh2o_acosf(C.c_float(x)) - np.arccos(np.float64(x))) < 2e-6
