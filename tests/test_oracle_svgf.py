"""The oracle's SVGF restatement against the reference's own filter kernels.

lib/CUDA/shared_kernel_code/finalize_shared.h (prepareFilterKernel, applyFilterKernel, TAApassKernel,
unsharpenTAAKernel, finalizeNoTAAKernel) and the packing helpers of tools_shared.h / sampling_shared.h are compiled
for the host by oracle/ref from the reference tree, and run over the same buffers as the oracle: feature buffers of
filter-core frames of the Cornell scene rendered by the oracle over a short camera path, with jitter, TAA on and off,
and a converging (camera-stationary) frame. Every buffer must agree bit for bit. CUDA math calls in the reference
code (__expf, powf(x, 128)) are routed to the oracle's own functions, as for the path-tracer kernels.
"""
import ctypes as C

import numpy as np
import pytest

from lighthouse2_gb300 import scenes as S
from oracle import bind as OB

REF = None


def ref():
    global REF
    if REF is None:
        try:
            path = OB.build_ref()
        except Exception as e:   # pragma: no cover
            pytest.skip(f"reference harness does not build: {e}")
        if path is None:
            pytest.skip("reference tree not available")
        L = C.CDLL(path)
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        L.ref_svgf_prepare.argtypes = [vp] * 10 + [f, f, f, f, i, i, f, f, f, i]
        L.ref_svgf_apply.argtypes = [vp] * 9 + [i, i, i, i]
        L.ref_svgf_taa.argtypes = [vp] * 4 + [i, i]
        L.ref_svgf_finalize.argtypes = [vp, vp, i, i, i]
        L.ref_pack_normal2.restype = C.c_uint32
        L.ref_pack_normal2.argtypes = [vp]
        L.ref_unpack_normal2.argtypes = [C.c_uint32, vp]
        L.ref_hdr_to_rgb32.restype = C.c_uint32
        L.ref_hdr_to_rgb32.argtypes = [vp]
        L.ref_rgb32_to_hdr.argtypes = [C.c_uint32, i, vp]
        L.ref_combine_to_float4.argtypes = [vp, vp, vp]
        L.ref_split_float4.argtypes = [vp, vp, vp]
        L.ref_rgb_to_ycocg.argtypes = [vp, vp]
        L.ref_ycocg_to_rgb.argtypes = [vp, vp]
        L.ref_luminance.restype = C.c_float
        L.ref_luminance.argtypes = [vp]
        L.ref_mitchell_netravali.restype = C.c_float
        L.ref_mitchell_netravali.argtypes = [f]
        REF = L
    return REF


def oracle_lib():
    o = OB.Oracle()
    L = o.lib
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    L.lh2o_pack_normal2.restype = C.c_uint32
    L.lh2o_pack_normal2.argtypes = [vp]
    L.lh2o_unpack_normal2.argtypes = [C.c_uint32, vp]
    L.lh2o_hdr_to_rgb32.restype = C.c_uint32
    L.lh2o_hdr_to_rgb32.argtypes = [vp]
    L.lh2o_rgb32_to_hdr.argtypes = [C.c_uint32, i, vp]
    L.lh2o_combine_to_float4.argtypes = [vp, vp, vp]
    L.lh2o_split_float4.argtypes = [vp, vp, vp]
    L.lh2o_rgb_to_ycocg.argtypes = [vp, vp]
    L.lh2o_ycocg_to_rgb.argtypes = [vp, vp]
    L.lh2o_luminance.restype = C.c_float
    L.lh2o_luminance.argtypes = [vp]
    L.lh2o_mitchell_netravali.restype = C.c_float
    L.lh2o_mitchell_netravali.argtypes = [f]
    L.lh2o_svgf_view.argtypes = [vp, i, vp]
    return o


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_packing_helpers_match_reference():
    R, O = ref(), oracle_lib().lib
    rng = np.random.default_rng(5)
    n3 = rng.normal(size=(400, 3)).astype(np.float32)
    n3 /= np.linalg.norm(n3, axis=1, keepdims=True)
    n3[:6] = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, -1], [-1.0000001, 0, 0]]
    for v in n3:
        v = np.ascontiguousarray(v, np.float32)
        assert R.ref_pack_normal2(_p(v)) == O.lh2o_pack_normal2(_p(v))
    for u in list(rng.integers(0, 2**32, 300, dtype=np.uint64)) + [0, 0xFFFFFFFF]:
        a, b = np.zeros(3, np.float32), np.zeros(3, np.float32)
        R.ref_unpack_normal2(int(u), _p(a)), O.lh2o_unpack_normal2(int(u), _p(b))
        assert bits(a).tolist() == bits(b).tolist()
        for m in (0, 1):
            R.ref_rgb32_to_hdr(int(u), m, _p(a)), O.lh2o_rgb32_to_hdr(int(u), m, _p(b))
            assert bits(a).tolist() == bits(b).tolist()
    cols = rng.uniform(0.0, 40.0, size=(400, 3)).astype(np.float32)
    # neither NaN nor negative values here: on the host, helper_math.h defines fminf as a < b ? a : b, which
    # differs from the device's fminf when an argument is NaN, and a negative float converted to unsigned is
    # undefined in C++ where the GPU's conversion (and the oracle's) gives 0
    cols[:4] = [[0, 0, 0], [1, 1, 1], [31.999, 32, 100], [0.0, 0.5, np.inf]]
    for c in cols:
        c = np.ascontiguousarray(c)
        assert R.ref_hdr_to_rgb32(_p(c)) == O.lh2o_hdr_to_rgb32(_p(c))
        a, b = np.zeros(3, np.float32), np.zeros(3, np.float32)
        R.ref_rgb_to_ycocg(_p(c), _p(a)), O.lh2o_rgb_to_ycocg(_p(c), _p(b))
        assert bits(a).tolist() == bits(b).tolist()
        R.ref_ycocg_to_rgb(_p(c), _p(a)), O.lh2o_ycocg_to_rgb(_p(c), _p(b))
        assert bits(a).tolist() == bits(b).tolist()
        assert bits(np.float32(R.ref_luminance(_p(c)))) == bits(np.float32(O.lh2o_luminance(_p(c))))
    for k in range(0, 400, 2):
        A, B = np.ascontiguousarray(np.abs(cols[k])), np.ascontiguousarray(np.abs(cols[k + 1]))
        a4, b4 = np.zeros(4, np.float32), np.zeros(4, np.float32)
        R.ref_combine_to_float4(_p(A), _p(B), _p(a4)), O.lh2o_combine_to_float4(_p(A), _p(B), _p(b4))
        assert bits(a4).tolist() == bits(b4).tolist()
        d1, i1, d2, i2 = (np.zeros(3, np.float32) for _ in range(4))
        R.ref_split_float4(_p(a4), _p(d1), _p(i1)), O.lh2o_split_float4(_p(a4), _p(d2), _p(i2))
        assert bits(d1).tolist() == bits(d2).tolist() and bits(i1).tolist() == bits(i2).tolist()
    for x in np.concatenate([rng.uniform(-3, 3, 200), [0, 1, -1, 2, -2, 0.5]]).astype(np.float32):
        assert bits(np.float32(R.ref_mitchell_netravali(float(x)))) == bits(np.float32(O.lh2o_mitchell_netravali(float(x))))


def svgf_view_numpy(view, h):
    """prepareFilter's host constants (finalize_shared.h:297-313) in float32 numpy arithmetic."""
    f = np.float32
    pos, p1, p2, p3 = (np.asarray(view[k], f) for k in ("pos", "p1", "p2", "p3"))

    def dot(a, b):
        return f(f(f(a[0] * b[0]) + f(a[1] * b[1])) + f(a[2] * b[2]))

    def normalize(v):
        inv = f(f(1) / np.sqrt(dot(v, v)))
        return (v * inv).astype(f)

    centre = (f(0.5) * (p2 + p3)).astype(f)
    direction = normalize((centre - pos).astype(f))
    right = normalize((p2 - p1).astype(f))
    up = normalize((p3 - p1).astype(f))
    d31 = (p3 - p1).astype(f)
    lenReci = f(f(h) / np.sqrt(dot(d31, d31)))
    out = np.zeros(16, f)
    out[0:3], out[3] = pos, -(dot(pos, direction) - dot(centre, direction))
    out[4:7], out[7] = direction, 0
    out[8:11], out[11] = (right * lenReci).astype(f), f(dot(p1, right) * lenReci)
    out[12:15], out[15] = (up * lenReci).astype(f), f(dot(p1, up) * lenReci)
    return out


HALTON = ([0.3, 0.7, 0.2, 0.8], [0.2, 0.8, 0.7, 0.3])


def jittered(view, W, H, j0, j1):
    jv = view.copy()
    right = view["p2"] - view["p1"]
    up = view["p3"] - view["p1"]
    jit = (np.float32(j0 / np.float32(W)) * right + np.float32(j1 / np.float32(H)) * up).astype(np.float32)
    for k in ("p1", "p2", "p3"):
        jv[k] = (view[k] + jit).astype(np.float32)
    jv["aperture"] = 0
    return jv


def xorshift(s):
    s ^= (s << 13) & 0xFFFFFFFF
    s ^= s >> 17
    s ^= (s << 5) & 0xFFFFFFFF
    return s


def run_reference_chain(R, st, accum, fp, view16, W, H):
    """The reference kernels over copies of the oracle state taken before the frame, with the core's swaps."""
    b = {k: st[k].copy() for k in OB.SVGF_SLOTS}
    f = lambda k: _p(b[k])
    R.ref_svgf_prepare(_p(accum), f("features"), f("worldPos"), f("prevWorldPos"), f("shading"), f("motion"), f("moments"),
                       f("prevMoments"), f("deltaDepth"), _p(view16), float(fp["j0"]), float(fp["j1"]), float(fp["prevj0"]),
                       float(fp["prevj1"]), W, H, float(np.float32(1) / np.float32(fp["samplesTaken"])), float(fp["clampDirect"]),
                       float(fp["clampIndirect"]), int(fp["camIsStationary"]))
    common = (f("features"), f("prevWorldPos"), f("worldPos"), f("deltaDepth"), f("motion"), f("moments"))
    R.ref_svgf_apply(*common, f("shading"), f("filteredIN"), f("filteredOUT"), W, H, 1, 0)
    R.ref_svgf_apply(*common, f("filteredOUT"), None, f("filteredIN"), W, H, 2, 0)
    R.ref_svgf_apply(*common, f("filteredIN"), None, f("shading"), W, H, 3, 1)
    if int(fp["taa"]):
        R.ref_svgf_taa(f("shading"), f("prevPixels"), f("motion"), f("taaPixels"), W, H)
        R.ref_svgf_finalize(f("taaPixels"), f("target"), W, H, 1)
        b["taaPixels"], b["prevPixels"] = b["prevPixels"], b["taaPixels"]
    else:
        R.ref_svgf_finalize(f("shading"), f("target"), W, H, 0)
        b["shading"], b["prevPixels"] = b["prevPixels"], b["shading"]
    for x, y in (("filteredIN", "filteredOUT"), ("prevWorldPos", "worldPos"), ("moments", "prevMoments")):
        b[x], b[y] = b[y], b[x]
    return b


@pytest.mark.parametrize("taa", [1, 0])
def test_svgf_chain_matches_reference_kernels(taa):
    R = ref()
    o = oracle_lib()
    sc = S.cornell_sphere(subdiv=3)
    o.set_scene(sc)
    W, H = 48, 36
    st = OB.SvgfState(o, W, H)
    seed = 0x12345678
    prev_view, pj = None, (0.0, 0.0)
    samples = 0
    # frames 0-3: moving camera (Restart each frame); frame 4: same pose as 3, converging
    for k, converge in enumerate([False, False, False, False, True]):
        view = S.cornell_view(W, H, frame=min(k, 3))
        if not converge:
            samples = 0
        j = (HALTON[0][k & 3], HALTON[1][k & 3]) if taa else (0.0, 0.0)
        seed = xorshift(seed)
        p = OB.make_params(W, H, 1, max_depth=4, rr_start=2, samples_taken=samples,
                           flags=OB.RP_FILTER | OB.RP_NEE | OB.RP_DEPTH_W, frame_seed=seed)
        if samples == 0:
            accum = np.zeros((2 * W * H, 4), np.float32)
        accum = o.render(jittered(view, W, H, *j), p, accum=accum, features=st)["accum"]
        samples += 1
        fp = OB.make_filter_params(prev_view if prev_view is not None else view, j[0], j[1], pj[0], pj[1], samples,
                                   0 if samples == 1 else 1, taa)
        v16 = np.zeros(16, np.float32)
        o.lib.lh2o_svgf_view(_p(fp["prevView"]), H, _p(v16))
        assert bits(v16).tolist() == bits(svgf_view_numpy(fp["prevView"], H)).tolist()
        expect = run_reference_chain(R, st, accum, fp, v16, W, H)
        st.frame(accum, fp)
        for name in OB.SVGF_SLOTS:
            a, b = bits(st[name]), bits(expect[name])
            bad = np.flatnonzero((a != b).any(axis=1))
            assert len(bad) == 0, f"frame {k} taa={taa} slot {name}: {len(bad)} pixels differ, first {bad[:5]}"
        prev_view, pj = view, j
    # the filter did real work: history accumulated, a non-trivial image inside the border
    feats = st["features"]
    assert (feats[:, 3] & 15).max() >= 3
    img = st["target"].reshape(H, W, 4)[1:-1, 1:-1, :3]
    assert np.isfinite(img).all() and img.mean() > 0.01
    # both reprojection branches ran: diffuse and specular first hits
    spec = (feats[:, 3] >> 4) & 3
    assert (spec == 0).any() and (spec != 0).any()
