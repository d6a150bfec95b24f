"""ctypes bindings of the CPU oracle (oracle/lh2o.cpp) and of the reference-kernel harness (oracle/ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from lighthouse2_gb300 import scenes as S

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liblh2o.so")
REF_LIB = os.path.join(HERE, "_ref", "libref.so")
# the Lighthouse 2 source tree, named by the caller (environment variable LH2_REFERENCE); without it the
# reference-kernel harness is not built and the tests that need it are skipped
REFERENCE_TREE = os.environ.get("LH2_REFERENCE", "")

PARAMS_DTYPE = np.dtype([("width", "<i4"), ("height", "<i4"), ("spp", "<i4"), ("maxDepth", "<i4"),
                         ("rrStartDepth", "<i4"), ("samplesTaken", "<i4"), ("cameraR0", "<u4"),
                         ("geometryEpsilon", "<f4"), ("clampValue", "<f4"), ("flags", "<i4"), ("frameSeed", "<u4")])
FILTER_PARAMS_DTYPE = np.dtype([("prevView", S.VIEW_DTYPE), ("j0", "<f4"), ("j1", "<f4"), ("prevj0", "<f4"), ("prevj1", "<f4"),
                                ("clampDirect", "<f4"), ("clampIndirect", "<f4"), ("samplesTaken", "<i4"),
                                ("camIsStationary", "<i4"), ("taa", "<i4")])
RP_NEE, RP_DEPTH_W, RP_FILTER = 1, 2, 4


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def build_ref():
    """Compile the reference's own kernels for the host (only where the reference tree exists)."""
    if not REFERENCE_TREE or not os.path.isdir(os.path.join(REFERENCE_TREE, "lib", "RenderCore_PrimeRef")):
        return None
    build_oracle()
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + REFERENCE_TREE], check=True)
    return REF_LIB


def make_params(width, height, spp=1, max_depth=3, rr_start=1, samples_taken=0, camera_r0=0, eps=1e-3,
                clamp=10.0, flags=RP_NEE, frame_seed=0):
    p = np.zeros((), PARAMS_DTYPE)
    p["width"], p["height"], p["spp"], p["maxDepth"] = width, height, spp, max_depth
    p["rrStartDepth"], p["samplesTaken"], p["cameraR0"] = rr_start, samples_taken, camera_r0
    p["geometryEpsilon"], p["clampValue"], p["flags"], p["frameSeed"] = eps, clamp, flags, frame_seed
    return p


def camera_r0(frame_index_since_restart):
    """R0 of the primary-ray kernel: RandomUInt(camRNGseed) with camRNGseed reset to 0x12345678 on Restart
    (lib/RenderCore_PrimeRef/rendercore.cpp:548,556; lib/platform/system.cpp:50)."""
    s = 0x12345678
    for _ in range(frame_index_since_restart + 1):
        s ^= (s << 13) & 0xFFFFFFFF
        s ^= s >> 17
        s ^= (s << 5) & 0xFFFFFFFF
    return s


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class _Capture(C.Structure):
    _fields_ = [("hits", C.c_void_p), ("seeds", C.c_void_p)]


class Oracle:
    def __init__(self):
        if not os.path.exists(LIB):
            build_oracle()
        self.lib = C.CDLL(LIB)
        L = self.lib
        L.lh2o_create.restype = C.c_void_p
        L.lh2o_destroy.argtypes = [C.c_void_p]
        L.lh2o_set_geometry.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.lh2o_set_instance.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.lh2o_set_materials.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.lh2o_set_textures.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.lh2o_set_lights.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        L.lh2o_set_sky.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.lh2o_finalize.argtypes = [C.c_void_p]
        L.lh2o_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        L.lh2o_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.lh2o_render_ex.argtypes = [C.c_void_p] * 8 + [C.c_int]
        L.lh2o_svgf_frame.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        self.s = L.lh2o_create()
        self._keep = []

    def __del__(self):
        try:
            self.lib.lh2o_destroy(self.s)
        except Exception:
            pass

    def set_scene(self, sc: S.Scene):
        L, s = self.lib, self.s
        for i, m in enumerate(sc.meshes):
            assert L.lh2o_set_geometry(s, i, _p(m.vertices), len(m.vertices), len(m.tris), _p(m.tris)) == 0
        for i, (mi, T) in enumerate(sc.instances):
            T = np.ascontiguousarray(T, np.float32)
            assert L.lh2o_set_instance(s, i, mi, _p(T)) == 0
        texdesc = texture_descs(sc.textures)
        self._keep.append(texdesc)
        assert L.lh2o_set_textures(s, _p(texdesc[0]) if len(sc.textures) else None, len(sc.textures)) == 0
        assert L.lh2o_set_materials(s, _p(sc.materials), len(sc.materials)) == 0
        assert L.lh2o_set_lights(s, _p(sc.tri_lights), len(sc.tri_lights), _p(sc.point_lights), len(sc.point_lights),
                                 _p(sc.spot_lights), len(sc.spot_lights), _p(sc.dir_lights), len(sc.dir_lights)) == 0
        if sc.sky is not None:
            rgb, w, h = sc.sky
            rgb = np.ascontiguousarray(rgb, np.float32)
            assert L.lh2o_set_sky(s, _p(rgb), w, h, None) == 0
        assert L.lh2o_finalize(s) == 0

    def trace(self, rays, mode=0, brute=False, nthreads=0):
        n = len(rays)
        if mode == 0:
            hits = np.zeros(n, S.HIT_DTYPE)
            assert self.lib.lh2o_trace(self.s, _p(rays), n, 0, int(brute), _p(hits), None, nthreads) == 0
            return hits
        occ = np.zeros(n, np.uint32)
        assert self.lib.lh2o_trace(self.s, _p(rays), n, 1, int(brute), None, _p(occ), nthreads) == 0
        return occ

    def render(self, view, params, accum=None, accum64=False, capture=False, nthreads=0, features=None):
        """One frame. LH2G_RP_FILTER frames accumulate 2*W*H pixels (direct, then indirect) and write the SVGF
        features into `features` (an SvgfState, or None)."""
        W, H, spp, D = int(params["width"]), int(params["height"]), int(params["spp"]), int(params["maxDepth"])
        halves = 2 if int(params["flags"]) & RP_FILTER else 1
        if accum is None:
            accum = np.zeros((halves * H * W, 4), np.float32)
        a64 = np.zeros((halves * H * W, 4), np.float64) if accum64 else None
        counters = np.zeros((D, 2), np.uint32)
        cap = None
        hits = seeds = None
        if capture:
            hits = np.zeros(D * W * H * spp, S.HIT_DTYPE)
            seeds = np.zeros(D * W * H * spp, np.uint32)
            cap = _Capture(hits.ctypes.data, seeds.ctypes.data)
        feat = _Features(features.ptr("features"), features.ptr("worldPos"), features.ptr("deltaDepth")) if features is not None else None
        rc = self.lib.lh2o_render_ex(self.s, _p(view), _p(params), _p(accum), _p(a64), _p(counters),
                                     C.byref(cap) if cap is not None else None, C.byref(feat) if feat is not None else None, nthreads)
        assert rc == 0
        out = {"accum": accum, "counters": counters}
        if accum64:
            out["accum64"] = a64
        if capture:
            out["hits"] = hits.reshape(D, -1)
            out["seeds"] = seeds.reshape(D, -1)
        return out


class NrcSpec(C.Structure):
    _fields_ = [("res", C.c_int * 12), ("dense", C.c_int * 12), ("bmin", C.c_float * 3), ("inv", C.c_float * 3)]


class NrcOracle:
    """The radiance cache's encoding, outputs and gradients restated on the CPU (oracle/lh2o.cpp)."""

    def __init__(self, res, dense, bmin, inv):
        if not os.path.exists(LIB):
            build_oracle()
        self.lib = C.CDLL(LIB)
        L = self.lib
        L.lh2o_nrc_encode.argtypes = [C.c_void_p] * 4
        L.lh2o_nrc_forward.argtypes = [C.c_void_p] * 4 + [C.c_longlong, C.c_void_p, C.c_int, C.c_int]
        L.lh2o_nrc_gradients.argtypes = [C.c_void_p] * 5 + [C.c_longlong, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.lh2o_nrc_adam.argtypes = [C.c_void_p] * 4 + [C.c_longlong, C.c_float, C.c_longlong]
        L.lh2o_nrc_forward64.argtypes = [C.c_void_p] * 4 + [C.c_longlong, C.c_void_p]
        self.spec = NrcSpec((C.c_int * 12)(*res), (C.c_int * 12)(*dense), (C.c_float * 3)(*bmin), (C.c_float * 3)(*inv))

    def encode(self, grid, query):
        e = np.zeros(64, np.float32)
        q = np.ascontiguousarray(query, np.float32)
        self.lib.lh2o_nrc_encode(C.byref(self.spec), _p(np.ascontiguousarray(grid, np.float32)), _p(q), _p(e))
        return e

    def forward(self, grid, mlp, queries, emulate=True):
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 16)
        out = np.zeros((len(q), 4), np.float32)
        assert self.lib.lh2o_nrc_forward(C.byref(self.spec), _p(np.ascontiguousarray(grid, np.float32)), _p(np.ascontiguousarray(mlp, np.float32)),
                                         _p(q), len(q), _p(out), int(emulate), 0) == 0
        return out

    def forward64(self, grid, mlp, queries):
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 16)
        out = np.zeros((len(q), 3), np.float64)
        assert self.lib.lh2o_nrc_forward64(C.byref(self.spec), _p(np.ascontiguousarray(grid, np.float32)), _p(np.ascontiguousarray(mlp, np.float32)),
                                           _p(q), len(q), _p(out)) == 0
        return out

    def gradients(self, grid, mlp, queries, targets, emulate=True, with_grid=True):
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 16)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 4)
        gm = np.zeros(len(mlp), np.float64)
        gg = np.zeros(len(grid), np.float64) if with_grid else None
        loss = C.c_double(0)
        assert self.lib.lh2o_nrc_gradients(C.byref(self.spec), _p(np.ascontiguousarray(grid, np.float32)), _p(np.ascontiguousarray(mlp, np.float32)),
                                           _p(q), _p(t), len(q), int(emulate), _p(gm), _p(gg), C.byref(loss)) == 0
        return gm, gg, loss.value

    def adam(self, p, m, v, g, lr, step):
        for a in (p, m, v, g):
            assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
        self.lib.lh2o_nrc_adam(_p(p), _p(m), _p(v), _p(g), len(p), lr, step)


class _Features(C.Structure):
    _fields_ = [("features", C.c_void_p), ("worldPos", C.c_void_p), ("deltaDepth", C.c_void_p)]


SVGF_SLOTS = ["features", "worldPos", "prevWorldPos", "deltaDepth", "motion", "moments", "prevMoments", "shading", "filteredIN",
              "filteredOUT", "prevPixels", "taaPixels", "target"]


class _Svgf(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int)] + [(n, C.c_void_p) for n in SVGF_SLOTS]


class SvgfState:
    """The oracle's SVGF buffers of one W x H target (zeroed, like the GPU core's at allocation). Slot names
    follow the GPU core's: lh2o_svgf_frame swaps the history slots exactly as the core does."""

    def __init__(self, oracle: Oracle, width, height):
        self.oracle, self.W, self.H = oracle, width, height
        n = width * height
        self.arrays = {}
        for name in SVGF_SLOTS:
            dt, comps = (np.uint32, 4) if name == "features" else (np.float32, 2 if name == "motion" else 4)
            self.arrays[name] = np.zeros((n, comps), dt)
        self.slot = {name: name for name in SVGF_SLOTS}       # slot -> array key

    def __getitem__(self, slot):
        return self.arrays[self.slot[slot]]

    def ptr(self, slot):
        return self[slot].ctypes.data

    def frame(self, accum, fparams, nthreads=0):
        st = _Svgf(self.W, self.H, *[self.ptr(n) for n in SVGF_SLOTS])
        assert self.oracle.lib.lh2o_svgf_frame(C.byref(st), _p(np.ascontiguousarray(accum)), _p(np.ascontiguousarray(fparams)),
                                               nthreads) == 0
        by_addr = {self.arrays[k].ctypes.data: k for k in self.arrays}
        self.slot = {n: by_addr[getattr(st, n)] for n in SVGF_SLOTS}


def make_filter_params(prev_view, j0, j1, prevj0, prevj1, samples_taken, cam_is_stationary, taa, clamp_direct=2.5, clamp_indirect=15.0):
    fp = np.zeros((), FILTER_PARAMS_DTYPE)
    fp["prevView"] = prev_view
    fp["j0"], fp["j1"], fp["prevj0"], fp["prevj1"] = j0, j1, prevj0, prevj1
    fp["clampDirect"], fp["clampIndirect"] = clamp_direct, clamp_indirect
    fp["samplesTaken"], fp["camIsStationary"], fp["taa"] = samples_taken, cam_is_stationary, taa
    return fp


TEXDESC_DTYPE = np.dtype([("texels", "<u8"), ("width", "<u4"), ("height", "<u4"), ("flags", "<u4"),
                          ("pixelCount", "<u4"), ("firstPixel", "<u4"), ("MIPlevels", "<u4"), ("storage", "<i4"),
                          ("pad", "<i4")])
assert TEXDESC_DTYPE.itemsize == 40


def texture_descs(textures):
    d = np.zeros(max(1, len(textures)), TEXDESC_DTYPE)
    keep = []
    for i, t in enumerate(textures):
        arr = np.ascontiguousarray(t.texels, np.uint32)
        keep.append(arr)
        d[i]["texels"] = arr.ctypes.data
        d[i]["width"], d[i]["height"] = t.width, t.height
        d[i]["pixelCount"] = len(arr)
        d[i]["MIPlevels"] = 5
    return d, keep


class RefKernels:
    """The reference's PrimeRef kernels compiled for the host (oracle/ref), driven through its own wave loop
    (lib/RenderCore_PrimeRef/rendercore.cpp:551-611) with the oracle answering the ray queries."""

    def __init__(self):
        if build_ref() is None:
            raise FileNotFoundError("reference tree not available")
        self.lib = C.CDLL(REF_LIB)
        L = self.lib
        L.ref_set_scene.argtypes = [C.c_void_p] * 2 + [C.c_void_p, C.c_int] * 4 + [C.c_void_p, C.c_float, C.c_int, C.c_void_p, C.c_int, C.c_int]
        L.ref_generate.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_float, C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.ref_shade.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int]
        L.ref_finalize_connections.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_next_counters.argtypes = [C.c_void_p]
        L.ref_init_counters.argtypes = [C.c_int]
        L.ref_wanghash.restype = C.c_uint32
        L.ref_random_float.restype = C.c_float
        L.ref_random_float.argtypes = [C.c_void_p]
        L.ref_pack_normal.restype = C.c_uint32
        L.ref_pack_normal.argtypes = [C.c_void_p]
        L.ref_unpack_normal.argtypes = [C.c_uint32, C.c_void_p]
        L.ref_random_barycentrics.argtypes = [C.c_float, C.c_void_p]
        L.ref_diffuse_cos.argtypes = [C.c_float, C.c_float, C.c_void_p]
        L.ref_tangent2world.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_consistent_normal.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
        L.ref_invert4x4.argtypes = [C.c_void_p, C.c_void_p]

    def render(self, oracle: Oracle, sc: S.Scene, view, params):
        """One frame through the reference's kernels; returns per-pixel accumulator and per-depth counters.
        Connections of the last wave are traced too (as the OptiX7 core's final shadow pass does,
        lib/rendercore_optix7/rendercore.cpp:919-922); the PrimeRef loop leaves them untraced only because its
        compile-time MAXPATHLENGTH of 64 is never reached."""
        L = self.lib
        W, H, spp, D = int(params["width"]), int(params["height"]), int(params["spp"]), int(params["maxDepth"])
        eps = float(params["geometryEpsilon"])
        nee = int(params["flags"]) & RP_NEE
        inst = np.zeros((len(sc.instances), 20), np.float32)
        keep = []
        for i, (mi, T) in enumerate(sc.instances):
            tris = sc.meshes[mi].tris
            inv = np.zeros(16, np.float32)
            L.ref_invert4x4(_p(np.ascontiguousarray(T, np.float32).reshape(-1)), _p(inv))
            inst[i].view(np.uint64)[0] = tris.ctypes.data
            inst[i, 4:] = inv
        packed = pack_materials(oracle, sc)
        texels = np.concatenate([t.texels for t in sc.textures]).astype(np.uint32) if sc.textures else np.zeros(16, np.uint32)
        sky4, sw, sh = None, 0, 0
        if sc.sky is not None:
            rgb, sw, sh = sc.sky
            sky4 = np.zeros((sw * sh, 4), np.float32)
            sky4[:, :3] = np.asarray(rgb, np.float32).reshape(-1, 3)
        keep += [inst, packed, texels, sky4]
        self._keep = keep
        L.ref_set_scene(_p(inst), _p(packed), _p(sc.tri_lights), len(sc.tri_lights), _p(sc.point_lights), len(sc.point_lights),
                        _p(sc.spot_lights), len(sc.spot_lights), _p(sc.dir_lights), len(sc.dir_lights), _p(texels), eps, D,
                        _p(sky4), sw, sh)
        P = W * H * spp
        rays = [np.zeros((P, 8), np.float32), np.zeros((P, 8), np.float32)]
        ps = [np.zeros((2 * P, 4), np.float32), np.zeros((2 * P, 4), np.float32)]
        conn = np.zeros((P, 8), np.float32)
        pot = np.zeros((P, 4), np.float32)
        acc = np.zeros((W * H, 4), np.float32)
        v = view
        right = (v["p2"] - v["p1"]).astype(np.float32)
        up = (v["p3"] - v["p1"]).astype(np.float32)
        L.ref_generate(_p(rays[0]), _p(ps[0]), int(params["cameraR0"]), int(params["samplesTaken"]), _p(v["pos"].copy()),
                       _p(right), _p(up), float(v["aperture"]), _p(v["p1"].copy()), W, H, spp)
        L.ref_init_counters(P)
        count, cin = P, 0
        counters = np.zeros((D, 2), np.uint32)
        tt = np.zeros(P, np.float32); ii = np.zeros(P, np.int32); pp = np.zeros(P, np.int32)
        uu = np.zeros(P, np.float32); vv = np.zeros(P, np.float32)
        isect = np.zeros(P, np.dtype([("t", "<f4"), ("triid", "<i4"), ("instid", "<i4"), ("u", "<f4"), ("v", "<f4")]))
        for pl in range(1, D + 1):
            r = np.ascontiguousarray(rays[cin][:count])
            oracle.lib.lh2o_trace_raw(oracle.s, _p(r), count, _p(tt), _p(ii), _p(pp), _p(uu), _p(vv), 0)
            isect["t"][:count], isect["triid"][:count], isect["instid"][:count] = tt[:count], pp[:count], ii[:count]
            isect["u"][:count], isect["v"][:count] = uu[:count], vv[:count]
            R0 = (int(params["samplesTaken"]) * 7907 + pl * 91771) & 0xFFFFFFFF
            L.ref_shade(count, _p(acc), _p(rays[cin]), _p(ps[cin]), _p(isect), _p(rays[1 - cin]), _p(ps[1 - cin]),
                        _p(conn), _p(pot), R0, int(params["samplesTaken"]), pl, W, H, float(v["spreadAngle"]), nee)
            c3 = np.zeros(3, np.uint32)
            L.ref_next_counters(_p(c3))
            counters[pl - 1] = c3[:2]
            if c3[1] > 0:
                occ = oracle.trace(np.ascontiguousarray(conn[:c3[1]]).view(S.RAY_DTYPE).reshape(-1), mode=1)
                bits = np.zeros((c3[1] + 31) // 32, np.uint32)
                idx = np.nonzero(occ)[0]
                np.bitwise_or.at(bits, idx >> 5, (np.uint32(1) << (idx & 31).astype(np.uint32)))
                L.ref_finalize_connections(int(c3[1]), _p(acc), _p(bits), _p(pot))
            count, cin = int(c3[0]), 1 - cin
            if count == 0:
                break
        return {"accum": acc, "counters": counters}


def pack_materials(oracle: Oracle, sc: S.Scene):
    first, wh, off = [], [], 0
    for t in sc.textures:
        first.append(off); wh += [t.width, t.height]; off += len(t.texels)
    first = np.array(first or [0], np.uint32); wh = np.array(wh or [0, 0], np.uint32)
    out = np.zeros((len(sc.materials), 32), np.uint32)
    fn = oracle.lib.lh2o_pack_material
    fn.argtypes = [C.c_void_p] * 4
    for i in range(len(sc.materials)):
        m = np.ascontiguousarray(sc.materials[i:i + 1])
        fn(_p(m), _p(first), _p(wh), out[i].ctypes.data_as(C.c_void_p))
    return out
