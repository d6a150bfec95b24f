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
                         ("geometryEpsilon", "<f4"), ("clampValue", "<f4"), ("flags", "<i4"), ("frameSeed", "<u4"),
                         ("shift", "<u4"), ("rowBegin", "<i4"), ("rowCount", "<i4")])
FILTER_PARAMS_DTYPE = np.dtype([("prevView", S.VIEW_DTYPE), ("j0", "<f4"), ("j1", "<f4"), ("prevj0", "<f4"), ("prevj1", "<f4"),
                                ("clampDirect", "<f4"), ("clampIndirect", "<f4"), ("samplesTaken", "<i4"),
                                ("camIsStationary", "<i4"), ("taa", "<i4")])
RP_NEE, RP_DEPTH_W, RP_FILTER, RP_OPTIX7, RP_ADAPTIVE, RP_DISNEY, RP_LIGHTTREE = 1, 2, 4, 16, 32, 64, 128


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
                clamp=10.0, flags=RP_NEE, frame_seed=0, shift=0):
    p = np.zeros((), PARAMS_DTYPE)
    p["width"], p["height"], p["spp"], p["maxDepth"] = width, height, spp, max_depth
    p["rrStartDepth"], p["samplesTaken"], p["cameraR0"] = rr_start, samples_taken, camera_r0
    p["geometryEpsilon"], p["clampValue"], p["flags"], p["frameSeed"] = eps, clamp, flags, frame_seed
    p["shift"] = shift
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
        L.lh2o_set_blue_noise.argtypes = [C.c_void_p] * 4
        L.lh2o_render_adaptive.argtypes = [C.c_void_p] * 12 + [C.c_int]
        L.lh2o_raster.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
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
        self.set_blue_noise(sc.blue_noise)
        assert L.lh2o_finalize(s) == 0

    def light_tree(self):
        """The light tree lh2o_set_lights built for the scene's lights (LIGHT_TREE_DTYPE records, record 0 the root)."""
        fn = self.lib.lh2o_light_tree
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        n = fn(self.s, None, 0)
        if n <= 0:
            return np.zeros(0, LIGHT_TREE_DTYPE)
        out = np.zeros(n, LIGHT_TREE_DTYPE)
        assert fn(self.s, _p(out), n) == n
        return out

    def set_blue_noise(self, tables):
        if tables is None:
            assert self.lib.lh2o_set_blue_noise(self.s, None, None, None) == 0
            return
        t = [np.ascontiguousarray(x, np.uint8) for x in tables]
        assert [len(x) for x in t] == [65536, 131072, 131072]
        assert self.lib.lh2o_set_blue_noise(self.s, _p(t[0]), _p(t[1]), _p(t[2])) == 0

    def render_adaptive(self, view, params, accum, dev_scale, capture=False, nthreads=0):
        """One PrimeAdaptive frame; accum (W*H float4) is updated in place. Returns the new devScale, the frame,
        per-wave counters, the second wave's path count and the intermediate buffers."""
        W, H, spp, D = int(params["width"]), int(params["height"]), int(params["spp"]), int(params["maxDepth"])
        P = W * H * spp
        frame = np.zeros((W * H, 4), np.float32)
        ds = np.array([dev_scale], np.float32)
        counters = np.zeros((2 * D, 2), np.uint32)
        n2 = np.zeros(1, np.uint32)
        facc = np.zeros((P, 4), np.float32)
        feat = np.zeros((P, 4), np.float32)
        dev = np.zeros(W * H, np.float32)
        cap = hits = seeds = None
        if capture:
            hits = np.zeros(D * P, S.HIT_DTYPE)
            seeds = np.zeros(D * P, np.uint32)
            cap = _Capture(hits.ctypes.data, seeds.ctypes.data)
        assert self.lib.lh2o_render_adaptive(self.s, _p(view), _p(params), _p(accum), _p(frame), _p(ds), _p(counters), _p(n2), _p(facc),
                                             _p(feat), _p(dev), C.byref(cap) if cap is not None else None, nthreads) == 0
        out = {"dev_scale": float(ds[0]), "frame": frame, "counters": counters, "adaptive_paths": int(n2[0]), "frame_acc": facc,
               "features": feat, "deviation": dev}
        if capture:
            out["hits"], out["seeds"] = hits.reshape(D, -1), seeds.reshape(D, -1)
        return out

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
        if int(params["rowCount"]) > 0:   # a band of rows: its pixels only
            H = int(params["rowCount"])
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


    def raster(self, view, W, H):
        """One SoftRasterizer frame: W*H RGBA8 pixels (uint32), the z-buffer (float32) and the depth-test passes."""
        px = np.zeros(W * H, np.uint32)
        zb = np.zeros(W * H, np.float32)
        frags = np.zeros(1, np.uint64)
        assert self.lib.lh2o_raster(self.s, _p(view), W, H, _p(px), _p(zb), _p(frags)) == 0
        return {"pixels": px, "zbuffer": zb, "fragments": int(frags[0])}


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


def _xorshift(x):
    x ^= (x << 13) & 0xFFFFFFFF
    x ^= x >> 17
    x ^= (x << 5) & 0xFFFFFFFF
    return x


def _sky_with_small(sc):
    """sky float4 pixels followed by the 64x scaled-down copy (RenderCore::SetSkyData, rendercore_optix7/
    rendercore.cpp:726-737): each tile summed in float32, row by row, then scaled by 1/4096"""
    if sc.sky is None:
        return None, 0, 0
    rgb, w, h = sc.sky
    px = np.asarray(rgb, np.float32).reshape(h, w, 3)
    sw, sh = w >> 6, h >> 6
    small = np.zeros((sh * sw, 4), np.float32)
    for y in range(sh):
        for x in range(sw):
            tile = px[y * 64:(y + 1) * 64, x * 64:(x + 1) * 64].reshape(-1, 3)
            small[x + y * sw, :3] = np.add.accumulate(tile, axis=0, dtype=np.float32)[-1] * np.float32(1.0 / 4096)
    sky4 = np.zeros((w * h + sw * sh, 4), np.float32)
    sky4[:w * h, :3] = px.reshape(-1, 3)
    sky4[w * h:] = small
    return sky4, w, h


def _ref_scene(lib, oracle, sc):
    inst = np.zeros((len(sc.instances), 20), np.float32)
    for i, (mi, T) in enumerate(sc.instances):
        inv = np.zeros(16, np.float32)
        lib.ref_invert4x4(_p(np.ascontiguousarray(T, np.float32).reshape(-1)), _p(inv))
        inst[i].view(np.uint64)[0] = sc.meshes[mi].tris.ctypes.data
        inst[i, 4:] = inv
    packed = pack_materials(oracle, sc)
    texels = np.concatenate([t.texels for t in sc.textures]).astype(np.uint32) if sc.textures else np.zeros(16, np.uint32)
    sky4, sw, sh = _sky_with_small(sc)
    return inst, packed, texels, sky4, sw, sh


def expand_blue_noise(tables):
    """the blue-noise tables as the OptiX 7 core expands them (rendercore.cpp:247-256), plus 64 zero entries"""
    bn = np.zeros(65536 * 5 + 64, np.uint32)
    bn[:65536] = tables[0]
    bn[65536:65536 + 131072] = tables[1]
    bn[3 * 65536:3 * 65536 + 131072] = tables[2]
    return bn


def reference_blue_noise():
    """the reference's own tables (common_bluenoise.h, compiled by path into the harness), as three byte arrays"""
    lib = C.CDLL(REF_LIB)
    out = []
    for name, n in (("ref_bluenoise_sobol", 65536), ("ref_bluenoise_scrambling", 131072), ("ref_bluenoise_ranking", 131072)):
        fn = getattr(lib, name)
        fn.restype = C.POINTER(C.c_uint8)
        out.append(np.ctypeslib.as_array(fn(), shape=(n,)).copy())
    return tuple(out)


LIGHT_TREE_DTYPE = np.dtype([("light", "<i4"), ("left", "<i4"), ("right", "<i4"), ("intensity", "<f4"), ("bmin", "<f4", 4),
                             ("bmax", "<f4", 4), ("N", "<f4", 3), ("parent", "<i4")])


def ref_light_tree(lib, tri, point, spot):
    """The light tree the reference's RenderCore::UpdateLightTree (rendercore_optix7/rendercore.cpp:625-680, compiled
    here by oracle/ref) builds for these lights: LIGHT_TREE_DTYPE records, record 0 the root."""
    fn = lib.ref_light_tree
    fn.argtypes = [C.c_void_p, C.c_int] * 3 + [C.c_void_p, C.c_int]
    cap = 2 * (len(tri) + len(point) + len(spot))
    out = np.zeros(max(cap, 1), LIGHT_TREE_DTYPE)
    n = fn(_p(tri) if len(tri) else None, len(tri), _p(point) if len(point) else None, len(point),
           _p(spot) if len(spot) else None, len(spot), _p(out), cap)
    assert n >= 0, "ref_light_tree: capacity"
    return out[:n]


class RefOptix7(RefKernels):
    """The OptiX 7 core's shading kernel and ray generation compiled for the host (oracle/ref/ref_optix7.cpp), driven
    through the core's wave loop (lib/rendercore_optix7/rendercore.cpp:874-922) with the oracle answering the ray
    queries. The connection buffer is made large enough that the loop's early flush (rendercore.cpp:906-913) never
    triggers."""

    def __init__(self, disney=False, light_tree=False):
        """disney: the kernel built with the Disney BSDF (ref_o7d_*) instead of lambert.h (ref_o7_*); light_tree: the
        kernel built with its light-tree calls and LIGHTTREE defined (ref_o7t_*, Lambert BSDF), reading the tree
        the reference's own UpdateLightTree builds (ref_light_tree)."""
        super().__init__()
        vp, i, f, u = C.c_void_p, C.c_int, C.c_float, C.c_uint32
        pre = "ref_o7t_" if light_tree else ("ref_o7d_" if disney else "ref_o7_")
        self.light_tree = light_tree
        sig = {"set_scene": [vp] * 2 + [vp, i] * 4 + [vp, f, f, i, vp, i, i, vp], "init_counters": [i], "next_counters": [],
               "counters": [vp], "generate": [vp, i, i, i, i, i, vp, f, vp, vp, vp, f], "shade": [i, vp, vp, vp, vp, u, u, i, i, i, i, i, f, i],
               "finalize_connections": [i, vp, vp, vp, i], "bluenoise4": [vp, i, i, i, i, vp], "set_shadow_count": [u]}
        if light_tree:
            sig["set_light_tree"] = [vp]

        class _Fns:
            pass
        self.fn = _Fns()
        for name, args in sig.items():
            fn = getattr(self.lib, pre + name)
            fn.argtypes = args
            setattr(self.fn, name, fn)

    def render(self, oracle: Oracle, sc: S.Scene, view, params, accum=None):
        """One frame; returns the accumulator, per path length the extension and connection counts, and whether the
        loop flushed its connection buffer early (pathCount + shadowRays >= 2 P: connections then reach the
        accumulator before later path lengths' terms)."""
        L = self.fn
        W, H, spp, D = int(params["width"]), int(params["height"]), int(params["spp"]), int(params["maxDepth"])
        P = W * H * spp
        eps = float(params["geometryEpsilon"])
        nee = int(params["flags"]) & RP_NEE
        inst, packed, texels, sky4, sw, sh = _ref_scene(self.lib, oracle, sc)
        bn = expand_blue_noise(sc.blue_noise)
        self._keep = [inst, packed, texels, sky4, bn]
        L.set_scene(_p(inst), _p(packed), _p(sc.tri_lights), len(sc.tri_lights), _p(sc.point_lights), len(sc.point_lights),
                           _p(sc.spot_lights), len(sc.spot_lights), _p(sc.dir_lights), len(sc.dir_lights), _p(texels), eps,
                           float(params["clampValue"]), D, _p(sky4), sw, sh, _p(bn))
        if self.light_tree:
            tree = ref_light_tree(self.lib, sc.tri_lights, sc.point_lights, sc.spot_lights)
            self._keep.append(tree)
            L.set_light_tree(_p(tree))
        ps = np.zeros((3 * P, 4), np.float32)
        hits = np.zeros((P, 4), np.float32)
        conn = np.zeros((6 * P, 4), np.float32)           # O4, D4, E4 at 0, 2 P, 4 P (rendercore.cpp:312)
        acc = np.zeros((W * H, 4), np.float32) if accum is None else accum
        v = view
        right = (v["p2"] - v["p1"]).astype(np.float32)
        up = (v["p3"] - v["p1"]).astype(np.float32)
        shift = int(params["shift"])
        L.generate(_p(ps), W, H, spp, int(params["samplesTaken"]), shift - (1 << 32) if shift >= 1 << 31 else shift,
                          _p(v["pos"].copy()), float(v["aperture"]), _p(right), _p(up), _p(v["p1"].copy()), float(v["distortion"]))
        L.init_counters(P)
        counters = np.zeros((D, 2), np.uint32)
        draw, count, seen, flushed = int(params["cameraR0"]), P, 0, False
        c2 = np.zeros(2, np.uint32)

        def connect(n):
            rays = np.zeros(n, S.RAY_DTYPE)
            rays["o"], rays["d"] = conn[:n, :3], conn[2 * P:2 * P + n, :3]
            rays["tmin"], rays["tmax"] = eps, conn[2 * P:2 * P + n, 3]
            occ = oracle.trace(rays, mode=1).astype(np.uint32)
            L.finalize_connections(n, _p(acc), _p(conn), _p(occ), P)

        for pl in range(1, D + 1):
            if pl > 1:
                L.next_counters()
                draw = _xorshift(draw)
            rays = np.zeros(count, S.RAY_DTYPE)
            rays["o"], rays["d"] = ps[:count, :3], ps[P:P + count, :3]
            rays["tmin"], rays["tmax"] = eps, 1e34
            h = oracle.trace(rays, mode=0)
            hits[:count, 0] = h["bary"].view(np.float32)
            hits[:count, 1] = h["inst"].view(np.float32)
            hits[:count, 2] = h["prim"].view(np.float32)
            hits[:count, 3] = h["t"]
            L.shade(count, _p(acc), _p(ps), _p(hits), _p(conn), (draw + pl * 91771) & 0xFFFFFFFF, shift,
                           int(params["samplesTaken"]), pl, W, H, spp, float(v["spreadAngle"]), nee)
            L.counters(_p(c2))
            counters[pl - 1] = (c2[0], c2[1] - seen)
            seen, count = int(c2[1]), int(c2[0])
            if count == 0:
                break
            if count + seen >= 2 * P and seen > 0:   # rendercore.cpp:906-913
                connect(seen)
                flushed = True
                L.set_shadow_count(0)
                seen = 0
        if seen:
            connect(seen)
        return {"accum": acc, "counters": counters, "flushed": flushed}

    def bluenoise4(self, bn, x, y, sample, dim):
        out = np.zeros(4, np.float32)
        self.fn.bluenoise4(_p(bn), x, y, sample, dim, _p(out))
        return out


class RefAdaptive(RefKernels):
    """The PrimeAdaptive core's kernels compiled for the host (oracle/ref/ref_adaptive.cpp), driven through the
    core's RenderImpl and FinalizeRender (lib/RenderCore_PrimeAdaptive/rendercore.cpp:600-755) with the oracle
    answering the ray queries. Launches run their threads in index order, so the adaptive ray generation's
    compaction gives slots in thread order."""

    ISECT = np.dtype([("t", "<f4"), ("triid", "<i4"), ("instid", "<i4"), ("u", "<f4"), ("v", "<f4")])

    def __init__(self):
        super().__init__()
        L = self.lib
        vp, i, f, u = C.c_void_p, C.c_int, C.c_float, C.c_uint32
        L.ref_ad_set_scene.argtypes = [vp] * 2 + [vp, i] * 4 + [vp, f, f, i, vp, i, i]
        L.ref_ad_init_extend.argtypes = [i]
        L.ref_ad_counters.argtypes = [vp]
        L.ref_ad_set_active.argtypes = [u]
        L.ref_ad_set_shadow.argtypes = [u]
        L.ref_ad_generate.argtypes = [vp, vp, u, vp, i, vp, f, vp, vp, vp, f, i, i, i]
        L.ref_ad_generate_adaptive.argtypes = [vp, vp, vp, u, i, vp, vp, f, vp, vp, vp, f, i, i, i]
        L.ref_ad_shade.argtypes = [i, vp, vp, vp, vp, vp, vp, vp, vp, vp, u, u, vp, i, i, i, i, f, i]
        L.ref_ad_finalize_connections.argtypes = [i, vp, vp, vp]
        L.ref_ad_estimate_variance.argtypes = [vp, vp, vp, f, i, i, i]
        L.ref_ad_finalize.argtypes = [vp, vp, vp, i, i, i, i]

    def render(self, oracle: Oracle, sc: S.Scene, view, params, accum, dev_scale):
        """One frame: accum (W*H float4) is updated in place. Returns the new devScale, the frame, the per-wave
        counters, the second wave's path count, the intermediate buffers and whether a wave loop flushed its
        connection buffer early (rendercore.cpp:636-645)."""
        L, O = self.lib, oracle.lib
        W, H, spp, D = int(params["width"]), int(params["height"]), int(params["spp"]), int(params["maxDepth"])
        P = W * H * spp
        eps = float(params["geometryEpsilon"])
        nee = int(params["flags"]) & RP_NEE
        st = int(params["samplesTaken"])
        shift = int(params["shift"])
        inst, packed, texels, sky4, sw, sh = _ref_scene(L, oracle, sc)
        bn = expand_blue_noise(sc.blue_noise)
        L.ref_ad_set_scene(_p(inst), _p(packed), _p(sc.tri_lights), len(sc.tri_lights), _p(sc.point_lights), len(sc.point_lights),
                           _p(sc.spot_lights), len(sc.spot_lights), _p(sc.dir_lights), len(sc.dir_lights), _p(texels), eps,
                           float(params["clampValue"]), D, _p(sky4), sw, sh)
        rays = [np.zeros((P, 8), np.float32), np.zeros((P, 8), np.float32)]
        ps = [np.zeros((2 * P, 4), np.float32), np.zeros((2 * P, 4), np.float32)]
        conn = np.zeros((2 * P, 8), np.float32)
        pot = np.zeros((2 * P, 4), np.float32)
        isect = np.zeros(P, self.ISECT)
        facc = np.zeros((P, 4), np.float32)
        feat = np.zeros((P, 4), np.float32)
        self._keep = [inst, packed, texels, sky4, bn, rays, ps, conn, pot, isect, facc, feat]
        v = view
        right = (v["p2"] - v["p1"]).astype(np.float32)
        up = (v["p3"] - v["p1"]).astype(np.float32)
        pos, p1 = v["pos"].copy(), v["p1"].copy()
        counters = np.zeros((2 * D, 2), np.uint32)
        c3 = np.zeros(3, np.uint32)
        tt = np.zeros(P, np.float32); ii = np.zeros(P, np.int32); pp = np.zeros(P, np.int32)
        uu = np.zeros(P, np.float32); vv = np.zeros(P, np.float32)
        flushed = [False]

        def connect():
            L.ref_ad_counters(_p(c3))
            n = int(c3[2])
            if n == 0:
                return
            occ = oracle.trace(np.ascontiguousarray(conn[:n]).view(S.RAY_DTYPE).reshape(-1), mode=1)
            bits = np.zeros((n + 31) // 32, np.uint32)
            idx = np.nonzero(occ)[0]
            np.bitwise_or.at(bits, idx >> 5, (np.uint32(1) << (idx & 31).astype(np.uint32)))
            L.ref_ad_finalize_connections(n, _p(facc), _p(bits), _p(pot))

        def wave_loop(count, cin, R0of, passv, row):
            seen = 0
            for pl in range(1, D + 1):
                r = np.ascontiguousarray(rays[cin][:count])
                O.lh2o_trace_raw(oracle.s, _p(r), count, _p(tt), _p(ii), _p(pp), _p(uu), _p(vv), 0)
                isect["t"][:count], isect["triid"][:count], isect["instid"][:count] = tt[:count], pp[:count], ii[:count]
                isect["u"][:count], isect["v"][:count] = uu[:count], vv[:count]
                L.ref_ad_shade(count, _p(facc), _p(feat), _p(rays[cin]), _p(ps[cin]), _p(isect), _p(rays[1 - cin]), _p(ps[1 - cin]),
                               _p(conn), _p(pot), R0of(pl) & 0xFFFFFFFF, shift, _p(bn), passv, pl, W, H, float(v["spreadAngle"]), nee)
                L.ref_ad_counters(_p(c3))
                counters[row + pl - 1] = (c3[1], int(c3[2]) - seen)
                seen = int(c3[2])
                if pl >= D:
                    break
                count, cin = int(c3[1]), 1 - cin
                if int(c3[2]) + count >= 2 * P:
                    connect()
                    L.ref_ad_set_shadow(0)
                    seen = 0
                    flushed[0] = True
                L.ref_ad_next()
            connect()
            return cin

        # first wave (rendercore.cpp:606-658)
        L.ref_ad_init_extend(P)
        L.ref_ad_generate(_p(rays[0]), _p(ps[0]), int(params["cameraR0"]), _p(bn), st, _p(pos), float(v["aperture"]), _p(right), _p(up), _p(p1),
                          float(v["distortion"]), W, H, spp)
        cin = wave_loop(P, 0, lambda pl: st * 7907 + pl * 91771, st, 0)
        # variance estimate and adaptive rays (rendercore.cpp:663-680)
        dev = np.zeros(W * H, np.float32)
        L.ref_ad_estimate_variance(_p(facc), _p(feat), _p(dev), float(np.float32(dev_scale)), W, H, spp)
        feat_wave1, facc_wave1 = feat.copy(), facc.copy()
        L.ref_ad_init_stage2()
        L.ref_ad_generate_adaptive(_p(dev), _p(rays[cin]), _p(ps[cin]), int(params["frameSeed"]), st, _p(bn), _p(pos), float(v["aperture"]),
                                   _p(right), _p(up), _p(p1), float(v["distortion"]), W, H, spp)
        L.ref_ad_counters(_p(c3))
        count = int(c3[0])
        budget = np.float32(W * H * spp)
        if np.float32(count) > budget:
            count = int(budget)
            L.ref_ad_set_active(count)
        ds = np.float32(dev_scale)
        fc = np.float32(count)
        if fc > np.float32(0.98) * budget:
            ds = np.float32(ds * np.float32(0.92))
        elif fc > np.float32(0.96) * budget:
            ds = np.float32(ds * np.float32(0.98))
        elif fc < np.float32(0.91) * budget:
            ds = np.float32(ds * np.float32(1.08))
        elif fc < np.float32(0.94) * budget:
            ds = np.float32(ds * np.float32(1.02))
        # second wave (rendercore.cpp:682-713)
        wave_loop(count, cin, lambda pl: st * 59071 + pl * 31771, st + spp, D)
        # FinalizeRender (rendercore.cpp:749-755)
        frame = np.zeros((W * H, 4), np.float32)
        L.ref_ad_finalize(_p(facc), _p(accum), _p(frame), W, H, st + spp, spp)
        return {"dev_scale": float(ds), "frame": frame, "counters": counters, "adaptive_paths": count, "frame_acc": facc,
                "frame_acc_wave1": facc_wave1, "features": feat_wave1, "deviation": dev, "flushed": flushed[0]}


class RefRaster:
    """The reference's SoftRasterizer core compiled for the host (oracle/ref/ref_raster.cpp), driven through its own
    RenderCore methods (lib/RenderCore_SoftRasterizer/rendercore.cpp)."""

    def __init__(self):
        if build_ref() is None:
            raise FileNotFoundError("reference tree not available")
        self.lib = C.CDLL(REF_LIB)
        self.lib.ref_raster.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]

    def raster(self, sc: S.Scene, view, W, H):
        nm = len(sc.meshes)
        tri_count = np.array([len(m.tris) for m in sc.meshes], np.int32)
        verts = [np.ascontiguousarray(m.vertices, np.float32) for m in sc.meshes]
        tris = [np.ascontiguousarray(m.tris) for m in sc.meshes]
        vp = (C.c_void_p * max(1, nm))(*[v.ctypes.data for v in verts])
        tp = (C.c_void_p * max(1, nm))(*[t.ctypes.data for t in tris])
        inst_mesh = np.array([mi for mi, _ in sc.instances], np.int32)
        inst_t = np.ascontiguousarray(np.array([np.asarray(T, np.float32).reshape(16) for _, T in sc.instances], np.float32).reshape(-1))
        texdesc, keep = texture_descs(sc.textures)
        px = np.zeros(W * H, np.uint32)
        zb = np.zeros(W * H, np.float32)
        rc = self.lib.ref_raster(W, H, nm, _p(tri_count), C.cast(vp, C.c_void_p), C.cast(tp, C.c_void_p), len(sc.instances), _p(inst_mesh),
                                 _p(inst_t), len(sc.materials), _p(sc.materials), len(sc.textures), _p(texdesc), _p(view), _p(px), _p(zb))
        assert rc == 0
        return {"pixels": px, "zbuffer": zb}


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
