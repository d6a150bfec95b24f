"""Python face of the GB300 render core: ctypes over the C ABI of include/lh2g.h.

The methods mirror the Lighthouse 2 RenderCore plugin interface (lib/RenderSystem/core_api_base.h:81-119):
SetGeometry / SetInstance / FinalizeInstances / SetMaterials / SetTextures / SetLights / SetSkyData / Setting /
SetTarget / Render / GetCoreStats, plus the ray-query entry points. Every call goes to the CUDA library; there is
no fallback: if libRenderCore_GB300.so is missing or cannot load, constructing a core raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import scenes as S

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libRenderCore_GB300.so")

PARAMS_DTYPE = np.dtype([("width", "<i4"), ("height", "<i4"), ("spp", "<i4"), ("maxDepth", "<i4"),
                         ("rrStartDepth", "<i4"), ("samplesTaken", "<i4"), ("cameraR0", "<u4"),
                         ("geometryEpsilon", "<f4"), ("clampValue", "<f4"), ("flags", "<i4"), ("frameSeed", "<u4"),
                         ("shift", "<u4"), ("rowBegin", "<i4"), ("rowCount", "<i4")])
FILTER_PARAMS_DTYPE = np.dtype([("prevView", S.VIEW_DTYPE), ("j0", "<f4"), ("j1", "<f4"), ("prevj0", "<f4"), ("prevj1", "<f4"),
                                ("clampDirect", "<f4"), ("clampIndirect", "<f4"), ("samplesTaken", "<i4"),
                                ("camIsStationary", "<i4"), ("taa", "<i4")])
TEXDESC_DTYPE = np.dtype([("texels", "<u8"), ("width", "<u4"), ("height", "<u4"), ("flags", "<u4"),
                          ("pixelCount", "<u4"), ("firstPixel", "<u4"), ("MIPlevels", "<u4"), ("storage", "<i4"),
                          ("pad", "<i4")])
STATS_FIELDS = ["totalRays", "totalExtensionRays", "totalShadowRays", "primaryRayCount", "bounce1RayCount", "deepRayCount",
                "renderTime", "traceTime0", "traceTime1", "traceTimeX", "shadowTraceTime", "shadeTime", "filterTime",
                "bvhBuildTime", "SMcount", "ccMajor", "ccMinor", "VRAM", "probedInstid", "probedTriid", "probedDist",
                "deviceStatus"]
STATS_DTYPE = np.dtype([(f, "<u4") for f in STATS_FIELDS[:6]] + [(f, "<f4") for f in STATS_FIELDS[6:14]] +
                       [(f, "<u4") for f in STATS_FIELDS[14:18]] + [("probedInstid", "<i4"), ("probedTriid", "<i4"),
                                                                    ("probedDist", "<f4"), ("deviceStatus", "<u4")])
RP_NEE, RP_DEPTH_W, RP_FILTER, RP_OPTIX7, RP_ADAPTIVE, RP_DISNEY, RP_LIGHTTREE = 1, 2, 4, 16, 32, 64, 128
# one light-tree record (lh2g_build_light_tree; the device LightCluster of common_classes.h:522-527)
LIGHT_TREE_DTYPE = np.dtype([("light", "<i4"), ("left", "<i4"), ("right", "<i4"), ("intensity", "<f4"), ("bmin", "<f4", 4),
                             ("bmax", "<f4", 4), ("N", "<f4", 3), ("parent", "<i4")])
# filter buffer slots (LH2G_FB_*): name -> (index, element dtype, components per pixel)
FILTER_SLOTS = {"features": (0, np.uint32, 4), "worldPos": (1, np.float32, 4), "prevWorldPos": (2, np.float32, 4),
                "deltaDepth": (3, np.float32, 4), "motion": (4, np.float32, 2), "moments": (5, np.float32, 4),
                "prevMoments": (6, np.float32, 4), "shading": (7, np.float32, 4), "filteredIN": (8, np.float32, 4),
                "filteredOUT": (9, np.float32, 4), "prevPixels": (10, np.float32, 4), "accum": (11, np.float32, 4)}
C_API = ["lh2g_create", "lh2g_destroy", "lh2g_last_error", "lh2g_set_geometry", "lh2g_set_instance", "lh2g_finalize_instances",
         "lh2g_set_materials", "lh2g_pack_materials", "lh2g_set_textures", "lh2g_set_lights", "lh2g_set_sky", "lh2g_setting",
         "lh2g_set_target", "lh2g_set_probe", "lh2g_render", "lh2g_render_ex", "lh2g_render_to_host", "lh2g_wait", "lh2g_get_stats",
         "lh2g_get_framebuffer", "lh2g_read_framebuffer", "lh2g_read_accumulator", "lh2g_trace", "lh2g_trace_host",
         "lh2g_get_stream", "lh2g_enable_launch_timing", "lh2g_get_launch_times", "lh2g_get_traversal_stats",
         "lh2g_render_noalloc", "lh2g_filter", "lh2g_read_filter_buffer", "lh2g_get_last_filter_frame",
         "lh2g_server_create", "lh2g_server_destroy", "lh2g_server_last_error", "lh2g_server_add_scene", "lh2g_server_submit_render",
         "lh2g_server_submit_trace", "lh2g_server_wait", "lh2g_server_release", "lh2g_server_get_stats", "lh2g_server_setting",
         "lh2g_nrc_create", "lh2g_nrc_destroy", "lh2g_nrc_last_error", "lh2g_nrc_get_spec", "lh2g_nrc_set_params", "lh2g_nrc_get_params",
         "lh2g_nrc_get_grads", "lh2g_nrc_infer", "lh2g_nrc_train", "lh2g_nrc_apply_update", "lh2g_nrc_infer_counted", "lh2g_nrc_train_counted",
         "lh2g_nrc_last_loss", "lh2g_nrc_wait_selftest", "lh2g_render_nrc", "lh2g_nrc_infer_host", "lh2g_nrc_train_host",
         "lh2g_set_blue_noise", "lh2g_render_adaptive", "lh2g_set_adaptive_scale", "lh2g_raster_render", "lh2g_raster_pixels_device", "lh2g_raster_read",
         "lh2g_build_light_tree"]

_lib = None


class CoreError(RuntimeError):
    pass


def build_light_tree(tri, point, spot, lib=None):
    """The light tree lh2g_set_lights builds for these lights (structured arrays of the scene's light dtypes),
    through the host-only lh2g_build_light_tree: an array of LIGHT_TREE_DTYPE records, record 0 the root."""
    lib = lib or load_library()
    arrs = [np.ascontiguousarray(a) for a in (tri, point, spot)]
    cap = 2 * sum(len(a) for a in arrs)
    out = np.zeros(max(cap, 1), LIGHT_TREE_DTYPE)
    n = lib.lh2g_build_light_tree(*[x for a in arrs for x in (_p(a) if len(a) else None, len(a))], _p(out), cap)
    if n < 0:
        raise CoreError(f"build_light_tree: status {-n}")
    return out[:n]


def load_library(path: str | None = None):
    """Load the CUDA core library (raises if it is not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise CoreError(f"{p} is not built: run `python -m lighthouse2_gb300.build`")
    lib = C.CDLL(p)
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    lib.lh2g_create.argtypes = [i, C.POINTER(vp)]
    lib.lh2g_destroy.argtypes = [vp]
    lib.lh2g_last_error.argtypes = [vp]
    lib.lh2g_last_error.restype = C.c_char_p
    lib.lh2g_set_geometry.argtypes = [vp, i, vp, i, i, vp]
    lib.lh2g_set_instance.argtypes = [vp, i, i, vp]
    lib.lh2g_finalize_instances.argtypes = [vp]
    lib.lh2g_set_materials.argtypes = [vp, vp, i]
    lib.lh2g_pack_materials.argtypes = [vp, i, vp, i, vp]
    lib.lh2g_set_textures.argtypes = [vp, vp, i]
    lib.lh2g_set_lights.argtypes = [vp, vp, i, vp, i, vp, i, vp, i]
    lib.lh2g_build_light_tree.argtypes = [vp, i, vp, i, vp, i, vp, i]
    lib.lh2g_set_sky.argtypes = [vp, vp, i, i, vp]
    lib.lh2g_setting.argtypes = [vp, C.c_char_p, f]
    lib.lh2g_set_target.argtypes = [vp, i, i, i]
    lib.lh2g_set_probe.argtypes = [vp, i, i]
    lib.lh2g_render.argtypes = [vp, vp, i]
    lib.lh2g_render_ex.argtypes = [vp, vp, vp, i, vp, vp, vp]
    lib.lh2g_render_to_host.argtypes = [vp, vp, vp, i, vp]
    lib.lh2g_wait.argtypes = [vp]
    lib.lh2g_get_stats.argtypes = [vp, vp]
    lib.lh2g_get_framebuffer.argtypes = [vp, C.POINTER(vp)]
    lib.lh2g_read_framebuffer.argtypes = [vp, vp]
    lib.lh2g_read_accumulator.argtypes = [vp, vp]
    lib.lh2g_trace.argtypes = [vp, vp, vp, C.c_longlong, i, vp]
    lib.lh2g_trace_host.argtypes = [vp, vp, vp, C.c_longlong, i]
    lib.lh2g_get_stream.argtypes = [vp, C.POINTER(vp)]
    lib.lh2g_enable_launch_timing.argtypes = [vp, i]
    lib.lh2g_get_launch_times.argtypes = [vp, vp, i, C.POINTER(i)]
    lib.lh2g_get_traversal_stats.argtypes = [vp, vp]
    lib.lh2g_render_noalloc.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.lh2g_filter.argtypes = [vp, vp]
    lib.lh2g_read_filter_buffer.argtypes = [vp, i, vp]
    lib.lh2g_get_last_filter_frame.argtypes = [vp, vp, vp, vp]
    lib.lh2g_render_nrc.argtypes = [vp, vp, vp, vp, i, i, vp]
    lib.lh2g_set_blue_noise.argtypes = [vp, vp, vp, vp]
    lib.lh2g_render_adaptive.argtypes = [vp, vp, vp, i, vp, vp, vp, vp]
    lib.lh2g_set_adaptive_scale.argtypes = [vp, f]
    lib.lh2g_raster_render.argtypes = [vp, vp, vp, vp, vp]
    lib.lh2g_raster_pixels_device.argtypes = [vp]
    lib.lh2g_raster_pixels_device.restype = vp
    if path is None:
        _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def texture_descs(textures):
    d = np.zeros(max(1, len(textures)), TEXDESC_DTYPE)
    keep = []
    for k, t in enumerate(textures):
        arr = np.ascontiguousarray(t.texels, np.uint32)
        keep.append(arr)
        d[k]["texels"] = arr.ctypes.data
        d[k]["width"], d[k]["height"] = t.width, t.height
        d[k]["pixelCount"] = len(arr)
        d[k]["MIPlevels"] = 5
    return d, keep


def make_params(width, height, spp=1, max_depth=3, rr_start=1, samples_taken=0, camera_r0=0, eps=1e-3, clamp=10.0, flags=RP_NEE,
                frame_seed=0, shift=0):
    p = np.zeros((), PARAMS_DTYPE)
    p["width"], p["height"], p["spp"], p["maxDepth"] = width, height, spp, max_depth
    p["rrStartDepth"], p["samplesTaken"], p["cameraR0"] = rr_start, samples_taken, camera_r0
    p["geometryEpsilon"], p["clampValue"], p["flags"], p["frameSeed"] = eps, clamp, flags, frame_seed
    p["shift"] = shift
    return p


def camera_r0(frames_since_restart: int) -> int:
    """RandomUInt(camRNGseed) of the n-th frame after a Restart (seed 0x12345678, xorshift32)."""
    s = 0x12345678
    for _ in range(frames_since_restart + 1):
        s ^= (s << 13) & 0xFFFFFFFF
        s ^= s >> 17
        s ^= (s << 5) & 0xFFFFFFFF
    return s


class RenderCore:
    """One GB300 render core (one C-ABI context, one CUDA stream)."""

    def __init__(self, device: int = 0, lib_path: str | None = None):
        self.lib = load_library(lib_path)
        self.ctx = C.c_void_p()
        rc = self.lib.lh2g_create(device, C.byref(self.ctx))
        if rc != 0:
            raise CoreError(f"lh2g_create failed with status {rc}")
        self._keep = []
        self.W = self.H = self.spp = 0

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.lh2g_last_error(self.ctx)
            raise CoreError(f"{what}: status {rc}: {msg.decode() if msg else ''}")

    def close(self):
        if self.ctx:
            self.lib.lh2g_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- CoreAPI_Base mirror -------------------------------------------------------------------------
    def SetGeometry(self, meshIdx, vertices, tris):
        vertices = np.ascontiguousarray(vertices, np.float32)
        tris = np.ascontiguousarray(tris)
        self._check(self.lib.lh2g_set_geometry(self.ctx, meshIdx, _p(vertices), len(vertices), len(tris), _p(tris)), "SetGeometry")

    def SetInstance(self, instIdx, meshIdx, transform=None):
        T = np.ascontiguousarray(np.eye(4, dtype=np.float32) if transform is None else transform, np.float32)
        self._check(self.lib.lh2g_set_instance(self.ctx, instIdx, meshIdx, _p(T)), "SetInstance")

    def FinalizeInstances(self):
        self._check(self.lib.lh2g_finalize_instances(self.ctx), "FinalizeInstances")

    def SetTextures(self, textures):
        d, keep = texture_descs(textures)
        self._keep.append((d, keep))
        self._check(self.lib.lh2g_set_textures(self.ctx, _p(d) if textures else None, len(textures)), "SetTextures")

    def SetMaterials(self, materials):
        m = np.ascontiguousarray(materials)
        self._check(self.lib.lh2g_set_materials(self.ctx, _p(m), len(m)), "SetMaterials")

    def SetLights(self, tri, point, spot, directional):
        arrs = [np.ascontiguousarray(a) for a in (tri, point, spot, directional)]
        self._check(self.lib.lh2g_set_lights(self.ctx, _p(arrs[0]), len(arrs[0]), _p(arrs[1]), len(arrs[1]), _p(arrs[2]), len(arrs[2]),
                                             _p(arrs[3]), len(arrs[3])), "SetLights")

    def SetSkyData(self, rgb, width, height, world_to_sky=None):
        rgb = np.ascontiguousarray(rgb, np.float32)
        m = None if world_to_sky is None else np.ascontiguousarray(world_to_sky, np.float32)
        self._check(self.lib.lh2g_set_sky(self.ctx, _p(rgb), width, height, _p(m)), "SetSkyData")

    def Setting(self, name, value):
        self._check(self.lib.lh2g_setting(self.ctx, name.encode(), float(value)), "Setting")

    def SetTarget(self, width, height, spp=1):
        self._check(self.lib.lh2g_set_target(self.ctx, width, height, spp), "SetTarget")
        self.W, self.H, self.spp = width, height, spp

    def SetProbePos(self, x, y):
        self._check(self.lib.lh2g_set_probe(self.ctx, x, y), "SetProbePos")

    def Render(self, view, converge=0):
        self._check(self.lib.lh2g_render(self.ctx, _p(np.ascontiguousarray(view)), int(converge)), "Render")

    def WaitForRender(self):
        self._check(self.lib.lh2g_wait(self.ctx), "WaitForRender")

    def GetCoreStats(self):
        s = np.zeros((), STATS_DTYPE)
        self._check(self.lib.lh2g_get_stats(self.ctx, _p(s)), "GetCoreStats")
        return {k: s[k].item() for k in STATS_DTYPE.names}

    # --- convenience --------------------------------------------------------------------------------
    def set_scene(self, sc: S.Scene):
        for k, m in enumerate(sc.meshes):
            self.SetGeometry(k, m.vertices, m.tris)
        for k, (mi, T) in enumerate(sc.instances):
            self.SetInstance(k, mi, T)
        self.SetTextures(sc.textures)
        self.SetMaterials(sc.materials)
        self.SetLights(sc.tri_lights, sc.point_lights, sc.spot_lights, sc.dir_lights)
        if sc.sky is not None:
            rgb, w, h = sc.sky
            self.SetSkyData(rgb, w, h)
        if sc.blue_noise is not None:
            self.set_blue_noise(sc.blue_noise)
        self.FinalizeInstances()

    def set_blue_noise(self, tables):
        """Blue-noise tables (sobol 65536, scrambling 131072, ranking 131072 bytes) or None to remove them."""
        if tables is None:
            self._check(self.lib.lh2g_set_blue_noise(self.ctx, None, None, None), "set_blue_noise")
            return
        t = [np.ascontiguousarray(x, np.uint8) for x in tables]
        assert [len(x) for x in t] == [65536, 131072, 131072]
        self._check(self.lib.lh2g_set_blue_noise(self.ctx, _p(t[0]), _p(t[1]), _p(t[2])), "set_blue_noise")

    def render_adaptive(self, view, params, accumulate=False, capture=False):
        """One PrimeAdaptive frame (lh2g_render_adaptive); waits and returns the per-wave counters, the devScale for
        the next frame, the second wave's path count and the samples requested (and first-wave captures)."""
        D, P = int(params["maxDepth"]), int(params["width"]) * int(params["height"]) * int(params["spp"])
        hits = np.zeros(D * P, S.HIT_DTYPE) if capture else None
        seeds = np.zeros(D * P, np.uint32) if capture else None
        cnt = np.zeros((2 * D, 2), np.uint32)
        st = np.zeros(3, np.uint32)
        self._check(self.lib.lh2g_render_adaptive(self.ctx, _p(np.ascontiguousarray(view)), _p(np.ascontiguousarray(params)), int(accumulate),
                                                  _p(hits), _p(seeds), _p(cnt), _p(st)), "render_adaptive")
        out = {"counters": cnt, "dev_scale": float(st[0:1].view(np.float32)[0]), "adaptive_paths": int(st[1]), "requested": int(st[2])}
        if capture:
            out["hits"], out["seeds"] = hits.reshape(D, P), seeds.reshape(D, P)
        return out

    def raster(self, view, pixels=True, depth=False, stats=False):
        """One SoftRasterizer frame of the target's size (lh2g_raster_render): RGBA8 pixels (uint32, W*H), the
        z-buffer (float32) and the frame's counts, as asked."""
        px = np.zeros(self.W * self.H, np.uint32) if pixels else None
        zb = np.zeros(self.W * self.H, np.float32) if depth else None
        st = np.zeros(6, np.uint32) if stats else None
        self._check(self.lib.lh2g_raster_render(self.ctx, _p(np.ascontiguousarray(view)), _p(px), _p(zb), _p(st)), "raster_render")
        out = {}
        if pixels:
            out["pixels"] = px
        if depth:
            out["zbuffer"] = zb
        if stats:
            out["stats"] = dict(zip(["instancesDrawn", "triangles", "smallTriangles", "bigTriangles", "fragments", "status"], map(int, st)))
        return out

    def raster_pixels_device(self):
        return self.lib.lh2g_raster_pixels_device(self.ctx)

    def set_adaptive_scale(self, dev_scale):
        self._check(self.lib.lh2g_set_adaptive_scale(self.ctx, float(dev_scale)), "set_adaptive_scale")

    def render_ex(self, view, params, accumulate=False, capture=False, counters=True):
        rows = int(params["rowCount"]) if int(params["rowCount"]) > 0 else int(params["height"])
        D, P = int(params["maxDepth"]), int(params["width"]) * rows * int(params["spp"])
        hits = np.zeros(D * P, S.HIT_DTYPE) if capture else None
        seeds = np.zeros(D * P, np.uint32) if capture else None
        cnt = np.zeros((D, 2), np.uint32) if counters else None
        self._check(self.lib.lh2g_render_ex(self.ctx, _p(np.ascontiguousarray(view)), _p(np.ascontiguousarray(params)), int(accumulate),
                                            _p(hits), _p(seeds), _p(cnt)), "render_ex")
        out = {}
        if capture:
            out["hits"], out["seeds"] = hits.reshape(D, P), seeds.reshape(D, P)
        if counters:
            out["counters"] = cnt
        return out

    def render_to_host(self, view, params, host_ptr, accumulate=False):
        """Queues a frame and the copy of its finalized image (W*H float4) into host memory at host_ptr (pinned for
        overlap); the image is there after WaitForRender or any call that reads results."""
        self._check(self.lib.lh2g_render_to_host(self.ctx, _p(np.ascontiguousarray(view)), _p(np.ascontiguousarray(params)), int(accumulate),
                                                 C.c_void_p(host_ptr)), "render_to_host")

    def read_framebuffer(self):
        out = np.zeros((self.W * self.H, 4), np.float32)
        self._check(self.lib.lh2g_read_framebuffer(self.ctx, _p(out)), "read_framebuffer")
        return out

    def read_accumulator(self):
        out = np.zeros((self.W * self.H, 4), np.float32)
        self._check(self.lib.lh2g_read_accumulator(self.ctx, _p(out)), "read_accumulator")
        return out

    def read_accumulator_into(self, out):
        """Copies the accumulator (direct half) into a preallocated (W*H, 4) float32 array."""
        assert out.dtype == np.float32 and out.size >= self.W * self.H * 4 and out.flags["C_CONTIGUOUS"]
        self._check(self.lib.lh2g_read_accumulator(self.ctx, _p(out)), "read_accumulator")

    def framebuffer_ptr(self):
        p = C.c_void_p()
        self._check(self.lib.lh2g_get_framebuffer(self.ctx, C.byref(p)), "get_framebuffer")
        return p.value

    def stream_ptr(self):
        p = C.c_void_p()
        self._check(self.lib.lh2g_get_stream(self.ctx, C.byref(p)), "get_stream")
        return p.value or 0

    def enable_launch_timing(self, on=True):
        self._check(self.lib.lh2g_enable_launch_timing(self.ctx, int(on)), "enable_launch_timing")

    def launch_times(self):
        """Durations (ms) of every launch timed since the previous call, frames in order."""
        buf = np.zeros(16384, np.float32)
        n = C.c_int(0)
        self._check(self.lib.lh2g_get_launch_times(self.ctx, _p(buf), len(buf), C.byref(n)), "get_launch_times")
        return buf[:n.value].copy()

    def traversal_stats(self):
        out = np.zeros(4, np.uint64)
        self._check(self.lib.lh2g_get_traversal_stats(self.ctx, _p(out)), "get_traversal_stats")
        return out

    # --- radiance cache ---------------------------------------------------------------------------------
    def render_nrc(self, cache, view, params, accumulate=False, train=True, stats=True):
        """One frame with the radiance cache (lh2g_render_nrc). stats: wait for the frame and return (queries,
        training samples, loss); else queue it (consecutive frames overlap) and return None."""
        st = np.zeros(3, np.uint32)
        self._check(self.lib.lh2g_render_nrc(self.ctx, cache.h, _p(np.ascontiguousarray(view)), _p(np.ascontiguousarray(params)),
                                             int(accumulate), int(train), _p(st) if stats else None), "render_nrc")
        return (int(st[0]), int(st[1]), float(st[2:3].view(np.float32)[0])) if stats else None

    # --- SVGF (filter core) ----------------------------------------------------------------------------
    def filter(self, fparams):
        self._check(self.lib.lh2g_filter(self.ctx, _p(np.ascontiguousarray(fparams))), "filter")

    def read_filter_buffer(self, name):
        """Copy of filter buffer slot `name` (FILTER_SLOTS) as an array of (pixels, components)."""
        idx, dt, comps = FILTER_SLOTS[name]
        n = self.W * self.H * (2 if name == "accum" else 1)
        out = np.zeros((n, comps), dt)
        self._check(self.lib.lh2g_read_filter_buffer(self.ctx, idx, _p(out)), "read_filter_buffer")
        return out

    def last_filter_frame(self):
        """(filter params, jittered view, render params) of the last filtered frame that Render produced."""
        fp, jv, rp = np.zeros((), FILTER_PARAMS_DTYPE), np.zeros((), S.VIEW_DTYPE), np.zeros((), PARAMS_DTYPE)
        self._check(self.lib.lh2g_get_last_filter_frame(self.ctx, _p(fp), _p(jv), _p(rp)), "get_last_filter_frame")
        return fp, jv, rp

    def read_framebuffer_into(self, host_ptr):
        self._check(self.lib.lh2g_read_framebuffer(self.ctx, C.c_void_p(host_ptr)), "read_framebuffer")

    def trace_host(self, rays, mode=0):
        rays = np.ascontiguousarray(rays)
        out = np.zeros(len(rays), S.HIT_DTYPE) if mode == 0 else np.zeros(len(rays), np.uint32)
        self._check(self.lib.lh2g_trace_host(self.ctx, _p(rays), _p(out), len(rays), mode), "trace_host")
        return out

    def trace(self, rays_dev_ptr, out_dev_ptr, n, mode=0, stream=None):
        self._check(self.lib.lh2g_trace(self.ctx, C.c_void_p(rays_dev_ptr), C.c_void_p(out_dev_ptr), int(n), mode,
                                        C.c_void_p(stream) if stream else None), "trace")
