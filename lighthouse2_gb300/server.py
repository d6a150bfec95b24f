"""Python face of the serving loop (lh2g_server_* in include/lh2g.h): render and ray-query jobs of several resident
scenes, continuously batched on one GPU. Every call goes to the CUDA library."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import scenes as S
from .core import CoreError, RenderCore, load_library


class JobTimes(C.Structure):
    _fields_ = [("submit", C.c_double), ("admit", C.c_double), ("done", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("ticks", C.c_ulonglong), ("raysTraced", C.c_ulonglong), ("jobsDone", C.c_longlong), ("pathsInFlight", C.c_longlong),
                ("pending", C.c_longlong), ("deviceStatus", C.c_uint32), ("loopLaunches", C.c_longlong)]


def _bind(lib):
    vp, i, ll = C.c_void_p, C.c_int, C.c_longlong
    lib.lh2g_server_create.argtypes = [i, ll, C.POINTER(vp)]
    lib.lh2g_server_destroy.argtypes = [vp]
    lib.lh2g_server_last_error.argtypes = [vp]
    lib.lh2g_server_last_error.restype = C.c_char_p
    lib.lh2g_server_add_scene.argtypes = [vp, vp, C.POINTER(i)]
    lib.lh2g_server_submit_render.argtypes = [vp, i, vp, vp, vp, C.POINTER(ll)]
    lib.lh2g_server_submit_trace.argtypes = [vp, i, vp, ll, i, vp, C.POINTER(ll)]
    lib.lh2g_server_wait.argtypes = [vp, ll, i, C.POINTER(JobTimes)]
    lib.lh2g_server_release.argtypes = [vp, ll]
    lib.lh2g_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
    lib.lh2g_server_setting.argtypes = [vp, C.c_char_p, C.c_double]


class RenderServer:
    """One serving loop on one GPU. Scenes are RenderCore objects whose scene is finalized; they must outlive the
    server. Results land in numpy arrays owned by the job handles returned by submit_*."""

    def __init__(self, path_capacity: int, device: int = 0, **settings):
        """settings: expressMaxPaths, expressBudget, tickBudget, maxWaitSeconds, largeJobPaths (lh2g_server_setting)."""
        self.lib = load_library()
        _bind(self.lib)
        self.srv = C.c_void_p()
        rc = self.lib.lh2g_server_create(device, int(path_capacity), C.byref(self.srv))
        if rc != 0:
            raise CoreError(f"lh2g_server_create failed with status {rc}")
        self._scenes = []
        self._keep = {}
        for k, v in settings.items():
            self.setting(k, v)

    def setting(self, name: str, value: float):
        self._check(self.lib.lh2g_server_setting(self.srv, name.encode(), float(value)), f"setting {name}")

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.lh2g_server_last_error(self.srv)
            raise CoreError(f"{what}: status {rc}: {msg.decode() if msg else ''}")

    def close(self):
        if self.srv:
            self.lib.lh2g_server_destroy(self.srv)
            self.srv = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, core: RenderCore) -> int:
        sid = C.c_int(-1)
        self._check(self.lib.lh2g_server_add_scene(self.srv, core.ctx, C.byref(sid)), "add_scene")
        self._scenes.append(core)
        return sid.value

    def submit_render(self, scene_id: int, view, params, out=None) -> int:
        """Queues a render job; returns its id. The image (width*height x 4 float32: per-pixel sums over the job's
        samples) is available from result(id) once wait(id) returned. `out` may supply the (width*height, 4)
        float32 host array to fill (pinned memory makes the copy asynchronous)."""
        W, H = int(params["width"]), int(params["height"])
        if out is None:
            out = np.zeros((W * H, 4), np.float32)
        elif out.dtype != np.float32 or out.shape != (W * H, 4) or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous (width*height, 4) float32 array")
        view, params = np.ascontiguousarray(view), np.ascontiguousarray(params)
        jid = C.c_longlong(0)
        self._check(self.lib.lh2g_server_submit_render(self.srv, scene_id, view.ctypes.data_as(C.c_void_p), params.ctypes.data_as(C.c_void_p),
                                                       out.ctypes.data_as(C.c_void_p), C.byref(jid)), "submit_render")
        self._keep[jid.value] = (out, view, params)
        return jid.value

    def submit_trace(self, scene_id: int, rays, mode: int = 0) -> int:
        rays = np.ascontiguousarray(rays)
        out = np.zeros(len(rays), S.HIT_DTYPE) if mode == 0 else np.zeros(len(rays), np.uint32)
        jid = C.c_longlong(0)
        self._check(self.lib.lh2g_server_submit_trace(self.srv, scene_id, rays.ctypes.data_as(C.c_void_p), len(rays), mode,
                                                      out.ctypes.data_as(C.c_void_p), C.byref(jid)), "submit_trace")
        self._keep[jid.value] = (out, rays)
        return jid.value

    def wait(self, job_id: int, timeout_ms: int = 120000):
        """Blocks until the job is done; returns (submit, admit, done) times in seconds on the server's clock."""
        t = JobTimes()
        rc = self.lib.lh2g_server_wait(self.srv, job_id, timeout_ms, C.byref(t))
        self._check(rc, f"wait job {job_id}")
        return t.submit, t.admit, t.done

    def result(self, job_id: int):
        return self._keep[job_id][0]

    def release(self, job_id: int):
        self._check(self.lib.lh2g_server_release(self.srv, job_id), "release")
        self._keep.pop(job_id, None)

    def stats(self):
        s = ServerStats()
        self._check(self.lib.lh2g_server_get_stats(self.srv, C.byref(s)), "get_stats")
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}
