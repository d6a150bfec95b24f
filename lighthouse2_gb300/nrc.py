"""Python face of the radiance cache (lh2g_nrc_* in include/lh2g.h): a hash-grid encoded 4 x 64 ReLU MLP trained
online on the GPU's tensor cores. Every call goes to the CUDA library."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from .core import CoreError, load_library

MLP_PARAMS = 16576
GRID_PARAMS = 12 * (1 << 19) * 2
LEVELS, TABLE = 12, 1 << 19


class NrcConfig(C.Structure):
    _fields_ = [("sceneMin", C.c_float * 3), ("sceneMax", C.c_float * 3), ("learningRate", C.c_float), ("seed", C.c_uint32)]


def _bind(lib):
    vp, i, ll, f = C.c_void_p, C.c_int, C.c_longlong, C.c_float
    lib.lh2g_nrc_create.argtypes = [i, vp, C.POINTER(vp)]
    lib.lh2g_nrc_destroy.argtypes = [vp]
    lib.lh2g_nrc_last_error.argtypes = [vp]
    lib.lh2g_nrc_last_error.restype = C.c_char_p
    lib.lh2g_nrc_get_spec.argtypes = [vp, vp, vp, vp]
    lib.lh2g_nrc_set_params.argtypes = [vp, vp, vp]
    lib.lh2g_nrc_get_params.argtypes = [vp, vp, vp]
    lib.lh2g_nrc_get_grads.argtypes = [vp, vp, vp]
    lib.lh2g_nrc_infer.argtypes = [vp, vp, ll, vp, vp]
    lib.lh2g_nrc_train.argtypes = [vp, vp, vp, ll, i, C.POINTER(f), vp]
    lib.lh2g_nrc_apply_update.argtypes = [vp, vp]
    lib.lh2g_nrc_infer_host.argtypes = [vp, vp, ll, vp]
    lib.lh2g_nrc_train_host.argtypes = [vp, vp, vp, ll, i, C.POINTER(f)]


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def grid_spec(scene_min, scene_max):
    """The encoding geometry the library computes (per-level resolution, dense flag, position mapping)."""
    growth = math.exp(math.log(2048.0 / 16.0) / (LEVELS - 1))
    res = [int(math.floor(16.0 * growth ** l)) for l in range(LEVELS)]
    dense = [1 if (r + 1.0) ** 3 <= TABLE else 0 for r in res]
    ext = [float(np.float32(b) - np.float32(a)) for a, b in zip(scene_min, scene_max)]
    inv = [float(np.float32(1.0) / np.float32(e)) if e > 0 else 1.0 for e in ext]
    return res, dense, list(map(float, scene_min)), inv


class RadianceCache:
    def __init__(self, scene_min, scene_max, learning_rate=1e-3, seed=1, device=0):
        self.lib = load_library()
        _bind(self.lib)
        cfg = NrcConfig((C.c_float * 3)(*scene_min), (C.c_float * 3)(*scene_max), learning_rate, seed)
        self.h = C.c_void_p()
        rc = self.lib.lh2g_nrc_create(device, C.byref(cfg), C.byref(self.h))
        if rc != 0:
            raise CoreError(f"lh2g_nrc_create failed with status {rc}")

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.lh2g_nrc_last_error(self.h)
            raise CoreError(f"{what}: status {rc}: {msg.decode() if msg else ''}")

    def close(self):
        if self.h:
            self.lib.lh2g_nrc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spec(self):
        res, dense, bi = np.zeros(12, np.int32), np.zeros(12, np.int32), np.zeros(6, np.float32)
        self._check(self.lib.lh2g_nrc_get_spec(self.h, _p(res), _p(dense), _p(bi)), "get_spec")
        return res, dense, bi

    def set_params(self, mlp=None, grid=None):
        mlp = None if mlp is None else np.ascontiguousarray(mlp, np.float32)
        grid = None if grid is None else np.ascontiguousarray(grid, np.float32)
        self._check(self.lib.lh2g_nrc_set_params(self.h, _p(mlp), _p(grid)), "set_params")

    def params(self):
        mlp, grid = np.zeros(MLP_PARAMS, np.float32), np.zeros(GRID_PARAMS, np.float32)
        self._check(self.lib.lh2g_nrc_get_params(self.h, _p(mlp), _p(grid)), "get_params")
        return mlp, grid

    def grads(self):
        mlp, grid = np.zeros(MLP_PARAMS, np.float32), np.zeros(GRID_PARAMS, np.float32)
        self._check(self.lib.lh2g_nrc_get_grads(self.h, _p(mlp), _p(grid)), "get_grads")
        return mlp, grid

    def infer(self, queries):
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 16)
        out = np.zeros((len(q), 4), np.float32)
        self._check(self.lib.lh2g_nrc_infer_host(self.h, _p(q), len(q), _p(out)), "infer")
        return out

    def train(self, queries, targets, update=True):
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 16)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 4)
        loss = C.c_float(0)
        self._check(self.lib.lh2g_nrc_train_host(self.h, _p(q), _p(t), len(q), int(update), C.byref(loss)), "train")
        return loss.value

    def apply_update(self):
        self._check(self.lib.lh2g_nrc_apply_update(self.h, None), "apply_update")
        self.lib.lh2g_nrc_get_params(self.h, None, None)   # waits for the update

    def infer_dev(self, queries_ptr, n, out_ptr, stream=None):
        self._check(self.lib.lh2g_nrc_infer(self.h, C.c_void_p(queries_ptr), int(n), C.c_void_p(out_ptr), C.c_void_p(stream) if stream else None),
                    "infer")

    def train_dev(self, queries_ptr, targets_ptr, n, update=True, stream=None):
        self._check(self.lib.lh2g_nrc_train(self.h, C.c_void_p(queries_ptr), C.c_void_p(targets_ptr), int(n), int(update), None,
                                            C.c_void_p(stream) if stream else None), "train")
