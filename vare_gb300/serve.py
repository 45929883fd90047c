"""ctypes binding of the serving layer (include/bora_serve.h): a stream of independent
FLIP requests on one GPU, admitted continuously against a device-memory budget.

The scheduler and the per-request workers are C++ threads inside the CUDA library; this
module only marshals arguments. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import flip

_vp = ctypes.c_void_p

REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = range(4)
WARN_TIMEOUT = 2


class ServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_running", ctypes.c_int), ("reserved", ctypes.c_int)]


class RequestStatus(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("status", ctypes.c_int), ("steps_total", ctypes.c_int),
                ("steps_done", ctypes.c_int), ("num_particles", ctypes.c_uint64),
                ("estimate_bytes", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64),
                ("queued_s", ctypes.c_double), ("run_s", ctypes.c_double), ("step_ms_p50", ctypes.c_double),
                ("step_ms_p99", ctypes.c_double), ("step_ms_max", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServeStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("admitted", ctypes.c_uint64), ("done", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("queued", ctypes.c_int), ("running", ctypes.c_int),
                ("bytes_reserved", ctypes.c_uint64), ("bytes_reserved_peak", ctypes.c_uint64),
                ("running_peak", ctypes.c_int), ("reserved", ctypes.c_int), ("particle_steps", ctypes.c_uint64),
                ("steps", ctypes.c_uint64), ("step_ms_p50", ctypes.c_double), ("step_ms_p99", ctypes.c_double),
                ("step_ms_max", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


_SIGS = {
    "bora_serve_default_config": (ctypes.c_int, [_vp]),
    "bora_serve_create": (ctypes.c_int, [_vp, _vp]),
    "bora_serve_destroy": (ctypes.c_int, [_vp]),
    "bora_serve_submit": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_float, _vp]),
    "bora_serve_set_colliders": (ctypes.c_int, [_vp, ctypes.c_uint64, _vp, ctypes.c_int, ctypes.c_float]),
    "bora_serve_poll": (ctypes.c_int, [_vp, ctypes.c_uint64, _vp]),
    "bora_serve_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_double]),
    "bora_serve_result": (ctypes.c_int, [_vp, ctypes.c_uint64, _vp, _vp, _vp, ctypes.c_size_t, _vp]),
    "bora_serve_release": (ctypes.c_int, [_vp, ctypes.c_uint64]),
    "bora_serve_drain": (ctypes.c_int, [_vp]),
    "bora_serve_get_stats": (ctypes.c_int, [_vp, _vp]),
    "bora_serve_estimate_bytes": (ctypes.c_uint64, [_vp, ctypes.c_size_t, ctypes.c_int]),
}

_BOUND = False


def load() -> ctypes.CDLL:
    global _BOUND
    lib = flip.load()
    if not _BOUND:
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _BOUND = True
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def _check(status: int, what: str) -> int:
    if status < 0:
        raise RuntimeError(f"{what}: {flip.status_string(status)} ({status})")
    return status


def _grid(scene) -> flip.GridDesc:
    g = flip.GridDesc()
    g.nx, g.ny, g.nz = scene.res
    g.min = (ctypes.c_float * 3)(*scene.bmin)
    g.max = (ctypes.c_float * 3)(*scene.bmax)
    return g


def estimate_bytes(scene, solver: int = flip.SOLVER_MIXED) -> int:
    g = _grid(scene)
    return int(load().bora_serve_estimate_bytes(ctypes.byref(g), scene.num_particles, solver))


class Server:
    """A running server: `submit` scenes, then `wait`/`result` per request."""

    def __init__(self, budget_bytes: int | None = None, max_running: int | None = None):
        self.lib = load()
        c = ServeConfig()
        _check(self.lib.bora_serve_default_config(ctypes.byref(c)), "default_config")
        if budget_bytes is not None:
            c.hbm_budget_bytes = int(budget_bytes)
        if max_running is not None:
            c.max_running = int(max_running)
        h = _vp()
        _check(self.lib.bora_serve_create(ctypes.byref(c), ctypes.byref(h)), "bora_serve_create")
        self.h = h
        self._keep = {}

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.bora_serve_destroy(self.h)
            self.h = None

    __del__ = close

    def submit(self, scene, steps: int, **overrides) -> int:
        """Queue `steps` substeps of a generated scene (vare_gb300.scenes.Scene)."""
        p = flip.scene_params(scene, **overrides)
        g = _grid(scene)
        pos = np.ascontiguousarray(scene.pos, np.float32)
        vel = np.ascontiguousarray(scene.vel, np.float32)
        rid = ctypes.c_uint64()
        _check(self.lib.bora_serve_submit(self.h, ctypes.byref(g), ctypes.byref(p), pos.ctypes.data,
                                          vel.ctypes.data, pos.shape[0], flip.SPACE_VOXEL, int(steps),
                                          ctypes.c_float(scene.dt), ctypes.byref(rid)), "bora_serve_submit")
        if scene.colliders:
            boxes = np.ascontiguousarray(np.array([np.concatenate([lo, hi, v]) for lo, hi, v in scene.colliders],
                                                  np.float32).reshape(-1))
            _check(self.lib.bora_serve_set_colliders(self.h, rid.value, boxes.ctypes.data, len(scene.colliders),
                                                     ctypes.c_float(scene.collider_band)), "set_colliders")
        return rid.value

    def poll(self, rid: int) -> dict:
        s = RequestStatus()
        _check(self.lib.bora_serve_poll(self.h, rid, ctypes.byref(s)), "bora_serve_poll")
        return s.as_dict()

    def wait(self, rid: int, timeout_s: float = -1.0) -> bool:
        st = _check(self.lib.bora_serve_wait(self.h, rid, ctypes.c_double(timeout_s)), "bora_serve_wait")
        return st != WARN_TIMEOUT

    def result(self, rid: int):
        n = ctypes.c_size_t()
        st = self.lib.bora_serve_result(self.h, rid, None, None, None, 0, ctypes.byref(n))
        if st not in (0, -6):
            _check(st, "bora_serve_result")
        m = n.value
        pos = np.empty((m, 3), np.float32)
        vel = np.empty((m, 3), np.float32)
        ids = np.empty(m, np.int32)
        _check(self.lib.bora_serve_result(self.h, rid, pos.ctypes.data, vel.ctypes.data, ids.ctypes.data, m,
                                          ctypes.byref(n)), "bora_serve_result")
        return pos, vel, ids

    def release(self, rid: int) -> None:
        _check(self.lib.bora_serve_release(self.h, rid), "bora_serve_release")

    def drain(self) -> None:
        _check(self.lib.bora_serve_drain(self.h), "bora_serve_drain")

    def stats(self) -> dict:
        s = ServeStats()
        _check(self.lib.bora_serve_get_stats(self.h, ctypes.byref(s)), "bora_serve_get_stats")
        return s.as_dict()
