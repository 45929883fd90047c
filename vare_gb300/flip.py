"""Python binding of the C ABI in include/bora_flip.h (ctypes, no torch types).

`FlipSim` mirrors the reference's Bora::FLIPMethod (base/header/FLIPMethod.h:13-126):
`initialize` is the constructor, `new_particles` batches FLIPMethod::newParticle,
`advance_one_step` / `advance_one_frame` are advanceOneStep / advanceOneFrame, and the
`field` / `tiles` accessors replace getVelocityField / getDensityField and the
SparseFrame internals. Errors raise `BoraError` with the library's status code.

The CUDA library must be built (vare_gb300.build.build()); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_vp = ctypes.c_void_p

BORA_OK = 0
BORA_WARN_NOT_CONVERGED = 1
SPACE_WORLD, SPACE_VOXEL = 0, 1
SOLVER_PLAIN, SOLVER_MIXED = 0, 1
FAULT_NONE, FAULT_BARRIER = 0, 1
ADVECT_EULER, ADVECT_RK2 = 0, 1
STAGE_REBUILD, STAGE_P2G, STAGE_BUILD_SYSTEM, STAGE_SOLVE, STAGE_UPDATE_VELOCITY, STAGE_UPDATE_PARTICLES = range(6)
POST_SPLAT, POST_TANK_SCAN, POST_REDISTANCE, POST_ATTRIBUTES = range(4)
FIELD_MASS, FIELD_SURF, FIELD_PRES, FIELD_VELO, FIELD_COMP, FIELD_FLAG, FIELD_RHS, FIELD_CODE = range(8)
VDB_SURFACE, VDB_VELOCITY = 0, 1
KERNEL_CLASSES = ["bin", "tiles", "sort", "p2g", "rhs", "pcg_direction", "pcg_update", "refine", "velocity", "g2p",
                  "mg_vcycle", "post"]
_FIELD_DTYPE = {FIELD_MASS: (np.float32, 1), FIELD_SURF: (np.float32, 1), FIELD_PRES: (np.float32, 1),
                FIELD_VELO: (np.float32, 3), FIELD_COMP: (np.float32, 3), FIELD_FLAG: (np.uint8, 1),
                FIELD_RHS: (np.float32, 1), FIELD_CODE: (np.uint16, 1)}


class BoraError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: status {status} ({status_string(status)})")


class GridDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("min", ctypes.c_float * 3), ("max", ctypes.c_float * 3)]


class Params(ctypes.Structure):
    _fields_ = [("ext_force", ctypes.c_float * 3), ("max_substeps", ctypes.c_int), ("dt", ctypes.c_float),
                ("wall_level", ctypes.c_float), ("enable_water_tank", ctypes.c_int), ("enable_curl", ctypes.c_int),
                ("damping_band", ctypes.c_float), ("voxel_size", ctypes.c_float), ("col_vel_scale", ctypes.c_float),
                ("pts_per_cell", ctypes.c_int), ("vort_pres_rate", ctypes.c_float),
                ("adjacency_under", ctypes.c_float), ("proj_iteration", ctypes.c_int),
                ("redist_iteration", ctypes.c_int), ("solver", ctypes.c_int), ("tolerance", ctypes.c_double),
                ("div_tolerance", ctypes.c_double), ("inner_tolerance", ctypes.c_double),
                ("max_refinements", ctypes.c_int), ("check_every", ctypes.c_int), ("advection", ctypes.c_int),
                ("post_process", ctypes.c_int), ("persistent", ctypes.c_int), ("warm_start", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint64), ("num_particles", ctypes.c_uint64), ("killed_last_step", ctypes.c_uint64),
                ("active_tiles", ctypes.c_int32), ("fluid_cells", ctypes.c_int32),
                ("solver_iterations", ctypes.c_int32), ("refinements", ctypes.c_int32),
                ("residual_rel", ctypes.c_double), ("residual_max", ctypes.c_double),
                ("residual_max_dx", ctypes.c_double), ("converged", ctypes.c_int32), ("mg_vcycle_launches", ctypes.c_int32),
                ("stage_ms", ctypes.c_double * 8), ("gpu_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("reserved", "stage_ms")}
        d["stage_ms"] = list(self.stage_ms)
        return d


class FrameInfo(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("tx", ctypes.c_int), ("ty", ctypes.c_int), ("tz", ctypes.c_int), ("tile", ctypes.c_int),
                ("active_tiles", ctypes.c_int), ("translate", ctypes.c_float * 3), ("scale", ctypes.c_float * 3),
                ("voxel_wall_level", ctypes.c_float), ("voxel_gravity", ctypes.c_float * 3)]


# name -> (restype, argtypes)
_SIGS = {
    "bora_flip_default_params": (ctypes.c_int, [ctypes.POINTER(Params)]),
    "bora_flip_create": (ctypes.c_int, [ctypes.POINTER(GridDesc), ctypes.POINTER(Params), ctypes.POINTER(_vp)]),
    "bora_flip_destroy": (ctypes.c_int, [_vp]),
    "bora_flip_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(Params)]),
    "bora_flip_add_particles": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_size_t, ctypes.c_int]),
    "bora_flip_set_particles": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_size_t, ctypes.c_int]),
    "bora_flip_clear_particles": (ctypes.c_int, [_vp]),
    "bora_flip_fill_water_tank": (ctypes.c_int, [_vp, _vp]),
    "bora_flip_set_collider_field": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_size_t]),
    "bora_flip_set_colliders": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_float]),
    "bora_flip_set_collider_voxels": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_float]),
    "bora_flip_step": (ctypes.c_int, [_vp, ctypes.c_float]),
    "bora_flip_step_batch": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_float, _vp]),
    "bora_flip_frame": (ctypes.c_int, [_vp]),
    "bora_flip_run_stage": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_float]),
    "bora_flip_post_process": (ctypes.c_int, [_vp]),
    "bora_flip_run_post_stage": (ctypes.c_int, [_vp, ctypes.c_int]),
    "bora_flip_get_particle_attributes": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_size_t,
                                                         ctypes.POINTER(ctypes.c_size_t)]),
    "bora_flip_set_particle_attributes": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_size_t]),
    "bora_flip_export_begin": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_size_t)]),
    "bora_flip_export_wait": (ctypes.c_int, [_vp]),
    "bora_flip_num_particles": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "bora_flip_get_particles": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_size_t,
                                               ctypes.POINTER(ctypes.c_size_t), ctypes.c_int]),
    "bora_flip_frame_info": (ctypes.c_int, [_vp, ctypes.POINTER(FrameInfo)]),
    "bora_flip_get_tiles": (ctypes.c_int, [_vp, _vp, ctypes.c_size_t]),
    "bora_flip_get_field": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_size_t]),
    "bora_flip_set_field": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_size_t]),
    "bora_flip_export_vdb": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, ctypes.c_size_t,
                                            ctypes.POINTER(ctypes.c_size_t), _vp, _vp]),
    "bora_flip_get_stats": (ctypes.c_int, [_vp, ctypes.POINTER(Stats)]),
    "bora_flip_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "bora_flip_set_profiling": (ctypes.c_int, [_vp, ctypes.c_uint32]),
    "bora_flip_set_profiling_sampling": (ctypes.c_int, [_vp, ctypes.c_uint32]),
    "bora_flip_get_kernel_times": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int]),
    "bora_flip_set_tuning": (ctypes.c_int, [ctypes.c_int]),
    "bora_flip_set_fault": (ctypes.c_int, [_vp, ctypes.c_int]),
    "bora_flip_tune_table": (ctypes.c_int, [_vp, ctypes.c_size_t, _vp]),
    "bora_scan_u32": (ctypes.c_int, [_vp, _vp, ctypes.c_size_t, _vp, _vp]),
    "bora_scan_u32_noalloc": (ctypes.c_int, [_vp, _vp, ctypes.c_size_t, _vp, _vp]),
}

_LIB: ctypes.CDLL | None = None


def library_path() -> str:
    return _build.LIB


def load() -> ctypes.CDLL:
    """Load the in-tree CUDA library; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA library {path} is missing: run vare_gb300.build.build() "
                               "(this package has no CPU fallback)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def exported_symbols() -> list[str]:
    return list(_SIGS)


def status_string(status: int) -> str:
    try:
        return load().bora_flip_status_string(status).decode()
    except Exception:  # pragma: no cover - only when the library is absent
        return "?"


def _check(status: int, what: str, allow_warn: bool = True) -> int:
    if status < 0 or (status > 0 and not allow_warn):
        raise BoraError(status, what)
    return status


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return _vp(a)
    return a.ctypes.data_as(_vp)


def default_params(**overrides) -> Params:
    p = Params()
    _check(load().bora_flip_default_params(ctypes.byref(p)), "default_params")
    for k, v in overrides.items():
        if k == "ext_force":
            p.ext_force = (ctypes.c_float * 3)(*v)
        else:
            setattr(p, k, v)
    return p


def scene_params(scene, **overrides) -> Params:
    """Parameters of a generated scene (vare_gb300.scenes.Scene)."""
    kw = dict(ext_force=scene.gravity, dt=scene.dt, wall_level=scene.wall_level, voxel_size=scene.voxel_size,
              proj_iteration=10000)
    kw.update(overrides)
    return default_params(**kw)


def set_tuning(on: bool) -> None:
    """bora_flip_set_tuning: the launch-shape autotuner on (default) or off."""
    _check(load().bora_flip_set_tuning(1 if on else 0), "set_tuning")


def tune_table() -> list[tuple[int, int, int, int, float]]:
    """bora_flip_tune_table: (group, device, size class, chosen shape or -1, median ms) rows."""
    lib = load()
    n = ctypes.c_size_t(0)
    _check(lib.bora_flip_tune_table(None, 0, ctypes.byref(n)), "tune_table")
    buf = ctypes.create_string_buffer(n.value + 1)
    _check(lib.bora_flip_tune_table(buf, n.value + 1, ctypes.byref(n)), "tune_table")
    rows = []
    for line in buf.value.decode().splitlines():
        g, d, c, v, m = line.split()
        rows.append((int(g), int(d), int(c), int(v), float(m)))
    return rows


def step_batch(sims, dt: float) -> list[int]:
    """bora_flip_step_batch: one step of every simulation, the pressure solve batched."""
    n = len(sims)
    if n == 0:
        return []
    hs = (_vp * n)(*[s.h for s in sims])
    st = np.zeros(n, np.int32)
    _check(load().bora_flip_step_batch(ctypes.cast(hs, _vp), n, float(dt), _ptr(st)), "step_batch")
    return [int(v) for v in st]


class FlipSim:
    """One simulation on the current CUDA device (Bora::FLIPMethod over the C ABI)."""

    def __init__(self, res, bmin, bmax, params: Params | None = None):
        lib = load()
        g = GridDesc()
        g.nx, g.ny, g.nz = (int(v) for v in res)
        g.min = (ctypes.c_float * 3)(*bmin)
        g.max = (ctypes.c_float * 3)(*bmax)
        h = _vp()
        _check(lib.bora_flip_create(ctypes.byref(g), ctypes.byref(params) if params is not None else None,
                                    ctypes.byref(h)), "bora_flip_create")
        self.lib = lib
        self.h = h
        self.params = params

    @classmethod
    def from_scene(cls, scene, **overrides) -> "FlipSim":
        sim = cls(scene.res, scene.bmin, scene.bmax, scene_params(scene, **overrides))
        if scene.colliders:
            sim.set_colliders(scene.colliders, scene.collider_band)
        sim.set_particles(scene.pos, scene.vel, space=SPACE_VOXEL)
        return sim

    def close(self):
        if getattr(self, "h", None):
            self.lib.bora_flip_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_params(self, params: Params) -> None:
        _check(self.lib.bora_flip_set_params(self.h, ctypes.byref(params)), "set_params")
        self.params = params

    def set_colliders(self, boxes, band: float) -> None:
        arr = np.ascontiguousarray(np.array([np.concatenate([lo, hi, v]) for lo, hi, v in boxes],
                                            np.float32).reshape(-1))
        _check(self.lib.bora_flip_set_colliders(self.h, _ptr(arr), len(boxes), band), "set_colliders")

    def add_particles(self, pos, vel=None, space: int = SPACE_WORLD) -> None:
        pos = np.ascontiguousarray(pos, np.float32)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
        _check(self.lib.bora_flip_add_particles(self.h, _ptr(pos), _ptr(vel), pos.shape[0], space), "add_particles")

    def set_particles(self, pos, vel=None, space: int = SPACE_WORLD) -> None:
        pos = np.ascontiguousarray(pos, np.float32)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
        _check(self.lib.bora_flip_set_particles(self.h, _ptr(pos), _ptr(vel), pos.shape[0], space), "set_particles")

    def set_collider_field(self, phi, vel=None) -> None:
        """Collider signed distance (and velocity) per frame cell, voxel units, x fastest."""
        if phi is None:
            _check(self.lib.bora_flip_set_collider_field(self.h, None, None, 0), "set_collider_field")
            return
        phi = np.ascontiguousarray(phi, np.float32).reshape(-1)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1)
        _check(self.lib.bora_flip_set_collider_field(self.h, _ptr(phi), _ptr(vel), phi.size), "set_collider_field")

    def set_collider_voxels(self, ijk, phi, vel=None, background: float = 0.0) -> None:
        """Sparse collider from a level set's active voxels (bora_flip_set_collider_voxels):
        ijk (N, 3) frame cells, phi (N,) world units, vel (N, 3) world units/s or None."""
        ijk = np.ascontiguousarray(ijk, np.int32).reshape(-1, 3)
        phi = np.ascontiguousarray(phi, np.float32).reshape(-1)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        _check(self.lib.bora_flip_set_collider_voxels(self.h, _ptr(ijk), _ptr(phi), _ptr(vel), len(phi),
                                                      float(background)), "set_collider_voxels")

    def fill_water_tank(self) -> int:
        """FLIPMethod::fillWaterTank: append the tank's particles; returns how many."""
        n = ctypes.c_size_t()
        _check(self.lib.bora_flip_fill_water_tank(self.h, ctypes.byref(n)), "fill_water_tank")
        return n.value

    def set_particles_ptr(self, pos_ptr: int, vel_ptr: int, n: int, space: int = SPACE_VOXEL) -> None:
        """Replace particles from raw host pointers (e.g. pinned torch buffers)."""
        _check(self.lib.bora_flip_set_particles(self.h, _vp(pos_ptr), _vp(vel_ptr), n, space), "set_particles")

    def step(self, dt: float) -> int:
        return _check(self.lib.bora_flip_step(self.h, dt), "bora_flip_step")

    advance_one_step = step

    def advance_one_frame(self) -> int:
        return _check(self.lib.bora_flip_frame(self.h), "bora_flip_frame")

    def run_stage(self, stage: int, dt: float = 0.0) -> int:
        return _check(self.lib.bora_flip_run_stage(self.h, stage, dt), f"run_stage({stage})")

    def post_process(self) -> None:
        """FLIPMethod::postProcess: surface splat, tank scan, redistancing, particle attributes."""
        _check(self.lib.bora_flip_post_process(self.h), "bora_flip_post_process")

    def run_post_stage(self, stage: int) -> None:
        _check(self.lib.bora_flip_run_post_stage(self.h, stage), f"run_post_stage({stage})")

    def particle_attributes(self):
        """(vorticity, curvature, ids) of the live particles, in particles()' order."""
        n = self.num_particles
        vort = np.zeros(n, np.float32)
        curv = np.zeros(n, np.float32)
        ids = np.zeros(n, np.int32)
        out = ctypes.c_size_t()
        _check(self.lib.bora_flip_get_particle_attributes(self.h, _ptr(vort), _ptr(curv), _ptr(ids), n,
                                                          ctypes.byref(out)), "get_particle_attributes")
        return vort, curv, ids

    def export_begin(self, pos_ptr: int, vel_ptr: int, vort_ptr: int = 0, curv_ptr: int = 0, ids_ptr: int = 0,
                     cap: int = 0, space: int = SPACE_VOXEL) -> int:
        """Start the asynchronous copy of the current particles to host memory (raw pointers,
        pinned for overlap; 0 = skip); returns the live count. Call export_wait before reading."""
        n = ctypes.c_size_t()
        _check(self.lib.bora_flip_export_begin(self.h, _vp(pos_ptr or None), _vp(vel_ptr or None),
                                               _vp(vort_ptr or None), _vp(curv_ptr or None), _vp(ids_ptr or None),
                                               cap, space, ctypes.byref(n)), "export_begin")
        return int(n.value)

    def export_wait(self) -> None:
        _check(self.lib.bora_flip_export_wait(self.h), "export_wait")

    def set_particle_attributes(self, vort, curv) -> None:
        vort = np.ascontiguousarray(vort, np.float32)
        curv = np.ascontiguousarray(curv, np.float32)
        _check(self.lib.bora_flip_set_particle_attributes(self.h, _ptr(vort), _ptr(curv), vort.shape[0]),
               "set_particle_attributes")

    @property
    def num_particles(self) -> int:
        n = ctypes.c_size_t()
        _check(self.lib.bora_flip_num_particles(self.h, ctypes.byref(n)), "num_particles")
        return int(n.value)

    def particles(self, space: int = SPACE_VOXEL):
        n = self.num_particles
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        adj = np.zeros(n, np.float32)
        ids = np.zeros(n, np.int32)
        out = ctypes.c_size_t()
        _check(self.lib.bora_flip_get_particles(self.h, _ptr(pos), _ptr(vel), _ptr(adj), _ptr(ids), n,
                                                ctypes.byref(out), space), "get_particles")
        return pos, vel, adj, ids

    def get_particles_ptr(self, pos_ptr: int, vel_ptr: int, cap: int, space: int = SPACE_VOXEL) -> int:
        out = ctypes.c_size_t()
        _check(self.lib.bora_flip_get_particles(self.h, _vp(pos_ptr), _vp(vel_ptr), None, None, cap,
                                                ctypes.byref(out), space), "get_particles")
        return int(out.value)

    def frame_info(self) -> dict:
        f = FrameInfo()
        _check(self.lib.bora_flip_frame_info(self.h, ctypes.byref(f)), "frame_info")
        return dict(nx=f.nx, ny=f.ny, nz=f.nz, tx=f.tx, ty=f.ty, tz=f.tz, tile=f.tile, ntiles=f.active_tiles,
                    translate=np.array(f.translate[:], np.float32), scale=np.array(f.scale[:], np.float32),
                    voxel_wall=f.voxel_wall_level, voxel_gravity=np.array(f.voxel_gravity[:], np.float32))

    def tiles(self) -> np.ndarray:
        n = self.frame_info()["ntiles"]
        out = np.zeros((n, 3), np.int32)
        _check(self.lib.bora_flip_get_tiles(self.h, _ptr(out), n), "get_tiles")
        return out.astype(np.int64)

    def field(self, which: int) -> np.ndarray:
        n = self.frame_info()["ntiles"] * 512
        dt, nc = _FIELD_DTYPE[which]
        out = np.zeros((n, 3) if nc == 3 else n, dt)
        _check(self.lib.bora_flip_get_field(self.h, which, _ptr(out), out.nbytes), "get_field")
        return out

    def set_field(self, which: int, data: np.ndarray) -> None:
        dt, nc = _FIELD_DTYPE[which]
        data = np.ascontiguousarray(data, dt)
        _check(self.lib.bora_flip_set_field(self.h, which, _ptr(data), data.nbytes), "set_field")

    def export_vdb(self, which: int) -> dict:
        """FieldCast's sparse -> VDB conversion as OpenVDB leaf blocks (bora_flip_export_vdb):
        origins (L, 3) int32, masks (L, 8) uint64, values (L, 512) or (L, 512, 3) float32,
        the transform (voxel size, translate xyz) and the background value."""
        n = ctypes.c_size_t(0)
        _check(self.lib.bora_flip_export_vdb(self.h, which, None, None, None, 0, ctypes.byref(n), None, None),
               "export_vdb")
        L = n.value
        comps = 1 if which == VDB_SURFACE else 3
        origins = np.zeros((L, 3), np.int32)
        masks = np.zeros((L, 8), np.uint64)
        values = np.zeros((L, 512) if comps == 1 else (L, 512, 3), np.float32)
        xform = np.zeros(4, np.float32)
        bg = np.zeros(1, np.float32)
        _check(self.lib.bora_flip_export_vdb(self.h, which, _ptr(origins), _ptr(masks), _ptr(values), L,
                                             ctypes.byref(n), _ptr(xform), _ptr(bg)), "export_vdb")
        return dict(origins=origins[:n.value], masks=masks[:n.value], values=values[:n.value], transform=xform,
                    background=float(bg[0]))

    def stats(self) -> dict:
        s = Stats()
        _check(self.lib.bora_flip_get_stats(self.h, ctypes.byref(s)), "get_stats")
        return s.as_dict()

    def set_fault(self, fault: int) -> None:
        """bora_flip_set_fault: inject a fault into the next solves (tests of the error paths)."""
        _check(self.lib.bora_flip_set_fault(self.h, int(fault)), "bora_flip_set_fault")

    def set_profiling(self, class_mask: int) -> None:
        _check(self.lib.bora_flip_set_profiling(self.h, class_mask), "set_profiling")

    def set_profiling_sampling(self, every: int) -> None:
        """Time one in `every` brackets of each profiled kernel class (1: all)."""
        _check(self.lib.bora_flip_set_profiling_sampling(self.h, every), "set_profiling_sampling")

    def kernel_times(self):
        ms = np.zeros(16, np.float64)
        n = np.zeros(16, np.uint64)
        _check(self.lib.bora_flip_get_kernel_times(self.h, _ptr(ms), _ptr(n), 16), "get_kernel_times")
        return ms, n

    def dense(self, which: int, background=0.0) -> np.ndarray:
        """Field scattered to a dense (nz, ny, nx[, 3]) array; inactive cells = background."""
        fi = self.frame_info()
        f = self.field(which)
        t = self.tiles()
        vec = f.ndim == 2
        shape = (fi["tz"] * 8, fi["ty"] * 8, fi["tx"] * 8) + ((3,) if vec else ())
        out = np.full(shape, background, dtype=f.dtype)
        if len(t):
            blk = f.reshape((len(t), 8, 8, 8) + ((3,) if vec else ()))
            for n, (i, j, k) in enumerate(t):
                out[k * 8:(k + 1) * 8, j * 8:(j + 1) * 8, i * 8:(i + 1) * 8] = blk[n]
        return out[:fi["nz"], :fi["ny"], :fi["nx"]]
