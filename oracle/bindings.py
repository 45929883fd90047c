"""ORACLE (test infrastructure only): ctypes bindings for the CPU oracles.

* `Oracle` wraps oracle/_build/liboracle_flip.so, the CPU restatement of the
  reference's FLIP substep (flip_oracle.cpp), in "compat" mode (4^3 tiles, the
  reference's tile-index wrap and CG rule) or "build" mode (8^3 tiles, FP64 solve).
* `RefSim` wraps oracle/_ref/libbora_ref*.so, the reference's own FLIP sources
  compiled for the host (only where the reference checkout exists; not on a GPU host).

Only tests, the smoke check and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle_flip.so")
REF_SO = os.path.join(HERE, "_ref", "libbora_ref.so")
REF64_SO = os.path.join(HERE, "_ref", "libbora_ref_cg64.so")

FIELD_MASS, FIELD_SURF, FIELD_PRES, FIELD_VELO, FIELD_COMP, FIELD_MARK = range(6)
K_AIR, K_SOLID, K_WALL, K_MARK, K_FLUID = range(5)

_vp = ctypes.c_void_p


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_vp)


def reference_dir() -> str | None:
    """The reference checkout named by BORA_REFERENCE (the directory holding base/source),
    or None when the variable is unset."""
    d = os.environ.get("BORA_REFERENCE")
    return d or None


def build(ref: bool | None = None, quiet: bool = True) -> None:
    """Compile the restatement, and the host build of the reference when BORA_REFERENCE
    names a checkout (ref=None: when it is set and holds base/source; ref=True: required,
    an error otherwise)."""
    targets = ["all"]
    refdir = reference_dir()
    has_ref = refdir is not None and os.path.isdir(os.path.join(refdir, "base", "source"))
    if ref is None:
        ref = has_ref
    elif ref and not has_ref:
        raise RuntimeError("building the reference needs BORA_REFERENCE set to a checkout holding base/source")
    args = ["make", "-C", HERE, "-j8", *targets]
    if ref:
        args += [f"REF={refdir}", "ref"]
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL if quiet else None)


class OracleConfig(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("bmin", ctypes.c_float * 3), ("bmax", ctypes.c_float * 3),
                ("block", ctypes.c_int), ("compat_wrap", ctypes.c_int), ("solver", ctypes.c_int),
                ("tol", ctypes.c_double), ("max_iter", ctypes.c_int),
                ("gravity", ctypes.c_float * 3), ("wall_level", ctypes.c_float),
                ("maxsubsteps", ctypes.c_int), ("col_vel_scale", ctypes.c_float),
                ("enable_tank", ctypes.c_int), ("damping_band", ctypes.c_float),
                ("voxel_size", ctypes.c_float), ("advection", ctypes.c_int)]


class RefParams(ctypes.Structure):
    _fields_ = [("extForce", ctypes.c_float * 3), ("maxsubsteps", ctypes.c_int), ("dt", ctypes.c_float),
                ("wallLevel", ctypes.c_float), ("enableWaterTank", ctypes.c_int), ("enableCurl", ctypes.c_int),
                ("dampingBand", ctypes.c_float), ("voxelSize", ctypes.c_float), ("colVelScale", ctypes.c_float),
                ("ptsPerCell", ctypes.c_int), ("vortPresRate", ctypes.c_float), ("adjacencyUnder", ctypes.c_float),
                ("projIteration", ctypes.c_int), ("redistIteration", ctypes.c_int)]


_LIBS: dict[str, ctypes.CDLL] = {}


def _load(path: str) -> ctypes.CDLL:
    if path not in _LIBS:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built; run oracle.bindings.build()")
        lib = ctypes.CDLL(path)
        _LIBS[path] = lib
    return _LIBS[path]


def _oracle_lib() -> ctypes.CDLL:
    lib = _load(ORACLE_SO)
    if not getattr(lib, "_typed", False):
        lib.ora_create.restype = _vp
        lib.ora_create.argtypes = [ctypes.POINTER(OracleConfig)]
        for name in ["ora_destroy", "ora_rebuild", "ora_p2g", "ora_mark", "ora_build_system",
                     "ora_update_velocity", "ora_compact"]:
            getattr(lib, name).argtypes = [_vp]
            getattr(lib, name).restype = None
        lib.ora_solve.argtypes = [_vp]
        lib.ora_solve.restype = ctypes.c_int
        lib.ora_step.argtypes = [_vp, ctypes.c_float]
        lib.ora_step.restype = ctypes.c_int
        lib.ora_update_particles.argtypes = [_vp, ctypes.c_float]
        lib.ora_set_threads.argtypes = [ctypes.c_int]
        lib.ora_get_threads.restype = ctypes.c_int
        lib.ora_set_colliders.argtypes = [_vp, ctypes.c_int, _vp, ctypes.c_float]
        lib.ora_set_collider_voxels.argtypes = [_vp, _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_float]
        lib.ora_set_particles.argtypes = [_vp, _vp, _vp, _vp, ctypes.c_size_t]
        lib.ora_num_particles.argtypes = [_vp]
        lib.ora_num_particles.restype = ctypes.c_size_t
        lib.ora_get_particles.argtypes = [_vp, _vp, _vp, _vp, _vp]
        lib.ora_get_removed.argtypes = [_vp, _vp]
        lib.ora_get_removed.restype = ctypes.c_size_t
        lib.ora_frame_info.argtypes = [_vp, _vp]
        lib.ora_grid_xform.argtypes = [_vp, _vp]
        lib.ora_get_tiles.argtypes = [_vp, _vp]
        lib.ora_get_markers.argtypes = [_vp, _vp]
        lib.ora_field_size.argtypes = [_vp]
        lib.ora_field_size.restype = ctypes.c_size_t
        lib.ora_get_field.argtypes = [_vp, ctypes.c_int, _vp]
        lib.ora_set_field.argtypes = [_vp, ctypes.c_int, _vp]
        lib.ora_num_unknowns.argtypes = [_vp]
        lib.ora_num_unknowns.restype = ctypes.c_size_t
        lib.ora_get_system.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp]
        lib.ora_set_solution.argtypes = [_vp, _vp]
        lib.ora_residual_max.argtypes = [_vp]
        lib.ora_residual_max.restype = ctypes.c_double
        lib.ora_last_rel.argtypes = [_vp]
        lib.ora_last_rel.restype = ctypes.c_double
        lib.ora_fill_water_tank.argtypes = [_vp, ctypes.c_int]
        lib.ora_fill_water_tank.restype = ctypes.c_size_t
        lib.ora_post_process.argtypes = [_vp, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int]
        lib.ora_post_splat.argtypes = [_vp]
        lib.ora_post_tank_scan.argtypes = [_vp, ctypes.c_int]
        lib.ora_post_redistance.argtypes = [_vp, ctypes.c_int]
        lib.ora_post_attributes.argtypes = [_vp, ctypes.c_float, ctypes.c_float]
        lib.ora_get_attributes.argtypes = [_vp, _vp, _vp]
        lib.ora_set_attributes.argtypes = [_vp, _vp, _vp]
        lib._typed = True
    return lib


class _SimBase:
    """Shared accessors of both CPU simulators (same field/tile conventions)."""

    _p = ""  # symbol prefix

    def frame_info(self) -> dict:
        out = np.zeros(8, np.int64)
        getattr(self.lib, self._p + "frame_info")(self.h, _ptr(out))
        return dict(fx=int(out[0]), fy=int(out[1]), fz=int(out[2]), block=int(out[3]),
                    nx=int(out[4]), ny=int(out[5]), nz=int(out[6]), ntiles=int(out[7]))

    def grid_xform(self) -> dict:
        out = np.zeros(10, np.float32)
        getattr(self.lib, self._p + "grid_xform")(self.h, _ptr(out))
        return dict(translate=out[0:3].copy(), scale=out[3:6].copy(), voxel_wall=float(out[6]),
                    voxel_gravity=out[7:10].copy())

    def tiles(self) -> np.ndarray:
        n = self.frame_info()["ntiles"]
        out = np.zeros((n, 3), np.int64)
        getattr(self.lib, self._p + "get_tiles")(self.h, _ptr(out))
        return out

    def markers(self) -> np.ndarray:
        fi = self.frame_info()
        out = np.zeros(fi["fx"] * fi["fy"] * fi["fz"], np.int32)
        getattr(self.lib, self._p + "get_markers")(self.h, _ptr(out))
        return out

    def field(self, which: int) -> np.ndarray:
        n = int(getattr(self.lib, self._p + "field_size")(self.h))
        if which in (FIELD_VELO, FIELD_COMP):
            out = np.zeros((n, 3), np.float32)
        elif which == FIELD_MARK:
            out = np.zeros(n, np.int64)
        else:
            out = np.zeros(n, np.float32)
        getattr(self.lib, self._p + "get_field")(self.h, which, _ptr(out))
        return out

    def dense(self, which: int, background=0.0) -> np.ndarray:
        """Field scattered to a dense (nz, ny, nx[, 3]) array over the frame grid;
        cells outside active tiles hold `background`."""
        fi = self.frame_info()
        B = fi["block"]
        f = self.field(which)
        t = self.tiles()
        vec = f.ndim == 2
        shape = (fi["fz"] * B, fi["fy"] * B, fi["fx"] * B) + ((3,) if vec else ())
        out = np.full(shape, background, dtype=f.dtype)
        if len(t):
            blk = f.reshape((len(t), B, B, B) + ((3,) if vec else ()))
            for n, (i, j, k) in enumerate(t):
                out[k * B:(k + 1) * B, j * B:(j + 1) * B, i * B:(i + 1) * B] = blk[n]
        return out[:fi["nz"], :fi["ny"], :fi["nx"]]

    def active_mask(self) -> np.ndarray:
        fi = self.frame_info()
        B = fi["block"]
        m = np.zeros((fi["fz"] * B, fi["fy"] * B, fi["fx"] * B), bool)
        for (i, j, k) in self.tiles():
            m[k * B:(k + 1) * B, j * B:(j + 1) * B, i * B:(i + 1) * B] = True
        return m[:fi["nz"], :fi["ny"], :fi["nx"]]


class Oracle(_SimBase):
    """CPU restatement of the reference FLIP substep (oracle/flip_oracle.cpp)."""

    _p = "ora_"

    def __init__(self, scene, block: int = 8, compat: bool = False, solver: str = "fp64",
                 tol: float = 1e-12, max_iter: int = 100000, threads: int | None = None, advection: int = 0,
                 tank: bool = False, damping_band: float = 0.0):
        self.lib = _oracle_lib()
        if threads is not None:
            self.lib.ora_set_threads(int(threads))
        c = OracleConfig()
        c.nx, c.ny, c.nz = scene.res
        c.bmin = (ctypes.c_float * 3)(*scene.bmin)
        c.bmax = (ctypes.c_float * 3)(*scene.bmax)
        c.block = block
        c.compat_wrap = 1 if compat else 0
        c.solver = {"reference": 0, "fp64": 1, "tol": 2}[solver]
        c.tol = tol
        c.max_iter = max_iter
        c.gravity = (ctypes.c_float * 3)(*scene.gravity)
        c.wall_level = scene.wall_level
        c.maxsubsteps = 1
        c.col_vel_scale = 1.0
        c.enable_tank = 1 if tank else 0
        c.damping_band = damping_band
        c.voxel_size = scene.voxel_size
        c.advection = advection
        self.cfg = c
        self.h = _vp(self.lib.ora_create(ctypes.byref(c)))
        if scene.colliders:
            self.set_colliders(scene.colliders, scene.collider_band)
        self.set_particles(scene.pos, scene.vel)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.ora_destroy(h)
            self.h = None

    def set_colliders(self, boxes, band: float) -> None:
        arr = np.ascontiguousarray(np.array([np.concatenate([lo, hi, v]) for lo, hi, v in boxes],
                                            np.float32).reshape(-1))
        self.lib.ora_set_colliders(self.h, len(boxes), _ptr(arr), band)

    def set_collider_voxels(self, ijk, phi, vel=None, background: float = 0.0) -> None:
        """Sparse collider from a level set's active voxels (world-unit phi and velocity)."""
        self._col_keep = (np.ascontiguousarray(ijk, np.int32).reshape(-1, 3),
                          np.ascontiguousarray(phi, np.float32).reshape(-1),
                          None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3))
        ijk, phi, vel = self._col_keep
        self.lib.ora_set_collider_voxels(self.h, _ptr(ijk), _ptr(phi), _ptr(vel), len(phi), float(background))

    def fill_water_tank(self, per_cell: int = 8) -> int:
        """FLIPMethod::fillWaterTank restated (particles appended in voxel space)."""
        return int(self.lib.ora_fill_water_tank(self.h, per_cell))

    def set_particles(self, pos, vel, ids=None) -> None:
        pos = np.ascontiguousarray(pos, np.float32)
        vel = np.ascontiguousarray(vel, np.float32)
        ids = None if ids is None else np.ascontiguousarray(ids, np.int32)
        self.lib.ora_set_particles(self.h, _ptr(pos), _ptr(vel), _ptr(ids), pos.shape[0])

    @property
    def num_particles(self) -> int:
        return int(self.lib.ora_num_particles(self.h))

    def particles(self):
        n = self.num_particles
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        adj = np.zeros(n, np.float32)
        ids = np.zeros(n, np.int32)
        self.lib.ora_get_particles(self.h, _ptr(pos), _ptr(vel), _ptr(adj), _ptr(ids))
        return pos, vel, adj, ids

    def removed(self) -> np.ndarray:
        n = int(self.lib.ora_get_removed(self.h, None))
        out = np.zeros(n, np.uint8)
        self.lib.ora_get_removed(self.h, _ptr(out))
        return out

    def step(self, dt: float) -> int:
        return int(self.lib.ora_step(self.h, dt))

    # stage-by-stage
    def rebuild(self): self.lib.ora_rebuild(self.h)
    def p2g(self): self.lib.ora_p2g(self.h)
    def mark(self): self.lib.ora_mark(self.h)
    def build_system(self): self.lib.ora_build_system(self.h)
    def solve(self) -> int: return int(self.lib.ora_solve(self.h))
    def update_velocity(self): self.lib.ora_update_velocity(self.h)
    def update_particles(self, dt): self.lib.ora_update_particles(self.h, dt)
    def compact(self): self.lib.ora_compact(self.h)

    def set_field(self, which: int, data: np.ndarray) -> None:
        data = np.ascontiguousarray(data)
        self.lib.ora_set_field(self.h, which, _ptr(data))

    def system(self):
        n = int(self.lib.ora_num_unknowns(self.h))
        b = np.zeros(n, np.float32)
        x = np.zeros(n, np.float32)
        cells = np.zeros(n, np.int64)
        vals = np.zeros((n, 7), np.float32)
        cols = np.zeros((n, 7), np.int64)
        self.lib.ora_get_system(self.h, _ptr(b), _ptr(x), _ptr(cells), _ptr(vals), _ptr(cols))
        return dict(b=b, x=x, cells=cells, vals=vals, cols=cols)

    def set_solution(self, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float32)
        self.lib.ora_set_solution(self.h, _ptr(x))

    def residual_max(self) -> float:
        return float(self.lib.ora_residual_max(self.h))

    def last_rel(self) -> float:
        return float(self.lib.ora_last_rel(self.h))

    # FLIPMethod::postProcess restated
    def post_process(self, dt: float, vort_pres_rate: float = 0.2, redist_iteration: int = 80,
                     literal_scan: bool = False) -> None:
        """literal_scan reproduces the reference's tank scan as it executes; the default is
        the 6-connected fill of the device path."""
        self.lib.ora_post_process(self.h, dt, vort_pres_rate, redist_iteration, 1 if literal_scan else 0)

    def post_splat(self): self.lib.ora_post_splat(self.h)
    def post_tank_scan(self, literal: bool = False): self.lib.ora_post_tank_scan(self.h, 1 if literal else 0)

    def post_redistance(self, iters: int = 80):
        self.lib.ora_post_redistance(self.h, iters)

    def post_attributes(self, dt: float, vort_pres_rate: float = 0.2):
        self.lib.ora_post_attributes(self.h, dt, vort_pres_rate)

    def attributes(self):
        n = self.num_particles
        vort = np.zeros(n, np.float32)
        curv = np.zeros(n, np.float32)
        self.lib.ora_get_attributes(self.h, _ptr(vort), _ptr(curv))
        return vort, curv

    def set_attributes(self, vort, curv) -> None:
        vort = np.ascontiguousarray(vort, np.float32)
        curv = np.ascontiguousarray(curv, np.float32)
        self.lib.ora_set_attributes(self.h, _ptr(vort), _ptr(curv))


def _ref_lib(path: str) -> ctypes.CDLL:
    lib = _load(path)
    if not getattr(lib, "_typed", False):
        lib.ref_create.restype = _vp
        lib.ref_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.POINTER(RefParams)]
        lib.ref_destroy.argtypes = [_vp]
        lib.ref_set_boxes.argtypes = [_vp, ctypes.c_int, _vp, ctypes.c_float]
        lib.ref_add_particles.argtypes = [_vp, _vp, _vp, ctypes.c_size_t]
        lib.ref_step.argtypes = [_vp, ctypes.c_float]
        lib.ref_num_particles.argtypes = [_vp]
        lib.ref_num_particles.restype = ctypes.c_size_t
        lib.ref_get_particles.argtypes = [_vp, _vp, _vp, _vp]
        lib.ref_get_removed.argtypes = [_vp, _vp]
        lib.ref_get_removed.restype = ctypes.c_size_t
        lib.ref_frame_info.argtypes = [_vp, _vp]
        lib.ref_grid_xform.argtypes = [_vp, _vp]
        lib.ref_get_tiles.argtypes = [_vp, _vp]
        lib.ref_get_markers.argtypes = [_vp, _vp]
        lib.ref_field_size.argtypes = [_vp]
        lib.ref_field_size.restype = ctypes.c_size_t
        lib.ref_get_field.argtypes = [_vp, ctypes.c_int, _vp]
        lib.ref_num_unknowns.argtypes = [_vp]
        lib.ref_num_unknowns.restype = ctypes.c_size_t
        lib.ref_get_system.argtypes = [_vp, _vp, _vp, _vp]
        lib.ref_fill_water_tank.argtypes = [_vp]
        lib.ref_fill_water_tank.restype = ctypes.c_size_t
        lib.ref_post_process.argtypes = [_vp]
        lib.ref_get_attributes.argtypes = [_vp, _vp, _vp]
        if hasattr(lib, "ref_cg64_set"):
            lib.ref_cg64_set.argtypes = [ctypes.c_double, ctypes.c_int]
            lib.ref_cg64_last_iters.restype = ctypes.c_int
        lib._typed = True
    return lib


def reference_available() -> bool:
    return os.path.exists(REF_SO) and os.path.exists(REF64_SO)


class RefSim(_SimBase):
    """The reference's own FLIPMethod compiled for the host (oracle/_ref)."""

    _p = "ref_"

    def __init__(self, scene, converged: bool = False, tol: float = 1e-12, proj_iteration: int = 200,
                 tank: bool = False, damping_band: float = 0.0):
        self.lib = _ref_lib(REF64_SO if converged else REF_SO)
        if converged:
            self.lib.ref_cg64_set(tol, 100000)
        p = RefParams()
        p.extForce = (ctypes.c_float * 3)(*scene.gravity)
        p.maxsubsteps = 1
        p.dt = scene.dt
        p.wallLevel = scene.wall_level
        p.enableWaterTank = 1 if tank else 0
        p.enableCurl = 0
        p.dampingBand = damping_band
        p.voxelSize = scene.voxel_size
        p.colVelScale = 1.0
        p.ptsPerCell = 8
        p.vortPresRate = 0.2
        p.adjacencyUnder = 2.0
        p.projIteration = proj_iteration
        p.redistIteration = 80
        bmin = (ctypes.c_float * 3)(*scene.bmin)
        bmax = (ctypes.c_float * 3)(*scene.bmax)
        self.h = _vp(self.lib.ref_create(scene.res[0], scene.res[1], scene.res[2], bmin, bmax, ctypes.byref(p)))
        if scene.colliders:
            arr = np.ascontiguousarray(np.array([np.concatenate([lo, hi, v]) for lo, hi, v in scene.colliders],
                                                np.float32).reshape(-1))
            self.lib.ref_set_boxes(self.h, len(scene.colliders), _ptr(arr), scene.collider_band)
        pos = np.ascontiguousarray(scene.pos, np.float32)
        vel = np.ascontiguousarray(scene.vel, np.float32)
        self.lib.ref_add_particles(self.h, _ptr(pos), _ptr(vel), pos.shape[0])

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.ref_destroy(h)
            self.h = None

    def fill_water_tank(self) -> int:
        """The reference's own FLIPMethod::fillWaterTank (new particles brought to voxel space)."""
        return int(self.lib.ref_fill_water_tank(self.h))

    @property
    def num_particles(self) -> int:
        return int(self.lib.ref_num_particles(self.h))

    def particles(self):
        n = self.num_particles
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        adj = np.zeros(n, np.float32)
        self.lib.ref_get_particles(self.h, _ptr(pos), _ptr(vel), _ptr(adj))
        return pos, vel, adj

    def removed(self) -> np.ndarray:
        n = int(self.lib.ref_get_removed(self.h, None))
        out = np.zeros(n, np.uint8)
        self.lib.ref_get_removed(self.h, _ptr(out))
        return out

    def step(self, dt: float) -> None:
        self.lib.ref_step(self.h, dt)

    def post_process(self) -> None:
        """The reference's own FLIPMethod::postProcess (params.dt, vortPresRate 0.2,
        redistIteration 80)."""
        self.lib.ref_post_process(self.h)

    def attributes(self):
        n = self.num_particles
        vort = np.zeros(n, np.float32)
        curv = np.zeros(n, np.float32)
        self.lib.ref_get_attributes(self.h, _ptr(vort), _ptr(curv))
        return vort, curv

    def system(self):
        n = int(self.lib.ref_num_unknowns(self.h))
        b = np.zeros(n, np.float32)
        x = np.zeros(n, np.float32)
        cells = np.zeros(n, np.int64)
        self.lib.ref_get_system(self.h, _ptr(b), _ptr(x), _ptr(cells))
        return dict(b=b, x=x, cells=cells)
