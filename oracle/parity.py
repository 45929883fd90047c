"""ORACLE (test infrastructure only): one FLIP step from an identical state on the device
and on the oracle, and the relative errors between the two.

The oracle runs the step in build mode (8^3 tiles, the reference's rules for every stage,
FluidProjection::solve's system solved by CG in FP64 to ||r||/||b|| < 1e-12), so it is the
FP64 projection the device's solver forms are judged against. Errors are
max|device - oracle| / max|oracle| over:

  pressure        the pressure field of the cells of active tiles after the step
                  (fluid cells and the air cells that take their neighbours' mean,
                  FluidProjection.cu:293-335)
  grid_velocity   the projected grid velocity ("comp", FluidProjection.cu:337-378)
  particle_velocity / particle_position   after G2P and advection (FLIPMethod.cu:54-175),
                  particles matched by id

Used by the GPU parity tests and, as a checker outside every timed region, by the
benchmark's parity report. Nothing here is part of the product path.
"""
from __future__ import annotations

import dataclasses
import os
import time

import numpy as np

from oracle import bindings as B


def rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a - b).max()) if a.size else 0.0


def real_cells(tiles, nx, ny, nz) -> np.ndarray:
    """Storage-order mask of the cells of active 8^3 tiles that lie inside the grid."""
    l = np.arange(512)
    li, lj, lk = l & 7, (l >> 3) & 7, l >> 6
    i = tiles[:, 0:1] * 8 + li[None, :]
    j = tiles[:, 1:2] * 8 + lj[None, :]
    k = tiles[:, 2:3] * 8 + lk[None, :]
    return ((i < nx) & (j < ny) & (k < nz)).reshape(-1)


def with_state(scene, pos, vel):
    """The scene with its particles replaced (voxel space)."""
    return dataclasses.replace(scene, pos=np.ascontiguousarray(pos, np.float32),
                               vel=np.ascontiguousarray(vel, np.float32))


def _by_id(pos, vel, ids):
    o = np.argsort(ids, kind="stable")
    return pos[o], vel[o], ids[o]


def oracle_step(scene, tol: float = 1e-12, threads: int | None = None) -> dict:
    """One oracle step (build mode, FP64 projection) from the scene's particles."""
    if not os.path.exists(B.ORACLE_SO):
        B.build(ref=False)
    t0 = time.perf_counter()
    ora = B.Oracle(scene, block=8, solver="fp64", tol=tol, threads=threads or os.cpu_count())
    ora.step(scene.dt)
    pos, vel, _, ids = ora.particles()
    out = dict(tiles=ora.tiles(), pres=ora.field(B.FIELD_PRES), comp=ora.field(B.FIELD_COMP),
               solver_rel=ora.last_rel(), seconds=time.perf_counter() - t0)
    out["pos"], out["vel"], out["ids"] = _by_id(pos, vel, ids)
    del ora
    return out


def device_step(flip, scene, **params) -> dict:
    """One device step through the C ABI from the scene's particles (params as for
    FlipSim.from_scene; none given = the library's defaults, the benchmark's settings)."""
    sim = flip.FlipSim.from_scene(scene, **params)
    status = sim.step(scene.dt)
    st = sim.stats()
    pos, vel, _, ids = sim.particles()
    fi = sim.frame_info()
    out = dict(status=status, stats=st, tiles=sim.tiles(), pres=sim.field(flip.FIELD_PRES),
               comp=sim.field(flip.FIELD_COMP), nx=fi["nx"], ny=fi["ny"], nz=fi["nz"])
    out["pos"], out["vel"], out["ids"] = _by_id(pos, vel, ids)
    sim.close()
    return out


def compare(dev: dict, ora: dict) -> dict:
    """Relative errors of a device step against the oracle step from the same state."""
    same_tiles = dev["tiles"].shape == ora["tiles"].shape and bool(np.array_equal(dev["tiles"], ora["tiles"]))
    same_ids = dev["ids"].shape == ora["ids"].shape and bool(np.array_equal(dev["ids"], ora["ids"]))
    out = {"same_tiles": same_tiles, "same_particles": same_ids}
    if same_tiles:
        real = real_cells(dev["tiles"], dev["nx"], dev["ny"], dev["nz"])
        out["pressure"] = rel_err(dev["pres"][real], ora["pres"][real])
        out["grid_velocity"] = rel_err(dev["comp"][real], ora["comp"][real])
    if same_ids:
        out["particle_velocity"] = rel_err(dev["vel"], ora["vel"])
        out["particle_position"] = rel_err(dev["pos"], ora["pos"])
    st = dev["stats"]
    out.update(residual_rel=st["residual_rel"], residual_max_dx=st["residual_max_dx"],
               solver_iterations=st["solver_iterations"], refinements=st["refinements"],
               converged=bool(st["converged"]))
    return out
