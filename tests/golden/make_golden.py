"""Generate golden vectors from the reference's own FLIP step.

Runs the reference's unmodified FLIP sources compiled for the host
(oracle/_ref/libbora_ref*.so, built by `make -C oracle ref` from a reference checkout)
on seeded scenes from vare_gb300.scenes, single-threaded, and writes the results as
.npz fixtures next to this script. The fixtures are committed; this script only needs
re-running when a scene definition changes.

Fixtures:
  ref_compat_small20.npz  20^3 dam break + sphere with two box colliders, the
                          reference's CG rule (absolute 1e-3, 201 iterations), 12 steps:
                          per-step SHA-256 of the particle arrays, final-step fields.
  ref_cg64_small24.npz    24^3 dam break + sphere, the same step with the pressure
                          system solved to 1e-10 relative in FP64 (libbora_ref_cg64),
                          3 steps: particle arrays after steps 1 and 3.
  ref_dam64.npz           64^3 dam break (505,856 particles), reference CG rule,
                          2 steps: SHA-256 of the particle arrays and summaries.
  ref_tank24.npz          24^3 dam break + sphere with the water tank on (wall level 0.25,
                          damping band 0.1): FLIPMethod::fillWaterTank's particles, then 3
                          steps with the reference CG rule: per-step SHA-256 and counts.

  ref_post_small20.npz    20^3 dam break + sphere (dt 1/60) set swirling (6 rad/s about
                          the vertical axis), two frames of step +
                          FLIPMethod::postProcess (redistIteration 80, vortPresRate 0.2):
                          per-frame SHA-256 of the surface, normal and velocity fields and
                          the particles' vorticity and curvature; final arrays.
  ref_post_bubble32.npz   32^3 water tank with an enclosed air bubble (vare_gb300.scenes.
                          tank_bubble), one postProcess: the tank's scan fills the bubble.

Usage: OMP_NUM_THREADS=1 python tests/golden/make_golden.py [fixture ...]
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from oracle import bindings as B  # noqa: E402
from vare_gb300 import scenes  # noqa: E402


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def remove_order(ids: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """Array::remove (base/header/Array.h:996-1024) applied to an id array."""
    a = ids.copy()
    size = len(a)
    end, dele = size - 1, 0
    for n in range(len(mask)):
        if n >= size:
            break
        if mask[n]:
            dele += 1
            q = end
            while q >= n + 1:
                if mask[q] == 0:
                    a[n] = a[q]
                    end = q - 1
                    break
                q -= 1
    return a[:size - dele]


def colliders_for(n: int):
    return [((n * 0.45, -2.0, n * 0.3), (n * 0.6, n * 0.3, n * 0.7), (0.0, 0.0, 0.0)),
            ((n * 0.8, n * 0.1, -1.0), (n * 0.95, n * 0.2, n * 0.4), (-3.0, 1.0, 0.0))]


def small20():
    n = 20
    sc = scenes.small(n, dt=1.0 / 60.0)
    sc.colliders = colliders_for(n)
    ref = B.RefSim(sc)
    ids = np.arange(sc.num_particles, dtype=np.int64)
    hashes, counts, ntiles = [], [], []
    for s in range(12):
        ref.step(sc.dt)
        pos, vel, adj = ref.particles()
        ids = remove_order(ids, ref.removed())
        hashes.append(sha(pos, vel, adj))
        counts.append(ref.num_particles)
        ntiles.append(ref.frame_info()["ntiles"])
    fi = ref.frame_info()
    out = dict(n=n, dt=sc.dt, seed=sc.seed, colliders=np.array([np.concatenate(c) for c in sc.colliders], np.float32),
               band=sc.collider_band, hashes=np.array(hashes), counts=np.array(counts), ntiles=np.array(ntiles),
               pos=pos, vel=vel, adj=adj, ids=ids, removed=ref.removed(), tiles=ref.tiles(),
               markers=ref.markers(), frame=np.array([fi[k] for k in ("fx", "fy", "fz", "block", "nx", "ny", "nz")]),
               mass=ref.field(B.FIELD_MASS), surf=ref.field(B.FIELD_SURF), pres=ref.field(B.FIELD_PRES),
               velo=ref.field(B.FIELD_VELO), comp=ref.field(B.FIELD_COMP), mark=ref.field(B.FIELD_MARK),
               b=ref.system()["b"], x=ref.system()["x"])
    np.savez_compressed(os.path.join(HERE, "ref_compat_small20.npz"), **out)
    print("small20", counts[-1], ntiles[-1])


def small24_cg64():
    n = 24
    sc = scenes.small(n)
    ref = B.RefSim(sc, converged=True, tol=1e-10)
    out = dict(n=n, dt=sc.dt, seed=sc.seed)
    ids = np.arange(sc.num_particles, dtype=np.int64)
    for s in range(3):
        ref.step(sc.dt)
        pos, vel, adj = ref.particles()
        ids = remove_order(ids, ref.removed())
        if s != 1:
            out[f"pos{s}"], out[f"vel{s}"], out[f"adj{s}"], out[f"ids{s}"] = pos, vel, adj, ids
    out["pres"] = ref.dense(B.FIELD_PRES)
    out["comp"] = ref.dense(B.FIELD_COMP)
    out["velo"] = ref.dense(B.FIELD_VELO)
    out["mass"] = ref.dense(B.FIELD_MASS)
    out["mark"] = (ref.dense(B.FIELD_MARK) >= B.K_FLUID).astype(np.uint8)
    np.savez_compressed(os.path.join(HERE, "ref_cg64_small24.npz"), **out)
    print("small24", len(ids))


def dam64():
    sc = scenes.config0()
    ref = B.RefSim(sc)
    hashes, counts, ke = [], [], []
    for s in range(2):
        ref.step(sc.dt)
        pos, vel, adj = ref.particles()
        hashes.append(sha(pos, vel, adj))
        counts.append(ref.num_particles)
        ke.append(float(0.5 * np.sum(vel.astype(np.float64) ** 2)))
    np.savez_compressed(os.path.join(HERE, "ref_dam64.npz"), hashes=np.array(hashes), counts=np.array(counts),
                        ke=np.array(ke), ntiles=ref.frame_info()["ntiles"], dt=sc.dt, seed=sc.seed)
    print("dam64", counts, ke)


def tank_scene():
    sc = scenes.small(24, seed=11)
    sc.wall_level = 0.25  # world units: the tank is 6 cells deep
    return sc


def tank24():
    sc = tank_scene()
    ref = B.RefSim(sc, tank=True, damping_band=0.1)
    added = ref.fill_water_tank()
    pos0, vel0, _ = ref.particles()
    ids = np.arange(ref.num_particles, dtype=np.int64)
    hashes, counts, ntiles = [], [], []
    for s in range(3):
        ref.step(sc.dt)
        pos, vel, adj = ref.particles()
        ids = remove_order(ids, ref.removed())
        hashes.append(sha(pos, vel, adj))
        counts.append(ref.num_particles)
        ntiles.append(ref.frame_info()["ntiles"])
    np.savez_compressed(os.path.join(HERE, "ref_tank24.npz"), added=added, pos0=pos0, vel0=vel0,
                        hashes=np.array(hashes), counts=np.array(counts), ntiles=np.array(ntiles), ids=ids,
                        wall_level=sc.wall_level, damping_band=0.1)
    print("tank24", added, counts, ntiles)


def _post_record(ref):
    surf = ref.field(B.FIELD_SURF)
    comp = ref.field(B.FIELD_COMP)
    velo = ref.field(B.FIELD_VELO)
    vort, curv = ref.attributes()
    return surf, comp, velo, vort, curv


def swirl(sc, omega: float = 6.0):
    """The scene with particles rotating about the vertical axis through the box centre
    (omega rad/s, voxel units), so that the vorticity threshold (0.2 world units) is
    exceeded."""
    c = np.array(sc.res, np.float32) * 0.5
    d = sc.pos - c
    vel = np.zeros_like(sc.pos)
    vel[:, 0] = -omega * d[:, 2]
    vel[:, 2] = omega * d[:, 0]
    sc.vel = vel.astype(np.float32)
    return sc


def post_small20():
    sc = swirl(scenes.small(20, dt=1.0 / 60.0))
    ref = B.RefSim(sc)
    hashes = []
    for f in range(2):
        ref.step(sc.dt)
        ref.post_process()
        hashes.append(sha(*_post_record(ref)))
    surf, comp, velo, vort, curv = _post_record(ref)
    pos, vel, adj = ref.particles()
    np.savez_compressed(os.path.join(HERE, "ref_post_small20.npz"), hashes=np.array(hashes), surf=surf, comp=comp,
                        velo=velo, vort=vort, curv=curv, pos=pos, tiles=ref.tiles(), dt=sc.dt)
    print("post_small20", hashes[-1][:16], float(np.abs(vort).max()), float(np.abs(curv).max()))


def post_bubble32():
    sc = scenes.tank_bubble(32)
    ref = B.RefSim(sc, tank=True)
    ref.post_process()
    surf, comp, velo, vort, curv = _post_record(ref)
    np.savez_compressed(os.path.join(HERE, "ref_post_bubble32.npz"), hash=sha(surf, comp, velo, vort, curv),
                        surf=surf, vort=vort, curv=curv, tiles=ref.tiles(), wall_level=sc.wall_level, dt=sc.dt)
    print("post_bubble32", int(np.sum(surf < 0)), float(np.abs(curv).max()))


if __name__ == "__main__":
    if not B.reference_available():
        B.build(ref=True)
    which = sys.argv[1:] or ["small20", "small24_cg64", "dam64", "tank24", "post_small20", "post_bubble32"]
    for name in which:
        globals()[name]()
