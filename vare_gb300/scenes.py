"""Seeded synthetic FLIP scenes (dam break, dam break + falling sphere, tanks).

The reference measures on no public data set; its Houdini node seeds particles from
input geometry (houdini/source/SOP_FlipWater.cpp:296-324) or fills a tank with a
hashed jitter (base/source/FLIPMethod.cu:407-478). Benchmarks and parity tests use
these generated scenes instead. Every particle position is a pure function of
(seed, cell index, sample index), so the oracle and the device see identical input:

    h = splitmix64(seed XOR (cell_linear * ppc + s))
    u = (bits 43..63, bits 22..42, bits 1..21 of h) * 2**-21      in [0, 1)^3
    voxel position = (i, j, k) + u        (computed in float64, rounded to float32)

`cell_linear = i + nx * (j + ny * k)` runs x-fastest over the grid, and particles are
emitted in that order, `s` innermost. A cell is filled when its centre lies inside
the scene's fluid region. Initial velocities are zero.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser over a uint64 array (Steele, Lea & Flood 2014)."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


@dataclasses.dataclass
class Scene:
    """A generated scene: grid, parameters and voxel-space particles."""

    name: str
    res: tuple[int, int, int]
    bmin: tuple[float, float, float]
    bmax: tuple[float, float, float]
    dt: float
    pos: np.ndarray  # (N, 3) float32, voxel space
    vel: np.ndarray  # (N, 3) float32, voxel units per second
    wall_level: float = 2.0  # world units; above the box top => solid walls on all faces
    gravity: tuple[float, float, float] = (0.0, -9.8, 0.0)
    colliders: list = dataclasses.field(default_factory=list)  # [(lo3, hi3, vel3)] voxel space
    collider_band: float = 3.0
    seed: int = 0

    @property
    def voxel_size(self) -> float:
        return (self.bmax[0] - self.bmin[0]) / self.res[0]

    @property
    def num_particles(self) -> int:
        return int(self.pos.shape[0])


def _jitter(cells: np.ndarray, ijk: np.ndarray, seed: int, ppc: int) -> np.ndarray:
    """Particles for the given cells (linear ids and (i,j,k)), `ppc` per cell."""
    n = cells.shape[0]
    s = np.arange(ppc, dtype=np.uint64)
    key = (cells.astype(np.uint64)[:, None] * np.uint64(ppc) + s[None, :]).reshape(-1)
    h = splitmix64(np.uint64(seed) ^ key)
    mask = np.uint64(0x1FFFFF)
    scale = 2.0 ** -21
    ux = ((h >> np.uint64(43)) & mask).astype(np.float64) * scale
    uy = ((h >> np.uint64(22)) & mask).astype(np.float64) * scale
    uz = ((h >> np.uint64(1)) & mask).astype(np.float64) * scale
    base = np.repeat(ijk.astype(np.float64), ppc, axis=0)
    pos = np.empty((n * ppc, 3), dtype=np.float32)
    pos[:, 0] = (base[:, 0] + ux).astype(np.float32)
    pos[:, 1] = (base[:, 1] + uy).astype(np.float32)
    pos[:, 2] = (base[:, 2] + uz).astype(np.float32)
    return pos


def _fill(res, bmin, bmax, inside, seed, ppc, chunk_k=16):
    """Emit particles for all cells whose world-space centre satisfies `inside`."""
    nx, ny, nz = res
    h = (bmax[0] - bmin[0]) / nx
    out = []
    ii = np.arange(nx)
    jj = np.arange(ny)
    for k0 in range(0, nz, chunk_k):
        kk = np.arange(k0, min(nz, k0 + chunk_k))
        K, J, I = np.meshgrid(kk, jj, ii, indexing="ij")
        cx = bmin[0] + (I + 0.5) * h
        cy = bmin[1] + (J + 0.5) * h
        cz = bmin[2] + (K + 0.5) * h
        m = inside(cx, cy, cz)
        if not m.any():
            continue
        I, J, K = I[m], J[m], K[m]
        lin = I.astype(np.int64) + nx * (J.astype(np.int64) + ny * K.astype(np.int64))
        ijk = np.stack([I, J, K], axis=1)
        out.append(_jitter(lin, ijk, seed, ppc))
    if not out:
        return np.zeros((0, 3), np.float32)
    return np.concatenate(out, axis=0)


def dam_break(n: int = 64, block=(0.4, 0.6), seed: int = 0x5EED0000, ppc: int = 8,
              dt: float = 1.0 / 240.0, sphere=None, name: str = "dam_break") -> Scene:
    """Unit-box dam break: fluid where the cell centre has x < block[0] and y < block[1]
    (all z), optionally plus a sphere (cx, cy, cz, r). Solid walls on all faces."""
    res = (n, n, n)
    bmin = (0.0, 0.0, 0.0)
    bmax = (1.0, 1.0, 1.0)

    def inside(x, y, z):
        m = (x < block[0]) & (y < block[1])
        if sphere is not None:
            cx, cy, cz, r = sphere
            m |= (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 < r * r
        return m

    pos = _fill(res, bmin, bmax, inside, seed, ppc)
    vel = np.zeros_like(pos)
    return Scene(name=name, res=res, bmin=bmin, bmax=bmax, dt=dt, pos=pos, vel=vel, seed=seed)


def config0() -> Scene:
    """64^3 dam break, dt = 1/240 (505,856 particles)."""
    return dam_break(64, (0.4, 0.6), seed=0x5EED0000, dt=1.0 / 240.0, name="dam_break_64")


def config1() -> Scene:
    """256^3 dam break (x<0.35, y<0.5) plus a sphere at (0.7, 0.8, 0.5), r = 0.12,
    dt = 1/480 (24,564,400 particles at 8 per cell)."""
    return dam_sphere(256)


def dam_sphere(n: int) -> Scene:
    """The 256^3 scene's geometry, seed and dt at n^3 (n = 160: about 6 M particles, a case
    larger than the 129 MB L2 that a profiler's kernel replays keep small)."""
    return dam_break(n, (0.35, 0.5), seed=0x5EED0001, dt=1.0 / 480.0,
                     sphere=(0.7, 0.8, 0.5, 0.12), name=f"dam_sphere_{n}")


def config3(scale: int = 1) -> Scene:
    """Large sparse domain: 1024x512x1024 cells (unit-wide box, 0.5 tall), a shallow tank
    8 cells deep over the whole floor, a wave column (x < 0.04, lower 30% of the height,
    all z) released at one end, and a static box obstacle at mid-span; dt = 1/960,
    seed 0x5EED0003. About 119 M particles at 8 per cell, about 6% of the 1,048,576
    tiles active. `scale` divides the resolution (8 gives a 128x64x128 copy with a
    1-cell tank for parity tests)."""
    nx, ny, nz = 1024 // scale, 512 // scale, 1024 // scale
    res = (nx, ny, nz)
    bmin = (0.0, 0.0, 0.0)
    bmax = (1.0, 0.5, 1.0)
    depth = 0.5 * 8.0 / 512.0

    def inside(x, y, z):
        return (y < depth) | ((x < 0.04) & (y < 0.15))

    seed = 0x5EED0003
    pos = _fill(res, bmin, bmax, inside, seed, 8, chunk_k=max(1, 16 // scale))
    vel = np.zeros_like(pos)
    sc = Scene(name="tank_1024" if scale == 1 else f"tank_{nx}", res=res, bmin=bmin, bmax=bmax, dt=1.0 / 960.0,
               pos=pos, vel=vel, seed=seed)
    # static box obstacle at mid-span (voxel space), below the column's release height
    sc.colliders = [((0.45 * nx, -2.0, 0.3 * nz), (0.55 * nx, 0.06 * ny, 0.7 * nz), (0.0, 0.0, 0.0))]
    return sc


def tank_bubble(n: int = 32, depth: float = 0.625, bubble=(0.5, 0.3, 0.5, 0.16), seed: int = 0x5EED0004,
                dt: float = 1.0 / 120.0) -> Scene:
    """Water tank with an air bubble: fluid below `depth` (unit box, world units) except a
    sphere (cx, cy, cz, r); the wall level is the tank's depth, so the water tank's scan
    fills the enclosed bubble. Run with the water tank enabled."""
    res = (n, n, n)
    bmin = (0.0, 0.0, 0.0)
    bmax = (1.0, 1.0, 1.0)
    cx, cy, cz, r = bubble

    def inside(x, y, z):
        return (y < depth) & ((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 >= r * r)

    pos = _fill(res, bmin, bmax, inside, seed, 8)
    sc = Scene(name=f"tank_bubble_{n}", res=res, bmin=bmin, bmax=bmax, dt=dt, pos=pos, vel=np.zeros_like(pos),
               seed=seed)
    sc.wall_level = depth
    return sc


def small(n: int = 24, seed: int = 7, sphere: bool = True, dt: float = 1.0 / 120.0) -> Scene:
    """Small dam break + sphere scene for parity tests."""
    return dam_break(n, (0.4, 0.55), seed=seed, dt=dt,
                     sphere=(0.7, 0.75, 0.5, 0.15) if sphere else None, name=f"small_{n}")


def serving_request(r: int, rng: np.random.Generator | None = None) -> tuple[Scene, int]:
    """One request of the mixed-size serving stream: cubic domain, edge log-uniform in
    [32, 192] cells, fill fraction in [0.2, 0.5], dam break or sphere drop by parity.
    Returns the scene and its number of steps (50..400)."""
    rng = rng or np.random.default_rng(0x5EED1000 + r)
    edge = int(round(math.exp(rng.uniform(math.log(32), math.log(192)))))
    fill = float(rng.uniform(0.2, 0.5))
    steps = int(rng.integers(50, 401))
    seed = 0x5EED1000 + r
    if r % 2 == 0:
        sc = dam_break(edge, (fill ** (1 / 2), fill ** (1 / 2)), seed=seed, dt=1.0 / 240.0,
                       name=f"req{r}_dam_{edge}")
    else:
        h = fill ** (1 / 3)
        sc = dam_break(edge, (1.0, 0.25 * h), seed=seed, dt=1.0 / 240.0,
                       sphere=(0.5, 0.7, 0.5, 0.25 * h + 0.05), name=f"req{r}_drop_{edge}")
    return sc, steps


def serving_arrivals(n: int = 64, rate: float = 20.0, seed: int = 0x5EED1000) -> np.ndarray:
    """Poisson arrival times (s) of the serving stream: exponential gaps at `rate`/s."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def serving_plan(n: int = 64) -> list[tuple[int, int, float]]:
    """(edge, steps, fill) of each request of the stream, without generating particles."""
    out = []
    for r in range(n):
        rng = np.random.default_rng(0x5EED1000 + r)
        edge = int(round(math.exp(rng.uniform(math.log(32), math.log(192)))))
        fill = float(rng.uniform(0.2, 0.5))
        steps = int(rng.integers(50, 401))
        out.append((edge, steps, fill))
    return out
