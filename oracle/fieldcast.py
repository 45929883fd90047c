"""ORACLE (test infrastructure only): FieldCast's sparse -> VDB conversions restated in
numpy float32, voxel by voxel, as the reference's loops write them.

* convert_surface (base/header/FieldCast.h:362-440, convertSurfaceVDB): every stored cell
  of the sparse field gets phi * dx; the grid's background is background * dx; with the
  water tank the five slabs of the 3-cell border band take
  Min(cellCenter.y - waterlevel, value), cellCenter = Grid::worldPoint(i+.5, j+.5, k+.5)
  (Grid.h:432-437), lv = int((waterlevel - min.y) / dx + 1).
* convert_velocity (FieldCast.h:14-48, convertVelocityVDB): v * dx (Grid::worldVector,
  Grid.h:440-443) on the stored cells whose length is not below 1e-30.

The stored cells are those of the given tiles inside the grid. The result is grouped into
8^3 leaves (origin -> (active mask, values)), the layout the device export returns.
OpenVDB itself is not available here, so the restatement is compared with the device, not
with an OpenVDB tree.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
PAD = 16  # voxels of margin around the grid for the band (>= 3, a multiple of 8)


def _stored(tiles, nx, ny, nz):
    """Voxel coordinates (N, 3) of the stored cells in tile storage order, and the mask of
    storage slots inside the grid."""
    l = np.arange(512)
    li, lj, lk = l & 7, (l >> 3) & 7, l >> 6
    i = (tiles[:, 0:1] * 8 + li[None, :]).reshape(-1)
    j = (tiles[:, 1:2] * 8 + lj[None, :]).reshape(-1)
    k = (tiles[:, 2:3] * 8 + lk[None, :]).reshape(-1)
    inside = (i < nx) & (j < ny) & (k < nz)
    return np.stack([i, j, k], 1), inside


def _shape(nx, ny, nz):
    r8 = lambda n: (n + 2 * PAD + 7) // 8 * 8
    return (r8(nz), r8(ny), r8(nx))


def _leaves(val, act, comps):
    """Group a padded voxel volume into 8^3 leaves with at least one active voxel."""
    out = {}
    Z, Y, X = act.shape
    for kz in range(0, Z, 8):
        for jy in range(0, Y, 8):
            for ix in range(0, X, 8):
                a = act[kz:kz + 8, jy:jy + 8, ix:ix + 8]
                if not a.any():
                    continue
                v = val[kz:kz + 8, jy:jy + 8, ix:ix + 8]
                origin = (ix - PAD, jy - PAD, kz - PAD)
                out[origin] = (a.reshape(512).copy(), v.reshape((512, comps) if comps > 1 else 512).copy())
    return out


def _level_index(level, miny, dx):
    return int(F32(F32(F32(level) - F32(miny)) / dx) + F32(1))


def convert_surface(surf, tiles, nx, ny, nz, translate, scale, background=10.0, tank=False, level=-1e10):
    dx = F32(scale[0])
    # the band may reach above the grid (a water level near or above the top)
    shape = _shape(nx, max(ny, _level_index(level, translate[1], dx) + 4) if tank else ny, nz)
    val = np.full(shape, F32(background) * dx, F32)
    act = np.zeros(shape, bool)
    ijk, inside = _stored(tiles, nx, ny, nz)
    ijk = ijk[inside]
    phi = np.asarray(surf, F32)[inside] * dx
    val[ijk[:, 2] + PAD, ijk[:, 1] + PAD, ijk[:, 0] + PAD] = phi
    act[ijk[:, 2] + PAD, ijk[:, 1] + PAD, ijk[:, 0] + PAD] = True
    if tank:
        ei, ek = nx - 1, nz - 1
        bnd = 3
        level = F32(level)
        miny = F32(translate[1])
        lv = _level_index(level, miny, dx)
        sy, ty = F32(scale[1]), F32(translate[1])

        def slab(i0, i1, j0, j1, k0, k1):
            for j in range(j0, j1 + 1):
                cy = F32(F32(F32(j) + F32(0.5)) * sy) + ty
                a = F32(cy - level)
                sl = (slice(k0 + PAD, k1 + PAD + 1), j + PAD, slice(i0 + PAD, i1 + PAD + 1))
                cur = val[sl]
                val[sl] = np.where(a < cur, a, cur)
                act[sl] = True

        slab(-bnd, ei + bnd, -bnd, 0, -bnd, ek + bnd)
        slab(-bnd, 0, -bnd, lv + bnd, -bnd, ek + bnd)
        slab(ei, ei + bnd, -bnd, lv + bnd, -bnd, ek + bnd)
        slab(-bnd, ei + bnd, -bnd, lv + bnd, -bnd, 0)
        slab(-bnd, ei + bnd, -bnd, lv + bnd, ek, ek + bnd)
    return _leaves(val, act, 1)


def convert_velocity(velo, tiles, nx, ny, nz, scale):
    sc = np.asarray(scale, F32)
    shape = _shape(nx, ny, nz)
    val = np.zeros(shape + (3,), F32)
    act = np.zeros(shape, bool)
    ijk, inside = _stored(tiles, nx, ny, nz)
    w = np.asarray(velo, F32)[inside] * sc[None, :]
    length = np.sqrt((w[:, 0] * w[:, 0] + w[:, 1] * w[:, 1]) + w[:, 2] * w[:, 2])
    keep = ~(length < F32(1e-30))
    ijk, w = ijk[inside][keep], w[keep]
    val[ijk[:, 2] + PAD, ijk[:, 1] + PAD, ijk[:, 0] + PAD] = w
    act[ijk[:, 2] + PAD, ijk[:, 1] + PAD, ijk[:, 0] + PAD] = True
    return _leaves(val, act, 3)
