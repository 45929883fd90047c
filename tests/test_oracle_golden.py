"""The CPU oracle against golden vectors produced by the reference's own FLIP code.

The fixtures in tests/golden were generated by tests/golden/make_golden.py from the
reference's unmodified FLIP sources compiled for the host. The oracle restatement
(oracle/flip_oracle.cpp) in its compat mode (4^3 tiles, the reference's tile-index
wrap and CG rule, one thread) must reproduce them bit for bit.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN
from vare_gb300 import scenes


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _small20_scene(g):
    n = int(g["n"])
    sc = scenes.small(n, dt=float(g["dt"]))
    sc.colliders = [(c[0:3], c[3:6], c[6:9]) for c in g["colliders"]]
    sc.collider_band = float(g["band"])
    return sc


def test_compat_small20_bit_exact(oracle_lib):
    B = oracle_lib
    g = np.load(os.path.join(GOLDEN, "ref_compat_small20.npz"))
    sc = _small20_scene(g)
    ora = B.Oracle(sc, block=4, compat=True, solver="reference", max_iter=200, threads=1)
    for s in range(len(g["hashes"])):
        ora.step(sc.dt)
        pos, vel, adj, ids = ora.particles()
        assert ora.num_particles == g["counts"][s], f"particle count, step {s}"
        assert ora.frame_info()["ntiles"] == g["ntiles"][s], f"active tiles, step {s}"
        assert sha(pos, vel, adj) == g["hashes"][s], f"particle arrays differ at step {s}"
    np.testing.assert_array_equal(ids, g["ids"])
    np.testing.assert_array_equal(ora.tiles(), g["tiles"])
    np.testing.assert_array_equal(ora.markers(), g["markers"])
    np.testing.assert_array_equal(ora.removed(), g["removed"])
    for which, key in [(B.FIELD_MASS, "mass"), (B.FIELD_SURF, "surf"), (B.FIELD_PRES, "pres"),
                       (B.FIELD_VELO, "velo"), (B.FIELD_COMP, "comp"), (B.FIELD_MARK, "mark")]:
        np.testing.assert_array_equal(ora.field(which), g[key], err_msg=key)
    sysm = ora.system()
    np.testing.assert_array_equal(sysm["b"], g["b"])
    np.testing.assert_array_equal(sysm["x"], g["x"])


def test_compat_cg64_small24_bit_exact(oracle_lib):
    B = oracle_lib
    g = np.load(os.path.join(GOLDEN, "ref_cg64_small24.npz"))
    sc = scenes.small(int(g["n"]))
    ora = B.Oracle(sc, block=4, compat=True, solver="fp64", tol=1e-10, threads=1)
    for s in range(3):
        ora.step(sc.dt)
        if f"pos{s}" not in g:
            continue
        pos, vel, adj, ids = ora.particles()
        np.testing.assert_array_equal(pos, g[f"pos{s}"])
        np.testing.assert_array_equal(vel, g[f"vel{s}"])
        np.testing.assert_array_equal(adj, g[f"adj{s}"])
        np.testing.assert_array_equal(ids, g[f"ids{s}"])
    np.testing.assert_array_equal(ora.dense(B.FIELD_PRES), g["pres"])
    np.testing.assert_array_equal(ora.dense(B.FIELD_COMP), g["comp"])


def test_compat_dam64_hashes(oracle_lib):
    B = oracle_lib
    g = np.load(os.path.join(GOLDEN, "ref_dam64.npz"))
    sc = scenes.config0()
    assert sc.num_particles == 505856
    ora = B.Oracle(sc, block=4, compat=True, solver="reference", max_iter=200, threads=1)
    for s in range(len(g["hashes"])):
        ora.step(sc.dt)
        pos, vel, adj, _ = ora.particles()
        assert ora.num_particles == g["counts"][s]
        assert sha(pos, vel, adj) == g["hashes"][s], f"step {s}"
    assert ora.frame_info()["ntiles"] == int(g["ntiles"])


def test_oracle_tile_rule_block8(oracle_lib):
    """8^3 activation: a tile is active iff some particle's tile (int(p)/8, clamped) is
    within one tile of it; slots follow linear tile order."""
    B = oracle_lib
    sc = scenes.small(32)
    ora = B.Oracle(sc, block=8, threads=1)
    ora.rebuild()
    fi = ora.frame_info()
    f = np.array([fi["fx"], fi["fy"], fi["fz"]])
    t = np.clip(np.maximum(np.trunc(sc.pos).astype(np.int64) // 8, 0), 0, f - 1)
    occ = np.zeros(f[::-1], bool)
    occ[t[:, 2], t[:, 1], t[:, 0]] = True
    act = np.zeros_like(occ)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sh = np.zeros_like(occ)
                src = occ[max(0, -dz):occ.shape[0] - max(0, dz), max(0, -dy):occ.shape[1] - max(0, dy),
                          max(0, -dx):occ.shape[2] - max(0, dx)]
                sh[max(0, dz):occ.shape[0] - max(0, -dz), max(0, dy):occ.shape[1] - max(0, -dy),
                   max(0, dx):occ.shape[2] - max(0, -dx)] = src
                act |= sh
    kk, jj, ii = np.nonzero(act)
    expect = np.stack([ii, jj, kk], 1)
    order = np.lexsort((expect[:, 0], expect[:, 1], expect[:, 2]))
    np.testing.assert_array_equal(ora.tiles(), expect[order])


def test_oracle_block8_matches_block4(oracle_lib):
    """The 8^3 layout changes storage order only: with the pressure system solved in FP64
    the particles after a step agree with the 4^3 (reference-layout) oracle to 1e-6."""
    B = oracle_lib
    sc = scenes.small(24)
    a = B.Oracle(sc, block=4, compat=False, solver="fp64", tol=1e-12, threads=1)
    b = B.Oracle(sc, block=8, compat=False, solver="fp64", tol=1e-12, threads=1)
    for _ in range(3):
        a.step(sc.dt)
        b.step(sc.dt)
    pa, va, _, ia = a.particles()
    pb, vb, _, ib = b.particles()
    np.testing.assert_array_equal(np.sort(ia), np.sort(ib))
    oa, ob = np.argsort(ia), np.argsort(ib)
    assert np.abs(pa[oa] - pb[ob]).max() <= 1e-6 * np.abs(pa).max()
    assert np.abs(va[oa] - vb[ob]).max() <= 1e-6 * np.abs(va).max()


def test_oracle_stages_equal_step(oracle_lib):
    B = oracle_lib
    sc = scenes.small(16)
    a = B.Oracle(sc, block=8, threads=1)
    b = B.Oracle(sc, block=8, threads=1)
    a.step(sc.dt)
    b.rebuild(); b.p2g(); b.mark(); b.build_system(); b.solve(); b.update_velocity()
    b.update_particles(sc.dt); b.compact()
    for x, y in zip(a.particles(), b.particles()):
        np.testing.assert_array_equal(x, y)


def test_reference_build_matches_oracle_live():
    """Where the reference checkout is present, its host build agrees with the oracle."""
    from oracle import bindings as B
    if not B.reference_available():
        pytest.skip("reference host build not available")
    sc = scenes.small(16, dt=1.0 / 60.0)
    ref = B.RefSim(sc)
    B._oracle_lib().ora_set_threads(1)
    ora = B.Oracle(sc, block=4, compat=True, solver="reference", max_iter=200, threads=1)
    for _ in range(4):
        ref.step(sc.dt)
        ora.step(sc.dt)
    pr, vr, ar = ref.particles()
    po, vo, ao, _ = ora.particles()
    np.testing.assert_array_equal(pr, po)
    np.testing.assert_array_equal(vr, vo)


def test_compat_tank24_bit_exact(oracle_lib):
    """Water tank (FLIPMethod::fillWaterTank, the tank's always-active tile rows, damping
    band): the restatement reproduces the reference's own fill and three steps bit for bit."""
    B = oracle_lib
    g = np.load(os.path.join(GOLDEN, "ref_tank24.npz"))
    sc = scenes.small(24, seed=11)
    sc.wall_level = float(g["wall_level"])
    ora = B.Oracle(sc, block=4, compat=True, solver="reference", max_iter=200, threads=1, tank=True,
                   damping_band=float(g["damping_band"]))
    assert ora.fill_water_tank(8) == int(g["added"])
    pos0, vel0, _, _ = ora.particles()
    np.testing.assert_array_equal(pos0, g["pos0"])
    np.testing.assert_array_equal(vel0, g["vel0"])
    for s in range(len(g["hashes"])):
        ora.step(sc.dt)
        pos, vel, adj, ids = ora.particles()
        assert ora.num_particles == g["counts"][s], f"particle count, step {s}"
        assert ora.frame_info()["ntiles"] == g["ntiles"][s], f"active tiles, step {s}"
        assert sha(pos, vel, adj) == g["hashes"][s], f"particle arrays differ at step {s}"
    np.testing.assert_array_equal(ids, g["ids"])
