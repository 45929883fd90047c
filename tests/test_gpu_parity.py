"""Parity of the CUDA FLIP substep (through the C ABI) with the CPU oracle.

Stage tests feed the device and the oracle identical inputs and require bit-exact
results wherever the stage's arithmetic is order-independent (tile set, dual-cell
binning via the count field, cell flags, right-hand side and stencil, velocity update,
G2P/advection). P2G sums and the pressure solve differ in summation order, so they are
compared with the relative tolerance max|gpu - ref| / max|ref| <= 1e-5.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from vare_gb300 import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative tolerance for order-dependent float results


def rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a - b).max())


def real_cells(tiles, nx, ny, nz) -> np.ndarray:
    """Storage-order mask of the cells of active tiles that lie inside the grid."""
    l = np.arange(512)
    li, lj, lk = l & 7, (l >> 3) & 7, l >> 6
    i = tiles[:, 0:1] * 8 + li[None, :]
    j = tiles[:, 1:2] * 8 + lj[None, :]
    k = tiles[:, 2:3] * 8 + lk[None, :]
    return ((i < nx) & (j < ny) & (k < nz)).reshape(-1)


def tight(**kw):
    d = dict(tolerance=1e-10, div_tolerance=1e-12, max_refinements=30, inner_tolerance=1e-4)
    d.update(kw)
    return d


def by_id(pos, vel, adj, ids):
    o = np.argsort(ids)
    return pos[o], vel[o], adj[o], ids[o]


def colliders_for(n):
    return [((n * 0.45, -2.0, n * 0.3), (n * 0.6, n * 0.3, n * 0.7), (0.0, 0.0, 0.0)),
            ((n * 0.8, n * 0.1, -1.0), (n * 0.95, n * 0.2, n * 0.4), (-3.0, 1.0, 0.0))]


def moving(sc, oracle_lib, steps: int = 1):
    """The scene after `steps` oracle steps from rest, as a new scene (ids renumbered in
    id order): from rest the first pressure solve is trivial (b = 0), so stage tests
    start from a moving state to exercise the solver."""
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=1)
    for _ in range(steps):
        ora.step(sc.dt)
    pos, vel, _, ids = ora.particles()
    o = np.argsort(ids)
    import dataclasses
    return dataclasses.replace(sc, pos=np.ascontiguousarray(pos[o]), vel=np.ascontiguousarray(vel[o]))


@pytest.fixture(params=["dam_sphere_24", "colliders_20", "padded_22", "slab_24x16x40"])
def scene(request, oracle_lib):
    name = request.param
    if name == "dam_sphere_24":
        sc = scenes.small(24)
    elif name == "colliders_20":
        sc = scenes.small(20, dt=1.0 / 60.0)
        sc.colliders = colliders_for(20)
    elif name == "padded_22":
        sc = scenes.small(22)
    else:
        sc = scenes.small(16)
        sc.res = (24, 16, 40)
        sc.bmax = (1.0, 16 / 24, 40 / 24)
        sc.pos = sc.pos[(sc.pos[:, 0] < 24) & (sc.pos[:, 1] < 16)]
        sc.vel = np.zeros_like(sc.pos)
    return moving(sc, oracle_lib, 2)


def _pair(gpu, oracle_lib, sc, **kw):
    sim = gpu.FlipSim.from_scene(sc, **tight(**kw))
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=1)
    return sim, ora


def test_frame_matches_oracle(gpu, oracle_lib, scene):
    sim, ora = _pair(gpu, oracle_lib, scene)
    fi, fo = sim.frame_info(), ora.frame_info()
    assert (fi["nx"], fi["ny"], fi["nz"]) == (fo["nx"], fo["ny"], fo["nz"])
    xo = ora.grid_xform()
    np.testing.assert_array_equal(fi["translate"], xo["translate"])
    np.testing.assert_array_equal(fi["scale"], xo["scale"])
    assert fi["voxel_wall"] == xo["voxel_wall"]
    np.testing.assert_array_equal(fi["voxel_gravity"], xo["voxel_gravity"])


def test_stages_bit_exact(gpu, oracle_lib, scene):
    B = oracle_lib
    sc = scene
    sim, ora = _pair(gpu, oracle_lib, sc)
    # rebuild + P2G + flags
    sim.run_stage(gpu.STAGE_REBUILD)
    sim.run_stage(gpu.STAGE_P2G)
    ora.rebuild(); ora.p2g(); ora.mark()
    tiles = sim.tiles()
    np.testing.assert_array_equal(tiles, ora.tiles())
    fi = sim.frame_info()
    real = real_cells(tiles, fi["nx"], fi["ny"], fi["nz"])
    # dual-cell binning: particle count per cell is exact
    np.testing.assert_array_equal(sim.field(gpu.FIELD_SURF)[real], ora.field(B.FIELD_SURF)[real])
    np.testing.assert_array_equal(sim.field(gpu.FIELD_FLAG)[real], ora.field(B.FIELD_MARK)[real].astype(np.uint8))
    assert rel_err(sim.field(gpu.FIELD_MASS)[real], ora.field(B.FIELD_MASS)[real]) <= 1e-6
    assert rel_err(sim.field(gpu.FIELD_VELO)[real], ora.field(B.FIELD_VELO)[real]) <= 1e-5
    # right-hand side and stencil from identical grid velocities
    velo = ora.field(B.FIELD_VELO)
    sim.set_field(gpu.FIELD_VELO, velo)
    sim.run_stage(gpu.STAGE_BUILD_SYSTEM)
    ora.build_system()
    sysm = ora.system()
    cells = sysm["cells"]
    rhs = sim.field(gpu.FIELD_RHS)
    np.testing.assert_array_equal(rhs[cells], sysm["b"])
    code = sim.field(gpu.FIELD_CODE).astype(np.int64)
    assert np.all(code[cells] & 0x8000)
    np.testing.assert_array_equal((code[cells] >> 8) & 15, sysm["vals"][:, 0].astype(np.int64))
    nbr_mask = np.zeros(len(cells), np.int64)
    for q in range(6):
        nbr_mask |= (sysm["cols"][:, 1 + q] >= 0).astype(np.int64) << q
    np.testing.assert_array_equal(code[cells] & 63, nbr_mask)
    others = np.ones(len(code), bool)
    others[cells] = False
    assert not np.any(code[others & real] & 0x8000)
    # velocity update from an identical pressure solution
    ora.solve()
    x = ora.system()["x"]
    pres = np.zeros(len(rhs), np.float32)
    pres[cells] = x
    sim.set_field(gpu.FIELD_PRES, pres)
    sim.run_stage(gpu.STAGE_UPDATE_VELOCITY)
    ora.update_velocity()
    np.testing.assert_array_equal(sim.field(gpu.FIELD_PRES)[real], ora.field(B.FIELD_PRES)[real])
    np.testing.assert_array_equal(sim.field(gpu.FIELD_COMP)[real], ora.field(B.FIELD_COMP)[real])
    # G2P + advection + kill from identical fields
    sim.run_stage(gpu.STAGE_UPDATE_PARTICLES, sc.dt)
    ora.update_particles(sc.dt)
    ora.compact()
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    for a, b, name in zip(g[:3], o[:3], ("pos", "vel", "adj")):
        np.testing.assert_array_equal(a, b, err_msg=name)


@pytest.mark.parametrize("solver", ["plain", "mixed"])
def test_solve_matches_fp64_oracle(gpu, oracle_lib, scene, solver):
    B = oracle_lib
    sc = scene
    sim, ora = _pair(gpu, oracle_lib, sc, solver=gpu.SOLVER_MIXED if solver == "mixed" else gpu.SOLVER_PLAIN)
    for st in (gpu.STAGE_REBUILD, gpu.STAGE_P2G, gpu.STAGE_BUILD_SYSTEM):
        sim.run_stage(st)
    ora.rebuild(); ora.p2g(); ora.mark()
    sim.set_field(gpu.FIELD_VELO, ora.field(B.FIELD_VELO))
    sim.run_stage(gpu.STAGE_BUILD_SYSTEM)
    ora.build_system()
    assert np.abs(ora.system()["b"]).max() > 0, "trivial right-hand side"
    status = sim.run_stage(gpu.STAGE_SOLVE)
    st = sim.stats()
    assert status == 0 and st["converged"] == 1, st
    assert st["solver_iterations"] > 0
    assert st["residual_rel"] <= 1e-10
    ora.solve()
    sysm = ora.system()
    p_gpu = sim.field(gpu.FIELD_PRES)[sysm["cells"]]
    assert rel_err(p_gpu, sysm["x"]) <= TOL
    # the oracle's FP64 residual of the device answer (rounded to float32, which adds up
    # to ~12 ulp(p) per row) agrees with the device's own FP64 residual report
    ora.set_solution(p_gpu)
    rmax = ora.residual_max()
    assert rmax <= 10 * st["residual_max"] + 16 * float(np.abs(sysm["x"]).max()) * 2.0 ** -24


@pytest.mark.parametrize("solver", ["plain", "mixed"])
def test_full_step_matches_oracle(gpu, oracle_lib, scene, solver):
    sc = scene
    sim, ora = _pair(gpu, oracle_lib, sc, solver=gpu.SOLVER_MIXED if solver == "mixed" else gpu.SOLVER_PLAIN)
    for _ in range(2):
        assert sim.step(sc.dt) == 0
        ora.step(sc.dt)
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    assert rel_err(g[0], o[0]) <= TOL
    assert rel_err(g[1], o[1]) <= TOL
    assert np.abs(g[2] - o[2]).max() <= 1e-3  # adjacency = min of integer counts


def test_step_matches_reference_golden(gpu):
    """One device step against the reference's own converged step (tests/golden)."""
    g = np.load(os.path.join(GOLDEN, "ref_cg64_small24.npz"))
    sc = scenes.small(int(g["n"]))
    sim = gpu.FlipSim.from_scene(sc, **tight())
    assert sim.step(sc.dt) == 0
    pos, vel, adj, ids = by_id(*sim.particles())
    ref_ids = g["ids0"]
    o = np.argsort(ref_ids)
    np.testing.assert_array_equal(ids, ref_ids[o])
    assert rel_err(pos, g["pos0"][o]) <= TOL
    assert rel_err(vel, g["vel0"][o]) <= TOL
    np.testing.assert_array_equal(adj, g["adj0"][o])
    # two more steps: chaotic amplification stays small over three steps
    sim.step(sc.dt)
    sim.step(sc.dt)
    pos, vel, adj, ids = by_id(*sim.particles())
    ref_ids = g["ids2"]
    o = np.argsort(ref_ids)
    np.testing.assert_array_equal(ids, ref_ids[o])
    assert rel_err(pos, g["pos2"][o]) <= TOL
    assert rel_err(vel, g["vel2"][o]) <= 1e-4


@pytest.mark.parametrize("solver", ["plain", "mixed"])
def test_deterministic(gpu, solver):
    sc = scenes.small(24)
    sv = gpu.SOLVER_MIXED if solver == "mixed" else gpu.SOLVER_PLAIN
    a = gpu.FlipSim.from_scene(sc, solver=sv)
    b = gpu.FlipSim.from_scene(sc, solver=sv)
    for _ in range(3):
        a.step(sc.dt)
        b.step(sc.dt)
    for x, y in zip(by_id(*a.particles()), by_id(*b.particles())):
        np.testing.assert_array_equal(x, y)


def test_multistep_statistics(gpu, oracle_lib):
    """Chaotic dynamics: after 20 steps compare conserved counts and bulk statistics."""
    sc = scenes.small(24)
    sim = gpu.FlipSim.from_scene(sc, tolerance=1e-8, div_tolerance=1e-9)
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-10, threads=os.cpu_count())
    for _ in range(20):
        sim.step(sc.dt)
        ora.step(sc.dt)
    gp, gv, _, _ = sim.particles()
    op, ov, _, _ = ora.particles()
    assert len(gp) == len(op)
    ke_g = 0.5 * np.sum(gv.astype(np.float64) ** 2)
    ke_o = 0.5 * np.sum(ov.astype(np.float64) ** 2)
    assert abs(ke_g - ke_o) <= 1e-3 * ke_o
    assert np.abs(gp.mean(0) - op.mean(0)).max() <= 1e-3


def test_edge_cases(gpu, oracle_lib):
    sc = scenes.small(16)
    # empty
    sim = gpu.FlipSim(sc.res, sc.bmin, sc.bmax, gpu.scene_params(sc))
    assert sim.step(sc.dt) == 0 and sim.num_particles == 0
    # a single particle, particles on the upper boundary and outside the grid
    pts = np.array([[3.3, 4.7, 5.1], [16.0, 16.0, 16.0], [15.99, 0.0, 8.0], [-0.5, 3.0, 3.0], [20.0, 3.0, 3.0],
                    [8.0, -3.0, 8.0]], np.float32)
    vel = np.array([[1, 2, 3], [0, 0, 0], [5, -5, 0], [0, 0, 0], [0, 0, 0], [0, -1, 0]], np.float32)
    sc2 = scenes.Scene(name="edge", res=sc.res, bmin=sc.bmin, bmax=sc.bmax, dt=sc.dt, pos=pts, vel=vel)
    sim.set_particles(pts, vel, space=gpu.SPACE_VOXEL)
    ora = oracle_lib.Oracle(sc2, block=8, solver="fp64", tol=1e-13, threads=1)
    for _ in range(2):
        sim.step(sc.dt)
        ora.step(sc.dt)
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    assert rel_err(g[0], o[0]) <= TOL and rel_err(g[1], o[1]) <= TOL


def test_world_space_round_trip(gpu):
    sc = scenes.small(16)
    sim = gpu.FlipSim(sc.res, sc.bmin, sc.bmax, gpu.scene_params(sc))
    fi = sim.frame_info()
    world = sc.pos * fi["scale"] + fi["translate"]
    sim.set_particles(world, sc.vel * fi["scale"], space=gpu.SPACE_WORLD)
    pos, _, _, ids = sim.particles(space=gpu.SPACE_VOXEL)
    np.testing.assert_allclose(pos[np.argsort(ids)], sc.pos, atol=2e-5 * 16)
    posw, _, _, ids = sim.particles(space=gpu.SPACE_WORLD)
    np.testing.assert_allclose(posw[np.argsort(ids)], world, atol=1e-6)


@pytest.mark.parametrize("solver", ["plain", "mixed"])
def test_full_size_invariants(gpu, solver):
    """The 256^3 dam-break + sphere scene (24,564,400 particles): size-independent
    properties after two steps - every particle kept once (solid walls), the count field
    sums to the stencil contributions, the tile set follows the activation rule, and the
    projection met max|b - Ap| * dx < 1e-5 with ||r||/||b|| < 1e-6."""
    sc = scenes.config1()
    assert sc.num_particles == 24564400
    sim = gpu.FlipSim.from_scene(sc, solver=gpu.SOLVER_MIXED if solver == "mixed" else gpu.SOLVER_PLAIN)
    for _ in range(2):
        status = sim.step(sc.dt)
        st = sim.stats()
        assert status == 0 and st["converged"] == 1, st
        assert st["residual_rel"] < 1e-6 and st["residual_max_dx"] < 1e-5
    pos, vel, adj, ids = sim.particles()
    assert len(ids) == sc.num_particles
    np.testing.assert_array_equal(np.sort(ids), np.arange(sc.num_particles, dtype=np.int32))
    assert np.isfinite(pos).all() and np.isfinite(vel).all()
    assert pos.min() >= 0.0 and pos.max() <= 256.0
    # rebuild for the current positions and check the tile rule and the count field
    sim.run_stage(gpu.STAGE_REBUILD)
    sim.run_stage(gpu.STAGE_P2G)
    fi = sim.frame_info()
    f = np.array([fi["tx"], fi["ty"], fi["tz"]])
    t = np.clip(np.maximum(np.trunc(pos).astype(np.int64) // 8, 0), 0, f - 1)
    occ = np.zeros(f[::-1], bool)
    occ[t[:, 2], t[:, 1], t[:, 0]] = True
    pad = np.pad(occ, 1)
    act = np.zeros_like(occ)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                act |= pad[dz:dz + f[2], dy:dy + f[1], dx:dx + f[0]]
    kk, jj, ii = np.nonzero(act)
    expect = np.stack([ii, jj, kk], 1)
    np.testing.assert_array_equal(sim.tiles(), expect[np.lexsort((ii, jj, kk))])
    # count field: each particle touches min(2, clipped) cells per axis
    d = np.maximum(np.trunc(pos - 0.5).astype(np.int64), 0)
    touched = np.prod(np.where(d + 1 <= 255, 2, 1), axis=1)
    assert int(sim.field(gpu.FIELD_SURF).astype(np.int64).sum()) == int(touched.sum())


def _read_store(f, with_origin):
    n = int(np.fromfile(f, np.int64, 1)[0])
    pos = np.fromfile(f, np.float32, 3 * n).reshape(n, 3)
    vel = np.fromfile(f, np.float32, 3 * n).reshape(n, 3)
    origin = np.fromfile(f, np.int32, n) if with_origin else None
    return pos, vel, origin


def test_cpp_harness_matches_oracle(gpu, oracle_lib, tmp_path):
    """The header-only FLIPMethod wrapper (include/BoraFLIPMethod.hpp) driven the way the
    Houdini node drives Bora::FLIPMethod - world-space particles, newParticle per point,
    advanceOneFrame (step + postProcess) three times, the library's default solver
    settings - against the oracle running the same frames: each frame's world -> voxel
    upload and voxel -> world read-back (Grid::voxelPoint / worldPoint, FLIPMethod.cu:
    481-513) restated in float32, one step with an FP64 projection in between; particles
    matched by their index in the initial store."""
    from vare_gb300 import build
    src = os.path.join(ROOT, "tests", "cpp", "flipmethod_harness.cpp")
    exe = os.path.join(ROOT, "tests", "cpp", "_build", "harness")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    libdir = os.path.dirname(build.LIB)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                    "-L", libdir, "-lbora_flip", f"-Wl,-rpath,{libdir}"], check=True)
    out = str(tmp_path / "harness.bin")
    frames = 3
    r = subprocess.run([exe, str(frames), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    with open(out, "rb") as f:
        pos0, vel0, _ = _read_store(f, False)
        pos1, vel1, origin = _read_store(f, True)
    f32 = np.float32
    dt = f32(1.0) / f32(24.0) / f32(4.0)  # the harness's params.dt
    sc = scenes.Scene(name="harness", res=(32, 32, 32), bmin=(0.0, 0.0, 0.0), bmax=(1.0, 1.0, 1.0), dt=float(dt),
                      pos=np.zeros((0, 3), f32), vel=np.zeros((0, 3), f32), wall_level=2.0,
                      gravity=(0.0, -9.80665, 0.0))
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-12, threads=os.cpu_count())
    xf = ora.grid_xform()
    tr, scl = xf["translate"].astype(f32), xf["scale"].astype(f32)
    wp, wv, ids = pos0, vel0, np.arange(len(pos0), dtype=np.int32)
    for _ in range(frames):
        ora.set_particles((wp - tr) / scl, wv / scl, ids)
        ora.step(dt)
        p, v, _, ids = ora.particles()
        wp, wv = p * scl + tr, v * scl
    o = np.argsort(ids)
    g = np.argsort(origin)
    np.testing.assert_array_equal(origin[g], ids[o])
    ep, ev = rel_err(pos1[g], wp[o]), rel_err(vel1[g], wv[o])
    print(f"\nC++ wrapper vs oracle after {frames} frames: position {ep:.3e}, velocity {ev:.3e}")
    assert ep <= TOL and ev <= 1e-4


def test_rk2_advection_matches_oracle(gpu, oracle_lib, scene):
    """The RK2 advection option (midpoint rule in the grid velocity per substep) against
    the oracle with the same option: G2P bit-exact from identical fields, and a full step
    within tolerance."""
    B = oracle_lib
    sc = scene
    sim = gpu.FlipSim.from_scene(sc, **tight(advection=gpu.ADVECT_RK2))
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=1, advection=1)
    for st in (gpu.STAGE_REBUILD, gpu.STAGE_P2G, gpu.STAGE_BUILD_SYSTEM, gpu.STAGE_SOLVE):
        sim.run_stage(st)
    ora.rebuild(); ora.p2g(); ora.mark(); ora.build_system(); ora.solve(); ora.update_velocity()
    # identical fields on both sides, then G2P + RK2 advection + kill
    for f in (B.FIELD_VELO, B.FIELD_COMP, B.FIELD_SURF):
        sim.set_field(f, ora.field(f))
    sim.run_stage(gpu.STAGE_UPDATE_PARTICLES, sc.dt)
    ora.update_particles(sc.dt)
    ora.compact()
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    for a, b, name in zip(g[:3], o[:3], ("pos", "vel", "adj")):
        np.testing.assert_array_equal(a, b, err_msg=name)
    # the option changes the motion: RK2 and Euler positions differ after a step
    eul = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=1)
    eul.step(sc.dt)
    sim2 = gpu.FlipSim.from_scene(sc, **tight(advection=gpu.ADVECT_RK2))
    ora2 = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=1, advection=1)
    assert sim2.step(sc.dt) == 0
    ora2.step(sc.dt)
    g2 = by_id(*sim2.particles())
    o2 = by_id(*ora2.particles())
    np.testing.assert_array_equal(g2[3], o2[3])
    assert rel_err(g2[0], o2[0]) <= TOL and rel_err(g2[1], o2[1]) <= TOL
    e = by_id(*eul.particles())
    if len(e[3]) == len(o2[3]) and np.array_equal(e[3], o2[3]):
        assert np.abs(e[0] - o2[0]).max() > 0


@pytest.mark.parametrize("solver", ["plain", "mixed"])
def test_tank_scene_matches_oracle(gpu, oracle_lib, solver):
    """The large-domain scene (shallow tank, wave column, static box obstacle) at 1/8 of
    its resolution, two full steps against the oracle."""
    sc = scenes.config3(8)
    sim = gpu.FlipSim.from_scene(sc, **tight(solver=gpu.SOLVER_MIXED if solver == "mixed" else gpu.SOLVER_PLAIN))
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13)
    for _ in range(2):
        assert sim.step(sc.dt) == 0
        ora.step(sc.dt)
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    assert rel_err(g[0], o[0]) <= TOL
    assert rel_err(g[1], o[1]) <= TOL


def test_emission_between_steps_matches_oracle(gpu, oracle_lib):
    """Particles emitted between steps (FLIPMethod::newParticle, FLIPMethod.h:75-99) join the
    next step. G2P bins only the particles it writes, so the rebuild after an emission must bin
    the particles again; the oracle gets the same particles appended with the same ids (the
    device hands ids out in order of addition)."""
    sc = scenes.small(24, seed=5)
    sim = gpu.FlipSim.from_scene(sc, **tight())
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=1)
    assert sim.step(sc.dt) == 0
    ora.step(sc.dt)
    n0, m = sc.pos.shape[0], 500
    rng = np.random.default_rng(3)
    new = (rng.random((m, 3)) * [6.0, 4.0, 6.0] + [9.0, 14.0, 9.0]).astype(np.float32)  # voxel space
    newv = np.tile(np.float32([0.0, -2.0, 0.0]), (m, 1))
    sim.add_particles(new, newv, space=gpu.SPACE_VOXEL)
    p, v, _, ids = ora.particles()
    ora.set_particles(np.concatenate([p, new]), np.concatenate([v, newv]),
                      np.concatenate([ids, np.arange(n0, n0 + m, dtype=np.int32)]))
    for _ in range(2):
        assert sim.step(sc.dt) == 0
        ora.step(sc.dt)
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    assert rel_err(g[0], o[0]) <= TOL and rel_err(g[1], o[1]) <= TOL


@pytest.mark.parametrize("solver", ["plain", "mixed"])
def test_warm_start_matches_oracle(gpu, oracle_lib, solver):
    """params.warm_start: each solve starts from the last step's pressure (the reference's starts
    from 0). Steps still match the oracle's (cold, FP64) steps, with fewer PCG iterations in
    all than the same steps started cold."""
    sc = scenes.small(32, seed=13)
    form = gpu.SOLVER_PLAIN if solver == "plain" else gpu.SOLVER_MIXED
    warm = gpu.FlipSim.from_scene(sc, **tight(solver=form, warm_start=1))
    cold = gpu.FlipSim.from_scene(sc, **tight(solver=form))
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=1)
    iters = {"warm": 0, "cold": 0}
    for n in range(5):
        assert warm.step(sc.dt) == 0 and cold.step(sc.dt) == 0
        ora.step(sc.dt)
        if n > 0:  # the first solve has no earlier pressure
            iters["warm"] += warm.stats()["solver_iterations"]
            iters["cold"] += cold.stats()["solver_iterations"]
    g = by_id(*warm.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    assert rel_err(g[0], o[0]) <= TOL and rel_err(g[1], o[1]) <= TOL
    assert iters["warm"] < iters["cold"], iters


def test_water_tank_matches_oracle(gpu, oracle_lib):
    """FLIPMethod::fillWaterTank on the device (bit-exact particles, in the reference's
    order) and steps with the tank on: its tile rows stay active, the damping band acts."""
    sc = scenes.small(24, seed=11)
    sc.wall_level = 0.25
    kw = dict(enable_water_tank=1, damping_band=0.1)
    sim = gpu.FlipSim.from_scene(sc, **tight(**kw))
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=1, tank=True, damping_band=0.1)
    n = sim.fill_water_tank()
    assert n > 0 and n == ora.fill_water_tank(8)
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    np.testing.assert_array_equal(g[0], o[0])
    np.testing.assert_array_equal(g[1], o[1])
    # tank rows active after a rebuild, the same tile set as the oracle
    sim.run_stage(gpu.STAGE_REBUILD)
    ora.rebuild()
    np.testing.assert_array_equal(sim.tiles(), ora.tiles())
    fi = sim.frame_info()
    rows = int(fi["voxel_wall"]) // 8
    tiles = sim.tiles()
    assert rows >= 0 and np.sum(tiles[:, 1] < rows) == fi["tx"] * fi["tz"] * min(rows, fi["ty"])
    for _ in range(2):
        assert sim.step(sc.dt) == 0
        ora.step(sc.dt)
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    assert rel_err(g[0], o[0]) <= TOL and rel_err(g[1], o[1]) <= TOL


def _sampled_boxes(boxes, band, nx, ny, nz):
    """Box colliders sampled at the frame's cell centres the way the device samples them
    (FP32, same operation order): clamped signed distance and the nearest box's velocity."""
    f32 = np.float32
    z, y, x = np.meshgrid(np.arange(nz, dtype=f32) + f32(0.5), np.arange(ny, dtype=f32) + f32(0.5),
                          np.arange(nx, dtype=f32) + f32(0.5), indexing="ij")
    band = f32(band)
    best = np.full(x.shape, band, f32)
    arg = np.full(x.shape, -1, np.int64)
    for n, (lo, hi, _) in enumerate(boxes):
        lo, hi = np.asarray(lo, f32), np.asarray(hi, f32)
        c, h = (lo + hi) * f32(0.5), (hi - lo) * f32(0.5)
        q = [np.abs(p - c[a]) - h[a] for a, p in enumerate((x, y, z))]
        o = [np.where(qa > 0, qa, f32(0)) for qa in q]
        outside = np.sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2])
        m = np.where(q[0] > q[1], q[0], q[1])
        m = np.where(m > q[2], m, q[2])
        d = outside + np.where(m < 0, m, f32(0))
        take = (arg < 0) | (d < best)
        best = np.where(take, d, best)
        arg = np.where(take, n, arg)
    best = np.where(best > band, band, best)
    best = np.where(best < -band, -band, best)
    vel = np.zeros(x.shape + (3,), f32)
    for n, (_, _, v) in enumerate(boxes):
        sel = (arg == n) & (best < band)
        vel[sel] = np.asarray(v, f32)
    return best.astype(f32), vel


def test_collider_field_ingest_matches_boxes(gpu):
    """Colliders given as per-cell signed distance and velocity buffers (the raw-buffer form
    of CollisionSource's sampled grids) reproduce the box colliders they were sampled from,
    bit for bit, through whole steps."""
    sc = scenes.small(20, dt=1.0 / 60.0)
    sc.colliders = colliders_for(20)
    box = gpu.FlipSim.from_scene(sc, **tight())
    fi = box.frame_info()
    phi, vel = _sampled_boxes(sc.colliders, sc.collider_band, fi["nx"], fi["ny"], fi["nz"])
    sc2 = scenes.small(20, dt=1.0 / 60.0)
    field = gpu.FlipSim.from_scene(sc2, **tight())
    field.set_collider_field(phi, vel)
    for _ in range(2):
        assert box.step(sc.dt) == 0
        assert field.step(sc.dt) == 0
    a = by_id(*box.particles())
    b = by_id(*field.particles())
    for u, v, name in zip(a, b, ("pos", "vel", "adj", "ids")):
        np.testing.assert_array_equal(u, v, err_msg=name)
    assert box.stats()["killed_last_step"] == field.stats()["killed_last_step"]


def test_dam_break_64_hundred_steps(gpu, oracle_lib):
    """The 64^3 dam break (505,856 particles, dt 1/240) over 100 steps - the chaotic regime,
    compared by bulk statistics against the oracle: particle count (solid walls keep every
    particle), kinetic energy, centre of mass and the dam front (largest x)."""
    sc = scenes.config0()
    sim = gpu.FlipSim.from_scene(sc, tolerance=1e-9, div_tolerance=1e-10, max_refinements=30)
    ora = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-11, threads=os.cpu_count())
    for _ in range(100):
        assert sim.step(sc.dt) == 0
        ora.step(sc.dt)
    gp, gv, _, _ = sim.particles()
    op, ov, _, _ = ora.particles()
    assert len(gp) == len(op) == sc.num_particles
    ke_g = 0.5 * np.sum(gv.astype(np.float64) ** 2)
    ke_o = 0.5 * np.sum(ov.astype(np.float64) ** 2)
    com = np.abs(gp.astype(np.float64).mean(0) - op.astype(np.float64).mean(0)).max()
    front = abs(float(gp[:, 0].max()) - float(op[:, 0].max()))
    print(f"KE {ke_g:.6e} vs {ke_o:.6e}, centre of mass {com:.2e} voxel, front {front:.3f} voxel")
    # measured on GB300: KE within 3e-7 relative, centre of mass within 2e-6 voxel, same front
    assert abs(ke_g - ke_o) <= 1e-4 * ke_o
    assert com <= 1e-3
    assert front <= 0.05


def _sphere_voxels(fi, center, radius, band_cells, vel):
    """A sphere collider as a level set's voxels: every frame cell whose signed distance at
    its centre (world units, float32) is below band_cells voxels - the narrow band and the
    interior - with a constant velocity; the background is band_cells voxels."""
    f32 = np.float32
    h = f32(fi["scale"][0])
    k, j, i = np.meshgrid(np.arange(fi["nz"]), np.arange(fi["ny"]), np.arange(fi["nx"]), indexing="ij")
    ijk = np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(np.int32)
    w = (ijk.astype(f32) + f32(0.5)) * fi["scale"][None, :].astype(f32) + fi["translate"][None, :].astype(f32)
    d = w - np.asarray(center, f32)[None, :]
    phi = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) - f32(radius)
    keep = phi < f32(band_cells) * h
    v = np.tile(np.asarray(vel, f32), (int(keep.sum()), 1))
    return ijk[keep], phi[keep].astype(f32), v, float(f32(band_cells) * h)


def test_collider_voxels_match_oracle(gpu, oracle_lib):
    """A collider given as a level set's voxels (CollisionSource::update, the sparse form):
    a moving sphere in the falling water. Identical inputs on both sides: the cell flags
    (solid where the sampled distance is negative) bit for bit, the collider velocity in the
    grid velocity within the P2G tolerance, G2P (collider carry, push-out along the
    normalised gradient, kill) bit for bit from identical fields, and two full steps within
    the tolerance."""
    B = oracle_lib
    sc = moving(scenes.small(24, dt=1.0 / 60.0), oracle_lib, 1)
    sim, ora = _pair(gpu, oracle_lib, sc)
    fi = sim.frame_info()
    ijk, phi, vel, bg = _sphere_voxels(fi, (0.55, 0.15, 0.5), 0.22, 3, (0.0, 0.0, 0.4))
    assert len(phi) > 0 and (phi < 0).any()
    sim.set_collider_voxels(ijk, phi, vel, bg)
    ora.set_collider_voxels(ijk, phi, vel, bg)
    sim.run_stage(gpu.STAGE_REBUILD)
    sim.run_stage(gpu.STAGE_P2G)
    ora.rebuild(); ora.p2g(); ora.mark()
    tiles = sim.tiles()
    np.testing.assert_array_equal(tiles, ora.tiles())
    real = real_cells(tiles, fi["nx"], fi["ny"], fi["nz"])
    gflag = sim.field(gpu.FIELD_FLAG)[real]
    np.testing.assert_array_equal(gflag, ora.field(B.FIELD_MARK)[real].astype(np.uint8))
    assert (gflag == 1).any(), "the sphere marks no solid cell"
    assert rel_err(sim.field(gpu.FIELD_VELO)[real], ora.field(B.FIELD_VELO)[real]) <= TOL
    # G2P + advection + collider push-out from identical fields
    sim.set_field(gpu.FIELD_VELO, ora.field(B.FIELD_VELO))
    sim.run_stage(gpu.STAGE_BUILD_SYSTEM)
    ora.build_system()
    ora.solve()
    ora.update_velocity()
    for f in (B.FIELD_VELO, B.FIELD_COMP, B.FIELD_SURF):
        sim.set_field(f, ora.field(f))
    sim.run_stage(gpu.STAGE_UPDATE_PARTICLES, sc.dt)
    ora.update_particles(sc.dt)
    ora.compact()
    g = by_id(*sim.particles())
    o = by_id(*ora.particles())
    np.testing.assert_array_equal(g[3], o[3])
    for a, b, name in zip(g[:3], o[:3], ("pos", "vel", "adj")):
        np.testing.assert_array_equal(a, b, err_msg=name)
    # two full steps
    sim2, ora2 = _pair(gpu, oracle_lib, sc)
    sim2.set_collider_voxels(ijk, phi, vel, bg)
    ora2.set_collider_voxels(ijk, phi, vel, bg)
    for _ in range(2):
        assert sim2.step(sc.dt) == 0
        ora2.step(sc.dt)
    g = by_id(*sim2.particles())
    o = by_id(*ora2.particles())
    np.testing.assert_array_equal(g[3], o[3])
    assert rel_err(g[0], o[0]) <= TOL and rel_err(g[1], o[1]) <= TOL
