"""Batched stepping (bora_flip_step_batch): several simulations per step with the pressure
solve's kernels launched once for all of them.

Each simulation runs its own tiles on its own grid and reduces into its own ring, with
stage_solve's control flow on its own, so a simulation's result does not depend on the
batch it runs in: bit-identical alone (a batch of one) and in any mix. Where the
simulation's multigrid hierarchy already has the batched shape (level 3 with more than 512
cells), a batch of one is also bit-identical to bora_flip_step. The batched path is checked
against the oracle like the single one."""
import os

import numpy as np
import pytest

from vare_gb300 import flip, scenes

pytestmark = pytest.mark.gpu


def _by_id(sim):
    pos, vel, adj, ids = sim.particles()
    o = np.argsort(ids)
    return pos[o], vel[o], adj[o], ids[o]


def _mix():
    return [scenes.small(24, seed=3), scenes.small(40, seed=4, sphere=False), scenes.small(32, seed=5),
            scenes.dam_break(48, (0.3, 0.5), seed=6, dt=1.0 / 120.0)]


def test_batch_matches_alone(gpu):
    scs = _mix()
    steps = 4
    dt = scs[0].dt
    mix = [flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED) for sc in scs]
    for _ in range(steps):
        st = flip.step_batch(mix, dt)
        assert all(v == 0 for v in st), st
    for sc, m in zip(scs, mix):
        alone = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
        for _ in range(steps):
            assert flip.step_batch([alone], dt) == [0]
        for a, b, name in zip(_by_id(m), _by_id(alone), ("pos", "vel", "adj", "ids")):
            np.testing.assert_array_equal(a, b, err_msg=name)
        sa, sb = m.stats(), alone.stats()
        assert sa["solver_iterations"] == sb["solver_iterations"] and sa["converged"] == 1


def test_batch_of_one_matches_single_step(gpu):
    """A scene with more than 512 active tiles: its own hierarchy already has the batched
    shape, so the batched step and bora_flip_step give the same bits."""
    sc = scenes.small(96, seed=2)
    a = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
    b = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
    for _ in range(3):
        assert a.step(sc.dt) == 0
        assert flip.step_batch([b], sc.dt) == [0]
    assert a.stats()["active_tiles"] > 512
    for u, v, name in zip(_by_id(a), _by_id(b), ("pos", "vel", "adj", "ids")):
        np.testing.assert_array_equal(u, v, err_msg=name)


def test_batch_matches_oracle(gpu, oracle_lib):
    """Two simulations stepped together against the oracle (FP64 projection), each within
    the parity tolerance, with the tight solver settings of the other parity tests."""
    scs = [scenes.small(24), scenes.small(20, seed=9, sphere=False)]
    kw = dict(tolerance=1e-10, div_tolerance=1e-12, max_refinements=30, inner_tolerance=1e-4)
    sims = [flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED, **kw) for sc in scs]
    oras = [oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13, threads=os.cpu_count()) for sc in scs]
    for _ in range(2):
        assert flip.step_batch(sims, scs[0].dt) == [0, 0]
        for o in oras:
            o.step(scs[0].dt)
    for sim, ora in zip(sims, oras):
        g = _by_id(sim)
        pos, vel, adj, ids = ora.particles()
        o = np.argsort(ids)
        np.testing.assert_array_equal(g[3], ids[o])
        for a, b in ((g[0], pos[o]), (g[1], vel[o])):
            err = np.abs(a.astype(np.float64) - b).max() / np.abs(b).max()
            assert err <= 1e-5, err


def test_batch_mixed_with_plain_and_empty(gpu):
    """A plain-form simulation and an empty one in the batch step on their own; the
    mixed-form ones batch as usual."""
    sc = scenes.small(24)
    mixed = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
    plain = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_PLAIN)
    empty = flip.FlipSim(sc.res, sc.bmin, sc.bmax, flip.scene_params(sc))
    ref = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_PLAIN)
    for _ in range(2):
        assert flip.step_batch([mixed, plain, empty], sc.dt) == [0, 0, 0]
        assert ref.step(sc.dt) == 0
    assert empty.num_particles == 0
    for u, v in zip(_by_id(plain), _by_id(ref)):
        np.testing.assert_array_equal(u, v)


def test_warm_start_member_steps_on_its_own(gpu):
    """A simulation with the warm start (params.warm_start) is taken out of the batched solve and
    stepped on its own: in a batch it gives the bits of bora_flip_step, and the others still
    give the bits they have alone."""
    scs = _mix()[:2]
    dt = scs[0].dt
    mix = [flip.FlipSim.from_scene(scs[0], solver=flip.SOLVER_MIXED, warm_start=1),
           flip.FlipSim.from_scene(scs[1], solver=flip.SOLVER_MIXED)]
    warm = flip.FlipSim.from_scene(scs[0], solver=flip.SOLVER_MIXED, warm_start=1)
    cold = flip.FlipSim.from_scene(scs[1], solver=flip.SOLVER_MIXED)
    for _ in range(3):
        assert flip.step_batch(mix, dt) == [0, 0]
        assert warm.step(dt) == 0
        assert flip.step_batch([cold], dt) == [0]
    for m, alone in zip(mix, (warm, cold)):
        for a, b, name in zip(_by_id(m), _by_id(alone), ("pos", "vel", "adj", "ids")):
            np.testing.assert_array_equal(a, b, err_msg=name)
