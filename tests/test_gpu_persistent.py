"""The plain form's persistent inner PCG (one cooperative launch per refinement pass, its
phases separated by grid barriers; bora_flip_params.persistent) and the bounded barrier.

The persistent pass runs the same direction and update tile loops as the per-phase kernels;
its sums are formed per block and added over blocks in a fixed order after each barrier,
and it checks convergence itself (the per-phase path reads the residual back one iteration
late), so the two paths agree within the solver tolerance rather than bit for bit; the
persistent path is also checked against the oracle's FP64 projection at the default stop rule
(the per-phase path, the default, in test_gpu_bench_settings.py).

The barrier test makes every wait run out - a barrier that waits for one block more than the
launch has (BORA_FAULT_BARRIER) - and checks that the kernel returns within its spin limit,
the step reports BORA_ERR_INTERNAL, and the handle then steps normally again.
"""
import time

import numpy as np
import pytest

from oracle import parity
from vare_gb300 import flip, scenes

pytestmark = pytest.mark.gpu


def _step(sc, steps, **params):
    sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_PLAIN, **params)
    for _ in range(steps):
        assert sim.step(sc.dt) == 0
    st = sim.stats()
    pos, vel, _, ids = sim.particles()
    pres = sim.field(flip.FIELD_PRES)
    sim.close()
    o = np.argsort(ids)
    return pos[o], vel[o], pres, st


@pytest.mark.parametrize("n", [24, 48])
def test_persistent_agrees_with_per_phase(n):
    sc = scenes.small(n)
    p1, v1, r1, s1 = _step(sc, 3, persistent=1)
    p0, v0, r0, s0 = _step(sc, 3, persistent=0)
    print(f"\n[{n}] iterations persistent {s1['solver_iterations']} per-phase {s0['solver_iterations']}, "
          f"pressure {parity.rel_err(r1, r0):.2e}, velocity {parity.rel_err(v1, v0):.2e}")
    assert s1["converged"] and s0["converged"]
    assert s1["residual_rel"] < 1e-6 and s1["residual_max_dx"] < 1e-5
    assert parity.rel_err(r1, r0) < 1e-5
    assert parity.rel_err(v1, v0) < 1e-5
    assert parity.rel_err(p1, p0) < 1e-6


def test_persistent_matches_fp64_oracle(oracle_lib):
    sc = scenes.small(24)
    ora0 = oracle_lib.Oracle(sc, block=8, solver="fp64", tol=1e-13)
    for _ in range(2):
        ora0.step(sc.dt)
    pos, vel, _, ids = ora0.particles()
    o = np.argsort(ids)
    state = parity.with_state(sc, pos[o], vel[o])
    ora = parity.oracle_step(state)
    dev = parity.device_step(flip, state, solver=flip.SOLVER_PLAIN, persistent=1)
    e = parity.compare(dev, ora)
    print("\n" + ", ".join(f"{k} {v:.3e}" if isinstance(v, float) else f"{k} {v}" for k, v in e.items()))
    assert e["same_tiles"] and e["same_particles"] and e["converged"]
    assert e["pressure"] <= 1e-5 and e["grid_velocity"] <= 1e-5 and e["particle_velocity"] <= 1e-5


def test_persistent_is_deterministic():
    sc = scenes.small(40)
    a = _step(sc, 2, persistent=1)
    b = _step(sc, 2, persistent=1)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)


def test_barrier_wait_runs_out_and_reports():
    sc = scenes.small(32)
    sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_PLAIN, persistent=1)
    assert sim.step(sc.dt) == 0  # from rest
    sim.set_fault(flip.FAULT_BARRIER)
    t0 = time.perf_counter()
    with pytest.raises(flip.BoraError) as e:
        sim.step(sc.dt)
    took = time.perf_counter() - t0
    assert e.value.status == -5  # BORA_ERR_INTERNAL
    assert took < 10.0, took
    # the context is intact: clear the fault, restore the particles, step again
    sim.set_fault(flip.FAULT_NONE)
    sim.set_particles(sc.pos, sc.vel, space=flip.SPACE_VOXEL)
    for _ in range(2):
        assert sim.step(sc.dt) == 0
    assert sim.stats()["converged"]
    sim.close()
