"""The launch-shape autotuner (bora_flip_set_tuning / bora_flip_tune_table).

The multigrid passes of levels 0-2 have several launch shapes that compute the same bits.
The tuner times each shape on live launches and keeps the fastest per size class. Tuning must
never change a result: a simulation stepped while the tuner measures (every shape in turn)
gives the same bits as one stepped with the default shapes, alone and in a batch; and the
table, once decided, is written to BORA_TUNE_FILE and read back by a new process.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from vare_gb300 import flip, scenes

pytestmark = pytest.mark.gpu

GROUPS_SINGLE = {0, 1, 2}  # levels 0, 1, 2 of single simulations
GROUPS_BATCH = {3, 4, 5}


def _run(sc, steps, tuning):
    flip.set_tuning(tuning)
    try:
        sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
        for _ in range(steps):
            assert sim.step(sc.dt) >= 0
        pos, vel, _, ids = sim.particles()
        sim.close()
    finally:
        flip.set_tuning(True)
    o = np.argsort(ids)
    return pos[o], vel[o]


def test_tuning_changes_no_result():
    sc = scenes.small(40)
    p0, v0 = _run(sc, 4, False)
    p1, v1 = _run(sc, 4, True)
    assert np.array_equal(p0, p1) and np.array_equal(v0, v1)
    rows = flip.tune_table()
    print("\n" + "\n".join(str(r) for r in rows))
    decided = {r[0] for r in rows if r[3] >= 0}
    assert GROUPS_SINGLE <= decided, rows


def _run_batch_of_one(sc, steps, tuning):
    flip.set_tuning(tuning)
    try:
        sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
        for _ in range(steps):
            assert flip.step_batch([sim], sc.dt) == [0]
        pos, vel, _, ids = sim.particles()
        sim.close()
    finally:
        flip.set_tuning(True)
    o = np.argsort(ids)
    return pos[o], vel[o]


def test_batch_tuning_changes_no_result():
    """Each simulation alone (a batch of one: a batched step keeps the hierarchy shape its
    launches need, so small scenes solve on more levels than bora_flip_step) with the default
    shapes, against all of them in one batch while the tuner measures."""
    scs = [scenes.small(24 + 8 * k) for k in range(3)]
    alone = [_run_batch_of_one(sc, 6, False) for sc in scs]
    sims = [flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED) for sc in scs]
    # a batch times one shape per step (the first step from rest solves nothing)
    for _ in range(6):
        st = flip.step_batch(sims, scs[0].dt)
        assert all(s >= 0 for s in st)
    for sim, (p0, v0) in zip(sims, alone):
        pos, vel, _, ids = sim.particles()
        sim.close()
        o = np.argsort(ids)
        assert np.array_equal(pos[o], p0) and np.array_equal(vel[o], v0)
    decided = {r[0] for r in flip.tune_table() if r[3] >= 0}
    assert GROUPS_BATCH <= decided


def test_table_file_round_trip(tmp_path):
    path = tmp_path / "tune.txt"
    code = textwrap.dedent("""
        from vare_gb300 import flip, scenes
        sc = scenes.small(32)
        sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
        decided = [r for r in flip.tune_table() if r[3] >= 0]
        print("BEFORE", len(decided))
        for _ in range(3):
            sim.step(sc.dt)
        print("AFTER", len([r for r in flip.tune_table() if r[3] >= 0]))
    """)
    env = dict(os.environ, BORA_TUNE_FILE=str(path))
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out1 = subprocess.run([sys.executable, "-c", code], env=env, cwd=repo, capture_output=True, text=True, timeout=600)
    assert out1.returncode == 0, out1.stderr
    lines = path.read_text().split("\n")
    entries = [l.split() for l in lines if l.strip()]
    assert entries and all(len(e) == 5 and int(e[3]) >= 0 for e in entries)
    out2 = subprocess.run([sys.executable, "-c", code], env=env, cwd=repo, capture_output=True, text=True, timeout=600)
    assert out2.returncode == 0, out2.stderr
    before = int([l for l in out2.stdout.splitlines() if l.startswith("BEFORE")][0].split()[1])
    assert before == len(entries)  # the second process starts from the saved table
