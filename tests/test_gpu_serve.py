"""Serving layer on the GPU: requests that overlap on the device give the same result as
the same request run alone; admission respects the memory budget and the slot count;
a request that arrives while others run starts before they have all finished."""
import time

import numpy as np
import pytest

from vare_gb300 import flip, scenes, serve

pytestmark = pytest.mark.gpu


def _requests():
    """Six small requests of uneven size: dam breaks and sphere drops."""
    out = []
    for r, (n, steps) in enumerate([(24, 12), (32, 6), (20, 15), (28, 9), (16, 20), (36, 5)]):
        sc = scenes.small(n, seed=100 + r, sphere=(r % 2 == 1), dt=1.0 / 120.0)
        out.append((sc, steps))
    return out


def _alone(sc, steps, **kw):
    """The request run alone: its own simulation stepped in batches of one."""
    sim = flip.FlipSim.from_scene(sc, **kw)
    for _ in range(steps):
        assert flip.step_batch([sim], sc.dt)[0] >= 0
    pos, vel, _, ids = sim.particles()
    o = np.argsort(ids)
    return pos[o], vel[o], ids[o]


@pytest.mark.parametrize("solver", [flip.SOLVER_MIXED, flip.SOLVER_PLAIN])
def test_results_match_alone_and_in_the_mix(gpu, solver):
    reqs = _requests()
    srv = serve.Server(max_running=4)
    try:
        ids = [srv.submit(sc, steps, solver=solver) for sc, steps in reqs]
        srv.drain()
        st = srv.stats()
        assert st["done"] == len(reqs) and st["failed"] == 0
        assert st["running_peak"] >= 2, "requests did not overlap"
        for rid, (sc, steps) in zip(ids, reqs):
            info = srv.poll(rid)
            assert info["state"] == serve.REQ_DONE and info["steps_done"] == steps
            assert info["device_bytes"] <= info["estimate_bytes"], info
            pos, vel, pid = srv.result(rid)
            apos, avel, aid = _alone(sc, steps, solver=solver)
            np.testing.assert_array_equal(pid, aid)
            np.testing.assert_array_equal(pos, apos)
            np.testing.assert_array_equal(vel, avel)
            srv.release(rid)
    finally:
        srv.close()


def test_budget_serialises_and_rejects(gpu):
    reqs = _requests()[:3]
    est = [serve.estimate_bytes(sc) for sc, _ in reqs]
    # room for the largest request only: one at a time
    srv = serve.Server(budget_bytes=max(est) + 1, max_running=8)
    try:
        ids = [srv.submit(sc, steps) for sc, steps in reqs]
        srv.drain()
        st = srv.stats()
        assert st["done"] == 3 and st["running_peak"] == 1
        assert st["bytes_reserved"] == 0 and st["bytes_reserved_peak"] <= max(est) + 1
        for rid in ids:
            srv.release(rid)
        # a request that can never fit fails without running
        small = scenes.small(16)
        srv2 = serve.Server(budget_bytes=1 << 20, max_running=2)
        try:
            rid = srv2.submit(small, 3)
            assert srv2.wait(rid, 30.0)
            info = srv2.poll(rid)
            assert info["state"] == serve.REQ_FAILED and info["status"] == -2
        finally:
            srv2.close()
    finally:
        srv.close()


def test_continuous_admission(gpu):
    """A request submitted while a long one runs is admitted and finishes first."""
    long_sc = scenes.small(40, seed=3)
    short_sc = scenes.small(16, seed=4)
    srv = serve.Server(max_running=4)
    try:
        a = srv.submit(long_sc, 120)
        t0 = time.time()
        while srv.poll(a)["steps_done"] < 3:
            assert time.time() - t0 < 60
            time.sleep(0.005)
        b = srv.submit(short_sc, 2)
        assert srv.wait(b, 60.0)
        info_a = srv.poll(a)
        assert srv.poll(b)["state"] == serve.REQ_DONE
        assert info_a["state"] == serve.REQ_RUNNING and info_a["steps_done"] < 120
        srv.drain()
        assert srv.poll(a)["state"] == serve.REQ_DONE
    finally:
        srv.close()
