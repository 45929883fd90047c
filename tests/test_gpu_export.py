"""Asynchronous export (bora_flip_export_begin / _wait): the copy of frame N's particles
runs on its own stream while step N+1 runs, and delivers exactly frame N's state."""
import numpy as np
import pytest

from vare_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_async_export_delivers_the_state_it_started_from(gpu):
    import torch
    sc = scenes.small(24)
    sim = gpu.FlipSim.from_scene(sc)
    assert sim.step(sc.dt) >= 0
    sim.post_process()
    pos, vel, _, ids = sim.particles(space=gpu.SPACE_WORLD)
    vort, curv, aids = sim.particle_attributes()
    np.testing.assert_array_equal(ids, aids)
    n = sim.num_particles
    hp = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    hv = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    ho = torch.empty(n, dtype=torch.float32, pin_memory=True)
    hc = torch.empty(n, dtype=torch.float32, pin_memory=True)
    hi = torch.empty(n, dtype=torch.int32, pin_memory=True)
    got = sim.export_begin(hp.data_ptr(), hv.data_ptr(), ho.data_ptr(), hc.data_ptr(), hi.data_ptr(), n,
                           space=gpu.SPACE_WORLD)
    assert got == n
    assert sim.step(sc.dt) >= 0  # overlaps the copy
    sim.export_wait()
    np.testing.assert_array_equal(hp.numpy(), pos)
    np.testing.assert_array_equal(hv.numpy(), vel)
    np.testing.assert_array_equal(ho.numpy(), vort)
    np.testing.assert_array_equal(hc.numpy(), curv)
    np.testing.assert_array_equal(hi.numpy(), ids)
    # a second export of the new state, back to back with the first finished
    pos2, _, _, ids2 = sim.particles()
    m = sim.export_begin(hp.data_ptr(), 0, 0, 0, hi.data_ptr(), n)
    sim.export_wait()
    np.testing.assert_array_equal(hp.numpy()[:m], pos2)
    np.testing.assert_array_equal(hi.numpy()[:m], ids2)
