"""Per-kernel-class device timing (bora_flip_set_profiling): every bracket or one in n of them,
and neither changes what a step computes."""
import numpy as np
import pytest

from vare_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_sampled_brackets_and_unchanged_results(gpu):
    sc = scenes.small(24, seed=9)
    cls = gpu.KERNEL_CLASSES.index("pcg_direction")
    sims = [gpu.FlipSim.from_scene(sc) for _ in range(2)]
    for sim in sims:
        assert sim.step(sc.dt) == 0  # a moving state: the next solve takes many iterations
    sims[0].set_profiling(1 << cls)
    sims[1].set_profiling(1 << cls)
    sims[1].set_profiling_sampling(4)
    for sim in sims:
        assert sim.step(sc.dt) == 0
    _, n_all = sims[0].kernel_times()
    ms, n_four = sims[1].kernel_times()
    assert n_all[cls] > 4
    assert n_four[cls] == (n_all[cls] + 3) // 4  # brackets 0, 4, 8, ... of the step
    assert ms[cls] > 0.0
    a, b = sims[0].particles(), sims[1].particles()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    with pytest.raises(Exception):
        sims[1].set_profiling_sampling(0)
