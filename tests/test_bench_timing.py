"""The bench's measurement of the timed steps (bench.timed_steps) on the CPU, against a stand-in
for the simulation handle that keeps the library's per-kernel timing rules: the dominant kernel
class is found in the warm-up, a few of its launches per timed step are bracketed by events (one
in `every`), the roofline's launch figures follow from the sampled brackets, and the timing is
off again afterwards, so that the steps measured next (end to end) record no events."""
import types

import numpy as np

import bench
from vare_gb300 import flip

UPDATE = flip.KERNEL_CLASSES.index("pcg_update")
DIRECTION = flip.KERNEL_CLASSES.index("pcg_direction")


class FakeSim:
    """Launches per step: 380 PCG updates (0.03 ms each), 380 directions (0.02 ms), one G2P."""

    def __init__(self):
        self.mask, self.every = 0, 1
        self.seen = np.zeros(16, np.int64)
        self.ms = np.zeros(16)
        self.n = np.zeros(16, np.uint64)
        self.launches = 0
        self.num_particles = 1000
        self.events_per_step = []

    def set_profiling(self, mask):
        self.mask = mask
        self.ms[:] = 0.0
        self.n[:] = 0
        self.seen[:] = 0

    def set_profiling_sampling(self, every):
        assert every >= 1
        self.every = every
        self.seen[:] = 0

    def _launch(self, cls, ms):
        self.launches += 1
        if (self.mask >> cls) & 1:
            if self.seen[cls] % self.every == 0:
                self.ms[cls] += ms
                self.n[cls] += 1
                self._events += 2
            self.seen[cls] += 1

    def step(self, dt):
        self._events = 0
        for _ in range(380):
            self._launch(DIRECTION, 0.02)
            self._launch(UPDATE, 0.03)
        self._launch(flip.KERNEL_CLASSES.index("g2p"), 0.4)
        self.events_per_step.append(self._events)
        return 0

    def kernel_times(self):
        return self.ms.copy(), self.n.copy()

    def stats(self):
        return {"kernel_launches": self.launches, "gpu_ms": 24.0, "solver_iterations": 380, "residual_rel": 1e-7,
                "residual_max_dx": 1e-8, "converged": 1, "refinements": 2, "mg_vcycle_launches": 0}

    def frame_info(self):
        return {"ntiles": 10}

    def field(self, which):
        f = np.zeros(10 * 512, np.uint8)
        f[:3000] = 4
        return f


def test_timed_steps_sample_the_dominant_class_and_switch_timing_off(monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    sim = FakeSim()
    args = types.SimpleNamespace(warmup=3, steps=5, nvtx=False)
    sc = types.SimpleNamespace(dt=1.0 / 480.0)
    m = bench.timed_steps(sim, sc, args, 1, flip, 0, False)
    roof = m["roofline"]
    assert roof["kernel"] == "pcg_update"
    assert roof["timed_every"] == 380 // 4
    assert roof["timed_launches"] == 4 * args.steps  # launches 0, 95, 190, 285 of each step
    assert roof["launches_per_step"] == 380.0
    assert abs(roof["avg_launch_ms"] - 0.03) < 1e-12
    assert abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-12
    for key in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert key in roof
    # a few brackets in each timed step, every launch of every class in the warm-up
    assert sim.events_per_step[:args.warmup] == [2 * 761] * args.warmup
    assert sim.events_per_step[args.warmup:] == [2 * 4] * args.steps
    # timing off afterwards: the steps measured next record no events
    assert sim.mask == 0 and sim.every == 1
    sim.step(sc.dt)
    assert sim.events_per_step[-1] == 0
    assert abs(m["value"] - sim.num_particles / 0.024) < 1e-6 * m["value"]
    assert m["ms_per_step"] == 24.0
