"""Benchmark of the GB300 FLIP substep (one JSON line on stdout, rank 0).

Workload (default): the 256^3 dam break + falling sphere (x<0.35, y<0.5 block plus a
sphere at (0.7, 0.8, 0.5), r = 0.12; 24,564,400 particles at 8 per cell, jittered
uniform, seeded), dt = 1/480, solid walls, pressure solved to ||b-Ap||/||b|| < 1e-6 and
max|b-Ap|*dx < 1e-5. A step is one FLIPMethod::advanceOneStep over all particles.

  value  = particle-steps/s with particles resident in HBM, device time of each step
           from CUDA events on the simulation's stream (max over ranks);
  e2e    = the same metric through the C ABI with host buffers: every step uploads the
           particles from pinned host memory, steps, and reads them back;
  roofline = the dominant kernel class: algorithmic bytes per launch / its average
           event-timed launch duration, against the measured HBM copy bandwidth;
  cpu_baseline = the reference's algorithm (oracle restatement, bit-exact with the
           reference's host build) on this host's cores, on a bounded sample.

Multi-GPU: replicas only - each rank advances its own independent simulation (weak
scaling, no collective on the data path); value sums all ranks' particle-steps over the
slowest rank's time.

--impl reference times the reference algorithm's CPU implementation (the oracle port,
all host threads) on the same workload, metric and unit.
"""
from __future__ import annotations

import argparse
import contextlib
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 256^3 FLIP (plain FP32 block-MIC(0)-PCG, max|div u|*dx < 1e-5)"
UNIT = "particle-steps/s"

# Algorithmic bytes per launch of each kernel class: (bytes per active cell, bytes per particle).
#   pcg_direction: read z, d (8) + stencil code (2) + e (4); write d', q (8) + e (4) -> 26 B/cell
#                  (the previous update's e += alpha d is applied here)
#   pcg_update:    read r, q (8) + M^-1 (4); write r, z (8)                   -> 20 B/cell
#   p2g:           per particle read idx (4) + pos, vel (24); per cell read dual-cell
#                  starts (4), write mass, count, velocity (20) + flag (1)      -> 25 B/cell, 28 B/particle
#   g2p:           per particle idx (4), read pos, vel, id (28), write (28), adjacency (4), the next
#                  rebuild's sort key (4); per cell read velo, comp, count (28)  -> 28 B/cell, 68 B/particle
#   velocity:      read flag (1), pres (4), velo (12); write pres (4), comp (12)  -> 33 B/cell
#   rhs:           read flag (1), velo (12); write b (4), code (2); MIC read code (2), write M (4) -> 25 B/cell
#   refine:        per pass read x (8), e (4), b (4), code (2); write x (8), r (4) -> 30 B/cell
#   sort:          per particle read vkey (4), write key (4), read key (4), write idx (4); per cell scan 12 B
#   bin:           per particle read id + pos (16), write vkey (4); only after the particles changed
#                  between steps (G2P bins the particles it writes)
#   mg_vcycle:     level 0 down: read r (4), code (2); write z0 (2), coarse r (0.25); level 0 up:
#                  read r (4), code (2), z0 (2), coarse z (0.25); write z (4) -> 20.5 B per fine
#                  cell, plus the coarser levels (1/8 of that per level)       -> 23 B/cell
ALG_BYTES = {
    "bin": (0, 20), "tiles": (0, 0), "sort": (12, 16), "p2g": (25, 28), "rhs": (25, 0),
    "pcg_direction": (26, 0), "pcg_update": (20, 0), "refine": (30, 0), "velocity": (33, 0), "g2p": (28, 68),
    "mg_vcycle": (23, 0),
}
# Mixed form: the PCG update has no preconditioner sweep (read r, q; write r: 12 B/cell) and
# runs inside the V-cycle's first passes, so a V-cycle moves 23 + 12 B per fine cell (the
# separate update kernel remains only for hierarchies whose level 0 is in the tail kernel).
ALG_BYTES_MIXED = dict(ALG_BYTES, pcg_update=(12, 0), mg_vcycle=(35, 0))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dam_sphere_256",
                    choices=["dam_sphere_256", "dam_sphere_160", "dam_break_64", "tank_1024", "serve_64"],
                    help="dam_sphere_160: the 256^3 scene at 160^3, for profiler captures")
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--serve-slots", type=int, default=64)
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-stream measurement of the default run")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-post", action="store_true", help="skip the post-processing measurement")
    ap.add_argument("--post-reps", type=int, default=5)
    ap.add_argument("--nvtx", action="store_true",
                    help="mark the timed steps and one post-processing frame with NVTX ranges 'step' and 'post' "
                         "(for a profiler's range filter)")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the parity report (one step of each solver form against the oracle's FP64 "
                         "projection from the state the timed steps left)")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-persistent", action="store_true", help="skip the persistent plain-PCG measurement")
    ap.add_argument("--no-warm", action="store_true",
                    help="skip the warm-start measurements (each solve started from the last step's pressure)")
    ap.add_argument("--solver", default="both", choices=["both", "plain", "mixed"],
                    help="plain only / mixed only (profiling runs); the default times both")
    return ap.parse_args()


def make_scene(name):
    from vare_gb300 import scenes
    if name == "tank_1024":
        return scenes.config3()
    if name == "dam_sphere_160":
        return scenes.dam_sphere(160)
    return scenes.config1() if name == "dam_sphere_256" else scenes.config0()


SOLVER_DESC = {"plain": "plain: FP32 PCG + block-MIC(0), FP64-accurate dots, double-float iterative refinement",
               "mixed": "mixed: FP32 PCG + geometric multigrid V(2,2) (FP16 level storage, FP32 arithmetic), "
                        "FP64-accurate dots, double-float iterative refinement"}


def workload_config(sc, extra=None, solver="plain"):
    cfg = {"workload": f"{sc.name}: {sc.res[0]}x{sc.res[1]}x{sc.res[2]} virtual grid in 8^3 tiles, "
                       f"{sc.num_particles} particles (8/cell jittered, seeded), dt={sc.dt:.6g}, solid walls"
                       + (", static box obstacle" if sc.colliders else ""),
           "grid": list(sc.res), "particles": sc.num_particles, "dt": sc.dt, "tile": 8,
           "solver": SOLVER_DESC.get(solver, solver),
           "tolerance": {"rel": 1e-6, "max_div_dx": 1e-5},
           "l2": f"inputs larger than L2 (particles alone are {sc.num_particles * 24 // 1000000} MB); no flush",
           "parallelism": "replicas (one independent simulation per GPU)"}
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return

        def read():
            for line in self.proc.stdout:
                self.samples.append([v.strip() for v in line.split(",")])
        self.thread = threading.Thread(target=read, daemon=True)
        self.thread.start()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, s[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel_class: str):
    """Per-launch DRAM bytes of a kernel class from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(path):
        return None, None
    with open(path) as f:
        d = json.load(f)
    e = d.get(kernel_class)
    if not e:
        return None, None
    return e.get("dram_bytes_per_launch_full_size"), e.get("note")


def cpu_model() -> str:
    """The host CPU's model name (lscpu), or the machine type."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.machine()


PHASES = ("rebuild", "p2g", "mark", "build_system", "solve", "update_velocity", "update_particles", "compact")


def _oracle_timed_step(ora, dt: float, phases: dict) -> float:
    """One oracle step stage by stage (the same sequence as its step()), phase times added
    into `phases`; returns the step's wall time."""
    t_start = time.perf_counter()
    iters = 0
    for name in PHASES:
        t0 = time.perf_counter()
        if name == "update_particles":
            ora.update_particles(dt)
        elif name == "solve":
            iters = ora.solve()
        else:
            getattr(ora, name)()
        phases[name] = phases.get(name, 0.0) + (time.perf_counter() - t0)
    phases.setdefault("_iterations", []).append(int(iters))
    return time.perf_counter() - t_start


def _oracle_leg(scene, steps: int, solver: str, threads: int, tol: float = 1e-6, timed_threads: int | None = None):
    """`steps` timed oracle steps (compat mode: 4^3 tiles, the reference's rules) after one
    warm-up step from rest on all `threads`; the timed steps run on `timed_threads`."""
    from oracle import bindings as B
    if not os.path.exists(B.ORACLE_SO):
        B.build(ref=False)
    ora = B.Oracle(scene, block=4, compat=True, solver=solver, tol=tol,
                   max_iter=200 if solver == "reference" else 10**6, threads=threads)
    ora.step(scene.dt)  # from rest the first solve is trivial; it serves as warm-up
    if timed_threads:
        ora.lib.ora_set_threads(int(timed_threads))
    times, nps, phases = [], [], {}
    for _ in range(steps):
        nps.append(ora.num_particles)
        times.append(_oracle_timed_step(ora, scene.dt, phases))
    if timed_threads:
        ora.lib.ora_set_threads(int(threads))
    iters = phases.pop("_iterations")
    tot = sum(times)
    return {"value": sum(nps) / tot, "ms_per_step": 1e3 * tot / len(times), "seconds": tot, "iterations": iters,
            "phase_ms_per_step": {k: round(1e3 * v / len(times), 1) for k, v in phases.items()}}


def cpu_baseline(scene, steps: int, threads: int | None = None, one_thread: bool = True):
    """The reference algorithm on the host cores: the oracle restatement in compat mode
    (4^3 tiles), bit-exact with the reference's code under its own CG rule.

    Variants: `o_ref` the reference's stop rule (|r| < 1e-3 absolute or 201 iterations,
    FP32 dots; at 256^3 it stops on the cap, unconverged); `o_tol` the same FP32 CG
    recurrence with FP64 dots run to ||r||/||b|| < 1e-6 with no cap - the like-for-like
    baseline of the device's converged solve; `o_ref_1_thread` one step of o_ref on one
    thread. The headline value is o_ref (the reference as shipped)."""
    threads = threads or os.cpu_count()
    model = cpu_model()
    ref = _oracle_leg(scene, steps, "reference", threads)
    tol = _oracle_leg(scene, steps, "tol", threads, tol=1e-6)
    out = {"value": ref["value"], "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": model,
           "sample": f"{steps} steps of the full workload after 1 warm-up step, oracle restatement of the "
                     f"reference step (4^3 tiles, reference CG rule: |r|<1e-3 or 201 iterations), "
                     f"{threads} OpenMP threads on {model}; {ref['seconds']:.1f} s",
           "ms_per_step": ref["ms_per_step"], "phase_ms_per_step": ref["phase_ms_per_step"],
           "cg_iterations_per_step": ref["iterations"],
           "variants": {"o_tol": {"value": tol["value"], "unit": UNIT, "cores": threads, "kind": "port",
                                  "ms_per_step": tol["ms_per_step"], "phase_ms_per_step": tol["phase_ms_per_step"],
                                  "cg_iterations_per_step": tol["iterations"],
                                  "sample": f"{steps} steps after 1 warm-up step; the reference's FP32 CG "
                                            f"recurrence with FP64 dots to ||r||/||b|| < 1e-6, no iteration cap "
                                            f"(the device's convergence level); {tol['seconds']:.1f} s"}}}
    if one_thread:
        one = _oracle_leg(scene, 1, "reference", threads, timed_threads=1)
        out["variants"]["o_ref_1_thread"] = {
            "value": one["value"], "unit": UNIT, "cores": 1, "kind": "port", "ms_per_step": one["ms_per_step"],
            "phase_ms_per_step": one["phase_ms_per_step"],
            "sample": f"1 step after 1 warm-up step (warm-up on {threads} threads), reference CG rule, one thread; "
                      f"{one['seconds']:.1f} s"}
    return out


def post_cpu_baseline(flip, reps: int = 2) -> dict:
    """FLIPMethod::postProcess on the host cores next to the device, both on the 64^3 dam
    break after one step (505,856 particles): the oracle restatement in compat mode (4^3
    tiles, the reference's rules; its splat adds in particle order on one thread, as the
    reference's host build does with one thread), all other loops on all cores."""
    import torch
    from oracle import bindings as B
    from vare_gb300 import scenes
    if not os.path.exists(B.ORACLE_SO):
        B.build(ref=False)
    sc = scenes.config0()
    sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
    sim.step(sc.dt)
    sim.post_process()
    gt = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.post_process()
        torch.cuda.synchronize()
        gt.append(time.perf_counter() - t0)
    del sim
    threads = os.cpu_count()
    ora = B.Oracle(sc, block=4, compat=True, solver="reference", max_iter=200, threads=threads)
    ora.step(sc.dt)
    ct = []
    for _ in range(reps):
        t0 = time.perf_counter()
        ora.post_process(sc.dt, literal_scan=True)
        ct.append(time.perf_counter() - t0)
    gt.sort()
    ct.sort()
    return {"workload": "dam_break_64 after one step (505,856 particles)", "gpu_ms": 1e3 * gt[len(gt) // 2],
            "cpu_ms": 1e3 * ct[len(ct) // 2], "cores": threads, "kind": "port",
            "sample": f"{reps} post-processing frames of the oracle restatement in compat mode"}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def allreduce_max(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    """The reference's algorithm on the host cores: every one of the --warmup and --steps
    steps of the workload runs (the first warm-up step starts from rest), all host threads."""
    if rank != 0:
        return
    sc = make_scene(args.workload)
    from oracle import bindings as B
    if not os.path.exists(B.ORACLE_SO):
        B.build(ref=False)
    threads = os.cpu_count()
    model = cpu_model()
    ora = B.Oracle(sc, block=4, compat=True, solver="reference", max_iter=200, threads=threads)
    for _ in range(args.warmup):
        ora.step(sc.dt)
    times, nps, phases = [], [], {}
    for _ in range(args.steps):
        nps.append(ora.num_particles)
        times.append(_oracle_timed_step(ora, sc.dt, phases))
    iters = phases.pop("_iterations")
    value = sum(nps) / sum(times)
    ms = sorted(1e3 * t for t in times)
    sample = (f"{args.steps} timed steps after {args.warmup} warm-up steps of the full workload; "
              f"oracle restatement of the reference FLIP step, bit-exact with the reference's host build "
              f"(4^3 tiles, reference CG rule), {threads} OpenMP threads on {model}")
    metric = METRIC if args.solver != "mixed" else METRIC.replace("plain FP32 block-MIC(0)-PCG", "mixed-precision MG-PCG")
    if args.workload != "dam_sphere_256":
        metric = metric.replace("at 256^3 FLIP", f"at {sc.res[0]}x{sc.res[1]}x{sc.res[2]} FLIP")
    out = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": sum(ms) / len(ms), "p50_ms": ms[len(ms) // 2], "p99_ms": ms[-1],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded jittered-uniform dam break + sphere)", "impl": "reference",
           "config": workload_config(sc, {"solver": "reference CG (absolute 1e-3, 201 iterations), FP32"}),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                            "cpu_model": model, "cg_iterations_per_step": iters,
                            "phase_ms_per_step": {k: round(1e3 * v / len(times), 1) for k, v in phases.items()}},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def timed_steps(sim, sc, args, world, flip, local, sample_clocks, alg=ALG_BYTES):
    """W warm-up steps (every kernel class timed, to find the dominant one), then K timed
    steps with the dominant class's launches bracketed by events, a few of them per step
    (every n-th bracket: an event record ends the programmatic overlap of the kernels around it,
    so bracketing all of a step's ~380 PCG launches would slow the step it measures). Returns
    the measurements."""
    import numpy as np
    import torch

    sim.set_profiling(0xFFFF)
    for _ in range(args.warmup):
        sim.step(sc.dt)
    ms, n = sim.kernel_times()
    classes = flip.KERNEL_CLASSES
    dom = int(np.argmax(ms[:len(classes)]))
    share = {c: float(ms[i]) for i, c in enumerate(classes)}
    # the warm-up's mean launches per step (its first step, from rest, solves little) set the stride
    every = max(1, int(float(n[dom]) / max(1, args.warmup)) // 4)
    sim.set_profiling(1 << dom)
    sim.set_profiling_sampling(every)
    clocks = ClockSampler(local) if sample_clocks else None
    if clocks:
        clocks.start()
    launches0 = sim.stats()["kernel_launches"]
    barrier(world)
    torch.cuda.synchronize()
    step_ms, particle_steps, iters, worst = [], 0, [], {"residual_rel": 0.0, "residual_max_dx": 0.0}
    all_conv = True
    with torch.cuda.nvtx.range("step") if getattr(args, "nvtx", False) else contextlib.nullcontext():
        for _ in range(args.steps):
            n0 = sim.num_particles
            status = sim.step(sc.dt)
            st = sim.stats()
            step_ms.append(st["gpu_ms"])
            particle_steps += n0
            iters.append(st["solver_iterations"])
            worst["residual_rel"] = max(worst["residual_rel"], st["residual_rel"])
            worst["residual_max_dx"] = max(worst["residual_max_dx"], st["residual_max_dx"])
            all_conv = all_conv and status == 0 and st["converged"] == 1
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop() if clocks else None
    launches = sim.stats()["kernel_launches"] - launches0
    kms, kn = sim.kernel_times()
    sim.set_profiling(0)  # untimed from here: the end-to-end steps that follow record no events
    sim.set_profiling_sampling(1)
    my_time = sum(step_ms) / 1e3
    t_max = allreduce_max(my_time, world)
    total_ps = allreduce_sum(float(particle_steps), world)

    # roofline of the dominant kernel class, measured over the timed region
    fi = sim.frame_info()
    ncells = fi["ntiles"] * 512
    name = classes[dom]
    cell_b, part_b = alg.get(name, (0, 0))
    avg_launch_ms = float(kms[dom] / max(1, kn[dom]))
    bytes_per_launch = cell_b * ncells + part_b * sim.num_particles
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_launch / (avg_launch_ms * 1e-3) / 1e9 if avg_launch_ms > 0 else 0.0
    traffic, tnote = ncu_traffic(name)
    roof = {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s",
            "alg_bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_launch_ms,
            "kernels_per_launch": (sim.stats()["mg_vcycle_launches"] if name == "mg_vcycle" else 1),
            "launches_per_step": float(kn[dom]) * every / args.steps, "timed_launches": int(kn[dom]),
            "timed_every": every, "active_cells": ncells,
            "share_of_warmup_device_time": {c: round(v / max(1e-9, sum(share.values())), 4)
                                            for c, v in share.items()}}
    if tnote:
        roof["traffic_note"] = tnote
    ms_sorted = sorted(step_ms)
    p99 = ms_sorted[min(len(ms_sorted) - 1, int(round(0.99 * (len(ms_sorted) - 1))))]
    # whole-step compulsory traffic (per particle, per active cell, per unknown and PCG
    # iteration, per refinement sweep) against the measured HBM bandwidth
    nu = int(np.count_nonzero(sim.field(flip.FIELD_FLAG) == 4))  # fluid cells = unknowns
    b_it = 87 if alg is ALG_BYTES_MIXED else 69
    passes = sim.stats()["refinements"]
    b_step = (92 * sim.num_particles + 90 * ncells + b_it * nu * float(np.mean(iters)) + 13 * nu * passes)
    step_roof = {"bytes_per_step": b_step, "achieved": b_step / (t_max / args.steps) / 1e9, "peak": peak,
                 "unit": "GB/s", "frac": b_step / (t_max / args.steps) / 1e9 / peak,
                 "model": f"92 B/particle + 90 B/active cell + {b_it} B/unknown/PCG iteration + 13 B/unknown/refinement"}
    return {"value": total_ps / t_max, "t_max": t_max, "ms_per_step": t_max * 1e3 / args.steps,
            "p50_ms": ms_sorted[len(ms_sorted) // 2], "p99_ms": p99, "roofline": roof, "step_roofline": step_roof,
            "clocks": clk,
            "launches": int(launches),
            "solver": {"iterations_per_step": iters, "all_converged": all_conv, **worst,
                       "active_tiles": fi["ntiles"]}}


def parity_report(flip, sc, sim, forms: dict) -> dict:
    """One step from the simulation's current particles on the device (each solver form,
    the library's default settings - the ones timed) and on the oracle (all host threads,
    8^3 tiles, the reference's rules, FluidProjection's system solved in FP64 to 1e-12):
    max|device - oracle| / max|oracle| of pressure, projected grid velocity and particle
    velocity and position."""
    import numpy as np

    from oracle import parity as OP
    pos, vel, _, ids = sim.particles()
    o = np.argsort(ids)
    state = OP.with_state(sc, pos[o], vel[o])
    del pos, vel, ids
    ora = OP.oracle_step(state)
    out = {}
    for name, solver in forms.items():
        e = OP.compare(OP.device_step(flip, state, solver=solver), ora)
        e["how"] = ("one step from the state after the timed steps; device at the timed settings vs the oracle's "
                    f"FP64 projection (CG to 1e-12, {ora['seconds']:.0f} s on {os.cpu_count()} host threads); "
                    "max|device - oracle| / max|oracle|")
        out[name] = e
    return out


def warm_parity(flip, sc, sim) -> dict:
    """One warm-started step of `sim` (its solve starts from its last pressure) against the
    oracle's step from the same particles (FP64 projection from p = 0): the errors of
    parity_report."""
    import numpy as np

    from oracle import parity as OP
    pos, vel, _, ids = sim.particles()
    o = np.argsort(ids)
    state = OP.with_state(sc, pos[o], vel[o])
    del pos, vel, ids
    ora = OP.oracle_step(state)
    status = sim.step(sc.dt)
    st = sim.stats()
    pos, vel, _, ids = sim.particles()
    o = np.argsort(ids, kind="stable")
    fi = sim.frame_info()
    dev = dict(status=status, stats=st, tiles=sim.tiles(), pres=sim.field(flip.FIELD_PRES),
               comp=sim.field(flip.FIELD_COMP), nx=fi["nx"], ny=fi["ny"], nz=fi["nz"],
               pos=pos[o], vel=vel[o], ids=ids[o])
    e = OP.compare(dev, ora)
    e["how"] = ("one warm-started device step from the state after the timed steps vs the oracle's step from the "
                "same particles with its FP64 projection (CG to 1e-12, from p = 0); max|device - oracle| / max|oracle|")
    return e


def post_measure(sim, sc, flip, reps: int = 5, nvtx: bool = False) -> dict:
    """FLIPMethod::postProcess on the state the timed steps left (one frame's surface
    pipeline): host wall time of bora_flip_post_process (synchronous; it includes the
    tile rebuild it starts with), then each stage on its own. The redistancing's
    algorithmic bytes are 8 per active cell and step (one read, one write; the tile's
    halo re-reads are not counted); its fields stay resident in L2 at this size."""
    import torch

    torch.cuda.synchronize()
    sim.post_process()  # warm-up (allocates the attribute buffers)
    times = []
    for r in range(max(1, reps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.nvtx.range("post") if nvtx and r == 0 else contextlib.nullcontext():
            sim.post_process()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    stages = {}
    sim.run_stage(flip.STAGE_REBUILD)
    for stage, label in [(flip.POST_SPLAT, "splat"), (flip.POST_TANK_SCAN, "tank_scan"),
                         (flip.POST_REDISTANCE, "redistance"), (flip.POST_ATTRIBUTES, "attributes")]:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.run_post_stage(stage)
        torch.cuda.synchronize()
        stages[label] = 1e3 * (time.perf_counter() - t0)
    st = sim.stats()
    cells = st["active_tiles"] * 512
    iters = 80
    red_s = stages["redistance"] / 1e3
    peak, src = measured_peaks()
    achieved = cells * 8.0 * iters / red_s / 1e9 if red_s > 0 else None
    times.sort()
    return {"ms_per_frame": 1e3 * times[len(times) // 2], "stage_ms": stages, "particles": sim.num_particles,
            "active_cells": cells, "redistance_steps": iters,
            "redistance_roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                    "frac": achieved / peak if achieved else None, "peak_source": src,
                                    "note": "8 B per active cell and step; the two fields (4 B per cell each) "
                                            "stay in L2 at this size, so the fraction can pass 1"},
            "how": "host wall time around synchronous calls; median of %d frames" % len(times)}


def run_ours(args, world, rank, local):
    import torch

    from vare_gb300 import build, flip

    build.build()
    torch.cuda.set_device(local)
    sc = make_scene(args.workload)
    if args.solver == "mixed":
        args.no_mixed = True
    sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED if args.solver == "mixed" else flip.SOLVER_PLAIN)
    meas = timed_steps(sim, sc, args, world, flip, local, True,
                       ALG_BYTES_MIXED if args.solver == "mixed" else ALG_BYTES)
    if args.solver == "plain":
        args.no_mixed = True
    value, roof, clk, launches = meas["value"], meas["roofline"], meas["clocks"], meas["launches"]

    # end to end through the C ABI with host buffers (pinned), rank-local
    e2e = None
    if args.e2e_steps > 0:
        n = sim.num_particles
        hp = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        hv = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        got = sim.get_particles_ptr(hp.data_ptr(), hv.data_ptr(), n)
        e_times, e_ps, h2d, d2h = [], 0, 0, 0
        for _ in range(args.e2e_steps):
            t0 = time.perf_counter()
            sim.set_particles_ptr(hp.data_ptr(), hv.data_ptr(), got)
            sim.step(sc.dt)
            m = sim.num_particles
            if m > hp.shape[0]:
                raise RuntimeError("particle count grew")
            got2 = sim.get_particles_ptr(hp.data_ptr(), hv.data_ptr(), hp.shape[0])
            e_times.append(time.perf_counter() - t0)
            e_ps += got
            h2d += got * 24
            d2h += got2 * 24
            got = got2
        et = allreduce_max(sum(e_times), world)
        eps = allreduce_sum(float(e_ps), world)
        e2e = {"value": eps / et, "unit": UNIT, "h2d_bytes_per_step": h2d // args.e2e_steps,
               "d2h_bytes_per_step": d2h // args.e2e_steps, "steps": args.e2e_steps,
               "ms_per_step": 1e3 * sum(e_times) / len(e_times),
               "how": "host wall time of bora_flip_set_particles (pinned host -> device) + bora_flip_step + "
                      "bora_flip_get_particles (device -> pinned host) per step"}

    # the plain form with each refinement pass's inner PCG in one cooperative launch
    # (bounded grid barriers between the phases; bora_flip_params.persistent = 1)
    persistent = None
    if args.solver != "mixed" and not args.no_persistent:
        del sim
        torch.cuda.empty_cache()
        sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_PLAIN, persistent=1)
        pm = timed_steps(sim, sc, args, world, flip, local, False, ALG_BYTES)
        persistent = {"value": pm["value"], "unit": UNIT, "ms_per_step": pm["ms_per_step"], "p50_ms": pm["p50_ms"],
                      "p99_ms": pm["p99_ms"], "gpu_launches": pm["launches"],
                      "iterations_per_step": pm["solver"]["iterations_per_step"],
                      "config": "same scene and stop rule; each refinement pass's inner PCG (first update, then "
                                "direction and update per iteration) in one cooperative launch whose phases meet at "
                                "grid barriers with bounded waits, convergence checked on the device"}

    # mixed-precision form on the same scene: MG-preconditioned CG, FP16 V-cycle storage
    mixed = None
    if not args.no_mixed:
        del sim
        torch.cuda.empty_cache()
        sim = flip.FlipSim.from_scene(sc, solver=flip.SOLVER_MIXED)
        mm = timed_steps(sim, sc, args, world, flip, local, False, ALG_BYTES_MIXED)
        mixed = {"value": mm["value"], "unit": UNIT, "ms_per_step": mm["ms_per_step"], "p50_ms": mm["p50_ms"],
                 "p99_ms": mm["p99_ms"], "roofline": mm["roofline"], "step_roofline": mm["step_roofline"],
                 "gpu_launches": mm["launches"],
                 "solver": mm["solver"], "speedup_over_plain": mm["value"] / value,
                 "launch_shapes": [{"group": ["L0", "L1", "L2", "L0 batch", "L1 batch", "L2 batch"][g], "size_class": c,
                                    "shape": ([2, 4, 8] if g % 3 == 0 else [64, 128, 256, 512])[v] if v >= 0 else None,
                                    "median_ms": m}
                                   for g, d, c, v, m in flip.tune_table() if d == local],
                 "config": "same scene; geometric-multigrid-preconditioned CG, V(2,2) damped Jacobi, FP16 level "
                           "storage with FP32 arithmetic, FP64-accurate dots and norms, double-float iterative refinement"}

    # parity at the benchmarked settings (a checker, outside every timed region): one step
    # of each solver form and of the oracle (FP64 projection) from the state left here
    if not args.no_parity and args.workload != "tank_1024":
        forms = {"plain": flip.SOLVER_PLAIN, "mixed": flip.SOLVER_MIXED}
        if args.solver != "both":
            forms = {args.solver: forms[args.solver]}
        rep = parity_report(flip, sc, sim, forms)
        meas["solver"]["parity"] = rep.get("plain") or rep.get("mixed")
        if mixed is not None:
            mixed["solver"]["parity"] = rep["mixed"]

    post = None if args.no_post else post_measure(sim, sc, flip, args.post_reps, args.nvtx)

    # both forms again with the warm start (bora_flip_params.warm_start = 1): each solve starts
    # from the last step's pressure instead of from 0 as the reference's does; same stop rule
    warm = None
    if not args.no_warm and args.workload == "dam_sphere_256":
        warm = {}
        cold_mixed = value if args.solver == "mixed" else (mixed["value"] if mixed else None)
        forms = {"plain": (flip.SOLVER_PLAIN, ALG_BYTES, value if args.solver != "mixed" else None),
                 "mixed": (flip.SOLVER_MIXED, ALG_BYTES_MIXED, cold_mixed)}
        if args.solver != "both":
            forms = {args.solver: forms[args.solver]}
        for name, (solver, alg, cold) in forms.items():
            del sim
            torch.cuda.empty_cache()
            sim = flip.FlipSim.from_scene(sc, solver=solver, warm_start=1)
            wm = timed_steps(sim, sc, args, world, flip, local, False, alg)
            warm[name] = {"value": wm["value"], "unit": UNIT, "ms_per_step": wm["ms_per_step"], "p50_ms": wm["p50_ms"],
                          "p99_ms": wm["p99_ms"], "iterations_per_step": wm["solver"]["iterations_per_step"],
                          "all_converged": wm["solver"]["all_converged"],
                          "speedup_over_cold_start": (wm["value"] / cold) if cold else None}
            if not args.no_parity:
                warm[name]["parity"] = warm_parity(flip, sc, sim)

    # the serving stream (64 uneven requests, Poisson arrivals) on the same GPU, after the timed steps
    serve_res = None
    if not args.no_serve and args.workload == "dam_sphere_256":
        del sim
        torch.cuda.empty_cache()
        sim = None
        serve_res = serve_stream(args, world, local, clocks_on=False)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        del sim
        torch.cuda.empty_cache()
        cpu = cpu_baseline(sc, args.cpu_steps)
        if post is not None:
            post["cpu_baseline"] = post_cpu_baseline(flip)

    if rank != 0:
        return
    metric = METRIC if args.solver != "mixed" else METRIC.replace("plain FP32 block-MIC(0)-PCG", "mixed-precision MG-PCG")
    if args.workload != "dam_sphere_256":
        metric = metric.replace("at 256^3 FLIP", f"at {sc.res[0]}x{sc.res[1]}x{sc.res[2]} FLIP")
    out = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": meas["ms_per_step"], "p50_ms": meas["p50_ms"],
           "p99_ms": meas["p99_ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": f"synthetic (seeded jittered-uniform {'tank + wave column' if sc.name.startswith('tank') else 'dam break + sphere'}; "
                   "no public data set exists for this path)",
           "config": workload_config(sc, solver=args.solver if args.solver != "both" else "plain"), "roofline": roof,
           "cpu_baseline": cpu, "e2e": e2e,
           "gpu_launches": int(launches), "clocks": clk, "solver": meas["solver"], "step_roofline": meas["step_roofline"],
           "plain_persistent": persistent, "mixed": mixed, "warm_start": warm, "post_process": post,
           "serve": serve_res}
    print(json.dumps(out), flush=True)


def serve_stream(args, world, local, clocks_on: bool = True) -> dict:
    """The serving stream: requests of uneven sizes arrive as a Poisson process at 20/s and
    are admitted continuously under a 120 GB budget (mixed-precision solver); running
    requests advance together in batched rounds (bora_flip_step_batch). Each rank serves its
    own copy of the stream (replicas)."""
    from vare_gb300 import flip, scenes, serve

    n = args.serve_requests
    reqs = [scenes.serving_request(r) for r in range(n)]
    arrivals = scenes.serving_arrivals(n, 20.0)
    srv = serve.Server(budget_bytes=120 * 10**9, max_running=args.serve_slots)
    clocks = ClockSampler(local) if clocks_on else None
    if clocks:
        clocks.start()
    barrier(world)
    t0 = time.perf_counter()
    ids = []
    for (sc, steps), ta in zip(reqs, arrivals):
        delay = t0 + ta - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        ids.append(srv.submit(sc, steps, solver=flip.SOLVER_MIXED))
    srv.drain()
    t1 = time.perf_counter()
    clk = clocks.stop() if clocks else None
    st = srv.stats()
    info = [srv.poll(i) for i in ids]
    srv.close()
    span = allreduce_max(t1 - t0, world)
    total = allreduce_sum(float(st["particle_steps"]), world)
    qs = sorted(x["queued_s"] for x in info)
    return {"value": total / span, "unit": UNIT,
            "step_ms_p50": st["step_ms_p50"], "step_ms_p99": st["step_ms_p99"], "step_ms_max": st["step_ms_max"],
            "makespan_s": span, "requests": n, "done": st["done"], "failed": st["failed"],
            "substeps": st["steps"], "particle_steps": st["particle_steps"], "running_peak": st["running_peak"],
            "bytes_reserved_peak": st["bytes_reserved_peak"],
            "queue_wait_s": {"p50": qs[len(qs) // 2], "p99": qs[min(len(qs) - 1, int(0.99 * (len(qs) - 1) + 0.5))]},
            "config": {"workload": f"serve_{n}: per request cubic edge log-uniform in [32, 192] cells, fill 0.2-0.5, "
                                   "50-400 substeps, dam break / sphere drop by parity, dt = 1/240, Poisson arrivals "
                                   "at 20/s",
                       "slots": args.serve_slots, "budget_bytes": 120 * 10**9,
                       "stepping": "one stepper thread; all running requests advance together, one "
                                   "bora_flip_step_batch per round (pressure-solve kernels launched once per round)",
                       "parallelism": "replicas (each GPU serves its own stream)"},
            "clocks": clk}


def run_serve(args, world, rank, local):
    import torch

    from vare_gb300 import build

    build.build()
    torch.cuda.set_device(local)
    res = serve_stream(args, world, local)
    if rank != 0:
        return
    n = args.serve_requests
    out = {"metric": f"particle-steps/s, serving stream of {n} FLIP requests (Poisson 20/s, edges 32-192, "
                     "mixed precision, 120 GB budget)",
           "value": res["value"], "unit": UNIT, "n_gpus": world, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam-break / sphere-drop requests)"}
    out.update({k: v for k, v in res.items() if k not in ("value", "unit")})
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "serve_64":
        run_serve(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
