#!/usr/bin/env python
"""Benchmark of the pairwise-interaction hot path on GB300.

Workload (one step = one stochastic Runge-Kutta step of the whole system):
second-order model, N = 4,194,304, density 2, interaction radius R = 1,
Verlet list with skin 0.3 R rebuilt on the max-displacement trigger, strong
order 1.5 stochastic Taylor stepper, dt = 0.005, inertia m = 1, v0 = 0.5,
sigma = 1, D = 0.1; uniform random positions and phases (seeded synthetic
field), mapped to the reference's unit box (L = sqrt(N / density)).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value`: particle-steps/s with the state resident in
HBM (CUDA events on the library's stream, max over ranks, summed over ranks).
`e2e`: the same through spss_step_host (host array in, host array out every
step, the host array page-locked), with `e2e.link` the host link's floor
under it (copy-engine copies of the same bytes).  `roofline`: the pair-and-update kernel's
algorithmic bytes over its CUDA-event duration.  `cpu_baseline` (rank 0): the oracle port of the
reference algorithm on this host's cores.  `allpairs_rk4_n1000`,
`cells_se_n65536`: two smaller workloads (first order N = 1000 all pairs RK4
FP64; second order N = 65,536 cell list SE) next to the oracle port.  `cells`: the
same workload with cell lists rebuilt every step (the reference's linked
list) next to the oracle port of that cell-list workload.  `sweep`: 512
independent systems of the batched parameter sweep stepped as one batch with
cell lists (phase-diagram points per hour at 20,000 steps per point);
`sweep_verlet`: the same with per-system Verlet lists.  `surrogate`
(rank 0): a 256 x 256 phase diagram from the learned surrogate with an
active-learning round, checked against a replica reference, against the
plain method timed at the same precision.  `--impl reference` times the
oracle port alone on the N = 4,194,304 workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 4194304
DENSITY, RADIUS, SKIN, DT = 2.0, 1.0, 0.3, 0.005
V0, MASS, SIGMA, NOISE = 0.5, 1.0, 1.0, 0.1
SRK = 2
L2_BYTES = 129 * 2 ** 20
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def workload(n):
    """Physical configuration mapped to the reference's unit box."""
    L = np.sqrt(n / DENSITY)
    rho = RADIUS / L
    r_max = (1.0 + SKIN) * rho
    return dict(model=2, n=n, rho=rho, v0=V0 / L, xi_r=1.0 / MASS, xi_phi=1.0 / MASS, D_r=0.0,
                D_phi=NOISE / MASS ** 2, sigma=SIGMA / MASS, alpha=0.0, r_max=r_max, nc_verlet=int(1.0 / r_max)), L


def initial_state(n, L, seed):
    rng = np.random.default_rng(seed)
    x = np.empty((n, 6))
    x[:, 0] = rng.random(n)
    x[:, 1] = rng.random(n)
    phi = rng.uniform(-np.pi, np.pi, n)
    x[:, 2] = np.cos(phi) / L
    x[:, 3] = np.sin(phi) / L
    x[:, 4] = phi
    x[:, 5] = 0.0
    return x.reshape(-1)


def mean_list_length(p):
    """Expected Verlet candidates per particle: pi r_max^2 n (unit box)."""
    return np.pi * p["r_max"] ** 2 * p["n"]


def algorithmic_bytes_per_particle(p):
    """Pair-and-update kernel, per particle-step: the 32-byte state read and
    written once (positions 2 x 8 B fixed point, v_x, v_y, phase, omega 4 B
    each) plus the Verlet list (4 B count + 4 B per entry)."""
    return 32 * 2 + 4 + 4 * mean_list_length(p)


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [c.strip() for c in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def traffic_per_launch():
    """DRAM bytes per launch of the pair-and-update kernel from the committed
    ncu summary (profiles/), scaled to the full system; None before a capture."""
    path = os.path.join(ROOT, "profiles", "fast_tile_kernel_srk2_verlet.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_particle"])
    except (OSError, KeyError, ValueError):
        return None


def host_link_ms(nbytes, reps=5):
    """Median times (ms) of copy-engine copies of `nbytes` from page-locked
    host memory to the device and back (CUDA events on torch's stream): the
    host link's floor under the end-to-end figure, whose upload and download
    kernels move the same bytes over the same link."""
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = []
    for src, dst in ((h, d), (d, h)):
        for _ in range(2):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        out.append(statistics.median(ts))
    del h, d
    return out


def cpu_baseline(n, budget_s=20.0, bench_lib=True):
    """The oracle port (FP64, OpenMP over particles as the reference's MPI
    decomposition) on this host's cores, on the same workload, for a bounded
    number of steps."""
    from oracle import binding as ob

    cores = os.cpu_count() or 1
    ob.set_threads(cores, bench=bench_lib)
    p, L = workload(n)
    sysm = ob.System(2, n, p["rho"], v0=p["v0"], xi_r=p["xi_r"], D_r=p["D_r"], xi_phi=p["xi_phi"],
                     D_phi=p["D_phi"], sigma=p["sigma"], alpha=p["alpha"], r_max=p["r_max"],
                     nc_verlet=p["nc_verlet"], bench=bench_lib)
    x = initial_state(n, L, 0)
    # warm-up step builds the Verlet list
    sysm.step(ob.SRK, 4, x, DT, DT, ob.philox_normals(0, 0, 0, 6 * n, bench=bench_lib))
    steps, t0 = 0, time.perf_counter()
    while True:
        normals = ob.philox_normals(0, steps + 1, 0, 6 * n, bench=bench_lib)
        sysm.step(ob.SRK, 4, x, DT * (steps + 2), DT, normals)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or steps >= 50:
            break
    sysm.close()
    return {"value": n * steps / el, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": "N=%d second-order SRK, linked-list+Verlet skin 0.3R, %d timed steps after 1 warm-up "
                      "step (%.1f s), FP64 oracle port, OpenMP %d threads" % (n, steps, el, cores)}


def cpu_cells_sample(n, budget_s=8.0):
    """The oracle port on this host's cores on the cell-list form of the
    workload (linked list rebuilt at every evaluation, as the reference's),
    for a bounded number of steps."""
    from oracle import binding as ob

    cores = os.cpu_count() or 1
    ob.set_threads(cores, bench=True)
    p, L = workload(n)
    sysm = ob.System(2, n, p["rho"], v0=p["v0"], xi_r=p["xi_r"], D_r=p["D_r"], xi_phi=p["xi_phi"],
                     D_phi=p["D_phi"], sigma=p["sigma"], alpha=p["alpha"], bench=True)
    x = initial_state(n, L, 0)
    steps, t0 = 0, time.perf_counter()
    while True:
        normals = ob.philox_normals(0, steps, 0, 6 * n, bench=True)
        sysm.step(ob.SRK, 2, x, DT * (steps + 1), DT, normals)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or steps >= 50:
            break
    sysm.close()
    return {"value": n * steps / el, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": "N=%d second-order SRK, linked list rebuilt every step, %d timed steps (%.1f s), FP64 "
                      "oracle port, OpenMP %d threads" % (n, steps, el, cores)}


def config_system(model, n, density, v0, m=1.0, sigma=1.0, D=0.1, xi=0.1):
    """A physical configuration in the reference's unit box (second order:
    xi_r = xi_phi = 1/m, sigma/m, D_phi = D/m^2, D_r = 0; first order the
    reference's friction xi = 0.1, D_phi = D)."""
    L = np.sqrt(n / density)
    if model == 1:
        kw = dict(v0=v0 / L, xi=xi, sigma=sigma, D_phi=D, alpha=0.0)
    else:
        kw = dict(v0=v0 / L, xi_r=1.0 / m, xi_phi=1.0 / m, D_r=0.0, D_phi=D / m ** 2, sigma=sigma / m, alpha=0.0)
    return RADIUS / L, kw, L


def first_order_initial(n, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 4))
    x[:, 0], x[:, 1] = rng.random(n), rng.random(n)
    x[:, 2] = rng.uniform(-np.pi, np.pi, n)
    return x.reshape(-1)


def run_config_legs(args, rank, world, barrier, max_over_ranks):
    """Two smaller workloads next to the oracle port of the same workload on
    this host's cores:
      allpairs_rk4_n1000: first order, N = 1000, density 1, all pairs called
         directly, RK4, D = 0, v0 = 0.1, sigma = 1, dt = 0.01, FP64 (the
         reference's arithmetic path), a run of 1000 steps;
      cells_se_n65536: second order, N = 65,536, density 2, cell list,
         StochasticEuler, D = 0.1, m = 1, v0 = 0.5, dt = 0.005, FP32 (GB300
         path), 2000 steps of a 10,000-step run timed."""
    import torch

    from oracle import binding as ob
    from spsslangevinintegration_gb300 import ALL_PAIRS, LINKED_LIST, PRECISION_F32, PRECISION_F64, RK4, \
        STOCHASTIC_EULER, Context

    out = {}
    cores = os.cpu_count() or 1
    ob.set_threads(cores, bench=True)
    cases = (("allpairs_rk4_n1000", 1, 1000, 1.0, 0.1, 0.0, RK4, ALL_PAIRS, PRECISION_F64, 0.01, 1000, 1000),
             ("cells_se_n65536", 2, 65536, 2.0, 0.5, 0.1, STOCHASTIC_EULER, LINKED_LIST, PRECISION_F32, DT, 2000,
              10000))
    for name, model, n, density, v0, D, stepper, variant, precision, dt, steps, full in cases:
        rho, kw, L = config_system(model, n, density, v0, D=D)
        x0 = first_order_initial(n, rank) if model == 1 else initial_state(n, L, rank)
        ctx = Context(model, n, rho, precision=precision, variant=variant, flavor=0, seed=12345, replica=rank, **kw)
        ctx.set_state(x0)
        ctx.steps(stepper, 0.0, dt, 5)
        barrier()
        launches0 = ctx.kernel_launches
        t0 = time.perf_counter()
        ctx.steps(stepper, 0.0, dt, steps)
        ctx.synchronize()
        barrier()
        el = max_over_ranks(time.perf_counter() - t0)
        launches = ctx.kernel_launches - launches0
        ctx.close()
        if rank != 0:
            continue
        entry = {"workload": "%s order, N=%d, density %g, R=1, %s, %s, dt=%g, %s" % (
                     "first" if model == 1 else "second", n, density,
                     "all pairs" if variant == ALL_PAIRS else "cell list",
                     "RK4, D=0, v0=0.1, sigma=1 (FP64 path)" if model == 1 else
                     "StochasticEuler, D=0.1, m=1, v0=0.5, sigma=1 (FP32 path)", dt,
                     "%d steps of a %d-step run timed" % (steps, full)),
                 "value": n * steps * world / el, "unit": "particle-steps/s", "ms_per_step": 1e3 * el / steps,
                 "steps_timed": steps, "gpu_launches_per_step": launches / steps,
                 "timing": "wall clock around %d steps (graph launches where the path has them, one host "
                           "synchronisation), max over ranks" % steps}
        if not args.no_cpu_baseline and world == 1:
            sysm = ob.System(model, n, rho, flavor=0, bench=True, **kw)
            x = x0.copy()
            per = 0 if stepper == RK4 else ob.normals_per_particle(model, stepper)
            k, c0 = 0, time.perf_counter()
            while True:
                normals = ob.philox_normals(0, k, 0, per * n, bench=True) if per else None
                sysm.step(stepper, variant, x, dt * (k + 1), dt, normals)
                k += 1
                cel = time.perf_counter() - c0
                if cel >= args.cpu_seconds / 4 or k >= steps:
                    break
            sysm.close()
            entry["cpu_baseline"] = {"value": n * k / cel, "unit": "particle-steps/s", "cores": cores,
                                     "kind": "port", "sample": "%d steps of the same workload (%.1f s), FP64 oracle "
                                     "port, OpenMP %d threads" % (k, cel, cores)}
            entry["speedup_vs_cpu"] = entry["value"] / entry["cpu_baseline"]["value"]
        out[name] = entry
    return out if rank == 0 else None


def run_cells_leg(args, rank, world, barrier, max_over_ranks):
    """The main leg's workload with cell lists rebuilt every step (the
    reference's linked list) instead of Verlet lists, device-timed, next to
    the oracle port of the same cell-list workload on the host cores."""
    import torch

    from spsslangevinintegration_gb300 import PRECISION_F32, Context, LINKED_LIST

    n = args.n
    p, L = workload(n)
    ctx = Context(2, n, p["rho"], precision=PRECISION_F32, variant=LINKED_LIST, v0=p["v0"], xi_r=p["xi_r"],
                  D_r=p["D_r"], xi_phi=p["xi_phi"], D_phi=p["D_phi"], sigma=p["sigma"], alpha=p["alpha"],
                  seed=12345, replica=rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.set_state(initial_state(n, L, rank))
    tune_ms = ctx.autotune(SRK, DT, steps=4)
    tiling = ctx.tiling()
    ctx.steps(SRK, 0.0, DT, max(3, args.warmup // 4))
    steps = max(20, min(args.steps, 100))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    ctx.steps(SRK, 0.0, DT, steps)
    e1.record(stream)
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1))
    ctx.close()
    if rank != 0:
        return None
    value = world * n * steps / (ms * 1e-3)
    out = {"workload": "the main workload (N=%d, SRK) with cell lists of side 1/int(1/rho) rebuilt every step "
                       "(slot re-sort and tile layout each step)" % n,
           "value": value, "unit": "particle-steps/s", "ms_per_step": ms / steps, "steps_timed": steps,
           "tiling": {"tile_cells": tiling[0], "persistent": tiling[1], "autotuned_ms_per_step": tune_ms},
           "timing": "CUDA events around %d graph steps on the library's stream, max over ranks" % steps}
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_cells_sample(n)
        out["cpu_baseline"] = cpu
        out["speedup_vs_cpu"] = value / cpu["value"]
    return out


SWEEP_SYSTEMS, SWEEP_STEPS_PER_POINT, SWEEP_SAMPLE_EVERY = 512, 20000, 10


def sweep_cpu_sample(points, budget_s=8.0):
    """The oracle port (FP64, all cores) on the sweep's most common system
    size: SE steps with cell lists, as particle-steps/s."""
    from oracle import binding as ob
    from spsslangevinintegration_gb300 import sweep

    cores = os.cpu_count() or 1
    ob.set_threads(cores, bench=True)
    pt = sorted(points, key=lambda q: q["n"])[len(points) // 2]
    kw = sweep.system_params(pt)
    sysm = ob.System(2, kw["n"], kw["rho"], v0=kw["v0"], xi_r=kw["xi_r"], D_r=kw["D_r"], xi_phi=kw["xi_phi"],
                     D_phi=kw["D_phi"], sigma=kw["sigma"], bench=True)
    x = sweep.initial_state(kw["n"], np.sqrt(kw["n"] / pt["density"]), 0)
    steps, t0 = 0, time.perf_counter()
    while True:
        normals = ob.philox_normals(0, steps, 0, 3 * kw["n"], bench=True)
        sysm.step(ob.SE, 2, x, DT * (steps + 1), DT, normals)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or steps >= 2000:
            break
    sysm.close()
    return kw["n"] * steps / el, cores, "N=%d (median system), %d SE steps with cell lists, FP64 oracle port, " \
        "OpenMP %d threads, %.1f s" % (kw["n"], steps, cores, el)


def run_sweep_leg(args, rank, world, barrier, max_over_ranks, verlet=False):
    """Batched parameter sweep: 512 independent systems in one batch context
    (one CUDA graph per step for all systems), tiling picked by the autotuner;
    phase-diagram points per hour at 20,000 steps per point.  Cell lists
    rebuilt every step (the sweep's prescribed method), or with `verlet` the
    reference's linked list + Verlet routine with skin 0.3 R, each system's
    lists rebuilt when its own displacement trigger fires (the same neighbour
    sets within R)."""
    import torch

    from spsslangevinintegration_gb300 import LINKED_LIST, LINKED_LIST_VERLET, STOCHASTIC_EULER, sweep
    from spsslangevinintegration_gb300.replicas import shard

    points = sweep.replica_table(SWEEP_SYSTEMS, seed=0)
    mine = [points[i] for i in shard(len(points), world, rank)]
    b = sweep.make_batch(mine, seed=0, first_replica=shard(len(points), world, rank)[0],
                         variant=LINKED_LIST_VERLET if verlet else LINKED_LIST, skin=SKIN if verlet else 0.0)
    b.steps(STOCHASTIC_EULER, 0.0, DT, 3)
    tune_ms = b.autotune(STOCHASTIC_EULER, DT, steps=4)
    b.run(STOCHASTIC_EULER, 0.0, DT, 10, sample_every=SWEEP_SAMPLE_EVERY, sample_from=0)
    steps = max(20, min(args.sweep_steps, 2000))
    launches0 = b.kernel_launches
    rebuilds0 = b.rebuild_count
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run(STOCHASTIC_EULER, 0.0, DT, steps, sample_every=SWEEP_SAMPLE_EVERY, sample_from=0)
    b.synchronize()
    barrier()
    el = max_over_ranks(time.perf_counter() - t0)
    launches = b.kernel_launches - launches0
    rebuild_steps = b.rebuild_count - rebuilds0
    tiling = b.tiling()
    total_n = sum(p["n"] for p in points)
    b.close()
    if rank != 0:
        return None
    s_per_step = el / steps
    lists = ("linked list + Verlet lists (skin 0.3R), each system rebuilt on its own displacement trigger"
             if verlet else "cell lists rebuilt every step")
    out = {
        "workload": "%d independent systems (second-order model): N log-uniform in [1024, 65536] (total %d), "
                    "sigma uniform in [0, 3], D log-uniform in [0.01, 1], m in {0.1, 1, 10}, density 2, R=1, "
                    "v0=0.5, %s, StochasticEuler dt=0.005, per-system time-averaged "
                    "phase and velocity order parameters sampled every %d steps" % (len(points), total_n, lists,
                                                                                   SWEEP_SAMPLE_EVERY),
        "steps_timed": steps, "ms_per_step": 1e3 * s_per_step, "particle_steps_per_s": total_n / s_per_step,
        "points_per_hour": len(points) * 3600.0 / (SWEEP_STEPS_PER_POINT * s_per_step),
        "points_per_hour_unit": "phase-diagram points per hour at %d steps per point" % SWEEP_STEPS_PER_POINT,
        "tiling": {"tile_cells": tiling[0], "persistent": tiling[1], "autotuned_ms_per_step": tune_ms},
        "gpu_launches_per_step": launches / steps, "steps_with_a_rebuild": rebuild_steps,
        "timing": "wall clock around %d steps (graph launches, one host synchronisation), max over ranks" % steps,
    }
    if not args.no_cpu_baseline and world == 1 and not verlet:
        rate, cores, sample = sweep_cpu_sample(points, budget_s=args.cpu_seconds / 2)
        out["cpu_baseline"] = {"particle_steps_per_s": rate, "cores": cores, "kind": "port", "sample": sample,
                               "points_per_hour": len(points) * 3600.0 * rate / (total_n * SWEEP_STEPS_PER_POINT)}
    return out


def run_surrogate_leg(args):
    """Phase diagram over a 256 x 256 (sigma, D) grid (N = 1024, density 2,
    m = 1, v0 = 0.5, 4000 SE steps per run) from the learned surrogate with one
    active-learning round, checked against a 256-replica reference at 48
    random grid points.  The plain method at the same precision is timed on
    the same workload: R runs at each of 80 grid points (the 48 checked ones
    and 32 more), R chosen so that a point's mean lands within 0.02 with 95 %
    probability (R = (1.96 std / 0.02)^2 averaged over the checked points, std
    the reference's run-to-run spread; the surrogate's own fraction within
    0.02 is measured at the same points), batched like the surrogate's
    training runs."""
    import torch

    from spsslangevinintegration_gb300 import surrogate as S

    grid = S.grid_points(256, 256)
    t0 = time.perf_counter()
    res = S.phase_diagram(grid, n_train=args.surrogate_train, steps=4000, epochs=100, rounds=1, flag_fraction=0.05)
    total = time.perf_counter() - t0
    idx = np.random.default_rng(11).choice(len(grid), 48, replace=False)
    mean, std = S.reference([grid[i] for i in idx], 256, steps=4000)
    err = np.abs(res["values"][idx] - mean).max(axis=1)
    runs_needed = float(np.maximum(1.0, (std.max(axis=1) / 0.02) ** 2).mean())
    single_rate = args.surrogate_train / res["seconds"]["simulate_training"]  # plain runs per second
    derived_pph = single_rate * 3600.0 / runs_needed
    sur_pph = len(grid) * 3600.0 / total
    # the plain replicated sweep, timed, at 95 % within 0.02
    reps = int(np.ceil(np.mean(np.maximum(1.0, (1.96 * std.max(axis=1) / 0.02) ** 2))))
    others = [i for i in np.random.default_rng(12).permutation(len(grid)) if i not in set(idx.tolist())][:32]
    subset = list(idx) + others
    torch.cuda.synchronize()
    p0 = time.perf_counter()
    runs = S.run_values(S.simulate([grid[i] for i in subset for _ in range(reps)], steps=4000, sample_every=10,
                                   seed=0, first_replica=2 * 10 ** 7))
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - p0
    plain_est = runs.reshape(len(subset), reps, 2).mean(axis=1)[:len(idx)]
    plain_err = np.abs(plain_est - mean).max(axis=1)
    plain_pph = len(subset) * 3600.0 / plain_s
    z = np.abs(res["judge_z"]).max(axis=1)
    return {
        "workload": "256 x 256 (sigma in [0, 3], D log in [0.01, 1]) phase diagram of the expected phase and "
                    "velocity order parameters, N=1024, density 2, m=1, v0=0.5, StochasticEuler dt=0.005, 4000 "
                    "steps per run (time average over the second half, every 10 steps), linked list + Verlet "
                    "lists (skin 0.3R) for the surrogate's runs and the plain method's alike",
        "network": "5-128-128-128-4 GELU, BF16 operands, FP32 accumulate (tcgen05, tensor memory), Adam",
        "training_runs": args.surrogate_train, "judge_runs": int(res["runs"] - args.surrogate_train),
        "seconds": {k: round(v, 3) for k, v in res["seconds"].items()}, "seconds_total": total,
        "note": "this leg's workload (N=1024, 4000 steps per run, the 256 x 256 grid) is not the batched sweep "
                "leg's (N log-uniform in [1024, 65536], 20,000 steps); both the surrogate and the plain method "
                "are timed here on this leg's workload",
        "points_per_hour": sur_pph,
        "plain_points_per_hour_at_0.02": plain_pph,
        "plain_timed": {"grid_points": len(subset), "runs_per_point": reps, "runs": len(subset) * reps,
                        "target": "a point's mean within 0.02 with 95 % probability",
                        "seconds": plain_s,
                        "accuracy": {"median_abs_error": float(np.median(plain_err)),
                                     "q90_abs_error": float(np.quantile(plain_err, 0.9)),
                                     "frac_within_0.02": float(np.mean(plain_err <= 0.02))}},
        "plain_points_per_hour_derived": derived_pph,
        "plain_runs_per_point_at_0.02_standard_error": runs_needed,
        "ratio_vs_plain": sur_pph / plain_pph,
        "accuracy": {"reference": "48 grid points x 256 plain runs", "median_abs_error": float(np.median(err)),
                     "q90_abs_error": float(np.quantile(err, 0.9)), "frac_within_0.02": float(np.mean(err <= 0.02))},
        "judge_calibration": {"frac_abs_z_le_2": float(np.mean(z <= 2.0)), "frac_abs_z_le_3": float(np.mean(z <= 3.0))},
        "network_kernel_launches": int(res["network_kernel_launches"]),
    }


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    n = args.n
    res = None
    per_step = []
    # W untimed samples then K timed ones, each sample one oracle-port step
    from oracle import binding as ob

    cores = os.cpu_count() or 1
    ob.set_threads(cores, bench=True)
    p, L = workload(n)
    sysm = ob.System(2, n, p["rho"], v0=p["v0"], xi_r=p["xi_r"], D_r=p["D_r"], xi_phi=p["xi_phi"],
                     D_phi=p["D_phi"], sigma=p["sigma"], alpha=p["alpha"], r_max=p["r_max"],
                     nc_verlet=p["nc_verlet"], bench=True)
    x = initial_state(n, L, 0)
    budget = 120.0
    t_start = time.perf_counter()
    for k in range(args.warmup + args.steps):
        normals = ob.philox_normals(0, k, 0, 6 * n, bench=True)
        t0 = time.perf_counter()
        sysm.step(ob.SRK, 4, x, DT * (k + 1), DT, normals)
        dt_s = time.perf_counter() - t0
        if k >= args.warmup:
            per_step.append(dt_s)
        if time.perf_counter() - t_start > budget and len(per_step) >= 1:
            break
    sysm.close()
    total = sum(per_step)
    value = n * len(per_step) / total
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": len(per_step), "warmup": args.warmup, "ms_per_step": 1e3 * total / len(per_step),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "second-order model, N=%d, density 2, R=1, Verlet skin 0.3R, StochasticRungeKutta, "
                               "dt=0.005, m=1, v0=0.5, sigma=1, D=0.1" % n, "n": n},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": "%d timed SRK steps of the full N=%d system (FP64 oracle port, OpenMP %d threads)"
                                   % (len(per_step), n, cores)},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_legs_only(args, rank, world, local_rank):
    """Only the smaller-workload, cell-list, sweep, Verlet-sweep and/or surrogate
    legs (for profiling them alone); the default run measures every leg."""
    import torch

    from spsslangevinintegration_gb300.replicas import max_over_ranks

    torch.cuda.set_device(local_rank)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    line = {"legs": sorted(args.legs)}
    if "configs" in args.legs:
        cf = run_config_legs(args, rank, world, barrier, max_over_ranks)
        if cf is not None:
            line.update(cf)
    if "cells" in args.legs:
        cl = run_cells_leg(args, rank, world, barrier, max_over_ranks)
        if cl is not None:
            line["cells"] = cl
    if "sweep" in args.legs:
        sw = run_sweep_leg(args, rank, world, barrier, max_over_ranks)
        if sw is not None:
            line["sweep"] = sw
    if "sweep_verlet" in args.legs:
        sv = run_sweep_leg(args, rank, world, barrier, max_over_ranks, verlet=True)
        if sv is not None:
            line["sweep_verlet"] = sv
    if "surrogate" in args.legs and rank == 0:
        line["surrogate"] = run_surrogate_leg(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_ours(args, rank, world, local_rank):
    import torch

    from spsslangevinintegration_gb300 import PRECISION_F32, Context, LINKED_LIST_VERLET, PinnedArray
    from spsslangevinintegration_gb300.replicas import max_over_ranks

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

    n = args.n
    p, L = workload(n)
    x0 = initial_state(n, L, seed=rank)
    ctx = Context(2, n, p["rho"], precision=PRECISION_F32, variant=LINKED_LIST_VERLET, v0=p["v0"], xi_r=p["xi_r"],
                  D_r=p["D_r"], xi_phi=p["xi_phi"], D_phi=p["D_phi"], sigma=p["sigma"], alpha=p["alpha"],
                  r_max=p["r_max"], nc_verlet=p["nc_verlet"], seed=12345, replica=rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.set_state(x0)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # tile width and launch form picked by the library's autotuner (trial
    # steps, state restored), then warm-up (graph capture, first list build)
    if args.tile_cells:
        ctx.set_tiling(args.tile_cells, False)
        tune_ms = None
    else:
        tune_ms = None if args.no_autotune else ctx.autotune(SRK, DT, steps=4)
    tiling = ctx.tiling()
    t = 0.0
    ctx.steps(SRK, t, DT, args.warmup)
    t += DT * args.warmup
    # start the timed window right after a Verlet rebuild: single steps until
    # the trigger has fired and the lists were rebuilt
    r_align = ctx.rebuild_count
    for _ in range(400):
        if ctx.rebuild_count != r_align:
            break
        ctx.step(SRK, t + DT, DT)
        t += DT
    barrier()
    launches0 = ctx.kernel_launches
    rebuilds0 = ctx.rebuild_count
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        barrier()
        e0.record(stream)
        ctx.steps(SRK, t, DT, args.steps)
        e1.record(stream)
        barrier()
    t += DT * args.steps
    window_ms = e0.elapsed_time(e1)
    launches = ctx.kernel_launches - launches0
    rebuilds_in_window = ctx.rebuild_count - rebuilds0

    # roofline: the pair-and-update kernel alone, CUDA events on the same stream
    ctx.set_timing(True)
    ctx.steps(SRK, t, DT, args.steps)
    t += DT * args.steps
    kernel_ms, kernel_count = ctx.timing()
    ctx.set_timing(False)
    avg_kernel_s = kernel_ms / max(kernel_count, 1) * 1e-3

    # steady state: the rebuild interval over a long untimed run, and the cost
    # of a rebuild (steps with a forced rebuild against plain steps, CUDA
    # events on the library's stream); rebuilds the window holds fewer of
    # than its share at that interval are added at that cost (never removed)
    interval_steps = 160
    r1 = ctx.rebuild_count
    ctx.steps(SRK, t, DT, interval_steps)
    t += DT * interval_steps
    rebuilds_long = ctx.rebuild_count - r1
    interval = interval_steps / rebuilds_long if rebuilds_long else None
    step_ms = {0: [], 1: []}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for k in range(12):
        forced = k % 2
        if forced:
            ctx.set_should_update_lists(1)
        ev[0].record(stream)
        ctx.step(SRK, t + DT, DT)
        ev[1].record(stream)
        ev[1].synchronize()
        t += DT
        step_ms[forced].append(ev[0].elapsed_time(ev[1]))
    rebuild_ms = max(0.0, statistics.median(step_ms[1]) - statistics.median(step_ms[0]))
    share = args.steps / interval if interval else 0.0
    added = max(0.0, share - rebuilds_in_window)
    ms = max_over_ranks(window_ms + added * rebuild_ms)
    value = world * n * args.steps / (ms * 1e-3)
    peak, peak_kind = hbm_peak()
    bytes_per_launch = n * algorithmic_bytes_per_particle(p)
    achieved = bytes_per_launch / avg_kernel_s / 1e9
    traffic = traffic_per_launch()

    # end to end through the host-array entry point (the drop-in DoStep path),
    # the state in a page-locked host array the kernels read and write over
    # the host link
    pinned = PinnedArray(ctx.length)
    host = pinned.array
    host[:] = ctx.get_state()
    e2e_steps = max(1, min(args.steps, 10))
    ctx.step_host(SRK, host, t, DT)
    t += DT
    barrier()
    r_e2e = ctx.rebuild_count
    w0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.step_host(SRK, host, t, DT)
        t += DT
    barrier()
    e2e_s = time.perf_counter() - w0
    e2e_added = max(0.0, (e2e_steps / interval if interval else 0.0) - (ctx.rebuild_count - r_e2e))
    e2e_s = max_over_ranks(e2e_s + e2e_added * rebuild_ms * 1e-3)
    e2e_value = world * n * e2e_steps / e2e_s
    pinned.free()
    h2d_ms, d2h_ms = host_link_ms(n * 6 * 8)
    link_floor_ms = h2d_ms + d2h_ms + ms / args.steps
    acc, flag, uses = ctx.verlet_state()
    ctx.close()

    if rank != 0:
        return 0
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "rebuilds_in_window": rebuilds_in_window,
        "timing": {"how": "CUDA events around the %d timed steps (graph launches) on the library's stream, max over "
                          "ranks; the window starts right after a Verlet rebuild, and the rebuilds it holds fewer "
                          "of than its share at the measured rebuild interval are added at the measured rebuild "
                          "cost (steady state; none are removed)" % args.steps,
                   "window_ms_per_step": window_ms / args.steps, "rebuilds_in_window": rebuilds_in_window,
                   "rebuild_interval_steps": interval, "rebuild_ms": rebuild_ms, "rebuilds_added": added},
        "scaling": "weak" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "second-order model, N=%d, density 2, R=1, Verlet skin 0.3R (rebuilt on the "
                               "max-displacement trigger), StochasticRungeKutta (strong order 1.5), dt=0.005, m=1, "
                               "v0=0.5, sigma=1, D=0.1; one independent replica per GPU" % n,
                   "n": n, "l2": "inputs larger than L2 (state %.0f MB + lists %.0f MB)" % (
                       n * 56 / 1e6, n * 4 * (mean_list_length(p) + 1) / 1e6),
                   "parallelism": "replicas x%d" % world,
                   "tiling": {"tile_cells": tiling[0], "persistent": tiling[1], "autotuned_ms_per_step": tune_ms}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "kernel": "fast_tile_kernel<2,2,2> (pair sums + SRK update)",
                     "kernel_ms": avg_kernel_s * 1e3,
                     "algorithmic_bytes_per_particle": algorithmic_bytes_per_particle(p),
                     "traffic": None if traffic is None else traffic * n},
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": n * 6 * 8,
                "d2h_bytes_per_step": n * 6 * 8, "steps": e2e_steps, "rebuilds_added": e2e_added,
                "path": "spss_step_host: host AoS float64 in, one SRK step, host AoS out (page-locked host "
                        "array from spss_pinned_alloc)",
                "link": {"h2d_ms": h2d_ms, "d2h_ms": d2h_ms, "h2d_gbs": n * 48 / h2d_ms / 1e6,
                         "d2h_gbs": n * 48 / d2h_ms / 1e6, "floor_ms_per_step": link_floor_ms,
                         "frac": link_floor_ms / (e2e_s * 1e3 / e2e_steps),
                         "how": "copy-engine copies of one step's state bytes each way (page-locked host memory, "
                                "CUDA events) plus ms_per_step: the host link's floor under the end-to-end step"}},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "verlet": {"accumulated_displacement": acc, "rebuild_pending": flag},
    }
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(n, budget_s=args.cpu_seconds)
    if not args.no_cells:
        cl = run_cells_leg(args, rank, world, barrier, max_over_ranks)
        if cl is not None:
            line["cells"] = cl
    if not args.no_configs:
        cf = run_config_legs(args, rank, world, barrier, max_over_ranks)
        if cf is not None:
            line.update(cf)
    if not args.no_sweep:
        sw = run_sweep_leg(args, rank, world, barrier, max_over_ranks)
        if sw is not None:
            line["sweep"] = sw
    if "sweep_verlet" in args.legs:
        sv = run_sweep_leg(args, rank, world, barrier, max_over_ranks, verlet=True)
        if sv is not None:
            line["sweep_verlet"] = sv
    if not args.no_surrogate and rank == 0:
        line["surrogate"] = run_surrogate_leg(args)
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="main leg: keep the default tiling (32 cells per tile, one launch per step)")
    ap.add_argument("--tile-cells", type=int, default=0,
                    help="main leg: this tiling (cells per tile, one launch per step) instead of the autotuner's")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--sweep-steps", type=int, default=400)
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--surrogate-train", type=int, default=50000)
    ap.add_argument("--legs", default="main,configs,cells,sweep,sweep_verlet,surrogate",
                    help="comma-separated subset of main, configs, cells, sweep, sweep_verlet, surrogate "
                         "(profiling a leg alone)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    args.legs = set(x.strip() for x in args.legs.split(",") if x.strip())
    args.no_cells = "cells" not in args.legs
    args.no_configs = "configs" not in args.legs
    if "main" in args.legs:
        args.no_sweep = args.no_sweep or "sweep" not in args.legs
        args.no_surrogate = args.no_surrogate or "surrogate" not in args.legs
        rc = run_ours(args, rank, world, local_rank)
    else:
        rc = run_legs_only(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
