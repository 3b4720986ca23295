"""Benchmark: pair-interactions/s of the all-pairs force + integrate step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (a "step" is one force + integrate iteration over the whole system):
N = 1,048,576 particles from a seeded Plummer sphere (scale radius 1, total mass
1), eps2 = 1e-4, dt = 1e-4, damping 1, FP32.  The inputs are generated on the
host by the library's seeded generator (no dataset).

Prints one JSON line.  `value` is device time with the state resident in HBM
(CUDA events on the simulation's stream, L2 flushed between timed steps);
`e2e` is the same metric through the C ABI with host buffers: every step copies
the state in from pinned host memory, advances, and copies it back.  Every
accumulator is measured (plain, compensated, and reference order -- the
reference kernel's own summation, bit for bit); the headline is the fastest one
whose force error against FP64 is within 1e-5 relative RMS.  The CPU baseline
times the reference kernel body as an OpenMP loop built for speed
(oracle/cpu_port.c, -O3 -ffast-math) on a bounded sample of i-rows against all N
j-particles.  Extra keys report the ensemble and adjoint speed-ups of the metric's
other two parts, and the headless render.

With --impl reference the line reports the reference's CPU path (that port, on
all host threads) on the same workload -- made by the oracle's bit-identical
restatement of the generator, so that arm never loads the library -- and, as an
extra key, the reference's own CUDA kernel built from its source for sm_103a.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "cuda-to-sycl-nbody_gb300"))

METRIC = "pair-interactions/s & %FP32 peak at N=1M; ensemble+adjoint speedup vs plain"
UNIT = "pair-interactions/s"
N_BENCH = 1 << 20
EPS2 = 1e-4
DT = 1e-4
SEED = 20261203
FLOP_PER_PAIR = 20


def workload_desc(n=N_BENCH):
    return {"workload": f"Plummer sphere N={n}, eps2={EPS2:g}, dt={DT:g}, FP32, one force+integrate "
                        "iteration per step", "N": n, "eps2": EPS2, "dt": DT, "seed": SEED,
            "pairs_per_step": n * n, "l2": "flushed between timed steps (512 MiB write)"}


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
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
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [s.strip() for s in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------- helpers
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("NB_BENCH_BACKEND") != "gloo" else "gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    """The largest of every rank's `v` (the whole job's time is the slowest rank's)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds_this_rank: float, world: int) -> float:
    """Units processed by all ranks divided by the slowest rank's time."""
    return units_per_rank * world / max_over_ranks(seconds_this_rank, world)


CPU_PORT_DESC = ("oracle/cpu_port.c: the reference kernel body (src/simulator.cu:193-211) "
                 "as an OpenMP loop over i-rows, built gcc -O3 -ffast-math -fopenmp (the j loop "
                 "vectorised; no -march=native, one recipe for both hosts)")


def cpu_sample_rate(pos, mass_G, target_s: float, max_rows: int | None = None):
    """The timed CPU port on strided i-rows against all N j, on every core this
    process may use.  Returns (pairs/s, rows, seconds, threads)."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_binding as orc

    # Every core this process may run on (a launcher may have set OMP_NUM_THREADS=1).
    orc.port_set_num_threads(len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity")
                             else (os.cpu_count() or 1))
    n = pos[0].size
    rows = 64
    while True:
        idx = np.linspace(0, n - 1, rows).astype(np.int64)
        t0 = time.perf_counter()
        orc.port_accel(pos, mass_G, EPS2, rows=idx)
        dt = time.perf_counter() - t0
        if dt >= target_s or (max_rows and rows >= max_rows):
            return rows * n / dt, rows, dt, orc.port_num_threads()
        grow = max(2.0, min(8.0, target_s / max(dt, 1e-3)))
        rows = int(rows * grow)
        if max_rows:
            rows = min(rows, max_rows)


def plummer_inputs(n=N_BENCH):
    """The workload from the library's seeded generator (nb_ic_plummer)."""
    import nbody_gb300 as nb

    (x, y, z), (vx, vy, vz), m = nb.plummer(SEED, n)
    return [x, y, z], [vx, vy, vz], m


def plummer_inputs_without_library(n=N_BENCH):
    """The same workload, bit for bit, from the oracle's restatement of the generator
    (oracle/workload_ic.c): the reference arm never loads the library under test."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_binding as orc

    (x, y, z), (vx, vy, vz), m = orc.plummer(SEED, n)
    return [x, y, z], [vx, vy, vz], m


# --------------------------------------------------------------------------- our arm
def force_error_vs_fp64(sim, n, rows_count=1024):
    """FP32 accelerations of the simulation's current state against GPU FP64
    accelerations on strided rows: (relative RMS, max per-row relative)."""
    rows = np.linspace(0, n - 1, rows_count).astype(np.uint64)
    a32 = sim.accelerations()
    a64 = sim.fp64_accelerations(rows)
    g = np.stack([a[rows.astype(np.int64)].astype(np.float64) for a in a32])
    r = np.stack(a64)
    err = np.linalg.norm(g - r, axis=0)
    mag = np.linalg.norm(r, axis=0)
    return (float(np.sqrt(np.mean(err ** 2) / np.mean(mag ** 2))),
            float(np.max(err / np.maximum(mag, 1e-300))), int(rows_count))


def time_steps(sim, stream, flush, steps, flush_mib):
    """Per-step CUDA-event times (ms) on `stream`, L2 flushed between steps."""
    import torch

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        if flush_mib:
            flush.zero_()
        starts[k].record(stream)
        sim.advance(1)
        ends[k].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in zip(starts, ends)]


def run_ours(args, rank, world) -> dict:
    import torch

    import nbody_gb300 as nb

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    n = args.n
    pos, vel, m = plummer_inputs(n)
    stream = torch.cuda.current_stream()
    flush = torch.empty(max(1, args.flush_mib) << 20, dtype=torch.uint8, device="cuda")
    peak_tf = nb.fp32_peak_tflops()
    peak_meas_tf = nb.measured_fp32_peak_tflops()

    # Every accumulator: force error against FP64 at the initial state, then the rate.
    modes = {}
    for name, acc in (("plain", nb.ACC_PLAIN), ("compensated", nb.ACC_COMPENSATED),
                      ("reference_order", nb.ACC_REFERENCE_ORDER)):
        if args.acc != "auto" and args.acc != name:
            continue
        p = nb.SimParam(numParticles=n, G=1.0, dt=DT, damping=1.0, distEps=EPS2, accumulator=acc)
        sim = nb.Simulation(p, pos, vel, m)
        sim.set_stream(stream.cuda_stream)
        if args.autotune:
            sim.autotune()
        rms, mx, nrows = force_error_vs_fp64(sim, n) if not args.no_accuracy else (None, None, 0)
        modes[name] = {"sim": sim, "force_rel_rms_vs_fp64": rms, "force_rel_max_vs_fp64": mx,
                       "rows": nrows}
    # Time every mode briefly; the headline is the fastest one whose force error
    # against FP64 meets the 1e-5 relative-RMS target.
    target = 1e-5
    for name, md in modes.items():
        sim = md["sim"]
        sim.advance(1)
        md["probe_ms"] = sim.time_iterations(2) / 2
    ok = [k for k, v in modes.items() if (v["force_rel_rms_vs_fp64"] or 0.0) <= target] or \
        list(modes)
    head = min(ok, key=lambda k: modes[k]["probe_ms"])
    order = [head] + [k for k in modes if k != head]

    result = None
    for name in order:
        sim = modes[name]["sim"]
        kinfo = sim.kernel_info()
        for _ in range(args.warmup):
            sim.advance(1)
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        if name == head:
            with ClockSampler(torch.cuda.current_device()) as clk:
                w0 = time.perf_counter()
                step_ms = time_steps(sim, stream, flush, args.steps, args.flush_mib)
                wall = time.perf_counter() - w0
        else:
            step_ms = time_steps(sim, stream, flush, min(args.steps, 5), args.flush_mib)
        sim.synchronize()
        barrier(world)
        dev_s = max_over_ranks(sum(step_ms) / 1e3, world)
        rate = float(n) * n * len(step_ms) * world / dev_s
        modes[name].update({"value": rate, "unit": UNIT, "ms_per_step": dev_s * 1e3 / len(step_ms),
                            "fp32_peak_frac": rate * FLOP_PER_PAIR / world / (peak_tf * 1e12),
                            "kernel": kinfo})
        if name != head:
            continue
        achieved_tf = FLOP_PER_PAIR * float(n) * n / (min(step_ms) * 1e-3) / 1e12
        roofline = {"bound": "fp32", "achieved": achieved_tf, "peak": peak_tf,
                    "unit": "TFLOP/s", "frac": achieved_tf / peak_tf,
                    "traffic": traffic_from_profile(),
                    "peak_source": "nominal: SMs x 128 FP32 lanes x 2 flop x max SM clock "
                                   "(no FP32 peak in MEASURED_PEAKS.json)",
                    "peak_measured": peak_meas_tf,
                    "frac_of_measured": achieved_tf / peak_meas_tf,
                    "peak_measured_source": "FFMA2 loop kernel over every SM, best of 20 "
                                            "(nb_measure_fp32_peak_tflops), this run",
                    "flop_per_pair": FLOP_PER_PAIR,
                    "kernel_ms": {"min": min(step_ms), "median": statistics.median(step_ms)}}
        # e2e through the C ABI with pinned host buffers
        host = [torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(6)]
        for h, src in zip(host, pos + vel):
            h[:] = src
        e2e_steps = max(1, min(args.steps, 5))
        sim.set_state(host[:3], host[3:])
        sim.advance(1)
        sim.get_state(host)
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            sim.set_state(host[:3], host[3:])   # 6 x N floats host -> device
            sim.advance(1)
            sim.get_state(host)                 # 6 x N floats device -> host (synchronizes)
        e2e_s = max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": float(n) * n * e2e_steps * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": 6 * 4 * n, "d2h_bytes_per_step": 6 * 4 * n,
               "ms_per_step": e2e_s * 1e3 / e2e_steps}
        result = {
            "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Plummer sphere generated by the library)",
            "config": dict(workload_desc(n), kernel=kinfo, accumulator=head, l2=(
                f"flushed between timed steps ({args.flush_mib} MiB write)"
                if args.flush_mib else "not flushed (profiling run)"),
                parallelism="replicas" if world > 1 else "single GPU"),
            "gflops": rate * FLOP_PER_PAIR / 1e9,
            "fp32_peak_frac": rate * FLOP_PER_PAIR / world / (peak_tf * 1e12),
            "force_rel_rms_vs_fp64": modes[head]["force_rel_rms_vs_fp64"],
            "force_rel_max_vs_fp64": modes[head]["force_rel_max_vs_fp64"],
            "roofline": roofline, "e2e": e2e, "gpu_launches": args.steps,
            "clocks": clk.summary(), "wall_s_timed_region": wall,
        }
    # The extras and the CPU baseline run at N = 1 only: under torchrun they would hold
    # every GPU of the job while rank 0 alone works.
    solo = rank == 0 and world == 1
    if solo and not args.no_extras:
        result["render"] = bench_render(modes[head]["sim"], n)
    result["accumulators"] = {k: {a: b for a, b in v.items() if a not in ("sim", "probe_ms")}
                              for k, v in modes.items()}
    result["accumulator_policy"] = ("fastest accumulator whose force error vs FP64 on "
                                    f"{modes[head]['rows']} rows is <= 1e-5 relative RMS")
    for v in modes.values():
        v["sim"].close()
    del flush
    if solo and not args.no_extras:
        result["ensemble"] = bench_ensemble(args)
        result["adjoint"] = bench_adjoint(args)
    if solo and not args.no_cpu:
        rate, rows, secs, thr = cpu_sample_rate(pos, float(np.float32(m[0])), args.cpu_seconds)
        result["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": thr, "kind": "port",
            "sample": f"{rows} strided i-rows x all {n} j-particles of the same workload "
                      f"({secs:.1f} s) on {thr} threads; {CPU_PORT_DESC}"}
    return result


def run_split(args, rank, world) -> dict:
    """One 1,048,576-particle system split over the job's GPUs (strong scaling): each
    rank integrates its shard of the particles against all N and the ranks
    all-gather their shards' positions after every step (nbody_gb300.shard over
    NCCL).  The timed step includes the all-gather."""
    import torch
    import torch.distributed as dist

    import nbody_gb300 as nb
    from nbody_gb300.shard import ShardedSimulation

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if not dist.is_initialized():                    # one GPU: a one-rank NCCL group
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29517")
        dist.init_process_group("nccl", rank=0, world_size=1)
    n = args.n
    pos, vel, m = plummer_inputs(n)
    stream = torch.cuda.current_stream()
    flush = torch.empty(max(1, args.flush_mib) << 20, dtype=torch.uint8, device="cuda")
    p = nb.SimParam(numParticles=n, G=1.0, dt=DT, damping=1.0, distEps=EPS2,
                    accumulator=nb.ACC_COMPENSATED)
    sim = nb.Simulation(p, pos, vel, m)
    sharded = ShardedSimulation(sim, rank, world, device="cuda")
    first, count = sharded.shard
    kinfo = sim.kernel_info()
    peak_tf = nb.fp32_peak_tflops()
    for _ in range(args.warmup):
        sharded.step(1)
    torch.cuda.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        for k in range(args.steps):
            if args.flush_mib:
                flush.zero_()
            starts[k].record(stream)
            sharded.step(1)
            ends[k].record(stream)
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    sim.synchronize()
    dist.barrier()
    dev_s = max_over_ranks(sum(step_ms) / 1e3, world)
    rate = float(n) * n * args.steps / dev_s          # the one system's pairs, whole job
    # e2e: every rank loads the state from pinned host memory, steps (with the
    # exchange) and reads its copy back.
    host = [torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(6)]
    for h, src in zip(host, pos + vel):
        h[:] = src
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.set_state(host[:3], host[3:])
        sharded.step(1)
        sharded.gather_velocities()
        sim.get_state(host)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    achieved_tf = FLOP_PER_PAIR * float(n) * count / (min(step_ms) * 1e-3) / 1e12
    result = {
        "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Plummer sphere generated by the library)",
        "config": dict(workload_desc(n), kernel=kinfo, accumulator="compensated",
                       parallelism=f"split{world}: i-shards of {count} particles, all-gather "
                                   "of positions after every step",
                       l2=(f"flushed between timed steps ({args.flush_mib} MiB write)"
                           if args.flush_mib else "not flushed (profiling run)")),
        "fp32_peak_frac": rate * FLOP_PER_PAIR / world / (peak_tf * 1e12),
        "roofline": {"bound": "fp32", "achieved": achieved_tf, "peak": peak_tf,
                     "unit": "TFLOP/s", "frac": achieved_tf / peak_tf, "traffic": None,
                     "peak_source": "nominal: SMs x 128 FP32 lanes x 2 flop x max SM clock",
                     "note": "per rank, this rank's shard over the whole step (all-gather "
                             "included)"},
        "e2e": {"value": float(n) * n * e2e_steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": 6 * 4 * n, "d2h_bytes_per_step": 6 * 4 * n,
                "ms_per_step": e2e_s * 1e3 / e2e_steps},
        "gpu_launches": args.steps, "clocks": clk.summary(),
    }
    sim.close()
    return result


def traffic_from_profile():
    """DRAM bytes per launch of the force kernel from the committed ncu summary."""
    f = ROOT / "profiles" / "force_kernel_plummer_1M.txt"
    try:
        for line in f.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch_full_size:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def bench_render(sim, n) -> dict:
    """Headless render math (nb_sim_render) of the current state at 1920 x 1080."""
    import math

    import torch

    import nbody_gb300 as nb

    w, h = 1920, 1080
    view, proj = nb.camera_matrices(0.0, math.pi / 4, 8.0, w, h)
    img = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    for _ in range(3):
        sim.render(view, proj, w, h, img.data_ptr())
    sim.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream()
    t0.record(stream)
    for _ in range(10):
        sim.render(view, proj, w, h, img.data_ptr())
    t1.record(stream)
    torch.cuda.synchronize()
    return {"width": w, "height": h, "particles": n, "ms_per_frame": t0.elapsed_time(t1) / 10,
            "pipeline": "flare splat (additive) + half-res separable bloom + mean luminance + "
                        "tonemap, float32 RGBA"}


def bench_ensemble(args) -> dict:
    """The ensemble workload: 4,096 Plummer systems, sizes log-uniform in [64, 8192]."""
    import torch

    import nbody_gb300 as nb

    sizes = nb.ensemble_sizes(SEED, 4096, 64, 8192)
    parts = [nb.plummer(SEED + 1 + k, int(s)) for k, s in enumerate(sizes)]
    pos = [np.concatenate([q[0][c] for q in parts]) for c in range(3)]
    vel = [np.concatenate([q[1][c] for q in parts]) for c in range(3)]
    m = np.concatenate([q[2] for q in parts])
    p = nb.SimParam(G=1.0, dt=1e-3, damping=1.0, distEps=1e-3)
    sim = nb.Simulation(p, pos, vel, m, sizes=sizes)
    stream = torch.cuda.Stream()          # graphs are captured on a non-default stream
    sim.set_stream(stream.cuda_stream)
    chosen = sim.autotune()
    pairs = float(np.sum(sizes.astype(np.float64) ** 2))
    sim.advance(2)
    with torch.cuda.nvtx.range("ensemble_persistent"):   # ncu --nvtx-include target
        persistent_ms = sim.time_iterations(10) / 10
    sim.graph_capture(100)
    sim.graph_launch()
    sim.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    sim.graph_launch()                    # 100 steps
    t1.record(stream)
    t1.synchronize()
    graph_ms = t0.elapsed_time(t1) / 100
    # The baseline: one launch per system (the reference's stepSim launches one grid
    # for its one system), each planned with the shape the system gets as a
    # simulation of its own.  Also reported: every system with the ensemble's shape.
    iters = 10
    sim.advance_per_system(1)
    per_sys_ms = sim.time_iterations(iters, per_system=1) / iters
    sim.time_iterations(1, per_system=2)
    per_sys_same_ms = sim.time_iterations(iters, per_system=2) / iters
    info = sim.kernel_info()
    sim.close()
    return {"systems": int(len(sizes)), "particles": int(sizes.sum()), "pairs_per_step": pairs,
            "persistent_ms_per_step": persistent_ms, "graph_ms_per_step": graph_ms,
            "graph_steps_timed": 100,
            "per_system_launch_ms_per_step": per_sys_ms,
            "per_system_policy": "one launch per system, each with the kernel shape it gets "
                                 "as a simulation of its own (nb_sim_advance_per_system)",
            "per_system_steps_timed": iters,
            "speedup_vs_per_system_launches": per_sys_ms / graph_ms,
            "per_system_launch_ensemble_shape_ms_per_step": per_sys_same_ms,
            "speedup_vs_per_system_launches_ensemble_shape": per_sys_same_ms / graph_ms,
            "pair_interactions_per_s": pairs / (graph_ms * 1e-3), "autotuned_config": chosen,
            "kernel": info}


def bench_adjoint(args) -> dict:
    """The adjoint workload: N = 16,384 disk, T = 256 iterations, checkpoints every 16.  Forward
    and backward are both timed with CUDA events on the simulation's stream; the
    backward runs on device-resident gradients (nb_sim_adjoint_backward_device)."""
    import torch

    import nbody_gb300 as nb

    n, T, every, repeats = 16384, 256, 16, 3
    (x, y, z), (vx, vy, vz), m = nb.thin_disk(SEED, n, 1e-3)
    p = nb.SimParam(numParticles=n, G=1.0, dt=1e-3, damping=0.999, distEps=1e-3)
    sim = nb.Simulation(p, (x, y, z), (vx, vy, vz), m)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.advance(2)
    fwd = [sim.time_iterations(T) / T for _ in range(repeats)]
    sim.set_state((x, y, z), (vx, vy, vz))
    gx = torch.full((3 * n,), 1.0 / n, dtype=torch.float32, device="cuda")
    out = [torch.empty(3 * n, dtype=torch.float32, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    sim.adjoint_forward(T, every)
    sim.adjoint_backward_device(gx.data_ptr(), None, out[0].data_ptr(), out[1].data_ptr())
    sim.synchronize()                      # warm-up
    bwd = []
    for _ in range(repeats):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.adjoint_backward_device(gx.data_ptr(), None, out[0].data_ptr(), out[1].data_ptr())
        e1.record(stream)
        e1.synchronize()
        bwd.append(e0.elapsed_time(e1) / T)
    sim.synchronize()
    sim.close()
    fwd_ms, bwd_ms = statistics.median(fwd), statistics.median(bwd)
    return {"N": n, "T": T, "checkpoint_every": every, "repeats": repeats,
            "forward_ms_per_step": fwd_ms, "forward_ms_per_step_all": fwd,
            "backward_ms_per_step": bwd_ms, "backward_ms_per_step_all": bwd,
            "adjoint_step_cost_vs_forward": bwd_ms / fwd_ms,
            "note": "medians of CUDA-event times on the simulation's stream; backward = "
                    "recompute from checkpoints + VJP kernel per step, gradients resident "
                    "on the device"}


# --------------------------------------------------------------------------- precision study
def run_precision_study(args) -> dict:
    """The precision study: N = 262,144 two-disk collision, plain vs compensated vs reference-order
    (the reference kernel's own summation, bit for bit) FP32 accumulation.
    FP64 energy and momenta (GPU) and the force error against FP64 accelerations on
    sampled rows every `every` steps.  Damping is 1 so that energy is conserved by the
    dynamics and its drift measures the arithmetic."""
    import nbody_gb300 as nb

    n, steps, every, eps, dt = args.n if args.n != N_BENCH else 262144, args.study_steps, 10, \
        1e-3, 1e-3
    (x, y, z), (vx, vy, vz), m = nb.two_disks(SEED, n, eps)
    rows = np.linspace(0, n - 1, 2048).astype(np.uint64)
    out = {"study": "precision", "N": n, "steps": steps, "every": every, "eps2": eps, "dt": dt,
           "damping": 1.0, "G": 1.0, "seed": SEED, "rows_sampled": int(rows.size),
           "modes": {}}
    for name, acc in (("plain", nb.ACC_PLAIN), ("compensated", nb.ACC_COMPENSATED),
                      ("reference_order", nb.ACC_REFERENCE_ORDER)):
        p = nb.SimParam(numParticles=n, G=1.0, dt=dt, damping=1.0, distEps=eps, accumulator=acc)
        sim = nb.Simulation(p, (x, y, z), (vx, vy, vz), m)
        series = []
        t_diag = t_step = 0.0
        for k in range(0, steps + 1, every):
            if k:
                w = time.perf_counter()
                sim.advance(every)
                sim.synchronize()
                t_step += time.perf_counter() - w
            w = time.perf_counter()
            d = sim.diagnostics()
            a32 = sim.accelerations()
            a64 = sim.fp64_accelerations(rows)
            t_diag += time.perf_counter() - w
            g = np.stack([a[rows.astype(np.int64)].astype(np.float64) for a in a32])
            r = np.stack(a64)
            err = np.linalg.norm(g - r, axis=0)
            mag = np.linalg.norm(r, axis=0)
            series.append({"step": k, "energy": d["total"], "kinetic": d["kinetic"],
                           "potential": d["potential"], "momentum": d["momentum"],
                           "angular_momentum": d["angular_momentum"],
                           "force_rel_rms": float(np.sqrt(np.mean(err ** 2) / np.mean(mag ** 2))),
                           "force_rel_max": float(np.max(err / np.maximum(mag, 1e-30)))})
        e0 = series[0]["energy"]
        p0 = np.array(series[0]["momentum"])
        out["modes"][name] = {
            "max_rel_energy_drift": max(abs(s_["energy"] - e0) / abs(e0) for s_ in series),
            "final_rel_energy_drift": (series[-1]["energy"] - e0) / abs(e0),
            "max_momentum_drift": max(float(np.linalg.norm(np.array(s_["momentum"]) - p0))
                                      for s_ in series),
            "force_rel_rms_mean": float(np.mean([s_["force_rel_rms"] for s_ in series])),
            "force_rel_rms_max": float(np.max([s_["force_rel_rms"] for s_ in series])),
            "force_rel_max_max": float(np.max([s_["force_rel_max"] for s_ in series])),
            "seconds_stepping": t_step, "seconds_diagnostics": t_diag, "series": series}
        sim.close()
    return out


# --------------------------------------------------------------------------- accuracy study
def run_accuracy_study(args) -> dict:
    """Force error of every accumulator against FP64 for the initial state of each
    configuration: FP32 accelerations of the library vs GPU FP64 accelerations on
    strided rows (for the ensemble: rows spread over all systems)."""
    import nbody_gb300 as nb

    cases = []
    (x, y, z), (vx, vy, vz), m = nb.thin_disk(SEED, 25600, 1e-3)
    cases.append(("thin_disk_25600", [x, y, z], [vx, vy, vz], m, None, 1e-3))
    (x, y, z), (vx, vy, vz), m = nb.plummer(SEED, 1 << 20)
    cases.append(("plummer_1048576", [x, y, z], [vx, vy, vz], m, None, 1e-4))
    (x, y, z), (vx, vy, vz), m = nb.two_disks(SEED, 262144, 1e-3)
    cases.append(("two_disks_262144", [x, y, z], [vx, vy, vz], m, None, 1e-3))
    sizes = nb.ensemble_sizes(SEED, 4096, 64, 8192)
    parts = [nb.plummer(SEED + 1 + k, int(s_)) for k, s_ in enumerate(sizes)]
    cases.append(("ensemble_4096_systems",
                  [np.concatenate([q[0][c] for q in parts]) for c in range(3)],
                  [np.concatenate([q[1][c] for q in parts]) for c in range(3)],
                  np.concatenate([q[2] for q in parts]), sizes, 1e-3))
    (x, y, z), (vx, vy, vz), m = nb.thin_disk(SEED, 16384, 1e-3)
    cases.append(("adjoint_disk_16384", [x, y, z], [vx, vy, vz], m, None, 1e-3))
    out = {"study": "accuracy", "rows": 2048, "reference": "GPU FP64 all-pairs rows "
           "(nb_sim_fp64_accelerations), checked against the CPU FP64 oracle in the tests",
           "cases": {}}
    for name, pos, vel, m, sizes_, eps in cases:
        n = pos[0].size
        res = {"N": int(n), "eps2": eps}
        for acc_name, acc in (("plain", nb.ACC_PLAIN), ("compensated", nb.ACC_COMPENSATED),
                              ("reference_order", nb.ACC_REFERENCE_ORDER)):
            p = nb.SimParam(G=1.0, dt=1e-3, damping=1.0, distEps=eps, accumulator=acc,
                            numParticles=n)
            sim = nb.Simulation(p, pos, vel, m, sizes=sizes_)
            rms, mx, rows = force_error_vs_fp64(sim, n, 2048)
            res[acc_name] = {"force_rel_rms_vs_fp64": rms, "force_rel_max_vs_fp64": mx}
            sim.close()
        out["cases"][name] = res
    return out


# --------------------------------------------------------------------------- sizes study
def run_sizes_study(args) -> dict:
    """ms per step of the tuned kernel (compensated, default shape), of the
    reference-order kernel (default shape) and of the PREDICATED compatibility kernel
    from N = 2,048 to 1,048,576 (thin disks, eps2 = 1e-3), CUDA events,
    median of repeated launches."""
    import nbody_gb300 as nb

    out = {"study": "sizes", "eps2": 1e-3, "cases": {}}
    for n in (2048, 25600, 65536, 262144, 1 << 20):
        (x, y, z), (vx, vy, vz), m = nb.thin_disk(SEED, n, 1e-3)
        row = {}
        for name, acc, method in (("compensated", nb.ACC_COMPENSATED, nb.BRANCH),
                                  ("reference_order", nb.ACC_REFERENCE_ORDER, nb.BRANCH),
                                  ("predicated", nb.ACC_COMPENSATED, nb.PREDICATED)):
            p = nb.SimParam(numParticles=n, G=1.0, dt=1e-3, damping=1.0, distEps=1e-3,
                            accumulator=acc, calcMethod=method)
            with nb.Simulation(p, (x, y, z), (vx, vy, vz), m) as sim:
                reps = 20 if n <= 65536 else (5 if n <= 262144 else 3)
                sim.advance(2)
                times = [sim.time_iterations(1) for _ in range(reps)]
                row[name] = {"ms_per_step": statistics.median(times),
                             "pairs_per_s": float(n) * n / (statistics.median(times) * 1e-3),
                             "kernel": sim.kernel_info()}
        out["cases"][str(n)] = row
    return out


# --------------------------------------------------------------------------- reference arm
def run_reference(args, rank, world) -> dict | None:
    if rank != 0:
        return None
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_binding as orc

    n = args.n
    pos, vel, m = plummer_inputs_without_library(n)
    G = float(np.float32(m[0]))
    # size each step to ~ cpu_seconds / (steps + warmup) of work
    per_step_s = max(1.0, args.cpu_seconds * 2 / max(1, args.steps + args.warmup))
    rate0, rows, _, thr = cpu_sample_rate(pos, G, per_step_s)
    idx = np.linspace(0, n - 1, rows).astype(np.int64)
    for _ in range(args.warmup):
        orc.port_accel(pos, G, EPS2, rows=idx)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.port_accel(pos, G, EPS2, rows=idx)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = rows * n * args.steps / total
    sample = (f"{rows} strided i-rows x all {n} j-particles per step on {thr} threads; "
              f"{CPU_PORT_DESC}.  The reference ships no CPU path, and its SYCL twin needs a "
              "DPC++ toolchain that is absent here")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": total * 1e3 / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded Plummer sphere; the oracle's bit-identical restatement of "
                   "the library's generator)",
           "config": workload_desc(n),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": thr, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    if orc.reference_available() and not args.no_extras:
        try:
            zeros = [np.zeros(n, np.float32)] * 3
            orc.reference_run(pos, zeros, G, DT, 1.0, EPS2, 1, gw_size=128)  # warm-up
            launches = [orc.reference_run(pos, zeros, G, DT, 1.0, EPS2, 1, gw_size=128)[1]
                        for _ in range(5)]
            ms = statistics.median(launches)
            out["reference_cuda_kernel"] = {
                "value": float(n) * n / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
                "ms_per_launch_all": launches, "ms_spread": max(launches) - min(launches),
                "launches_timed": len(launches),
                "source": "src/simulator.cu particle_interaction<BRANCH> compiled unmodified "
                          "for sm_103a with -use_fast_math, gwSize 128; median of 5 single "
                          "launches, CUDA events"}
        except Exception as e:  # reported, not fatal
            out["reference_cuda_kernel"] = {"unavailable": str(e).splitlines()[0]}
    return out


def main() -> int:
    ap = argparse.ArgumentParser(description="GB300 n-body benchmark")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--n", type=int, default=N_BENCH,
                    help="particles (default: the 1,048,576-particle workload; smaller values "
                         "are for profiling only)")
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--split", action="store_true",
                    help="split the one system over the job's GPUs (strong scaling: shards of "
                         "particles, an all-gather of positions per step) instead of running "
                         "one replica per GPU")
    ap.add_argument("--study", choices=["precision", "accuracy", "ensemble", "sizes"],
                    default=None,
                    help="run a study instead of the benchmark (precision: the two-disk collision over time; "
                         "accuracy: force error vs FP64 of every workload, every accumulator; "
                         "ensemble: the 4,096-system ensemble leg alone, for profiling; "
                         "sizes: both kernels from N = 2,048 to 1M)")
    ap.add_argument("--study-steps", type=int, default=1000)
    ap.add_argument("--flush-mib", type=int, default=512,
                    help="L2 flush buffer written between timed steps (0: no flush; profiling)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--acc", choices=["auto", "plain", "compensated", "reference_order"],
                    default="auto",
                    help="accumulator(s) to measure; auto: all three, headline = the fastest of "
                         "those whose force error vs FP64 is <= 1e-5 relative RMS "
                         "(reference_order: the reference's own summation, bit-identical to "
                         "its kernel)")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP64 force-error check (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)  # at least 3 untimed warm-up steps
    if args.study == "precision":
        print(json.dumps(run_precision_study(args)), flush=True)
        return 0
    if args.study == "accuracy":
        print(json.dumps(run_accuracy_study(args)), flush=True)
        return 0
    if args.study == "ensemble":
        print(json.dumps(bench_ensemble(args)), flush=True)
        return 0
    if args.study == "sizes":
        print(json.dumps(run_sizes_study(args)), flush=True)
        return 0
    rank, world = dist_init()
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    elif args.split:
        res = run_split(args, rank, world)
    else:
        res = run_ours(args, rank, world)
    if rank == 0 and res is not None:
        # Libraries below Python (NCCL announces its version on stdout) write through C
        # stdio buffers: flush them first, so that the JSON line is the last line.
        import ctypes

        try:
            ctypes.CDLL(None).fflush(None)
        except (OSError, AttributeError):
            pass
        print(json.dumps(res), flush=True)
    dist = sys.modules.get("torch.distributed")
    if dist is not None and dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
