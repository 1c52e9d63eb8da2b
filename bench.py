"""Benchmark of the GB300 timestep: particle-steps/s on the 2-D production
workload (N = 1e7 particles, grid 128x128x1x32x1, box 40x40, Dt 0.1, Dr 1.0,
active stress -2, dt 0.005, 1 % sinusoidal density perturbation along x),
plain FP64 path (the headline `value`), with sections for the same FP64
mode with the update's increments in two-float arithmetic (f32x2), the FP32
mixed path (FP64 and fixed-point positions), the batched ensemble of 64 parameter
sets, the learned denoiser in the loop and the 3-D magnetic workload (2e7
particles, grid 64^3 x 16 x 8; FP64 and FP32 mixed).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--no-mixed] [--no-ensemble] [--no-denoise] [--no-c2] [--only SECTION]

One JSON line on stdout (rank 0).  --impl reference times the CPU path of the
same workload instead: the FP64 C restatement of the reference timestep
(oracle/), parallel like the reference (serial histogram and stress
contraction, parallel FFT components and particle loop) on all host threads.
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

METRIC_NAME = "particle-steps/s on 1 GB300 at fixed L2 field error vs FP64 oracle; plain vs denoised/FP32"
UNIT = "particle-steps/s"
GRID = (128, 128, 1, 32, 1)
BOX = (40.0, 40.0, 1.0)
N = 10_000_000
PARAMS = dict(timestep=0.005, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-2.0)
WORKLOAD = "2-D production size, plain FP64: N=1e7, grid 128x128x1x32x1, box 40x40, 1% sin(2 pi x/40) density"
TWOPI = 2 * np.pi


def workload_config(n):
    """The `config` object of the JSON line, identical in both arms."""
    return {"workload": WORKLOAD, "particles": n, "grid": list(GRID), "box": list(BOX), **PARAMS,
            "l2": "inputs larger than L2 (400 MB particle state per step)"}


E2E_MIN_STEPS = 20


def e2e_median(step, n, steps, world, dist):
    """End-to-end throughput from `steps` host-timed calls of step(k) (each
    synchronised), the median step time: returns (particle-steps/s,
    median ms, steps)."""
    import torch
    times = []
    for k in range(steps):
        t0 = time.perf_counter()
        step(k)
        torch.cuda.synchronize()
        times.append(1e3 * (time.perf_counter() - t0))
    med = statistics.median(times)
    value, ms = aggregate(med, n, 1, world, dist)
    return value, ms, steps


def c1_particles(n, seed=1):
    rng = np.random.default_rng(seed)
    L = BOX[0]
    u = rng.random(n)
    x = u * L
    for _ in range(30):
        f = x / L + 0.01 * (1 - np.cos(TWOPI * x / L)) / TWOPI - u
        x -= f / ((1 + 0.01 * np.sin(TWOPI * x / L)) / L)
    return np.column_stack([np.mod(x, L), BOX[1] * rng.random(n), np.zeros(n), TWOPI * rng.random(n),
                            np.full(n, np.pi / 2)])


def traffic_per_launch(key, n):
    """DRAM bytes per launch of a kernel at n particles, from the ncu
    figures in profiles/traffic.txt (bytes per particle, measured on a smaller
    case of the same workload); None when absent."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.txt")) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 2 and parts[0] == key:
                    return float(parts[1]) * n
    except OSError:
        pass
    return None


def fp64_per_particle(key):
    """FP64 thread-instructions (DFMA + DMUL + DADD) per particle of a kernel,
    from the ncu instruction counts in profiles/fp64_inst.txt; None when absent."""
    try:
        with open(os.path.join(ROOT, "profiles", "fp64_inst.txt")) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 2 and parts[0] == key:
                    return float(parts[1])
    except OSError:
        pass
    return None


def fp64_rate():
    """Measured FP64 FMA rate of this GPU (thread-FMAs/s, ss_fp64_rate probe)."""
    import ctypes

    from stochasticsampling_gb300 import _lib
    r = ctypes.c_double()
    _lib.check(_lib.load().ss_fp64_rate(ctypes.byref(r)))
    return r.value


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi clock sampling (every 20 ms) during the timed region: start()
    before the warm-up, mark() just before the timed region begins; stop()
    summarises the samples taken from the mark on (the last one before it
    when the region is shorter than one sampling interval)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        """Starts the sampler and returns once its first sample has arrived (at
        most 3 s), so that nvidia-smi's own start-up stays out of the timed
        region that follows."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def mark(self):
        self.first = len(self.lines)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        first = getattr(self, "first", 0)
        lines = self.lines[first:] if len(self.lines) > first else self.lines[max(0, first - 1):]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_step_rate(n, steps, nthreads, seed=1):
    """Time the oracle (the reference restatement) on n particles of the
    workload: returns (particle-steps/s, seconds)."""
    from oracle import oracle as O
    s = O.make_settings(GRID, BOX, timestep=PARAMS["timestep"], trans_diff=PARAMS["trans_diffusion"],
                        rot_diff=PARAMS["rot_diffusion"], active=PARAMS["stress_active"], quasi2d=True, seed=seed)
    sim = O.Simulation(s, n, nthreads=nthreads)
    sim.init(c1_particles(n, seed))
    sim.do_timestep()  # warm
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.do_timestep()
    dt = time.perf_counter() - t0
    return n * steps / dt, dt


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def run_reference(args, rank, world):
    """--impl reference: the CPU path of the workload on all host threads."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    nthreads = os.cpu_count() or 1
    # size the per-step sample so the whole run ends within a few minutes
    probe_n = 1_000_000
    rate, _ = cpu_step_rate(probe_n, 1, nthreads)
    budget_s = 150.0
    n_sample = int(min(N, max(100_000, rate * budget_s / max(1, args.steps + args.warmup))))
    # the whole workload per step whenever the budget allows it (the GPU arm's config)
    from oracle import oracle as O2
    s = O2.make_settings(GRID, BOX, timestep=PARAMS["timestep"], trans_diff=PARAMS["trans_diffusion"],
                         rot_diff=PARAMS["rot_diffusion"], active=PARAMS["stress_active"], quasi2d=True)
    sim = O2.Simulation(s, n_sample, nthreads=nthreads)
    sim.init(c1_particles(n_sample))
    for _ in range(args.warmup):
        sim.do_timestep()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.do_timestep()
    dt = time.perf_counter() - t0
    value = n_sample * args.steps / dt
    sample = (f"{n_sample} particles of the workload (grid 128x128x1x32x1) per step, {args.steps} timed steps "
              f"after {args.warmup} warm-up; FP64 C restatement of do_timestep on {nthreads} threads "
              f"({cpu_model()})")
    line = {
        "impl": "reference", "metric": METRIC_NAME, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n_sample),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def aggregate(ms_local, n_local, steps, world, dist):
    """Replicas: every rank steps its own n_local particles.  The job's time
    is the slowest rank's (max over ranks) and its throughput all particles
    of all ranks over that time.  Returns (particle-steps/s, ms)."""
    import torch
    t = torch.tensor([float(ms_local)], dtype=torch.float64)
    n = torch.tensor([float(n_local)], dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(n, op=dist.ReduceOp.SUM)
    ms = float(t[0])
    return float(n[0]) * steps / (ms / 1e3), ms


def measure_sorted(args, stream, p0, params, world, dist, barrier):
    """The same FP64 workload with the counting sort by cell each step."""
    import torch

    import stochasticsampling_gb300 as ss
    sim = ss.Simulation(grid=GRID, box=BOX, params=params, quasi2d=True, sort=True, stream=stream.cuda_stream)
    sim.init(p0)
    with torch.cuda.stream(stream):
        sim.run(args.warmup)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
    sim.close()
    value, ms_max = aggregate(ms, N, args.steps, world, dist)
    return {"value": value, "unit": UNIT, "ms_per_step": ms_max / args.steps}


def measure_f32x2(args, stream, p0, params, world, dist, barrier):
    """The same workload in the FP64 mode with SS_FLAG_F32X2 (the canonical
    update's increments in two-float arithmetic, the state in FP64):
    throughput over K graph-replayed steps, the update kernel's time from
    per-stage events and its HBM roofline, end to end through ss_step_host,
    and the largest deviation of x, y, phi from the FP64 mode after one step
    from identical state and noise."""
    import torch

    import stochasticsampling_gb300 as ss
    sim = ss.Simulation(grid=GRID, box=BOX, params=params, quasi2d=True, sort=False, f32x2=True,
                        stream=stream.cuda_stream)
    sim.init(p0)
    with torch.cuda.stream(stream):
        sim.run(args.warmup)
        torch.cuda.synchronize()
        barrier()
        l0 = sim.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
        launches = sim.launch_count() - l0
    value, ms_max = aggregate(ms, N, args.steps, world, dist)
    sim.profile(True)
    sim.run(args.steps)
    stage_ms, nprof = sim.profile_read()
    sim.profile(False)
    stage_avg = {k: v / max(1, nprof) for k, v in stage_ms.items()}
    # end to end: ss_step_host with pinned host rows, as the FP64 headline
    host_in = torch.empty((N, 5), dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty((N, 5), dtype=torch.float64, pin_memory=True).numpy()
    host_in[:] = sim.get_particles()
    for _ in range(2):
        sim.step_host(host_in, out=host_out)
    torch.cuda.synchronize()
    barrier()
    bufs = [host_in, host_out]

    def one(k):
        sim.step_host(bufs[k % 2], out=bufs[1 - k % 2])

    e2e, e2e_ms, e2e_steps = e2e_median(one, N, max(E2E_MIN_STEPS, min(args.steps, 50)), world, dist)
    # one step from identical state and noise in both modes
    state = sim.get_particles()
    ts = sim.get_timestep()
    ref = ss.Simulation(grid=GRID, box=BOX, params=params, quasi2d=True, sort=False, stream=stream.cuda_stream)
    dev = []
    for g in (sim, ref):
        g.resume(state, ts)
        g.do_timestep()
        dev.append(g.get_particles())
    ref.close()
    sim.close()
    d = np.abs(dev[0] - dev[1])
    d = np.minimum(d, np.array([BOX[0], BOX[1], BOX[2], 2 * np.pi, np.pi]) - d)
    gx, gy, gz, gp, gt = GRID
    ncell, nbins = gx * gy * gz, gx * gy * gz * gp * gt
    upd_bytes = N * (24 + 24 + 4 + 4 + 4) + ncell * 16 * 8 + nbins * 4
    upd_ms = stage_avg["update"]
    peak, peak_kind = peaks()
    achieved = upd_bytes / (upd_ms / 1e3) / 1e9
    return {"value": value, "unit": UNIT, "ms_per_step": ms_max / args.steps, "gpu_launches": launches,
            "dtype": "f64 state and sums, f32x2 increments",
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "kernel": "k_update (two-float canonical chain)",
                         "peak_source": peak_kind, "bytes_per_launch": upd_bytes, "avg_launch_ms": upd_ms},
            "stage_ms": stage_avg,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": N * 5 * 8, "d2h_bytes_per_step": N * 5 * 8,
                    "steps": e2e_steps, "median_ms_per_step": e2e_ms, "api": "ss_step_host, pinned"},
            "max_abs_dev_vs_fp64_one_step": {"x": float(d[:, 0].max()), "y": float(d[:, 1].max()),
                                             "phi": float(d[:, 3].max())}}


def measure_mixed(args, stream, p0, rank, world, dist, barrier, mode=True):
    """The FP32 mixed-precision path on the same workload: throughput over K
    graph-replayed steps, and each field's error against the FP64 path after
    one step from identical state and noise."""
    import torch

    import stochasticsampling_gb300 as ss
    params = dict(PARAMS, number_of_particles=N, seed=1 + rank)
    sim = ss.Simulation(grid=GRID, box=BOX, params=params, quasi2d=True, mixed=mode, stream=stream.cuda_stream)
    sim.init(p0)
    with torch.cuda.stream(stream):
        sim.run(args.warmup)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
    sim.profile(True)
    sim.run(min(args.steps, 20))
    stage_ms, nprof = sim.profile_read()
    sim.profile(False)
    value, ms_max = aggregate(ms, N, args.steps, world, dist)
    # errors against the FP64 path (itself within 1e-15 of the FP64 oracle)
    start = sim.get_particles()
    sim.close()
    m = ss.Simulation(grid=GRID, box=BOX, params=params, quasi2d=True, mixed=mode)
    d = ss.Simulation(grid=GRID, box=BOX, params=params, quasi2d=True)
    m.init(start)
    d.init(start)
    cm, cd = m.get_counts().astype(np.float64), d.get_counts().astype(np.float64)
    noise = m.noise(0)
    m.do_timestep()
    d.do_timestep(noise)
    um, ud = m.get_flow_field(), d.get_flow_field()
    pm, pd = m.get_particles(), d.get_particles()
    disp = np.linalg.norm((pd - start)[:, :2])
    dphi = np.abs(pm[:, 3] - pd[:, 3])
    dphi = np.minimum(dphi, 2 * np.pi - dphi)
    errors = {
        "histogram_l1_rel": float(np.abs(cm - cd).sum() / cd.sum()),
        "flow_l2_rel": float(np.linalg.norm(um - ud) / np.linalg.norm(ud)),
        "position_l2_rel_to_displacement": float(np.linalg.norm((pm - pd)[:, :2]) / disp),
        "phi_rms_rad": float(np.sqrt(np.mean(dphi ** 2))),
    }
    m.close()
    d.close()
    dtype = "f32 + 64-bit fixed-point positions" if mode == "fixed64" else "f32 + f64 positions"
    stage = {k: v / max(1, nprof) for k, v in stage_ms.items()}
    # k_update_m, algorithmic bytes per launch: x, y (8 B each), phi and the
    # cell key (4 B each) read and written; the table (16 floats per cell)
    # and the next histogram once
    gx, gy, gz, gp, gt = GRID
    upd_bytes = N * 48 + gx * gy * gz * 16 * 4 + gx * gy * gz * gp * gt * 4
    peak, peak_kind = peaks()
    achieved = upd_bytes / (stage["update"] / 1e3) / 1e9
    key = "k_update_m_fixed64_c1" if mode == "fixed64" else "k_update_m_c1"
    return {"value": value, "unit": UNIT, "ms_per_step": ms_max / args.steps, "dtype": dtype,
            "stage_ms": stage,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic_per_launch(key, N),
                         "kernel": "k_update_m", "peak_source": peak_kind, "bytes_per_launch": upd_bytes,
                         "avg_launch_ms": stage["update"]},
            "errors_vs_fp64_one_step": errors}


# the driver's loop with due outputs on the production workload: the
# distribution (4.2 MB) and the flow field (0.4 MB) every 10 steps, all
# particles (400 MB) every 100 steps, over 300 steps
OUT_STEPS = 300
OUT_EVERY = dict(distribution=10, flowfield=10, particles=100)


def measure_outputs(args, stream, p0, params):
    """run_simulation (src/bin/main.rs:139-289) on the production workload
    with an IO sink that drops the entries (the IO worker's compression runs
    on its own thread and is not timed): the overlapped hand-off
    (ss_output_begin into page-locked buffers, two outputs in flight)
    against the blocking getters into fresh arrays.  Wall time of the whole
    loop on the host, synchronised at both ends; each arm runs once untimed
    first over 30 steps with the particles every 10 (the overlapped arm's
    page-locked buffers, 2 x 405 MB, are allocated there and reused, as for
    a long run)."""
    import types

    import torch

    import stochasticsampling_gb300 as ss
    from stochasticsampling_gb300 import driver

    class Sink:
        def __init__(self):
            self.entries = 0

        def append(self, e):
            self.entries += 1

        def write_snapshot(self, snap):
            self.entries += 1

    def settings(steps, every):
        o = types.SimpleNamespace(initial_condition=False, final_snapshot=False, magneticfield=None,
                                  particles_head=None, snapshot=None, **every)
        return types.SimpleNamespace(simulation=types.SimpleNamespace(output_at_timestep=o,
                                                                      number_of_timesteps=steps - 1))

    res = {}
    for overlap in (False, True):
        sim = ss.Simulation(grid=GRID, box=BOX, params=params, quasi2d=True, sort=False, stream=stream.cuda_stream)
        sim.init(p0)
        with torch.cuda.stream(stream):
            sim.run(args.warmup)
            # untimed: every output kind in both slots (the buffers of the first use)
            driver.run_simulation(settings(30, dict(OUT_EVERY, particles=10)), sim, Sink(), overlap=overlap)
            sim.synchronize()
            sink = Sink()
            t0 = time.perf_counter()
            driver.run_simulation(settings(OUT_STEPS, OUT_EVERY), sim, sink, overlap=overlap)
            sim.synchronize()
            secs = time.perf_counter() - t0
        sim.close()
        res["overlapped" if overlap else "blocking"] = {
            "ms_per_step": secs * 1e3 / OUT_STEPS, "value": N * OUT_STEPS / secs, "unit": UNIT,
            "entries": sink.entries}
    res["steps"] = OUT_STEPS
    res["outputs"] = {k: f"every {v} steps" for k, v in OUT_EVERY.items()}
    res["d2h_bytes_per_100_steps"] = 10 * (GRID[0] * GRID[1] * GRID[3] + 3 * GRID[0] * GRID[1]) * 8 + N * 40
    res["timing"] = "host wall clock of the loop, synchronised at both ends"
    return res


# the reference's CPU-runnable 2-D case: box 10x10, grid 32x32x1x16x1,
# 1e5 particles (uniform positions and phi), Dt 0.1, Dr 0.5, active stress
# -1, dt 0.01, 100 steps, FP64
C0_GRID = (32, 32, 1, 16, 1)
C0_BOX = (10.0, 10.0, 1.0)
C0_N = 100_000
C0_STEPS = 100
C0_PARAMS = dict(timestep=0.01, trans_diffusion=0.1, rot_diffusion=0.5, stress_active=-1.0)


def measure_c0(stream, cpu=True):
    """The small 2-D workload in full (100 steps of 1e5 particles): the FP64
    GPU path (one CUDA graph per step) and, on the host cores, the oracle
    (the FP64 C restatement of the reference step, OpenMP like the reference's
    rayon loops)."""
    import torch

    import stochasticsampling_gb300 as ss
    rng = np.random.default_rng(4)
    p0 = np.column_stack([C0_BOX[0] * rng.random(C0_N), C0_BOX[1] * rng.random(C0_N), np.zeros(C0_N),
                          TWOPI * rng.random(C0_N), np.full(C0_N, np.pi / 2)])
    params = dict(C0_PARAMS, number_of_particles=C0_N, seed=1)
    sim = ss.Simulation(grid=C0_GRID, box=C0_BOX, params=params, quasi2d=True, sort=False, stream=stream.cuda_stream)
    sim.init(p0)
    with torch.cuda.stream(stream):
        sim.run(5)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run(C0_STEPS)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
    sim.close()
    out = {"workload": "2-D, box 10x10, grid 32x32x1x16x1, N=1e5, Dt 0.1, Dr 0.5, active -1, dt 0.01, 100 steps, FP64",
           "gpu": {"value": C0_N * C0_STEPS / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / C0_STEPS,
                   "note": "latency-bound small kernels: the 32x32 transforms and k space take about 53 us of the step"}}
    if cpu:
        from oracle import oracle as O
        nthreads = os.cpu_count() or 1
        st = O.make_settings(C0_GRID, C0_BOX, timestep=C0_PARAMS["timestep"], trans_diff=C0_PARAMS["trans_diffusion"],
                             rot_diff=C0_PARAMS["rot_diffusion"], active=C0_PARAMS["stress_active"], quasi2d=True,
                             seed=1)
        o = O.Simulation(st, C0_N, nthreads=nthreads)
        o.init(p0)
        t0 = time.perf_counter()
        for _ in range(C0_STEPS):
            o.do_timestep()
        secs = time.perf_counter() - t0
        out["cpu"] = {"value": C0_N * C0_STEPS / secs, "unit": UNIT, "ms_per_step": 1e3 * secs / C0_STEPS,
                      "cores": nthreads, "kind": "port",
                      "sample": f"all {C0_STEPS} steps, FP64 C restatement of do_timestep, OpenMP on {nthreads} "
                                f"threads ({cpu_model()})"}
    return out


# 3-D workload with the dipolar solver: box 20^3, grid 64x64x64x16x8,
# 2e7 particles (uniform positions, orientations uniform on the sphere),
# dipolar coupling 0.5, external field 1 (along the reference's field axis),
# active stress -1, Dt 0.1, Dr 1.0, dt 0.002
C2_GRID = (64, 64, 64, 16, 8)
C2_BOX = (20.0, 20.0, 20.0)
C2_N = 20_000_000
C2_PARAMS = dict(timestep=0.002, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-1.0,
                 magnetic_reorientation=1.0, magnetic_dipole_dipole=0.5)


def c2_particles(n, seed=3):
    rng = np.random.default_rng(seed)
    return np.column_stack([C2_BOX[0] * rng.random(n), C2_BOX[1] * rng.random(n), C2_BOX[2] * rng.random(n),
                            TWOPI * rng.random(n), np.arccos(1 - 2 * rng.random(n))])


def measure_c2(args, stream, rank, world, dist, barrier):
    """The 3-D magnetic workload: the plain FP64 path, the FP64 mode with
    two-float increments (SS_FLAG_F32X2) and the FP32 mixed path (FP64
    positions), each over graph-replayed steps; the mixed path's errors per
    field and the two-float mode's largest deviations against the FP64 path
    after one step from identical state and noise."""
    import torch

    import stochasticsampling_gb300 as ss
    n = C2_N if not args.particles else max(1, args.particles * 2)
    steps = max(1, min(args.steps, 20))
    params = dict(C2_PARAMS, number_of_particles=n, seed=5 + rank)
    p0 = c2_particles(n, seed=3 + rank)
    out = {"workload": "3-D with the dipolar solver: box 20^3, grid 64x64x64x16x8, uniform positions and "
                       "orientations on the sphere, dipolar coupling 0.5, external field 1, active stress -1, "
                       "Dt 0.1, Dr 1.0, dt 0.002", "particles": n, "steps": steps}
    for name, mode, f32x2 in (("fp64", False, False), ("f32x2", False, True), ("mixed", True, False)):
        # rows counting-sorted by cell at init keep their locality over these steps: no per-step sort
        sim = ss.Simulation(grid=C2_GRID, box=C2_BOX, params=params, mixed=mode, sort=False, f32x2=f32x2,
                            stream=stream.cuda_stream)
        sim.init(p0)
        with torch.cuda.stream(stream):
            sim.run(args.warmup)
            torch.cuda.synchronize()
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sim.run(steps)
            e1.record(stream)
            torch.cuda.synchronize()
            barrier()
            ms = e0.elapsed_time(e1)
        sim.profile(True)
        sim.run(min(steps, 5))
        stage_ms, nprof = sim.profile_read()
        sim.profile(False)
        sim.close()
        value, ms_max = aggregate(ms, n, steps, world, dist)
        out[name] = {"value": value, "unit": UNIT, "ms_per_step": ms_max / steps,
                     "dtype": "f32 + f64 positions" if mode else
                     ("f64 state and sums, f32x2 increments" if f32x2 else "f64"),
                     "stage_ms": {k: v / max(1, nprof) for k, v in stage_ms.items()}}
    m = ss.Simulation(grid=C2_GRID, box=C2_BOX, params=params, mixed=True)
    d = ss.Simulation(grid=C2_GRID, box=C2_BOX, params=params)
    f = ss.Simulation(grid=C2_GRID, box=C2_BOX, params=params, f32x2=True)
    m.init(p0)
    d.init(p0)
    f.init(p0)
    cm, cd = m.get_counts().astype(np.float64), d.get_counts().astype(np.float64)
    noise = m.noise(0)
    m.do_timestep()
    d.do_timestep(noise)
    f.do_timestep(noise)
    pf, pd0 = f.get_particles(), d.get_particles()
    df = np.abs(pf - pd0)
    df[:, 3] = np.minimum(df[:, 3], 2 * np.pi - df[:, 3]) * np.sin(pd0[:, 4])
    out["f32x2"]["max_abs_dev_vs_fp64_one_step"] = {
        "position": float(df[:, :3].max()), "theta": float(df[:, 4].max()),
        "phi_times_sin_theta": float(df[:, 3].max())}
    f.close()
    um, ud = m.get_flow_field(), d.get_flow_field()
    bm, bd = m.get_magnetic_field(), d.get_magnetic_field()
    pm, pd = m.get_particles(), d.get_particles()
    disp = np.linalg.norm(pd[:, :3] - p0[:, :3])
    ang = np.abs(pm[:, 3] - pd[:, 3])
    ang = np.minimum(ang, 2 * np.pi - ang)
    out["mixed"]["errors_vs_fp64_one_step"] = {
        "histogram_l1_rel": float(np.abs(cm - cd).sum() / cd.sum()),
        "flow_l2_rel": float(np.linalg.norm(um - ud) / np.linalg.norm(ud)),
        "magnetic_l2_rel": float(np.linalg.norm(bm - bd) / np.linalg.norm(bd)),
        "position_l2_rel_to_displacement": float(np.linalg.norm((pm - pd)[:, :3]) / disp),
        "phi_rms_rad": float(np.sqrt(np.mean(ang ** 2))),
        "theta_rms_rad": float(np.sqrt(np.mean((pm[:, 4] - pd[:, 4]) ** 2))),
    }
    m.close()
    d.close()
    return out


def measure_ensemble(args, stream, rank, world, dist, barrier):
    """The batched ensemble: 64 independent 2-D simulations (particle counts
    log-uniform in [50k, 2M], grid edges {32, 64, 128}, 16 or 32 phi bins,
    active stress uniform in [-3, 0], own Philox seed each) stepped by one
    CUDA graph per step; against the same members as 64 separate mixed
    contexts stepped one after the other."""
    import torch

    import stochasticsampling_gb300 as ss
    from stochasticsampling_gb300.ensemble import parameter_scan, uniform_particles
    members = parameter_scan(args.ensemble_members, seed=1 + rank)
    rows = uniform_particles(members, seed=2 + rank)
    ntot = int(rows.shape[0])
    ens = ss.Ensemble(members, stream=stream.cuda_stream)
    ens.init(rows)
    t0 = time.perf_counter()
    if args.ensemble_config:
        cfg = tuple(int(v) for v in args.ensemble_config.split(","))
        ens.set_config(cfg)
    else:
        cfg = ens.autotune()
    tune_s = time.perf_counter() - t0
    steps = args.steps
    with torch.cuda.stream(stream):
        ens.run(args.warmup)
        torch.cuda.synchronize()
        barrier()
        _, _, l0 = ens.info()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ens.run(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
        _, groups, l1 = ens.info()
    ens.close()
    value, ms_max = aggregate(ms, ntot, steps, world, dist)
    # the same members as separate contexts, one after the other per step
    sep_steps = max(3, min(steps, 20))
    off = np.cumsum([0] + [m["params"]["number_of_particles"] for m in members])
    sims = []
    for i, m in enumerate(members):
        s_ = ss.Simulation(grid=m["grid"], box=m["box"], params=m["params"], quasi2d=True, mixed=True,
                           stream=stream.cuda_stream)
        s_.init(rows[off[i]:off[i + 1]])
        sims.append(s_)
    with torch.cuda.stream(stream):
        for s_ in sims:
            s_.run(args.warmup)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(sep_steps):
            for s_ in sims:
                s_.run(1)
        e1.record(stream)
        torch.cuda.synchronize()
        sep_ms = e0.elapsed_time(e1) / sep_steps
    for s_ in sims:
        s_.close()
    nbins = sum(m["grid"][0] * m["grid"][1] * m["grid"][3] for m in members)
    ncell = sum(m["grid"][0] * m["grid"][1] for m in members)
    # algorithmic bytes per step: particles x, y (f64), phi, cell key (f32/u32)
    # read and written; both histograms (zero, count, contract read); 9 + 12
    # complex FP32 spectra read and written by the FFTs and their neighbours;
    # the table (16 floats per cell) written and read
    step_bytes = ntot * 48 + nbins * 12 + ncell * 21 * 8 * 4 + ncell * 16 * 4 * 2
    ns = [m["params"]["number_of_particles"] for m in members]
    return {"value": value, "unit": UNIT, "ms_per_step": ms_max / steps, "steps": steps,
            "dtype": "f32 + f64 positions",
            "workload": "64 independent 2-D simulations, N log-uniform in [50k, 2M], grid edge in {32, 64, 128}, "
                        "16 or 32 phi bins, box edge = 0.3125 x grid edge, active stress U[-3, 0], Dt 0.1, Dr 1.0, "
                        "dt 0.005, own Philox seed per member",
            "particles": ntot, "particles_min_max": [min(ns), max(ns)], "grid_shapes": groups,
            "autotune": {"threads": cfg[0], "blocks_per_sm": cfg[1], "particles_per_unit": cfg[2],
                         "seconds": tune_s},
            "gpu_launches_per_step": (l1 - l0) / steps,
            "step_algorithmic_bytes": step_bytes,
            "step_achieved_gbs": step_bytes / (ms_max / steps / 1e3) / 1e9,
            "separate_contexts": {"ms_per_step": sep_ms, "value": ntot / (sep_ms / 1e3),
                                  "note": "the same 64 members as SS_FLAG_MIXED contexts, each graph-stepped, "
                                          "one after the other"}}


def measure_denoised(args, rank):
    """The learned denoiser in the loop: trained on pairs (1e6-particle
    histogram, independent 6.4e7-particle histogram) of the workload's
    initial-condition family, then run for a number of steps beside plain
    FP64 runs and a 6.4e7-particle FP64 reference from independent samples of
    the workload's initial condition; errors of the distribution and flow
    field against the reference, and the plain FP64 cost of the denoised
    run's error."""
    from stochasticsampling_gb300 import denoise_eval as de
    dn, info = de.train_denoiser(pairs=args.denoise_pairs, epochs=args.denoise_epochs, seed=rank)
    res = de.evaluate(dn, steps=args.denoise_steps, every=max(1, args.denoise_steps // 4), seed=10 + rank)
    dn.close()
    ms = res["ms_per_step"]["denoised"]
    return {"value": res["n_low"] / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "dtype": "f32 step (fixed-point positions) + bf16 tensor-core CNN (fp32 accumulation)",
            "particles": res["n_low"], "cnn_ms_per_step": ms - res["ms_per_step"]["fp32_plain"],
            "training": {k: v for k, v in info.items() if k != "history"} | {"history": info["history"]},
            "steps": res["steps"], "mean_errors_vs_64M_fp64": res["mean_errors"],
            "plain_fp64_ms_per_step": {k: v for k, v in res["ms_per_step"].items() if k.startswith("plain") or k == "ref"},
            "equal_error_cost": {"distribution": res["dist_fit"], "flow": res["flow_fit"]}}


def run_gpu(args, rank, world, dist):
    import torch

    import stochasticsampling_gb300 as ss

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    params = dict(PARAMS, number_of_particles=N, seed=1 + rank)
    p0 = c1_particles(N, seed=1 + rank)

    def barrier():
        if dist is not None:
            dist.barrier()

    if args.only:
        if args.only == "ensemble":
            res = measure_ensemble(args, stream, rank, world, dist, barrier)
        elif args.only == "c2":
            res = measure_c2(args, stream, rank, world, dist, barrier)
        elif args.only == "denoised":
            res = measure_denoised(args, rank)
        elif args.only == "c0":
            res = measure_c0(stream, cpu=rank == 0)
        elif args.only == "f32x2":
            res = measure_f32x2(args, stream, p0, params, world, dist, barrier)
        elif args.only == "outputs":
            res = measure_outputs(args, stream, p0, params)
        else:
            res = measure_mixed(args, stream, p0, rank, world, dist, barrier,
                                "fixed64" if args.only == "fixed64" else True)
        if rank == 0:
            print(json.dumps({"section": args.only, **res}), flush=True)
        return
    # the counting sort by cell is off: the FP64 update is FP64-issue bound on
    # GB300, so the sort's locality saves nothing and its pass costs 0.2 ms
    # per step (the sorted step is measured below, as "sorted")
    sim = ss.Simulation(grid=GRID, box=BOX, params=params, quasi2d=True, sort=False, stream=stream.cuda_stream)
    sim.init(p0)

    with torch.cuda.stream(stream):
        clocks = Clocks(local)
        clocks.start()  # (its start-up stays ahead of the warm-up)
        sim.run(args.warmup)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        l0 = sim.launch_count()
        clocks.mark()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        clk = clocks.stop()
        ms = e0.elapsed_time(e1)
        launches = sim.launch_count() - l0
    sim.synchronize()
    value, ms_max = aggregate(ms, N, args.steps, world, dist)
    sorted_line = measure_sorted(args, stream, p0, params, world, dist, barrier)

    # per-stage CUDA events over K direct-launch steps (same stream, same
    # workload), each step on its own: the median per stage, so that a step
    # delayed on the shared host cores (direct launches are enqueued one by
    # one) does not move the figures
    per_step = []
    for _ in range(args.steps):
        sim.profile(True)
        sim.run(1)
        st, k = sim.profile_read()
        per_step.append({name: v / max(1, k) for name, v in st.items()})
    sim.profile(False)
    stage_avg = {name: statistics.median(r[name] for r in per_step) for name in per_step[0]}

    # end to end through the C ABI with pinned host buffers: per step the host
    # particle array goes in, the step runs, the particles come out.  The
    # headline uses ss_step_host (one call, read-back overlapping the chunked
    # update); the same loop over ss_resume + ss_do_timestep +
    # ss_get_particles is reported beside it.
    host_in = torch.empty((N, 5), dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty((N, 5), dtype=torch.float64, pin_memory=True).numpy()
    host_in[:] = sim.get_particles()
    e2e_steps = max(E2E_MIN_STEPS, min(args.steps, 50))

    def e2e_loop(fused):
        nonlocal host_in, host_out

        def one(k0):
            if fused:
                sim.step_host(host_in, out=host_out)
            else:
                sim.resume(host_in, k0)
                sim.do_timestep()
                sim.get_particles(out=host_out)

        # untimed warm-up steps: the first launch of each kernel loads it
        for _ in range(2):
            one(sim.get_timestep())
        ts = sim.get_timestep()
        torch.cuda.synchronize()
        barrier()

        def timed(k):
            nonlocal host_in, host_out
            one(ts + k)
            host_in, host_out = host_out, host_in

        return e2e_median(timed, N, e2e_steps, world, dist)

    e2e_sep, e2e_sep_ms, _ = e2e_loop(False)
    e2e_value, e2e_ms, _ = e2e_loop(True)
    sim.close()
    f32x2 = measure_f32x2(args, stream, p0, params, world, dist, barrier)
    mixed = None if args.no_mixed else measure_mixed(args, stream, p0, rank, world, dist, barrier)
    mixed_fixed = None if args.no_mixed else measure_mixed(args, stream, p0, rank, world, dist, barrier, "fixed64")
    ensemble = None if args.no_ensemble else measure_ensemble(args, stream, rank, world, dist, barrier)
    c2 = None if args.no_c2 else measure_c2(args, stream, rank, world, dist, barrier)
    denoised = None if args.no_denoise else measure_denoised(args, rank)
    c0 = measure_c0(stream, cpu=(rank == 0 and not args.no_cpu_baseline))
    outputs = measure_outputs(args, stream, p0, params)

    if rank != 0:
        return
    peak, peak_kind = peaks()
    gx, gy, gz, gp, gt = GRID
    ncell, nbins = gx * gy * gz, gx * gy * gz * gp * gt
    # update kernel (the canonical quasi-2-D variant: every particle holds
    # z = 0, theta = pi/2, which it neither reads nor writes), algorithmic
    # bytes per launch: x, y, phi read + written (3 f64), cell key read +
    # written, particle id read, the field table once, the next histogram
    # once (u32)
    upd_bytes = N * (24 + 24 + 4 + 4 + 4) + ncell * 16 * 8 + nbins * 4
    upd_ms = stage_avg["update"]
    achieved = upd_bytes / (upd_ms / 1e3) / 1e9
    # whole step, algorithmic bytes: particles 80 B, histogram 12 B
    # per bin, 21 FFT components read+written as 16 B complex, field table
    step_bytes = N * 80 + nbins * 12 + ncell * 16 * 2 * 21 + ncell * 13 * 8
    traffic = traffic_per_launch("k_update_c1", N)
    # the bound of k_update on GB300: FP64 issue (instructions from ncu)
    inst = fp64_per_particle("k_update_c1")
    rate = fp64_rate()
    fp64_roof = {"bound": "fp64", "achieved": inst * N / (upd_ms / 1e3) if inst else None, "peak": rate,
                 "unit": "FP64 thread-instructions/s",
                 "frac": inst * N / (upd_ms / 1e3) / rate if inst else None,
                 "instructions_per_particle": inst,
                 "peak_source": "ss_fp64_rate: independent FMA chains on every SM, measured in this run",
                 "instructions_source": "DFMA + DMUL + DADD per particle, ncu (profiles/fp64_inst.txt)"}
    cpu = None
    if not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        n_cpu = N
        rate, secs = cpu_step_rate(1_000_000, 1, nthreads)
        steps_cpu = max(2, min(10, int(20.0 / max(1e-9, N / rate))))
        if N / rate * steps_cpu > 40:
            n_cpu = int(rate * 20 / steps_cpu)
        v, secs = cpu_step_rate(n_cpu, steps_cpu, nthreads)
        cpu = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"{steps_cpu} steps of {n_cpu} particles of the workload, FP64 C restatement of "
                         f"do_timestep, OpenMP on {nthreads} threads ({cpu_model()}), {secs:.1f} s"}
    line = {
        "metric": METRIC_NAME, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(N),
        "execution": {"noise": "on-device Philox4x32-10",
                      "graph": "CUDA graph per step, particles in input order (no counting sort)",
                      "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "k_update (fused Langevin step + next-step binning)",
                     "peak_source": peak_kind, "bytes_per_launch": upd_bytes, "avg_launch_ms": upd_ms,
                     "note": "FP64-issue bound on GB300 (low FP64 rate); HBM fraction reported as required"},
        "fp64_roofline": fp64_roof,
        "step_roofline": {"algorithmic_bytes": step_bytes,
                          "achieved_gbs": step_bytes / (ms_max / args.steps / 1e3) / 1e9},
        "stage_ms": stage_avg,
        "sorted": sorted_line,
        "f32x2": f32x2,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": N * 5 * 8, "d2h_bytes_per_step": N * 5 * 8,
                "steps": e2e_steps, "median_ms_per_step": e2e_ms,
                "timing": "each step timed on the host (synchronised), median of the steps",
                "api": "ss_step_host(host rows in, host rows out), pinned",
                "separate_calls": {"value": e2e_sep, "median_ms_per_step": e2e_sep_ms,
                                   "api": "ss_resume(host) + ss_do_timestep + ss_get_particles(host)"}},
        "gpu_launches": launches,
        "clocks": clk,
        "cpu_baseline": cpu,
        "mixed": mixed,
        "mixed_fixed64": mixed_fixed,
        "ensemble": ensemble,
        "c2_3d_magnetic": c2,
        "c0_small_2d": c0,
        "driver_outputs": outputs,
        "denoised": denoised,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the FP32 mixed-precision measurement")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--no-denoise", action="store_true", help="skip the learned-denoiser measurement")
    ap.add_argument("--no-c2", action="store_true", help="skip the 3-D magnetic measurement")
    ap.add_argument("--denoise-pairs", type=int, default=1000)
    ap.add_argument("--denoise-epochs", type=int, default=6)
    ap.add_argument("--denoise-steps", type=int, default=400)
    ap.add_argument("--only", choices=["mixed", "fixed64", "ensemble", "denoised", "c2", "f32x2", "c0", "outputs"], default=None,
                    help="run one section alone (a smaller command for profiling); prints its JSON")
    ap.add_argument("--ensemble-members", type=int, default=64)
    ap.add_argument("--ensemble-config", default=None,
                    help="threads,blocks_per_sm,unit,plan of the ensemble update instead of autotuning")
    ap.add_argument("--particles", type=int, default=None,
                    help="override N (profiling a smaller case of the same workload)")
    args = ap.parse_args()
    if args.particles:
        global N
        N = args.particles
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_gpu(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
