"""Train the histogram denoiser on pairs the method generates and evaluate it
in the loop of the production workload (2-D, grid 128x128x1x32x1, box
40x40, Dt 0.1, Dr 1.0, active stress -2, dt 0.005).

    python -m stochasticsampling_gb300.denoise_eval [--pairs 4000] [--epochs 2] [--steps 2000]
                                                    [--moment-weight 16]

Training: pairs (histogram of n_in = 1e6 particles, independent histogram of
n_target - n_in = 63e6 particles) that the method generates: snapshots along
plain FP64 runs of n_target = 64e6 particles from initial conditions of the
workload's family (perturbation amplitude uniform in [0, 5 %], random phase
and axis), each snapshot split into 64 disjoint 1e6-particle sets
(method_pairs).  The loss adds to the mean-square error the second angular
harmonic of the residual per cell, the part of the error that reaches the
flow (ss_dn_set_loss).

Evaluation: independent samples of the workload's initial condition (1 %
sinusoidal density along x) run side by side -- a plain FP64 reference with
64e6 particles, plain FP64 runs with 1e6, 4e6 and 1.6e7 particles, and the
FP32 (fixed-point positions) run with 1e6 particles and the denoiser in the
loop.  Every `every` steps the L2 errors of the distribution (histogram /
mean count; for the denoised run the network's output) and of the flow field
against the reference are recorded, and the flow's size relative to the
reference's (the workload's infinite-N flow is zero: its orientations stay
isotropic).  The particle-steps cost of reaching the
denoised run's error with the plain FP64 path follows from the plain runs'
errors (error^2 = a / N + b) and their measured step times.
"""
import argparse
import json
import time

import numpy as np

GRID = (128, 128, 1, 32, 1)
BOX = (40.0, 40.0, 1.0)
PARAMS = dict(timestep=0.005, trans_diffusion=0.1, rot_diffusion=1.0, stress_active=-2.0)
SHAPE = (GRID[0], GRID[1], GRID[3])


def initial_rows(n, amp=0.01, seed=1, phase=0.0, axis=0, out=None):
    """n particles of the workload's initial-condition family: density
    1 + amp sin(2 pi s / L + phase) along `axis` (0: x, 1: y; inverse CDF by
    Newton), uniform along the other axis and in phi.  Large n is drawn in
    chunks of 2^22 rows on a thread pool (numpy releases the interpreter lock
    inside its array loops), chunk k from its own stream (seed, k)."""
    from concurrent.futures import ThreadPoolExecutor
    rows = np.empty((n, 5)) if out is None else out
    L = BOX[axis]
    w = 2 * np.pi / L
    chunk = 1 << 22

    def fill(k):
        lo, hi = k * chunk, min(n, (k + 1) * chunk)
        rng = np.random.default_rng([seed, k]) if n > chunk else np.random.default_rng(seed)
        m = hi - lo
        u = rng.random(m)
        s = u * L
        for _ in range(8):
            f = s / L + amp * (np.cos(phase) - np.cos(w * s + phase)) / (2 * np.pi) - u
            s -= f / ((1 + amp * np.sin(w * s + phase)) / L)
        r = rows[lo:hi]
        r[:, axis] = np.mod(s, L)
        r[:, 1 - axis] = BOX[1 - axis] * rng.random(m)
        r[:, 2] = 0.0
        r[:, 3] = 2 * np.pi * rng.random(m)
        r[:, 4] = np.pi / 2

    nchunks = -(-n // chunk)
    if nchunks == 1:
        fill(0)
    else:
        import os
        with ThreadPoolExecutor(max_workers=min(nchunks, os.cpu_count() or 1)) as ex:
            list(ex.map(fill, range(nchunks)))
    return rows


def _subset_counts(lib, rows_dev, first, count, den_over_vol, out_dist):
    """Counts per bin of rows first .. first + count of a device particle
    array [n][5] (ss_sample_distribution_noalloc gives (c / D) V; c is
    recovered exactly by rounding c = dist * D / V)."""
    import ctypes

    import torch

    from . import _lib
    g, b = _lib.Grid(*GRID), _lib.Box(*BOX)
    ptr = rows_dev.data_ptr() + 5 * 8 * int(first)
    _lib.check(lib.ss_sample_distribution_noalloc(ctypes.byref(g), ctypes.byref(b), ctypes.c_void_p(ptr), int(count),
                                                  ctypes.c_void_p(out_dist.data_ptr()), None))
    torch.cuda.synchronize()
    return torch.round(out_dist * (den_over_vol * count))


def method_pairs(npairs, n_in=1_000_000, n_target=64_000_000, amp_max=0.05, steps=2000, snapshots=8, seed=0):
    """Training pairs the method itself generates.  Runs of the plain FP64
    path with n_target particles start from the workload's initial-condition
    family (density 1 + amp sin along x or y, amp uniform in [0, amp_max],
    random phase; uniform orientations) and are stepped for `steps` steps;
    `snapshots` states along each run, evenly spaced from step 0, give pairs:
    the particles of a snapshot are split into disjoint sets of n_in (by
    caller index; the rows are independent draws), and each set's histogram
    (the input) is paired with the histogram of the snapshot's other
    n_target - n_in particles (the target, independent of the input).  Both
    are normalised to mean 1.  Returns (inputs, targets, info): CUDA float
    tensors [npairs, *SHAPE]."""
    import torch

    import stochasticsampling_gb300 as ss
    from . import _lib
    lib = _lib.load()
    per_snap = n_target // n_in
    nruns = max(1, -(-npairs // (per_snap * snapshots)))
    X = torch.empty((npairs, *SHAPE), device="cuda", dtype=torch.float32)
    T = torch.empty_like(X)
    nbins = int(np.prod(SHAPE))
    gw = [BOX[0] / GRID[0], BOX[1] / GRID[1], BOX[2] / GRID[2], 2 * np.pi / GRID[3], np.pi / GRID[4]]
    den_over_vol = gw[0] * gw[1] * gw[2] * gw[3] * gw[4] / (BOX[0] * BOX[1] * BOX[2])  # D / (V n)
    dist = torch.empty(nbins, device="cuda", dtype=torch.float64)
    rng = np.random.default_rng(seed)
    every = max(1, steps // snapshots)
    k = 0
    t_sim = 0.0
    # one pinned host buffer and one device buffer for every snapshot's rows
    host = torch.empty((n_target, 5), dtype=torch.float64, pin_memory=True)
    dev = torch.empty((n_target, 5), dtype=torch.float64, device="cuda")
    for run in range(nruns):
        amp, phase, axis = rng.uniform(0.0, amp_max), rng.uniform(0.0, 2 * np.pi), int(rng.integers(2))
        rows = initial_rows(n_target, amp=amp, seed=int(rng.integers(1 << 31)), phase=phase, axis=axis,
                            out=host.numpy())
        p = dict(PARAMS, number_of_particles=n_target, seed=int(rng.integers(1 << 31)))
        sim = ss.Simulation(grid=GRID, box=BOX, params=p, quasi2d=True, sort=False)
        sim.init(rows)
        for snap in range(snapshots):
            if k >= npairs:
                break
            if snap:
                t0 = time.perf_counter()
                sim.run(every)
                sim.synchronize()
                t_sim += time.perf_counter() - t0
            sim.get_particles(out=host.numpy())
            dev.copy_(host)
            full = _subset_counts(lib, dev, 0, n_target, den_over_vol, dist)
            for j in range(per_snap):
                if k >= npairs:
                    break
                c = _subset_counts(lib, dev, j * n_in, n_in, den_over_vol, dist)
                X[k] = (c * (nbins / n_in)).float().reshape(SHAPE)
                T[k] = ((full - c) * (nbins / (n_target - n_in))).float().reshape(SHAPE)
                k += 1
        sim.close()
    del host, dev
    torch.cuda.synchronize()
    info = {"runs": nruns, "snapshots_per_run": snapshots, "steps_between_snapshots": every,
            "pairs_per_snapshot": per_snap, "simulation_seconds": t_sim}
    return X, T, info


def train_denoiser(pairs=4000, epochs=2, batch=8, lr=1e-3, n_in=1_000_000, n_target=64_000_000, seed=0,
                   val_pairs=64, steps=2000, snapshots=8, moment_weight=16.0):
    import torch

    from .denoiser import Denoiser, train
    t0 = time.perf_counter()
    X, T, gen = method_pairs(pairs, n_in, n_target, steps=steps, snapshots=snapshots, seed=seed)
    # validation: one snapshot of an independent run, midway through it
    Xv, Tv, _ = method_pairs(val_pairs, n_in, n_target, steps=steps // 2, snapshots=2, seed=seed + 1000)
    t_data = time.perf_counter() - t0
    dn = Denoiser(SHAPE, seed=seed)
    dn.set_loss(moment_weight)
    base = loss_of(Xv, Tv, moment_weight)
    start = dn.loss(Xv, Tv)
    t0 = time.perf_counter()
    hist = train(dn, X, T, epochs=epochs, batch=batch, lr=lr, seed=seed, val=(Xv, Tv))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del X, T
    info = {"pairs": pairs, "epochs": epochs, "batch": batch, "lr": lr, "n_in": n_in, "n_target": n_target,
            "generation": gen, "moment_weight": moment_weight,
            "data_seconds": t_data, "train_seconds": t_train,
            "val_loss_identity": base, "val_loss_start": start, "history": hist}
    return dn, info


def loss_of(Y, T, moment_weight):
    """The training loss of outputs Y against targets T (ss_dn_set_loss):
    mean-square error plus moment_weight times the squared second angular
    harmonic of the residual per cell, over the voxel count; batch mean."""
    import torch
    r = (Y - T).double()
    nphi = SHAPE[2]
    phi2 = 2 * (torch.arange(nphi, dtype=torch.float64, device=r.device) + 0.5) * 2 * np.pi / nphi
    c2 = (r * torch.cos(phi2)).sum(-1)
    s2 = (r * torch.sin(phi2)).sum(-1)
    per = (r ** 2).mean(dim=(1, 2, 3)) + moment_weight * (c2 ** 2 + s2 ** 2).sum(dim=(1, 2)) / float(np.prod(SHAPE))
    return float(per.mean().item())


def _unit(counts):
    c = counts.astype(np.float64).reshape(SHAPE)
    return c / c.mean()


def evaluate(dn, steps=2000, every=200, n_low=1_000_000, n_ref=64_000_000, plain=(1_000_000, 4_000_000, 16_000_000),
             seed=10):
    import torch

    import stochasticsampling_gb300 as ss
    runs = {}

    def make(n, s, mixed=False):
        # without the per-step counting sort: the plain FP64 runs' fastest form
        p = dict(PARAMS, number_of_particles=n, seed=s)
        sim = ss.Simulation(grid=GRID, box=BOX, params=p, quasi2d=True, mixed=mixed, sort=False)
        sim.init(initial_rows(n, seed=s))
        return sim

    runs["ref"] = make(n_ref, seed)
    for k, n in enumerate(plain):
        runs[f"plain_{n}"] = make(n, seed + 1 + k)
    runs["denoised"] = make(n_low, seed + 10, mixed="fixed64")
    runs["denoised"].set_denoiser(dn)
    runs["fp32_plain"] = make(n_low, seed + 10, mixed="fixed64")

    def fields(name, sim):
        f = _unit(sim.get_counts())
        if name == "denoised":
            x = torch.as_tensor(f.astype(np.float32)).cuda().contiguous()
            f = dn.forward(x).cpu().numpy().astype(np.float64)
        return f, sim.get_flow_field()

    errs = {k: {"dist": [], "flow": [], "flow_norm": []} for k in runs if k != "ref"}
    times = {k: 0.0 for k in runs}
    done = 0
    while True:
        # step 0 is the initial histogram (the flow of step 0 is solved from it)
        for name, sim in runs.items():
            t0 = time.perf_counter()
            sim.run(1 if done == 0 else every)
            sim.synchronize()
            times[name] += time.perf_counter() - t0
        done += 1 if done == 0 else every
        fr, ur = fields("ref", runs["ref"])
        for name, sim in runs.items():
            if name == "ref":
                continue
            f, u = fields(name, sim)
            errs[name]["dist"].append(float(np.linalg.norm(f - fr) / np.linalg.norm(fr)))
            errs[name]["flow"].append(float(np.linalg.norm(u - ur) / np.linalg.norm(ur)))
            # the flow's size against the reference's: with isotropic
            # orientations the workload's mean-field flow is zero (the density
            # modulation only adds a pressure, which the Oseen projection
            # removes), so this is the error against the infinite-N flow
            errs[name]["flow_norm"].append(float(np.linalg.norm(u) / np.linalg.norm(ur)))
        if done >= steps:
            break
    ms = {k: 1e3 * v / done for k, v in times.items()}
    for sim in runs.values():
        sim.close()
    mean_err = {k: {q: float(np.mean(v[q])) for q in v} for k, v in errs.items()}
    # plain FP64: error^2 = a / N + b, fitted on the plain runs; N at the denoised error
    ns = np.array(plain, dtype=np.float64)
    out = {"steps": done, "every": every, "n_low": n_low, "n_ref": n_ref, "errors": errs, "mean_errors": mean_err,
           "ms_per_step": ms}
    for q in ("dist", "flow", "flow_norm"):
        e2 = np.array([mean_err[f"plain_{n}"][q] ** 2 for n in plain])
        A = np.column_stack([1.0 / ns, np.ones_like(ns)])
        (a, b), *_ = np.linalg.lstsq(A, e2, rcond=None)
        target = mean_err["denoised"][q] ** 2
        n_eq = a / (target - b) if target > b and a > 0 else float("inf")
        per_particle_ms = ms[f"plain_{plain[-1]}"] / plain[-1]
        cost_plain = n_eq * per_particle_ms
        out[f"{q}_fit"] = {"a": float(a), "b": float(b), "plain_particles_at_denoised_error": float(n_eq),
                           "plain_ms_per_step_at_that_error": float(cost_plain),
                           "denoised_ms_per_step": ms["denoised"],
                           "cost_ratio": float(cost_plain / ms["denoised"]) if np.isfinite(cost_plain) else None}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=4000)
    ap.add_argument("--epochs", type=int, default=2)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=200)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--moment-weight", type=float, default=16.0)
    ap.add_argument("--snapshots", type=int, default=8, help="training snapshots per 64e6-particle run")
    ap.add_argument("--save", default=None, help="write the trained parameters (.npy)")
    args = ap.parse_args()
    dn, info = train_denoiser(pairs=args.pairs, epochs=args.epochs, lr=args.lr, steps=args.steps,
                              snapshots=args.snapshots, moment_weight=args.moment_weight)
    if args.save:
        dn.save(args.save)
    res = evaluate(dn, steps=args.steps, every=args.every)
    print(json.dumps({"training": info, "evaluation": res}))


if __name__ == "__main__":
    main()
