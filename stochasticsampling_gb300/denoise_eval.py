"""Train the histogram denoiser on pairs the method generates and evaluate it
in the loop of the production workload (2-D, grid 128x128x1x32x1, box
40x40, Dt 0.1, Dr 1.0, active stress -2, dt 0.005).

    python -m stochasticsampling_gb300.denoise_eval [--pairs 4000] [--epochs 2] [--steps 2000]

Training: pairs (histogram of n_in = 1e6 particles, independent histogram of
n_target = 64e6 particles) of initial conditions of the workload's family,
perturbation amplitude uniform in [0, 5 %] (random phase and axis).

Evaluation: independent samples of the workload's initial condition (1 %
sinusoidal density along x) run side by side -- a plain FP64 reference with
64e6 particles, plain FP64 runs with 1e6, 4e6 and 1.6e7 particles, and the
FP32 (fixed-point positions) run with 1e6 particles and the denoiser in the
loop.  Every `every` steps the L2 errors of the distribution (histogram /
mean count; for the denoised run the network's output) and of the flow field
against the reference are recorded.  The particle-steps cost of reaching the
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


def initial_rows(n, amp=0.01, seed=1):
    """n particles of the workload's initial condition: density
    1 + amp sin(2 pi x / L) along x (inverse CDF by Newton), uniform y and phi."""
    rng = np.random.default_rng(seed)
    L = BOX[0]
    u = rng.random(n)
    x = u * L
    for _ in range(8):
        f = x / L + amp * (1 - np.cos(2 * np.pi * x / L)) / (2 * np.pi) - u
        x -= f / ((1 + amp * np.sin(2 * np.pi * x / L)) / L)
    rows = np.empty((n, 5))
    rows[:, 0] = np.mod(x, L)
    rows[:, 1] = BOX[1] * rng.random(n)
    rows[:, 2] = 0.0
    rows[:, 3] = 2 * np.pi * rng.random(n)
    rows[:, 4] = np.pi / 2
    return rows


def train_denoiser(pairs=4000, epochs=2, batch=8, lr=1e-3, n_in=1_000_000, n_target=64_000_000, seed=0,
                   val_pairs=64):
    import torch

    from .denoiser import Denoiser, make_pairs, train
    t0 = time.perf_counter()
    X, T = make_pairs(pairs, SHAPE, n_in, n_target, seed=seed)
    Xv, Tv = make_pairs(val_pairs, SHAPE, n_in, n_target, seed=seed + 1000)
    t_data = time.perf_counter() - t0
    dn = Denoiser(SHAPE, seed=seed)
    base = float(((Xv - Tv) ** 2).mean().item())
    start = dn.loss(Xv, Tv)
    t0 = time.perf_counter()
    hist = train(dn, X, T, epochs=epochs, batch=batch, lr=lr, seed=seed, val=(Xv, Tv))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del X, T
    info = {"pairs": pairs, "epochs": epochs, "batch": batch, "lr": lr, "n_in": n_in, "n_target": n_target,
            "data_seconds": t_data, "train_seconds": t_train,
            "val_loss_identity": base, "val_loss_start": start, "history": hist}
    return dn, info


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

    errs = {k: {"dist": [], "flow": []} for k in runs if k != "ref"}
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
    for q in ("dist", "flow"):
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
    ap.add_argument("--save", default=None, help="write the trained parameters (.npy)")
    args = ap.parse_args()
    dn, info = train_denoiser(pairs=args.pairs, epochs=args.epochs, lr=args.lr)
    if args.save:
        dn.save(args.save)
    res = evaluate(dn, steps=args.steps, every=args.every)
    print(json.dumps({"training": info, "evaluation": res}))


if __name__ == "__main__":
    main()
