"""Batched ensemble of independent Taylor-Green solves (uneven grids and parameters).

  python -m cbns3d_cart_mpi_gb300.ensemble [--solves 64] [--steps 200] [--precision both]

Draws the ensemble with numpy.random.default_rng(seed): N per axis from
{32, 48, 64, 96, 128}, Re log-uniform in [400, 3200], Ma uniform in [0.05, 0.3];
each solve starts from the Taylor-Green state plus a solenoidal perturbation of
16 random Fourier modes with |k| <= 4 and total amplitude 1e-3
(cbns_host_initial_condition_perturbed, seeded per solve).  All solves of one
precision step together as one batch (one launch per kernel over every solve's
tiles, a batch step replayed as one CUDA graph, launch shape autotuned), for
`steps` RK3 steps.  Prints one JSON line: cell-RK3-steps/s per precision, the
autotuner's choice, and the FP32-mixed error against the binary64 batch.
"""
import argparse
import json
import math
import time

import numpy as np

from ._abi import NG, tgv_params
from .solver import Batch, Solver, initial_condition_perturbed

GRIDS = (32, 48, 64, 96, 128)


def draw(n, seed=0):
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(n):
        N = int(rng.choice(GRIDS))
        Re = float(math.exp(rng.uniform(math.log(400.0), math.log(3200.0))))
        Ma = float(rng.uniform(0.05, 0.3))
        cases.append({"N": N, "Re": Re, "Mach": Ma, "seed": 1000 + i})
    return cases


def build_solvers(cases, precision, t_end=20.0):
    solvers = []
    for c in cases:
        p = tgv_params(c["N"], Re=c["Re"], Mach=c["Mach"], t_end=t_end)
        s = Solver(p, precision=precision)
        s.upload_Q(initial_condition_perturbed(p, seed=c["seed"], amp=1e-3, nmodes=16, kmax=4), 0.0)
        solvers.append(s)
    return solvers


def run_batch(cases, precision, steps, tune=True, reps=2):
    import torch
    solvers = build_solvers(cases, precision)
    b = Batch(solvers)
    tuned = b.autotune(reps=reps) if tune else []
    stream = torch.cuda.ExternalStream(b.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    taken = b.run(steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    cells = sum(c["N"] ** 3 for c in cases)
    res = {"precision": precision, "ms": ms, "ms_per_step": ms / steps,
           "cell_rk3_steps_per_s": cells * steps / (ms * 1e-3), "steps_taken_min": min(taken),
           "config": b.config, "autotune_ms_per_step": [[r, c, m] for r, c, m in tuned]}
    return res, b, solvers


def rel_linf(a, b):
    a = a[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)
    b = b[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)
    return np.abs(a - b).max(axis=0) / np.abs(b).max(axis=0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--solves", type=int, default=64)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", default="both",
                    help="fp64, fp32_mixed, fp64_ff, a comma-separated list, or both (fp64,fp32_mixed)")
    ap.add_argument("--no-tune", action="store_true")
    args = ap.parse_args()
    cases = draw(args.solves, args.seed)
    cells = sum(c["N"] ** 3 for c in cases)
    out = {"workload": "TGV ensemble, %d solves, N in %s, Re log-U[400,3200], Ma U[0.05,0.3], seed %d, %d steps"
                       % (args.solves, list(GRIDS), args.seed, args.steps),
           "cells": cells, "grid_counts": {str(g): sum(c["N"] == g for c in cases) for g in GRIDS}}
    states = {}
    t0 = time.perf_counter()
    precs = ["fp64", "fp32_mixed"] if args.precision == "both" else args.precision.split(",")
    for prec in precs:
        res, b, solvers = run_batch(cases, prec, args.steps, tune=not args.no_tune)
        out[prec] = res
        states[prec] = [s.download_Q() for s in solvers]
        b.close()
        for s in solvers:
            s.close()
    for prec in states:
        if prec == "fp64" or "fp64" not in states:
            continue
        errs = np.array([rel_linf(m, d) for m, d in zip(states[prec], states["fp64"])])
        out[prec + "_vs_fp64_rel_linf_max"] = dict(zip(["rho", "rho*u", "rho*v", "rho*w", "E"],
                                                       errs.max(axis=0).tolist()))
        out[prec + "_vs_fp64_rel_linf_median"] = dict(zip(["rho", "rho*u", "rho*v", "rho*w", "E"],
                                                          np.median(errs, axis=0).tolist()))
        out[prec + "_speedup"] = out[prec]["cell_rk3_steps_per_s"] / out["fp64"]["cell_rk3_steps_per_s"]
    out["wall_s"] = time.perf_counter() - t0
    print(json.dumps(out))


if __name__ == "__main__":
    main()
