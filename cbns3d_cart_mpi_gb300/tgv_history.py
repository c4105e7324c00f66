"""Taylor-Green vortex history: precisions side by side.

  python -m cbns3d_cart_mpi_gb300.tgv_history [--N 256] [--times 0.5,1,2] [--every 10] [--out FILE]
      [--precisions fp64,fp32_mixed] [--history-vs FILE]

Runs the reference's Taylor-Green case (Re 1600, Ma 0.1, CFL 0.5, its mesh and
initial condition) on one GPU in each precision (default binary64 and
FP32-mixed), each as replayed step graphs, recording kinetic energy and
enstrophy every `every` steps.  Each listed time is an end time the solve clips
its last step to (the reference's t_end rule), so all precisions reach exactly
the same times; there each state is compared with the binary64 one when
binary64 is among the runs (relative L-inf and L2 per conserved field).
--history-vs names the text history of an earlier binary64 run (columns: step,
t, KE, enstrophy, ...): each run's KE and enstrophy are compared with it at the
same steps.  Writes a JSON file with the histories, the errors and the wall
time of each run.
"""
import argparse
import json
import time

import numpy as np

from ._abi import NG, tgv_params
from .solver import Solver, initial_condition

FIELDS = ["rho", "rho*u", "rho*v", "rho*w", "E"]


def run(N, precision, times, every, Q0):
    import torch
    p = tgv_params(N, t_end=max(times))
    s = Solver(p, precision=precision)
    s.upload_Q(Q0, 0.0)
    hist = []
    ke, en = s.diagnostics()
    hist.append((0, 0.0, ke, en))
    states = {}
    steps = 0
    gpu_ms = 0.0
    stream = torch.cuda.ExternalStream(s.stream)
    for te in times:
        while True:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            n = s.run(every, t_end=te)
            e1.record(stream)
            e1.synchronize()
            gpu_ms += e0.elapsed_time(e1)
            steps += n
            t, _ = s.time()
            ke, en = s.diagnostics()
            hist.append((steps, t, ke, en))
            if n < every:
                break
        states[te] = s.download_Q()
    s.close()
    return hist, states, steps, gpu_ms


def errors(a, b):
    a = a[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)
    b = b[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)
    linf = np.abs(a - b).max(axis=0) / np.abs(b).max(axis=0)
    l2 = np.sqrt(((a - b) ** 2).sum(axis=0) / (b ** 2).sum(axis=0))
    return dict(zip(FIELDS, linf.tolist())), dict(zip(FIELDS, l2.tolist()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--times", default="0.5,1,2")
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--out", default="tgv_history.json")
    ap.add_argument("--precisions", default="fp64,fp32_mixed")
    ap.add_argument("--history-vs", default=None)
    args = ap.parse_args()
    precs = args.precisions.split(",")
    times = [float(x) for x in args.times.split(",")]
    Q0 = initial_condition(tgv_params(args.N))
    out = {"case": "TGV %d^3, Re 1600, Ma 0.1, CFL 0.5, reference mesh and initial condition" % args.N,
           "times": times, "every": args.every}
    states = {}
    for prec in precs:
        t0 = time.perf_counter()
        hist, st, steps, gpu_ms = run(args.N, prec, times, args.every, Q0)
        out[prec] = {"steps": steps, "gpu_ms": gpu_ms, "wall_s": time.perf_counter() - t0,
                     "cell_rk3_steps_per_s": args.N ** 3 * steps / (gpu_ms * 1e-3),
                     "history": [list(h) for h in hist]}
        states[prec] = st
    for prec in precs:
        if prec == "fp64" or "fp64" not in states:
            continue
        out[prec + "_vs_fp64"] = {}
        for te in times:
            linf, l2 = errors(states[prec][te], states["fp64"][te])
            out[prec + "_vs_fp64"][str(te)] = {"rel_linf": linf, "rel_l2": l2}
    if args.history_vs:
        ref = {}
        with open(args.history_vs) as f:
            for line in f:
                if line.strip() and not line.startswith("#"):
                    c = line.split()
                    ref[int(c[0])] = (float(c[2]), float(c[3]))
        for prec in precs:
            common = [h for h in out[prec]["history"] if h[0] in ref]
            out[prec + "_vs_history"] = {
                "file": args.history_vs, "points": len(common),
                "ke_rel_max": max(abs(h[2] - ref[h[0]][0]) / abs(ref[h[0]][0]) for h in common),
                "enstrophy_rel_max": max(abs(h[3] - ref[h[0]][1]) / abs(ref[h[0]][1]) for h in common)}
    with open(args.out, "w") as f:
        json.dump(out, f)
    print(json.dumps({k: v for k, v in out.items() if k not in precs}))
    for prec in precs:
        print(prec, {k: v for k, v in out[prec].items() if k != "history"})


if __name__ == "__main__":
    main()
