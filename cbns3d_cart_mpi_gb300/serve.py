"""Serving benchmark: Poisson-arrival solve requests through the continuous-batching server.

  python -m cbns3d_cart_mpi_gb300.serve [--rates 0.25,0.5,1] [--requests 24] [--precision fp32_mixed]
                                        [--grids 32:192:16]

Each request: grid N per axis uniform in {32, 48, ..., 192} (--grids), Re log-uniform in
[400, 3200], Ma uniform in [0.05, 0.3], the Taylor-Green state plus a seeded
solenoidal perturbation (16 modes, |k| <= 4, amplitude 1e-3) built on the
device, run to t = 1.  Arrivals are a Poisson process at each swept rate
(numpy.random.default_rng(seed)); a submitter thread sleeps the exponential
gaps.  Reports per rate: p50/p99 latency (submit to done), p50 queueing delay,
aggregate cell-RK3-steps/s over the makespan, and the server's peak
concurrency.  One JSON line.
"""
import argparse
import json
import math
import threading
import time

import numpy as np

from ._abi import CBNS_OK, tgv_params
from .solver import Server

GRIDS = tuple(range(32, 193, 16))


def draw(n, seed, grids=GRIDS):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        out.append({"N": int(rng.choice(grids)),
                    "Re": float(math.exp(rng.uniform(math.log(400.0), math.log(3200.0)))),
                    "Mach": float(rng.uniform(0.05, 0.3)), "seed": 5000 + i})
    return out


def run_rate(rate, reqs, precision, seed, t_end, steps_per_round, memory_budget):
    rng = np.random.default_rng(seed + 1)
    gaps = rng.exponential(1.0 / rate, size=len(reqs))
    sv = Server(precision=precision, steps_per_round=steps_per_round, memory_budget_bytes=memory_budget)
    ids = [None] * len(reqs)

    def submitter():
        for i, r in enumerate(reqs):
            time.sleep(gaps[i])
            p = tgv_params(r["N"], Re=r["Re"], Mach=r["Mach"], t_end=t_end)
            ids[i] = sv.submit_tgv(p, seed=r["seed"], amp=1e-3, nmodes=16, kmax=4)

    th = threading.Thread(target=submitter)
    t0 = time.perf_counter()
    th.start()
    th.join()
    infos = [sv.wait(i) for i in ids]
    makespan = time.perf_counter() - t0
    st = sv.stats()
    sv.close()
    ok = [x for x in infos if x["status"] == CBNS_OK]
    lat = np.array([x["done_s"] - x["submit_s"] for x in ok])
    queue = np.array([x["admit_s"] - x["submit_s"] for x in ok])
    cell_steps = sum(r["N"] ** 3 * x["steps"] for r, x in zip(reqs, infos) if x["status"] == CBNS_OK)
    return {"rate_req_per_s": rate, "requests": len(reqs), "completed": len(ok),
            "latency_p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "queue_p50_s": float(np.percentile(queue, 50)) if len(queue) else None,
            "cell_rk3_steps_per_s": cell_steps / makespan, "makespan_s": makespan,
            "peak_active": st["peak_active"], "rounds": st["rounds"], "batch_builds": st["batch_builds"],
            "steps_per_request_mean": float(np.mean([x["steps"] for x in ok])) if ok else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rates", default="0.25,0.5,1.0")
    ap.add_argument("--requests", type=int, default=24)
    ap.add_argument("--precision", default="fp32_mixed", choices=["fp64", "fp32_mixed", "fp64_ff"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--t-end", type=float, default=1.0)
    ap.add_argument("--steps-per-round", type=int, default=20)
    ap.add_argument("--memory-budget-gb", type=float, default=0.0)
    ap.add_argument("--grids", default="32:192:16", help="first:last:step of the grid sizes N drawn from")
    args = ap.parse_args()
    g0, g1, gs = (int(x) for x in args.grids.split(":"))
    grids = tuple(range(g0, g1 + 1, gs))
    reqs = draw(args.requests, args.seed, grids)
    out = {"workload": "Poisson solve requests, N in %d..%d step %d, Re log-U[400,3200], Ma U[0.05,0.3], "
                       "TGV + 1e-3 solenoidal perturbation built on the device, run to t=%g" % (
                           g0, g1, gs, args.t_end),
           "precision": args.precision, "steps_per_round": args.steps_per_round, "rates": []}
    for k, rate in enumerate(float(x) for x in args.rates.split(",")):
        out["rates"].append(run_rate(rate, reqs, args.precision, args.seed + k, args.t_end, args.steps_per_round,
                                     int(args.memory_budget_gb * 2 ** 30)))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
