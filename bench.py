"""Throughput of one RK3 step of the cbns3d right-hand side on GB300.

Metric: cell-RK3-steps/s (interior cells x full 3-stage RK3 steps per second).
Workload: Taylor-Green vortex 256^3, binary64, Re 1600, Ma 0.1, CFL 0.5, the
reference's initial condition and mesh (synthetic analytic data; no dataset).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:       W untimed steps, then K steps timed with CUDA events on the solve's
            stream (the replayed step graph; state resident in HBM, 1.5 GB of
            state per step >> the 129 MB L2).  Then, inside the same run:
              * per-kernel timing of K more steps (events around every launch),
                giving the dominant kernel's roofline against the FP64 FMA peak
                measured live by cbns_probe_peak;
              * e2e: K steps through the C ABI with host buffers: upload Q from
                pinned memory, one step, download Q, every step, through the
                asynchronous entry points of one handle (copies on its second
                stream under the neighbouring steps' kernels); the synchronous
                calls timed beside it;
              * cpu_baseline: the oracle's CPU restatement of the reference (all
                host threads) on a bounded sample of the same workload.
reference:  the reference algorithm on the host cores (the oracle's restatement,
            bitwise equal to the reference compiled unmodified), W + K steps.
Multi-GPU: replicas only (independent solves, one per rank, no collective on the
data path); the JSON value is the aggregate over ranks, time = max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cell-RK3-steps/s TGV 256^3 FP64"
UNIT = "cell-RK3-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--cpu-steps", type=int, default=1, help="steps of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the FP32-mixed leg")
    ap.add_argument("--no-ff", action="store_true", help="skip the float-float faces leg (CBNS_FP64_FF)")
    ap.add_argument("--no-large", action="store_true", help="skip the 512^3 and 768^3 blocks")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(value, world):
    """Max of a float over ranks (identity at world size 1)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(world, cells, steps, ms_max):
    """Whole-job throughput of `world` replicas, each advancing `cells` cells by
    `steps` steps, timed by the slowest rank (ms_max)."""
    return world * cells * steps / (ms_max * 1e-3)


def hbm_peak():
    """The measured HBM copy bandwidth (GB/s) of the GB300s, else the fallback figure."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def workload_config(N):
    """The `config` both arms print: the same workload, so the two lines compare
    like for like (where each arm runs is in its `placement` key)."""
    from cbns3d_cart_mpi_gb300._abi import NEQ, NG
    return {"workload": "taylor-green vortex %d^3 FP64, Re 1600, Ma 0.1, CFL 0.5" % N, "grid": [N, N, N],
            "precision": "fp64",
            "l2": "state 2x%.0f MB per step, larger than the 129 MB L2; no flush" % (
                NEQ * (N + 2 * NG) ** 3 * 8 / 1e6)}


def cpu_sample(N, steps):
    """The oracle's CPU restatement of the reference on `steps` steps of the N^3
    workload, all host threads; returns (cell-steps/s, threads, seconds)."""
    from cbns3d_cart_mpi_gb300._abi import tgv_params
    from oracle.build import build_port
    from oracle.oracle import OracleBlock, num_threads
    build_port()
    b = OracleBlock(tgv_params(N, t_end=2.0))
    b.initial_condition()
    t0 = time.perf_counter()
    for _ in range(steps):
        b.step()
    sec = time.perf_counter() - t0
    th = num_threads()
    b.close()
    return N ** 3 * steps / sec, th, sec


def ncu_counts():
    """Per-launch figures from the committed ncu summaries (profiles/traffic.json):
    DRAM bytes per launch at 256^3 and binary64 instructions per face."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle.build import build_port
    from oracle.oracle import OracleBlock, num_threads
    from cbns3d_cart_mpi_gb300._abi import tgv_params
    build_port()
    N = args.N
    b = OracleBlock(tgv_params(N, t_end=2.0))
    b.initial_condition()
    for _ in range(args.warmup):
        b.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.step()
    sec = time.perf_counter() - t0
    value = N ** 3 * args.steps / sec
    th = num_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(N),
        "placement": "host cores (%d OpenMP threads over k-planes)" % th,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": th, "kind": "port",
                         "sample": "%d warm-up + %d timed full RK3 steps of the %d^3 workload" % (
                             args.warmup, args.steps, N)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
        "note": "oracle/cbns_oracle.c: the reference's arithmetic restated in C, bitwise equal to the reference "
                "compiled unmodified (tests/test_oracle_golden.py); the reference binary itself is built only "
                "where its sources are present, and the box has no MPI",
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    from cbns3d_cart_mpi_gb300 import build as pkg_build
    from cbns3d_cart_mpi_gb300._abi import NEQ, NG, tgv_params
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition
    from cbns3d_cart_mpi_gb300.workload import kernel_flops, mixed_update_bytes, probe_peak, state_bytes_per_step

    pkg_build.build()
    os.environ["CBNS_DEVICE"] = str(local)
    torch.cuda.set_device(local)
    N = args.N
    p = tgv_params(N, t_end=2.0)
    Q0 = initial_condition(p)
    s = Solver(p)
    s.upload_Q(Q0, 0.0)
    stream = torch.cuda.ExternalStream(s.stream)

    # Warm-up (also builds the step graph).
    s.run(args.warmup)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    done = s.run(args.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    ms = reduce_max(ms, world)
    assert done == args.steps, "solve finished early (%d of %d steps)" % (done, args.steps)
    cells = N ** 3
    value = aggregate_value(world, cells, args.steps, ms)
    launches_per_step = 2 + 3 * 5

    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(N),
            "placement": ("%d replicas, one solve per GPU" % world) if world > 1 else "one solve on one GPU",
            "clocks": clocks,
            "gpu_launches": launches_per_step * args.steps,
        }

    # Per-kernel timing over K more steps: roofline of the dominant kernel.
    s.profile_begin()
    s.run(args.steps)
    prof = s.profile_end()
    if rank == 0:
        tot = sum(v[1] for v in prof.values())
        kernels = {k: {"launches": v[0], "ms_per_launch": v[1] / v[0], "share": v[1] / tot} for k, v in prof.items()}
        dom = max(prof, key=lambda k: prof[k][1])
        if dom.startswith("inviscid_"):
            # One kernel template per direction with equal shares (29.1% each); the
            # x-direction launch is the one whose ncu counts are recorded.
            dom = "inviscid_x"
        per_launch_ms = prof[dom][1] / prof[dom][0]
        flops = kernel_flops(dom, N, N, N)
        achieved = flops / (per_launch_ms * 1e-3) * 1e-12
        peak = probe_peak(fp64=True)
        counts = ncu_counts()
        traffic = counts.get(dom)
        line["roofline"] = {
            "bound": "fp64-pipe", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic,
            "peak_source": "binary64 FMA throughput measured live on this GPU (cbns_probe_peak); "
                           "MEASURED_PEAKS.json holds no FP64 figure",
            "algorithmic_flops_per_launch": flops,
            "flop_count": "reference's own op count per face (tests/golden/opcount.txt) x N^3 distinct "
                          "periodic faces; a division counts 1",
            "note": "frac counts the reference's FLOPs against the FMA peak and can exceed 1; pipe_frac is "
                    "the binary64 instructions the kernel issues (ncu) over the pipe's measured issue rate",
        }
        inst = counts.get(dom + "_fp64_inst_per_face")
        if inst:
            # Binary64 instructions issued per second over the probe's FMA rate
            # (peak TFLOP/s / 2 FLOPs per FMA): the FP64 pipe's busy fraction.
            issued = inst * N ** 3 / (per_launch_ms * 1e-3)
            line["roofline"]["pipe_frac"] = issued / (peak * 1e12 / 2.0)
            line["roofline"]["fp64_inst_per_face"] = inst
        step_ms = ms / args.steps
        line["kernels"] = kernels
        line["step_roofline"] = {
            "algorithmic_tflops": 15198.25 * cells / (step_ms * 1e-3) * 1e-12,
            "hbm_gbs_min_state": state_bytes_per_step(N, N, N) / (step_ms * 1e-3) * 1e-9,
        }

    # The other precisions' legs: same workload, same number of steps (warm-up,
    # timed, profiled), and the error against the binary64 state after them.
    Q64 = s.download_Q() if not (args.no_mixed and args.no_ff) else None

    def precision_leg(prec, e2e=False):
        sx = Solver(p, precision=prec)
        sx.upload_Q(Q0, 0.0)
        xstream = torch.cuda.ExternalStream(sx.stream)
        sx.run(args.warmup)
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(xstream)
        sx.run(args.steps)
        e1.record(xstream)
        e1.synchronize()
        xms = reduce_max(e0.elapsed_time(e1), world)
        sx.profile_begin()
        sx.run(args.steps)
        xprof = sx.profile_end()
        a = sx.download_Q()[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)
        xe2e = None
        if e2e:
            # end to end as the headline's e2e: host state uploaded and downloaded
            # every step through the asynchronous calls of one handle
            xin, xout = sx.pinned_state(), sx.pinned_state()
            xin[...] = Q0
            sx.upload_Q_async(xin, 0.0)
            sx.step_async()
            sx.download_Q_async(xout)
            sx.wait()
            barrier(world)
            t0 = time.perf_counter()
            for _ in range(args.steps):
                sx.upload_Q_async(xin, 0.0)
                sx.step_async()
                sx.download_Q_async(xout)
            sx.wait()
            xe2e = reduce_max(time.perf_counter() - t0, world)
        sx.close()
        b = Q64[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)
        # L-inf error over each field's scale; the three momentum fields share
        # the largest momentum magnitude (rho w starts at exactly zero, so its own
        # maximum is no scale in the first steps).
        scale = np.abs(b).max(axis=0)
        scale[1:4] = scale[1:4].max()
        err = (np.abs(a - b).max(axis=0) / scale).tolist()
        return (xms, xprof, err, xe2e) if e2e else (xms, xprof, err)

    # FP32-mixed leg.
    if not args.no_mixed:
        mms, mprof, err = precision_leg("fp32_mixed")
        if rank == 0:
            mtot = sum(v[1] for v in mprof.values())
            mdom = max(mprof, key=lambda k: mprof[k][1])
            if mdom.startswith("inviscid_"):
                mdom = "inviscid_x"
            mper = mprof[mdom][1] / mprof[mdom][0]
            mflops = kernel_flops(mdom, N, N, N)
            peak32 = probe_peak(fp64=False)
            if mdom == "update":
                # The binary32 update is bound by memory and its binary64 remnant, not
                # binary32 arithmetic: its compulsory bytes against the measured HBM peak.
                hbm, hbm_src = hbm_peak()
                mbytes = mixed_update_bytes(N, N, N)
                # ncu DRAM bytes of the three update launches of one step at 256^3, averaged.
                traffic = ncu_counts().get("update_f32") if N == 256 else None
                mroof = {"bound": "hbm", "kernel": mdom, "achieved": mbytes / (mper * 1e-3) * 1e-9, "peak": hbm,
                         "unit": "GB/s", "frac": mbytes / (mper * 1e-3) * 1e-9 / hbm, "traffic": traffic,
                         "algorithmic_bytes_per_launch": mbytes, "peak_source": hbm_src,
                         "bytes_count": "compulsory bytes per cell by stage (workload.MIXED_UPDATE_BYTES_PER_CELL)"}
            else:
                mroof = {"bound": "fp32-pipe", "kernel": mdom, "achieved": mflops / (mper * 1e-3) * 1e-12,
                         "peak": peak32, "unit": "TFLOP/s", "frac": mflops / (mper * 1e-3) * 1e-12 / peak32,
                         "peak_source": "binary32 FMA throughput measured live (cbns_probe_peak)"}
            line["fp32_mixed"] = {
                "value": world * cells * args.steps / (mms * 1e-3), "unit": UNIT, "ms_per_step": mms / args.steps,
                "speedup_vs_fp64": ms / mms,
                "linf_vs_fp64_over_field_scale": dict(zip(["rho", "rho*u", "rho*v", "rho*w", "E"], err)),
                "error_after_steps": args.warmup + 2 * args.steps,
                "kernels": {k: {"launches": v[0], "ms_per_launch": v[1] / v[0], "share": v[1] / mtot}
                            for k, v in mprof.items()},
                "roofline": mroof,
            }

    # Float-float faces leg (CBNS_FP64_FF): the binary64 solve with its face
    # fluxes in float-float arithmetic on the binary32 pipes.  The face kernel's
    # roofline: binary32 instructions issued (ncu count per face) over the
    # binary32 FMA pipe's measured instruction rate.
    if not args.no_ff:
        fms, fprof, ferr, fe2e = precision_leg("fp64_ff", e2e=not args.no_e2e)
        if rank == 0:
            ftot = sum(v[1] for v in fprof.values())
            fper = fprof["inviscid_x"][1] / fprof["inviscid_x"][0]
            froof = {"bound": "fp32-pipe", "kernel": "inviscid_x", "unit": "TFLOP/s",
                     "peak": probe_peak(fp64=False), "peak_source": "binary32 FMA throughput measured live "
                                                                  "(cbns_probe_peak)"}
            finst = counts.get("inviscid_x_ff_fp32_inst_per_face")
            if finst:
                issued = finst * N ** 3 / (fper * 1e-3)  # binary32 instructions per second
                froof["fp32_inst_per_face"] = finst
                froof["achieved"] = issued * 2.0 * 1e-12  # as FMA-equivalent TFLOP/s
                froof["frac"] = froof["achieved"] / froof["peak"]
                ref_per_face = kernel_flops("inviscid_x", N, N, N) / N ** 3
                froof["note"] = ("float-float arithmetic: binary32 instructions per face (ncu) over the pipe's "
                                 "instruction rate; the reference's %d FLOPs per face take about %.1f of them each"
                                 % (round(ref_per_face), finst / ref_per_face))
            line["fp64_ff"] = {
                "value": world * cells * args.steps / (fms * 1e-3), "unit": UNIT, "ms_per_step": fms / args.steps,
                "dtype": "f64 state and RK3; float-float (binary32 pairs) faces, viscous terms, flux "
                         "differences, primitives and time-step speeds",
                "speedup_vs_fp64": ms / fms,
                "linf_vs_fp64_over_field_scale": dict(zip(["rho", "rho*u", "rho*v", "rho*w", "E"], ferr)),
                "error_after_steps": args.warmup + 2 * args.steps,
                "kernels": {k: {"launches": v[0], "ms_per_launch": v[1] / v[0], "share": v[1] / ftot}
                            for k, v in fprof.items()},
                "roofline": froof,
            }
            if fe2e:
                nst = int(np.prod(s.shape))
                line["fp64_ff"]["e2e"] = {"value": world * cells * args.steps / fe2e, "unit": UNIT,
                                          "h2d_bytes_per_step": nst * 8, "d2h_bytes_per_step": nst * 8,
                                          "path": "as e2e, on a CBNS_FP64_FF handle"}

    # e2e: host buffers through the C ABI, copies inside the timed region.  Every
    # step uploads its input state from pinned host memory, steps, and downloads
    # its result, through the asynchronous entry points of one handle: the copies
    # run on the handle's second stream under the neighbouring steps' kernels, and
    # the timed region ends when cbns_wait has seen the last download land.  The
    # synchronous calls (each waits for its own copy) are timed beside it.
    if not args.no_e2e:
        n = int(np.prod(s.shape))
        hin, hout = s.pinned_state(), s.pinned_state()
        hin[...] = Q0
        s.upload_Q_async(hin, 0.0)
        s.step_async()
        s.download_Q_async(hout)
        s.wait()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.upload_Q_async(hin, 0.0)
            s.step_async()
            s.download_Q_async(hout)
        s.wait()
        sec = reduce_max(time.perf_counter() - t0, world)
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.upload_Q(hin, 0.0)
            s.step()
            s.download_Q(out=hout)
        seq = reduce_max(time.perf_counter() - t0, world)
        if rank == 0:
            line["e2e"] = {"value": world * cells * args.steps / sec, "unit": UNIT,
                           "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8,
                           "path": "cbns_upload_Q_async (pinned) + cbns_step_async + cbns_download_Q_async (pinned) "
                                   "per step on one handle, %d steps, then cbns_wait" % args.steps,
                           "synchronous_calls": world * cells * args.steps / seq}
    s.close()

    # Larger blocks, state built on the device: binary64 at 512^3 (50 GB),
    # float-float at 512^3 (78 GB) and 768^3 (259 GB), and FP32-mixed at 512^3 and
    # at 768^3 (165 GB), above the old 31-bit-index limit (N ~ 745).
    if not args.no_large and rank == 0:
        large = []
        for NL, prec in ((512, "fp64"), (512, "fp64_ff"), (768, "fp64_ff"), (512, "fp32_mixed"), (768, "fp32_mixed")):
            pl = tgv_params(NL, t_end=2.0)
            try:
                sl = Solver(pl, precision=prec)
            except Exception as e:  # not enough device memory on this GPU
                large.append({"N": NL, "precision": prec, "skipped": str(e)[:200]})
                continue
            sl.init_tgv()
            lstream = torch.cuda.ExternalStream(sl.stream)
            nwarm, ntimed = (1, 2) if prec == "fp64" else (2, 3)
            sl.run(nwarm)
            torch.cuda.synchronize()
            l0 = torch.cuda.Event(enable_timing=True)
            l1 = torch.cuda.Event(enable_timing=True)
            l0.record(lstream)
            nl = sl.run(ntimed)
            l1.record(lstream)
            l1.synchronize()
            lms = l0.elapsed_time(l1) / nl
            large.append({"N": NL, "precision": prec, "steps": nl, "ms_per_step": lms,
                          "value": NL ** 3 / (lms * 1e-3), "device_bytes": sl.info()["device_bytes"]})
            sl.close()
        line["large_blocks"] = large

    if rank == 0 and world == 1 and not args.no_cpu_baseline:  # the host baseline is an N=1 figure
        v, th, sec = cpu_sample(N, args.cpu_steps)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": th, "kind": "port",
                                "sample": "%d full RK3 step(s) of the %d^3 workload, %.1f s" % (args.cpu_steps, N, sec)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        if world > 1:
            # The CPU reference runs once on rank 0; other ranks exit without work.
            run_reference(args, rank, world)
            return
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
