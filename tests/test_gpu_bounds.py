"""The kernels, compiled with every global index checked (-DCBNS_BOUNDS_CHECK).

compute-sanitizer is not available on the GPUs these tests run on, so the
library is built a second time with each array access of its kernels going
through a checked accessor: an index outside its array sets the solve's
bounds bit (CBNS_ERR_BOUNDS from the next call that reads the status) and the
access goes to element 0 instead, so nothing faults.  A child process loads
that build (CBNS_GPU_LIB) and runs the stage, step-graph, batch, asynchronous
and allocation-free paths on blocks at and near the smallest extents (NG = 4),
odd and non-cubic shapes and an odd JM for the FP32-mixed two-row face kernel,
in every precision.  Every call must return CBNS_OK and every state must be
bitwise the one the normal build gives (a check changes addresses, never
arithmetic).  tests/test_index_bounds.py restates the same offset arithmetic
on the CPU.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

SHAPES = [(4, 5, 6), (12, 16, 20), (33, 17, 9), (20, 13, 10)]


def run_cases(out_path):
    """Every path on every shape; all states into one .npz (run with either build)."""
    import ctypes
    import math

    sys.path.insert(0, ROOT)
    import torch

    from cbns3d_cart_mpi_gb300 import _lib
    from cbns3d_cart_mpi_gb300._abi import CBNS_OK, tgv_params
    from cbns3d_cart_mpi_gb300.solver import Batch, Solver, initial_condition_perturbed

    res = {}
    for prec in ("fp64", "fp32_mixed", "fp64_ff"):
        solves = []
        for q, (IM, JM, KM) in enumerate(SHAPES):
            p = tgv_params(IM, JM=JM, KM=KM, Re=800.0, Mach=0.2)
            Q0 = initial_condition_perturbed(p, seed=60 + q, amp=1e-3)
            tag = "%s_%dx%dx%d" % (prec, IM, JM, KM)
            s = Solver(p, precision=prec)
            s.upload_Q(Q0, 0.0)
            s.stage(1e-3, 1)
            res[tag + "_stage1"] = s.download_Q_p()
            s.upload_Q(Q0, 0.0)
            s.step()
            assert s.run(2) == 2
            res[tag + "_steps"] = s.download_Q()
            res[tag + "_diag"] = np.array(s.diagnostics())
            res[tag + "_prims"] = np.stack([s.download_prims()[k] for k in ("rho", "u", "v", "w", "p", "T")])
            # asynchronous path
            a_in, a_out = s.pinned_state(), s.pinned_state()
            a_in[...] = Q0
            s.upload_Q_async(a_in, 0.0)
            s.step_async()
            s.download_Q_async(a_out)
            s.wait()
            res[tag + "_async"] = a_out.copy()
            # allocation-free diagnostics on a device copy of the state
            if prec == "fp64":
                dev = torch.device("cuda", torch.cuda.current_device())
                Qd = torch.from_numpy(np.ascontiguousarray(res[tag + "_steps"]).reshape(-1)).to(dev)
                out = torch.empty(2, dtype=torch.float64, device=dev)
                st = _lib.gpu().cbns_diagnostics_noalloc(
                    ctypes.c_void_p(Qd.data_ptr()), IM, JM, KM, 2 * math.pi / IM, 2 * math.pi / JM,
                    2 * math.pi / KM, ctypes.c_void_p(out.data_ptr()),
                    ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
                assert st == CBNS_OK, _lib.last_error()
                torch.cuda.synchronize()
                res[tag + "_noalloc"] = out.cpu().numpy()
            s.upload_Q(Q0, 0.0)
            solves.append(s)
        # the same solves stepped as one batch, persistent launch shape included
        b = Batch(solves)
        assert b.run(2) == [2] * len(solves)
        b.set_config(2, 2)
        assert b.run(1) == [3] * len(solves)
        for (IM, JM, KM), s in zip(SHAPES, solves):
            res["%s_%dx%dx%d_batch" % (prec, IM, JM, KM)] = s.download_Q()
            s.check_state()
        b.close()
        for s in solves:
            s.close()
    np.savez(out_path, **res)


def _child(lib, out_path):
    env = dict(os.environ)
    if lib:
        env["CBNS_GPU_LIB"] = lib
    r = subprocess.run([sys.executable, os.path.abspath(__file__), out_path], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return np.load(out_path)


@pytest.mark.gpu
def test_checked_build_reports_no_access_outside_its_arrays(tmp_path, built):
    from cbns3d_cart_mpi_gb300 import build
    checked = build.build_checked()
    plain = _child(None, str(tmp_path / "plain.npz"))
    chk = _child(checked, str(tmp_path / "checked.npz"))
    assert sorted(plain.files) == sorted(chk.files)
    assert len(plain.files) >= 8 * len(SHAPES)
    for k in plain.files:
        assert np.array_equal(plain[k], chk[k]), k


if __name__ == "__main__":
    run_cases(sys.argv[1])
