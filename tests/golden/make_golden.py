"""Generate the golden fixtures of tests/golden/ from the reference solver itself.

Runs ``oracle/_ref/ref_harness`` — the reference's own sources compiled
unmodified by ``oracle/build.py`` — on small Taylor-Green cases and stores what
it produced.  Needs the reference sources on this machine; the fixtures are
committed so the tests never need them.

  python tests/golden/make_golden.py

Fixtures (states hold the interior cells only, shape (KM, JM, IM, 5); ghosts
follow from the periodic fill):
  tgv16.npz      16^3: Q0, Q_p after stage 1 of step 1, Q after 3 steps, dt/t per step
  tgv_odd.npz    12x16x20 (non-cubic, not a multiple of the tile): Q0, Q after 2 steps
  tgv_min.npz    4x5x6 (every extent at or near NG = 4): Q0, Q after 2 steps
  tgv_pert.npz   12^3, Re 800, Ma 0.2, perturbed initial state injected through the
                 reference's checkpoint reader: Q0, Q after 3 steps
  tgv64_hist.npz 64^3, Re 1600, Ma 0.1, CFL 0.5, 100 steps: dt/t per step; kinetic
                 energy, enstrophy and per-field sums/maxima every 10 steps; every 4th
                 cell of Q after step 100
  ckpt_4x5x6.dat the reference's own Block3d::output_bin file after 2 steps of tgv_min
  vtk/           the reference's VTK XML output (output_vtk_xml) for tgv_min at start/end
  opcount.txt    FLOPs per unit of the reference's hot-path functions (oracle/opcount)
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cbns3d_cart_mpi_gb300._abi import NG, tgv_params  # noqa: E402
from cbns3d_cart_mpi_gb300.params import write_input_txt  # noqa: E402
from oracle.build import build_ref  # noqa: E402
from oracle.oracle import diagnostics, read_state, write_state  # noqa: E402

# Run directories of the reference harness: a fresh temporary directory per
# invocation of this script, removed by the operating system's temp cleanup.
WORK = tempfile.mkdtemp(prefix="cbns_golden_runs_")


def interior(Q):
    return np.ascontiguousarray(Q[NG:-NG, NG:-NG, NG:-NG, :])


def run(harness, name, params, nsteps, dump_every, extra=(), inject=None):
    wd = os.path.join(WORK, name)
    if os.path.isdir(wd):
        shutil.rmtree(wd)
    os.makedirs(wd)
    write_input_txt(params, os.path.join(wd, "input.txt"))
    args = [harness, wd, str(nsteps), str(dump_every)] + list(extra)
    if inject is not None:
        Q0, t0 = inject
        write_state(os.path.join(wd, "inject.dat"), Q0, t0)
        args += ["--inject", "inject.dat"]
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s failed: %s" % (name, r.stderr))
    steps = np.loadtxt(os.path.join(wd, "steps.txt"), ndmin=2)
    return wd, steps


def state(wd, n):
    return read_state(os.path.join(wd, "q_%06d.bin" % n))


def main():
    res = build_ref()
    if res is None:
        sys.exit("reference sources not found; cannot generate golden fixtures")
    harness, opcount = res

    # 16^3: one stage, then three steps.
    p = tgv_params(16)
    wd, _ = run(harness, "tgv16_stage1", p, 1, 1, ["--stage1"])
    _, Qp1 = read_state(os.path.join(wd, "qp_stage1.bin"))
    wd, steps = run(harness, "tgv16", p, 3, 1)
    np.savez(os.path.join(HERE, "tgv16.npz"), Q0=interior(state(wd, 0)[1]), Qp_stage1=interior(Qp1),
             Q3=interior(state(wd, 3)[1]), dt=steps[:, 1], t=steps[:, 2], N=np.array([16, 16, 16]))

    p = tgv_params(12, JM=16, KM=20)
    wd, steps = run(harness, "tgv_odd", p, 2, 1)
    np.savez(os.path.join(HERE, "tgv_odd.npz"), Q0=interior(state(wd, 0)[1]), Q2=interior(state(wd, 2)[1]),
             dt=steps[:, 1], t=steps[:, 2], N=np.array([12, 16, 20]))

    p = tgv_params(4, JM=5, KM=6)
    wd, steps = run(harness, "tgv_min", p, 2, 1, ["--vtk", "--ckpt"])
    np.savez(os.path.join(HERE, "tgv_min.npz"), Q0=interior(state(wd, 0)[1]), Q2=interior(state(wd, 2)[1]),
             dt=steps[:, 1], t=steps[:, 2], N=np.array([4, 5, 6]))
    shutil.copy(os.path.join(wd, "checkpoint_ref.dat"), os.path.join(HERE, "ckpt_4x5x6.dat"))
    vdir = os.path.join(HERE, "vtk")
    if os.path.isdir(vdir):
        shutil.rmtree(vdir)
    os.makedirs(vdir)
    for sub in ("vtk_init", "vtk_final"):
        for f in os.listdir(os.path.join(wd, sub)):
            shutil.copy(os.path.join(wd, sub, f), os.path.join(vdir, sub + "_" + f))

    # Perturbed initial state (host library generator), injected via read_bin.
    from cbns3d_cart_mpi_gb300 import build as pkg_build
    from cbns3d_cart_mpi_gb300.solver import initial_condition_perturbed
    pkg_build.build()
    p = tgv_params(12, Re=800.0, Mach=0.2)
    Qinj = initial_condition_perturbed(p, seed=7, amp=1e-3)
    wd, steps = run(harness, "tgv_pert", p, 3, 1, inject=(Qinj, 0.0))
    np.savez(os.path.join(HERE, "tgv_pert.npz"), Q0=interior(state(wd, 0)[1]), Q3=interior(state(wd, 3)[1]),
             dt=steps[:, 1], t=steps[:, 2], N=np.array([12, 12, 12]), Re=800.0, Mach=0.2)

    # 64^3 history: the 100-step parity case.
    p = tgv_params(64)
    wd, steps = run(harness, "tgv64", p, 100, 10)
    dx = 2.0 * np.pi / 64
    ke, en, sums, amax, tt = [], [], [], [], []
    for n in range(0, 101, 10):
        t, Q = state(wd, n)
        k, e = diagnostics(Q, 64, 64, 64, dx, dx, dx)
        ke.append(k)
        en.append(e)
        qi = interior(Q)
        sums.append(qi.reshape(-1, 5).sum(axis=0))
        amax.append(np.abs(qi).reshape(-1, 5).max(axis=0))
        tt.append(t)
    _, Q100 = state(wd, 100)
    np.savez(os.path.join(HERE, "tgv64_hist.npz"), dt=steps[:, 1], t=steps[:, 2], diag_steps=np.arange(0, 101, 10),
             diag_t=np.array(tt), ke=np.array(ke), enstrophy=np.array(en), sums=np.array(sums),
             absmax=np.array(amax), Q100_sub=interior(Q100)[::4, ::4, ::4, :].copy(), N=np.array([64, 64, 64]))

    r = subprocess.run([opcount, "64", "256"], capture_output=True, text=True, check=True)
    with open(os.path.join(HERE, "opcount.txt"), "w") as f:
        f.write(r.stdout)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
