"""The C++ driver (lib/cbns3d_gb300): the reference's time loop on one GPU.

Runs it in a scratch directory from an input.txt, as the reference is run, and
checks its console protocol ("n, dt, t" per step), its output directories, the
VTK files (text-identical to the host writer fed with the library's state after
the same steps) and its checkpoint (bitwise the library's state)."""
import subprocess

import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import tgv_params

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("built")]


def test_driver_run(tmp_path):
    from cbns3d_cart_mpi_gb300 import build
    from cbns3d_cart_mpi_gb300.params import write_input_txt
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition, output_vtk_xml, read_bin

    # dt is about 0.0103, so t_end = 0.06 takes six steps (the last one clipped);
    # outputs at start, after t = 0.03 and at the end; checkpoints after steps 3, 6.
    p = tgv_params(12, JM=8, KM=10, t_end=0.06, nstep_max=100)
    p.checkpoint_freq = 3
    p.num_output = 2
    write_input_txt(p, str(tmp_path / "input.txt"))
    r = subprocess.run([build.DRIVER, "1", "1", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    steps = [ln for ln in r.stdout.splitlines() if ln.count(",") == 2 and ln.split(",")[0].strip().isdigit()]
    assert len(steps) == 6 and "Finished!" in r.stdout
    for d in ("output000", "output001", "output002"):
        assert (tmp_path / d / "output000.vtr").exists() and (tmp_path / d / "output.vtm").exists()

    # The same six steps through the library.
    s = Solver(p)
    s.upload_Q(initial_condition(p), 0.0)
    for _ in range(6):
        s.step()
    t_lib, _ = s.time()
    t_ck, Qck = read_bin(str(tmp_path / "checkpoint000.dat"), 12, 8, 10)
    assert np.array_equal(Qck, s.download_Q()) and t_ck == t_lib
    last = "output002"
    ref_dir = tmp_path / "ref"
    ref_dir.mkdir()
    output_vtk_xml(str(ref_dir), "output", p, s.download_prims())
    assert (tmp_path / last / "output000.vtr").read_text() == (ref_dir / "output000.vtr").read_text()


def test_driver_restarts_from_its_checkpoint(tmp_path):
    """is_restart = 0 resumes from checkpoint000.dat (src/cbns3d.cpp:136-144),
    which the driver streams to the device; the resumed run ends bitwise where
    the library ends after loading the same file and taking the same steps."""
    from cbns3d_cart_mpi_gb300 import build
    from cbns3d_cart_mpi_gb300.params import write_input_txt
    from cbns3d_cart_mpi_gb300.solver import Solver, read_bin

    p = tgv_params(12, JM=8, KM=10, t_end=0.03, nstep_max=100)
    p.checkpoint_freq = 3
    p.num_output = 1
    write_input_txt(p, str(tmp_path / "input.txt"))
    r = subprocess.run([build.DRIVER, "1", "1", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    first = (tmp_path / "checkpoint000.dat").read_bytes()
    (tmp_path / "first.dat").write_bytes(first)
    p.is_restart = 0
    p.t_end = 0.06
    write_input_txt(p, str(tmp_path / "input.txt"))
    r = subprocess.run([build.DRIVER, "1", "1", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    steps = [ln for ln in r.stdout.splitlines() if ln.count(",") == 2 and ln.split(",")[0].strip().isdigit()]
    assert len(steps) == 3 and "Finished!" in r.stdout

    s = Solver(p)
    s.load_checkpoint(str(tmp_path / "first.dat"))
    for _ in range(3):
        s.step()
    t_ck, Qck = read_bin(str(tmp_path / "checkpoint000.dat"), 12, 8, 10)
    assert np.array_equal(Qck, s.download_Q()) and t_ck == s.time()[0]


def test_driver_rejects_more_than_one_process(tmp_path):
    from cbns3d_cart_mpi_gb300 import build
    from cbns3d_cart_mpi_gb300.params import write_input_txt
    write_input_txt(tgv_params(8), str(tmp_path / "input.txt"))
    r = subprocess.run([build.DRIVER, "2", "1", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "dimX * dimY * dimZ" in r.stderr


def test_driver_float_float_precision(tmp_path):
    """CBNS_PRECISION=fp64_ff runs the reference's loop with float-float
    arithmetic: the driver's checkpoint is bitwise the library's fp64_ff state
    after the same steps, and within the binary64 parity bar of binary64's."""
    import os

    from cbns3d_cart_mpi_gb300 import build
    from cbns3d_cart_mpi_gb300.params import write_input_txt
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition, read_bin

    p = tgv_params(12, JM=8, KM=10, t_end=0.06, nstep_max=100)
    p.checkpoint_freq = 3
    p.num_output = 1
    write_input_txt(p, str(tmp_path / "input.txt"))
    env = dict(os.environ, CBNS_PRECISION="fp64_ff")
    r = subprocess.run([build.DRIVER, "1", "1", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=120,
                       env=env)
    assert r.returncode == 0, r.stderr
    t_ck, Qck = read_bin(str(tmp_path / "checkpoint000.dat"), 12, 8, 10)
    states = {}
    for prec in ("fp64_ff", "fp64"):
        s = Solver(p, precision=prec)
        s.upload_Q(initial_condition(p), 0.0)
        for _ in range(6):
            s.step()
        states[prec] = s.download_Q()
        s.close()
    assert np.array_equal(Qck, states["fp64_ff"])
    a = Qck[4:-4, 4:-4, 4:-4].reshape(-1, 5)
    b = states["fp64"][4:-4, 4:-4, 4:-4].reshape(-1, 5)
    assert (np.abs(a - b).max(axis=0) / np.abs(b).max(axis=0) <= 1e-11).all()


def test_driver_rejects_an_unknown_precision(tmp_path):
    import os

    from cbns3d_cart_mpi_gb300 import build
    from cbns3d_cart_mpi_gb300.params import write_input_txt
    write_input_txt(tgv_params(8), str(tmp_path / "input.txt"))
    env = dict(os.environ, CBNS_PRECISION="fp16")
    r = subprocess.run([build.DRIVER, "1", "1", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=60,
                       env=env)
    assert r.returncode != 0 and "CBNS_PRECISION" in r.stderr
