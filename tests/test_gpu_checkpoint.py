"""Checkpoints streamed between a file and the device (cbns_load_checkpoint,
cbns_save_checkpoint) in the reference's output_bin format (Block3d::read_bin /
output_bin, src/Block3d.cpp:318-357 and :964-987).

Loading must equal read_bin + cbns_upload_Q (the reference's restart path),
saving must write the bytes the host writer writes for the downloaded state, a
saved state must continue bitwise like the solve it came from at a given dt,
shapes whose
state spans several pinned chunks (8 MiB) included, and a failed load must leave
the solve unchanged.  The serving loop can start a request from a checkpoint
file that its worker reads at admission."""
import os

import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import CBNS_ERR_FORMAT, CBNS_ERR_IO, CBNS_OK, NG, tgv_params

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("built")]


def test_load_reference_checkpoint(golden_dir):
    from cbns3d_cart_mpi_gb300.solver import Solver, read_bin
    path = os.path.join(golden_dir, "ckpt_4x5x6.dat")  # written by the reference's output_bin
    p = tgv_params(4, JM=5, KM=6)
    t_h, Q = read_bin(path, 4, 5, 6)
    a = Solver(p)
    t = a.load_checkpoint(path)
    b = Solver(p)
    b.upload_Q(Q, t_h)
    assert t == t_h and a.time()[0] == t_h
    assert np.array_equal(a.download_Q(), b.download_Q())
    a.step()
    b.step()
    assert np.array_equal(a.download_Q(), b.download_Q()) and a.time() == b.time()


@pytest.mark.parametrize("shape,precision", [((4, 5, 6), "fp64"), ((60, 52, 44), "fp64"), ((96, 96, 96), "fp64"),
                                             ((16, 12, 20), "fp32_mixed")])  # 1, 2 and 6 chunks
def test_save_matches_host_writer_and_continues(tmp_path, shape, precision):
    from cbns3d_cart_mpi_gb300.solver import Solver, output_bin
    IM, JM, KM = shape
    p = tgv_params(IM, JM=JM, KM=KM)
    s = Solver(p, precision=precision)
    s.init_tgv(seed=3, amp=1e-3, nmodes=8, kmax=3)
    s.step()
    s.step()
    s.save_checkpoint(str(tmp_path / "a.dat"))
    t, _ = s.time()
    output_bin(str(tmp_path / "b.dat"), t, s.download_Q(), IM, JM, KM)
    assert (tmp_path / "a.dat").read_bytes() == (tmp_path / "b.dat").read_bytes()
    r = Solver(p, precision=precision)
    assert r.load_checkpoint(str(tmp_path / "a.dat")) == t
    assert np.array_equal(r.download_Q(), s.download_Q())
    # A restart sets the lagged mu to 1 before its first calc_dt, so the solves
    # continue identically at a given dt (mu is recomputed before every use in
    # the viscous fluxes).
    for stage in (1, 2, 3):
        s.stage(1.0e-3, stage)
        r.stage(1.0e-3, stage)
    assert np.array_equal(r.download_Q(), s.download_Q())


def test_failed_loads_leave_the_state_unchanged(tmp_path):
    from cbns3d_cart_mpi_gb300.solver import CbnsError, Solver
    p = tgv_params(8, JM=8, KM=8)
    s = Solver(p)
    s.init_tgv(seed=2, amp=1e-3, nmodes=4, kmax=2)
    s.step()
    Q0, t0 = s.download_Q(), s.time()
    other = Solver(tgv_params(8, JM=8, KM=9))
    other.init_tgv()
    other.save_checkpoint(str(tmp_path / "wrong.dat"))
    s.save_checkpoint(str(tmp_path / "good.dat"))
    (tmp_path / "short.dat").write_bytes((tmp_path / "good.dat").read_bytes()[:10000])
    for name, status in [("wrong.dat", CBNS_ERR_FORMAT), ("short.dat", CBNS_ERR_FORMAT),
                         ("missing.dat", CBNS_ERR_IO)]:
        with pytest.raises(CbnsError) as e:
            s.load_checkpoint(str(tmp_path / name))
        assert e.value.status == status, name
        assert np.array_equal(s.download_Q(), Q0) and s.time() == t0
    with pytest.raises(CbnsError) as e:
        s.save_checkpoint(str(tmp_path / "no_such_dir" / "x.dat"))
    assert e.value.status == CBNS_ERR_IO


def test_server_request_from_checkpoint(tmp_path):
    from cbns3d_cart_mpi_gb300.solver import Server, Solver
    p = tgv_params(16, JM=12, KM=20, t_end=0.05)
    s = Solver(p)
    s.init_tgv(seed=1, amp=1e-3, nmodes=8, kmax=3)
    s.step()
    ck = str(tmp_path / "ck.dat")
    s.save_checkpoint(ck)
    ref = Solver(p)
    ref.load_checkpoint(ck)
    while ref.run(25) == 25:
        pass
    sv = Server(precision="fp64", steps_per_round=3)
    rid = sv.submit_checkpoint(p, ck, keep_state=True)
    bad = sv.submit_checkpoint(p, str(tmp_path / "missing.dat"))
    info = sv.wait(rid, timeout=120.0)
    assert info["status"] == CBNS_OK
    shape = (p.KM + 2 * NG, p.JM + 2 * NG, p.IM + 2 * NG, 5)
    assert np.array_equal(sv.result(rid, shape), ref.download_Q())
    assert sv.wait(bad, timeout=60.0)["status"] == CBNS_ERR_IO
    sv.close()
