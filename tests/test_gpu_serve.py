"""Serving loop: continuous batching of solve requests.

Each request's final state must be bitwise the state of the same solve stepped
alone (batching only regroups launches), whether it ran with others, arrived
while others were running, or waited for memory.  Failures and cancellations
are injected on the host (a request whose initial state holds a negative
density, a cancel call) and must leave the other requests' results unchanged.
"""
import time

import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import (CBNS_ERR_CANCELLED, CBNS_ERR_NONPHYSICAL, CBNS_ERR_TIMEOUT, CBNS_OK, NG,
                                        tgv_params)

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("built")]

REQS = [dict(N=16, JM=16, KM=16, Re=1600.0, Mach=0.1, t_end=0.10, seed=1),
        dict(N=12, JM=20, KM=24, Re=500.0, Mach=0.25, t_end=0.05, seed=2),
        dict(N=24, JM=8, KM=12, Re=3000.0, Mach=0.05, t_end=0.02, seed=3),
        dict(N=20, JM=20, KM=20, Re=900.0, Mach=0.15, t_end=0.08, seed=4)]


def params(r):
    return tgv_params(r["N"], JM=r["JM"], KM=r["KM"], Re=r["Re"], Mach=r["Mach"], t_end=r["t_end"])


def shape(p):
    return (p.KM + 2 * NG, p.JM + 2 * NG, p.IM + 2 * NG, 5)


def solo(r, precision):
    from cbns3d_cart_mpi_gb300.solver import Solver
    p = params(r)
    s = Solver(p, precision=precision)
    s.init_tgv(seed=r["seed"], amp=1e-3, nmodes=16, kmax=4)
    steps = 0
    while True:
        n = s.run(25)
        steps += n
        if n < 25:
            break
    return s.download_Q(), steps


def test_device_initial_condition_matches_host():
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition_perturbed
    p = tgv_params(24, JM=20, KM=16, Re=700.0, Mach=0.2)
    a = Solver(p)
    a.init_tgv(seed=5, amp=1e-3, nmodes=16, kmax=4)
    b = Solver(p)
    b.upload_Q(initial_condition_perturbed(p, seed=5, amp=1e-3, nmodes=16, kmax=4), 0.0)
    np.testing.assert_allclose(a.download_Q(), b.download_Q(), rtol=1e-14, atol=1e-15)


# A request long enough (about 340 steps of 32^3) that later ones arrive while it runs.
LONG = dict(N=32, JM=32, KM=32, Re=1200.0, Mach=0.1, t_end=1.0, seed=7)


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed", "fp64_ff"])
def test_results_same_alone_and_in_the_mix(precision):
    """Two requests start; once the server has stepped them for a round, two more
    arrive.  The late ones must be admitted after the first ones and before the
    long one is done (their work overlaps on the device: at least three requests
    active at once), and every result must be bitwise its solo result."""
    from cbns3d_cart_mpi_gb300.solver import Server
    reqs = [LONG, REQS[1], REQS[2], REQS[3]]
    ref = [solo(r, precision) for r in reqs]
    sv = Server(precision=precision, steps_per_round=7)
    ids = [sv.submit_tgv(params(r), seed=r["seed"], amp=1e-3, nmodes=16, kmax=4, keep_state=True)
           for r in reqs[:2]]
    t0 = time.time()
    while sv.stats()["rounds"] < 1:  # the first two are on the device
        assert time.time() - t0 < 60.0, "the server did not start a round"
        time.sleep(0.001)
    ids += [sv.submit_tgv(params(r), seed=r["seed"], amp=1e-3, nmodes=16, kmax=4, keep_state=True)
            for r in reqs[2:]]
    infos = []
    for rid, r, (Qref, nref) in zip(ids, reqs, ref):
        info = sv.wait(rid, timeout=120.0)
        assert info["status"] == CBNS_OK, info
        assert info["steps"] == nref
        assert abs(info["t_final"] - r["t_end"]) < 1e-5 + 1e-15
        Q = sv.result(rid, shape(params(r)))
        assert np.array_equal(Q, Qref), r
        infos.append(info)
    long_info = infos[0]
    for late in infos[2:]:
        assert long_info["admit_s"] < late["admit_s"] < long_info["done_s"], (long_info, late)
    st = sv.stats()
    assert st["peak_active"] >= 3, st
    assert st["completed"] == 4 and st["failed"] == 0
    print(precision, "long request admitted %.4f done %.4f; late requests admitted %s; peak active %d" % (
        long_info["admit_s"], long_info["done_s"], [round(x["admit_s"], 4) for x in infos[2:]],
        st["peak_active"]))
    sv.close()


def test_admission_respects_the_memory_budget():
    from cbns3d_cart_mpi_gb300.solver import Server, footprint
    fps = [footprint(r["N"], r["JM"], r["KM"]) for r in REQS]
    budget = int(1.5 * max(fps))
    sv = Server(precision="fp64", memory_budget_bytes=budget, steps_per_round=5)
    ids = [sv.submit_tgv(params(r), seed=r["seed"], amp=1e-3, nmodes=16, kmax=4) for r in REQS]
    infos = [sv.wait(i, timeout=120.0) for i in ids]
    assert all(x["status"] == CBNS_OK for x in infos)
    assert [x["device_bytes"] for x in infos] == fps
    st = sv.stats()
    assert st["completed"] == 4 and st["budget_bytes"] == budget and st["used_bytes"] == 0
    # At every admission, the requests then running fit the budget together ...
    for a in infos:
        running = [x for x in infos if x["admit_s"] <= a["admit_s"] < x["done_s"]]
        assert sum(x["device_bytes"] for x in running) <= budget
    # ... and the budget made some of them wait (all four together do not fit).
    assert sum(fps) > budget and st["peak_active"] < 4
    assert max(x["admit_s"] - x["submit_s"] for x in infos) > 0
    sv.close()


def test_a_failing_request_leaves_the_others_unchanged():
    from cbns3d_cart_mpi_gb300.solver import Server, initial_condition_perturbed
    ref = [solo(r, "fp64") for r in REQS[:2]]
    sv = Server(precision="fp64", steps_per_round=4)
    ok = [sv.submit_tgv(params(r), seed=r["seed"], amp=1e-3, nmodes=16, kmax=4, keep_state=True) for r in REQS[:2]]
    pb = params(REQS[3])
    Qbad = initial_condition_perturbed(pb, seed=9, amp=1e-3)
    Qbad[NG + 2, NG + 3, NG + 4, 0] = -1.0  # host-injected non-physical cell
    bad = sv.submit(pb, Qbad)
    assert sv.wait(bad, timeout=120.0)["status"] == CBNS_ERR_NONPHYSICAL
    for rid, r, (Qref, _) in zip(ok, REQS[:2], ref):
        assert sv.wait(rid, timeout=120.0)["status"] == CBNS_OK
        assert np.array_equal(sv.result(rid, shape(params(r))), Qref)
    sv.close()


def test_cancel_and_wait_timeout():
    from cbns3d_cart_mpi_gb300.solver import Server
    sv = Server(precision="fp64", steps_per_round=2)
    long = dict(REQS[0], t_end=1e9)
    rid = sv.submit_tgv(params(long), seed=1, amp=1e-3, nmodes=16, kmax=4)
    other = sv.submit_tgv(params(REQS[2]), seed=3, amp=1e-3, nmodes=16, kmax=4, keep_state=True)
    assert sv.wait(rid, timeout=0.01)["status"] == CBNS_ERR_TIMEOUT
    sv.cancel(rid)
    assert sv.wait(rid, timeout=60.0)["status"] == CBNS_ERR_CANCELLED
    assert sv.wait(other, timeout=60.0)["status"] == CBNS_OK
    Qref, _ = solo(REQS[2], "fp64")
    assert np.array_equal(sv.result(other, shape(params(REQS[2]))), Qref)
    sv.close()
