"""Asynchronous single-handle path (cbns_upload_Q_async, cbns_step_async,
cbns_download_Q_async, cbns_wait, cbns_poll).

Enqueuing only reorders when the host waits, never what the device computes:
every state must be bitwise the one the synchronous calls give, also when the
upload of one state, the steps and the download of another are in flight
together (host copies on the handle's second stream, kernels on its first).
"""
import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import tgv_params

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("built")]


def states(p, n):
    from cbns3d_cart_mpi_gb300.solver import initial_condition_perturbed
    return [initial_condition_perturbed(p, seed=40 + q, amp=1e-3) for q in range(n)]


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_async_pipeline_equals_synchronous_calls(precision):
    from cbns3d_cart_mpi_gb300.solver import Solver
    p = tgv_params(24, JM=20, KM=28, Re=900.0, Mach=0.15)
    Qs = states(p, 4)
    ref = []
    s = Solver(p, precision=precision)
    for Q in Qs:
        s.upload_Q(Q, 0.0)
        for _ in range(2):
            s.step()
        ref.append(s.download_Q())
    s.close()

    a = Solver(p, precision=precision)
    ins = [a.pinned_state() for _ in Qs]
    outs = [a.pinned_state() for _ in Qs]
    for q, Q in enumerate(Qs):
        ins[q][...] = Q
        outs[q][...] = np.nan
    # Everything enqueued before the first wait: upload n+1 overlaps the steps of n.
    for q in range(len(Qs)):
        a.upload_Q_async(ins[q], 0.0)
        a.step_async()
        a.step_async()
        a.download_Q_async(outs[q])
    dt_t = a.wait()
    assert dt_t is not None and a.poll()
    for q in range(len(Qs)):
        assert np.array_equal(outs[q], ref[q]), q
    a.close()


def test_async_reuses_one_pinned_pair_and_reports_finish():
    """The bench's end-to-end loop: one input and one output buffer reused every
    step.  Downloads are ordered behind the previous one, so the last result is
    the last step's; cbns_wait reports CBNS_FINISHED once t_end is reached."""
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition
    p = tgv_params(16, JM=12, KM=20, t_end=0.02)
    Q0 = initial_condition(p)
    s = Solver(p)
    s.upload_Q(Q0, 0.0)
    s.step()
    one = s.download_Q()
    a = Solver(p)
    hin, hout = a.pinned_state(), a.pinned_state()
    hin[...] = Q0
    for _ in range(5):
        a.upload_Q_async(hin, 0.0)
        a.step_async()
        a.download_Q_async(hout)
    a.wait()
    assert np.array_equal(hout, one)
    # run past t_end asynchronously: the step graph stops by itself
    a.upload_Q_async(hin, 0.0)
    for _ in range(40):
        a.step_async()
    assert a.wait() is None
    s.close()
    a.close()


def test_async_rejects_bad_arguments():
    """Null handles and buffers come back as CBNS_ERR_INVALID_ARG, before any
    work is enqueued; the handle stays usable."""
    import ctypes

    from cbns3d_cart_mpi_gb300 import _lib
    from cbns3d_cart_mpi_gb300._abi import CBNS_ERR_INVALID_ARG
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition
    lib = _lib.gpu()
    p = tgv_params(8, JM=8, KM=9)
    s = Solver(p)
    assert lib.cbns_upload_Q_async(None, None, 0.0) == CBNS_ERR_INVALID_ARG
    assert lib.cbns_upload_Q_async(s._h, None, 0.0) == CBNS_ERR_INVALID_ARG
    assert lib.cbns_download_Q_async(s._h, None) == CBNS_ERR_INVALID_ARG
    assert lib.cbns_step_async(None, 1.0) == CBNS_ERR_INVALID_ARG
    assert lib.cbns_wait(None, None, None) == CBNS_ERR_INVALID_ARG
    assert lib.cbns_poll(s._h, None) == CBNS_ERR_INVALID_ARG
    done = ctypes.c_int(-1)
    assert lib.cbns_poll(s._h, ctypes.byref(done)) == 0 and done.value == 1
    hin = s.pinned_state()
    hin[...] = initial_condition(p)
    s.upload_Q_async(hin, 0.0)
    s.step_async()
    assert s.wait() is not None
    s.close()
