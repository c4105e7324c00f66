"""Batched ensembles: many solves of uneven size and parameters in one set of
launches over a flattened tile table, replayed as a CUDA graph.  Stepping a
solve in a batch must give bitwise the state stepping it alone gives, under
every launch shape the autotuner may pick, and each solve stops at its own t_end."""
import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import tgv_params

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("built")]

# The last case has an odd JM: the FP32-mixed face kernels take two rows per
# thread, and its last row runs unpaired.
CASES = [dict(N=16, JM=16, KM=16, Re=1600.0, Mach=0.1), dict(N=12, JM=20, KM=24, Re=500.0, Mach=0.25),
         dict(N=40, JM=8, KM=12, Re=3000.0, Mach=0.05), dict(N=20, JM=13, KM=10, Re=800.0, Mach=0.15)]


def make(precision, t_ends=None):
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition_perturbed
    out = []
    for i, c in enumerate(CASES):
        te = 20.0 if t_ends is None else t_ends[i]
        p = tgv_params(c["N"], JM=c["JM"], KM=c["KM"], Re=c["Re"], Mach=c["Mach"], t_end=te)
        s = Solver(p, precision=precision)
        s.upload_Q(initial_condition_perturbed(p, seed=100 + i, amp=1e-3), 0.0)
        out.append(s)
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed", "fp64_ff"])
def test_batch_equals_alone_bitwise(precision):
    from cbns3d_cart_mpi_gb300.solver import Batch
    alone = make(precision)
    for s in alone:
        for _ in range(4):
            s.step()
    batched = make(precision)
    b = Batch(batched)
    assert b.run(4) == [4] * len(CASES)
    for a, s in zip(alone, batched):
        assert np.array_equal(a.download_Q(), s.download_Q())
        assert a.time() == s.time()


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed", "fp64_ff"])
def test_every_launch_shape_gives_the_same_bits(precision):
    from cbns3d_cart_mpi_gb300.solver import Batch
    ref = None
    for rows, cps in [(4, 0), (2, 2), (8, 4), (4, 8)]:
        ss = make(precision)
        b = Batch(ss)
        b.set_config(rows, cps)
        assert b.config == {"tile_rows": rows, "ctas_per_sm": cps}
        b.run(3)
        got = [s.download_Q() for s in ss]
        if ref is None:
            ref = got
        else:
            for x, y in zip(ref, got):
                assert np.array_equal(x, y), (rows, cps)


def test_autotune_restores_state_and_picks_a_candidate():
    from cbns3d_cart_mpi_gb300.solver import Batch
    plain = make("fp32_mixed")
    Batch(plain).run(3)
    tuned = make("fp32_mixed")
    b = Batch(tuned)
    res = b.autotune(reps=1)
    assert len(res) == 12 and all(ms > 0 for _, _, ms in res)
    best = min(res, key=lambda r: r[2])
    assert b.config == {"tile_rows": best[0], "ctas_per_sm": best[1]}
    assert b.run(3) == [3] * len(CASES)
    for x, y in zip(plain, tuned):
        assert np.array_equal(x.download_Q(), y.download_Q())


def test_each_solve_stops_at_its_own_t_end():
    from cbns3d_cart_mpi_gb300.solver import Batch
    ss = make("fp64", t_ends=[0.02, 20.0, 0.005, 20.0])
    b = Batch(ss)
    steps = b.run(10)
    assert steps[1] == 10 and steps[0] < 10 and steps[2] < steps[0]
    for s, te in zip(ss, [0.02, 20.0, 0.005, 20.0]):
        t, _ = s.time()
        if te < 1:
            assert abs(t - te) < 1e-5 + 1e-15 and t + 1e-5 > te


def test_batch_rejects_a_handle_listed_twice():
    """A handle listed twice would put its tiles in the table twice, and two CTAs
    would update the same cells and control block in every stage."""
    from cbns3d_cart_mpi_gb300._abi import CBNS_ERR_INVALID_ARG
    from cbns3d_cart_mpi_gb300.solver import Batch, CbnsError
    solves = make("fp64")
    with pytest.raises(CbnsError) as e:
        Batch([solves[0], solves[1], solves[0]])
    assert e.value.status == CBNS_ERR_INVALID_ARG
    assert "more than once" in str(e.value)
