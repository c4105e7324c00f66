"""The oracle's CPU restatement against the reference's own outputs (CPU only).

tests/golden/ holds states produced by the reference solver compiled
unmodified from its sources (tests/golden/make_golden.py).  The restatement in
oracle/cbns_oracle.c must reproduce them bit for bit; that pins the oracle
before any GPU result is compared with it.
"""
import os

import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import NG, tgv_params

pytestmark = pytest.mark.usefixtures("built")


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def pad(Qi):
    """Interior state (KM, JM, IM, 5) -> padded array with zero ghosts."""
    KM, JM, IM, _ = Qi.shape
    Q = np.zeros((KM + 2 * NG, JM + 2 * NG, IM + 2 * NG, 5))
    Q[NG:-NG, NG:-NG, NG:-NG] = Qi
    return Q


def interior(Q):
    return Q[NG:-NG, NG:-NG, NG:-NG]


def oracle_from(golden, params):
    from oracle.oracle import OracleBlock
    b = OracleBlock(params)
    b.set_Q(pad(golden["Q0"]), 0.0)
    return b


def test_initial_condition_bitwise(golden_dir):
    from oracle.oracle import OracleBlock
    g = load(golden_dir, "tgv16.npz")
    b = OracleBlock(tgv_params(16))
    b.initial_condition()
    # libm sin/cos on another host may differ in the last place; here they agree.
    np.testing.assert_allclose(interior(b.get_Q()), g["Q0"], rtol=4e-16, atol=0)


def test_stage1_bitwise(golden_dir):
    g = load(golden_dir, "tgv16.npz")
    b = oracle_from(g, tgv_params(16))
    dt = b.calc_dt()
    assert dt == g["dt"][0]
    b.stage(dt, 1)
    assert np.array_equal(interior(b.get_Q_p()), g["Qp_stage1"])


def test_three_steps_bitwise(golden_dir):
    g = load(golden_dir, "tgv16.npz")
    b = oracle_from(g, tgv_params(16))
    for n in range(3):
        dt, t = b.step()
        assert dt == g["dt"][n] and t == g["t"][n]
    assert np.array_equal(interior(b.get_Q()), g["Q3"])


def test_ghost_fill_is_periodic_wrap(golden_dir):
    g = load(golden_dir, "tgv16.npz")
    b = oracle_from(g, tgv_params(16))
    Q = b.get_Q()
    Qi = g["Q0"]
    # Every padded cell holds the interior cell congruent to it modulo N.
    idx = (np.arange(-NG, 16 + NG) % 16)
    expect = Qi[np.ix_(idx, idx, idx)]
    assert np.array_equal(Q, expect)


@pytest.mark.parametrize("name,steps,key", [("tgv_odd.npz", 2, "Q2"), ("tgv_min.npz", 2, "Q2"),
                                            ("tgv_pert.npz", 3, "Q3")])
def test_cases_bitwise(golden_dir, name, steps, key):
    g = load(golden_dir, name)
    IM, JM, KM = (int(x) for x in g["N"])
    kw = {}
    if "Re" in g.files:
        kw = dict(Re=float(g["Re"]), Mach=float(g["Mach"]))
    p = tgv_params(IM, JM=JM, KM=KM, **kw)
    b = oracle_from(g, p)
    for n in range(steps):
        dt, t = b.step()
        assert dt == g["dt"][n] and t == g["t"][n]
    assert np.array_equal(interior(b.get_Q()), g[key])


def test_history_64_first_steps(golden_dir):
    """64^3: the first 10 steps of the reference's 100-step history, bitwise."""
    from oracle.oracle import OracleBlock
    g = load(golden_dir, "tgv64_hist.npz")
    b = OracleBlock(tgv_params(64))
    b.initial_condition()
    for n in range(10):
        dt, t = b.step()
        assert dt == g["dt"][n], n
    Qi = interior(b.get_Q()).reshape(-1, 5)
    np.testing.assert_array_equal(Qi.sum(axis=0), g["sums"][1])
    np.testing.assert_array_equal(np.abs(Qi).max(axis=0), g["absmax"][1])
    ke, en = b.diagnostics()
    assert ke == g["ke"][1] and en == g["enstrophy"][1]


def test_thread_count_does_not_change_results(golden_dir):
    """The oracle's OpenMP loops are per-cell independent: 1 thread == many."""
    import subprocess
    import sys
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r)\n"
        "from oracle.oracle import OracleBlock\n"
        "from cbns3d_cart_mpi_gb300._abi import tgv_params\n"
        "b = OracleBlock(tgv_params(12, JM=16, KM=20)); b.initial_condition(); b.step(); b.step()\n"
        "sys.stdout.buffer.write(b.get_Q().tobytes())\n" % os.path.dirname(os.path.dirname(golden_dir)))
    outs = []
    for th in ("1", "3"):
        env = dict(os.environ, OMP_NUM_THREADS=th)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, env=env, check=True)
        outs.append(r.stdout)
    assert outs[0] == outs[1] and len(outs[0]) > 0


def test_live_reference_matches_port(tmp_path):
    """When the reference's sources are present (oracle/_ref built), run it on a
    fresh perturbed case and compare with the port bit for bit."""
    import subprocess
    from oracle.build import build_ref
    from oracle.oracle import OracleBlock, read_state, write_state
    from cbns3d_cart_mpi_gb300.params import write_input_txt
    from cbns3d_cart_mpi_gb300.solver import initial_condition_perturbed
    res = build_ref()
    if res is None:
        pytest.skip("reference sources not present on this machine")
    p = tgv_params(10, JM=9, KM=11, Re=2000.0, Mach=0.15)
    Q0 = initial_condition_perturbed(p, seed=11, amp=2e-3)
    write_input_txt(p, str(tmp_path / "input.txt"))
    write_state(str(tmp_path / "inj.dat"), Q0, 0.0)
    subprocess.run([res[0], str(tmp_path), "2", "1", "--inject", "inj.dat"], check=True, capture_output=True)
    _, Qref = read_state(str(tmp_path / "q_000002.bin"))
    b = OracleBlock(p)
    b.set_Q(Q0, 0.0)
    b.step()
    b.step()
    assert np.array_equal(b.get_Q(), Qref)
