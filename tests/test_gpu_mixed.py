"""FP32-mixed precision mode against the binary64 oracle.

FP32-mixed runs the WENO5 reconstruction, the Roe eigenvector projections and
the inviscid and viscous fluxes in binary32, on the perturbation of the state
about the free stream (rho = 1, p = 1/(gamma M^2)); the RK3 accumulation of the
conserved state stays binary64.  The bound is 1e-5 relative L-inf
per conserved field against the binary64 oracle; the tests check it on the
64^3 100-step case and state the measured error.
"""
import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import NG, tgv_params

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("built")]


def interior(Q):
    return Q[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)


def field_errors(a, b):
    a, b = interior(a), interior(b)
    return np.abs(a - b).max(axis=0) / np.abs(b).max(axis=0)


def test_mixed_64_100_steps_within_1e5_of_oracle():
    from oracle.oracle import OracleBlock
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition
    p = tgv_params(64)
    Q0 = initial_condition(p)
    s = Solver(p, precision="fp32_mixed")
    s.upload_Q(Q0, 0.0)
    o = OracleBlock(p)
    o.set_Q(Q0, 0.0)
    for n in range(100):
        dt, t = s.step()
        dto, to = o.step()
        assert abs(dt - dto) <= 1e-6 * dto, n
    err = field_errors(s.download_Q(), o.get_Q())
    print("FP32-mixed 64^3 100 steps, rel Linf per field:", err)
    assert (err <= 1e-5).all(), err
    ke, en = s.diagnostics()
    ko, eo = o.diagnostics()
    assert abs(ke - ko) <= 1e-6 * ko and abs(en - eo) <= 1e-5 * eo


def test_mixed_free_stream_is_preserved():
    from cbns3d_cart_mpi_gb300.solver import Solver
    p = tgv_params(12, JM=8, KM=10)
    Q = np.zeros((10 + 2 * NG, 8 + 2 * NG, 12 + 2 * NG, 5))
    rho, u, v, w, pr = 1.1, 0.3, -0.2, 0.15, 1.02 * p.p_inf
    Q[...] = [rho, rho * u, rho * v, rho * w, pr / p.gam1 + 0.5 * rho * (u * u + v * v + w * w)]
    s = Solver(p, precision="fp32_mixed")
    s.upload_Q(Q, 0.0)
    s.stage(1e-3, 1)
    assert np.array_equal(s.download_Q_p(), Q)


def test_mixed_graph_matches_step_loop():
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition_perturbed
    p = tgv_params(24, JM=20, KM=28, Re=900.0, Mach=0.15, t_end=0.05)
    Q0 = initial_condition_perturbed(p, seed=2, amp=1e-3)
    a = Solver(p, precision="fp32_mixed")
    b = Solver(p, precision="fp32_mixed")
    a.upload_Q(Q0, 0.0)
    b.upload_Q(Q0, 0.0)
    n = 0
    while a.step() is not None:
        n += 1
    assert b.run(100) == n
    assert np.array_equal(a.download_Q(), b.download_Q())


def test_mixed_prims_download_is_binary64_of_Q():
    from oracle.oracle import OracleBlock
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition
    p = tgv_params(16)
    s = Solver(p, precision="fp32_mixed")
    s.upload_Q(initial_condition(p), 0.0)
    s.step()
    Q = s.download_Q()
    o = OracleBlock(p)
    o.set_Q(Q, 0.0)
    gp, op = s.download_prims(), o.get_prims()
    for k in ("rho", "u", "v", "w", "p", "T"):
        np.testing.assert_allclose(gp[k], op[k], rtol=1e-15, atol=1e-15, err_msg=k)


@pytest.mark.parametrize("Re,Mach,seed", [(400.0, 0.3, 21), (3200.0, 0.05, 22)])
def test_mixed_parameter_corners_within_1e5_of_oracle(Re, Mach, seed):
    """Corners of the ensemble/serving parameter range (Ma 0.05 has the largest
    mean pressure relative to the fluctuations, the hardest case for the
    perturbation form): 40 steps of perturbed data against the binary64 oracle,
    per field over its scale (the momentum fields share one)."""
    from oracle.oracle import OracleBlock
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition_perturbed
    p = tgv_params(24, JM=20, KM=16, Re=Re, Mach=Mach)
    Q0 = initial_condition_perturbed(p, seed=seed, amp=1e-3, nmodes=16, kmax=4)
    s = Solver(p, precision="fp32_mixed")
    s.upload_Q(Q0, 0.0)
    o = OracleBlock(p)
    o.set_Q(Q0, 0.0)
    for _ in range(40):
        s.step()
        o.step()
    a = s.download_Q()[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)
    b = o.get_Q()[NG:-NG, NG:-NG, NG:-NG].reshape(-1, 5)
    scale = np.abs(b).max(axis=0)
    scale[1:4] = scale[1:4].max()
    err = np.abs(a - b).max(axis=0) / scale
    print("FP32-mixed Re %g Ma %g, 40 steps: error over field scale" % (Re, Mach), err)
    assert (err <= 1e-5).all(), err
