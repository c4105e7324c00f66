"""GPU path (through the C ABI) against the reference's golden states and the oracle.

Tolerances:
  * per conserved field (rho, rho*u, rho*v, rho*w, E), max|a-b| / max|b| <= 1e-11
    (the parity bar, checked after 100 RK3 steps at 64^3 and on every
    short case); the kinetic-energy and enstrophy histories to 1e-10;
  * on short runs also an absolute bound: max|a-b| <= 1e-13 times the field's
    scale, where the three momentum components share the momentum scale.  The
    per-field bound alone is loose for rho*w early on, because w starts at 0
    (max|rho*w| is 1.4e-3 after one step at 16^3).  The GPU kernels reorder
    binary64 operations (shared projections, one division per ten WENO weights,
    fused multiply-adds), so they differ from the reference by rounding only.
"""
import os

import numpy as np
import pytest

from cbns3d_cart_mpi_gb300._abi import CBNS_ERR_BAD_DIMS, CBNS_ERR_NONPHYSICAL, NG, tgv_params

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("built")]

FIELDS = ["rho", "rho*u", "rho*v", "rho*w", "E"]


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def pad(Qi):
    KM, JM, IM, _ = Qi.shape
    Q = np.zeros((KM + 2 * NG, JM + 2 * NG, IM + 2 * NG, 5))
    Q[NG:-NG, NG:-NG, NG:-NG] = Qi
    return Q


def interior(Q):
    return Q[NG:-NG, NG:-NG, NG:-NG]


def rel_linf(a, b):
    """Per-field max|a-b| / max|b| over the last axis."""
    a = a.reshape(-1, 5)
    b = b.reshape(-1, 5)
    return np.abs(a - b).max(axis=0) / np.abs(b).max(axis=0)


def assert_close(a, b, tol, what="", tight=None):
    err = rel_linf(a, b)
    assert (err <= tol).all(), "%s rel Linf %s > %g" % (what, dict(zip(FIELDS, err)), tol)
    if tight is not None:
        a2, b2 = a.reshape(-1, 5), b.reshape(-1, 5)
        scale = np.abs(b2).max(axis=0)
        scale[1:4] = scale[1:4].max()
        e2 = np.abs(a2 - b2).max(axis=0) / scale
        assert (e2 <= tight).all(), "%s scaled error %s > %g" % (what, dict(zip(FIELDS, e2)), tight)


def solver_from(Qi, params):
    from cbns3d_cart_mpi_gb300.solver import Solver
    s = Solver(params)
    s.upload_Q(pad(Qi), 0.0)
    return s


def test_upload_ghost_fill_and_prims(golden_dir):
    from oracle.oracle import OracleBlock
    g = load(golden_dir, "tgv16.npz")
    p = tgv_params(16)
    s = solver_from(g["Q0"], p)
    o = OracleBlock(p)
    o.set_Q(pad(g["Q0"]), 0.0)
    # Ghost fill is an exact copy: bitwise equal to the reference's halo sweeps.
    assert np.array_equal(s.download_Q(), o.get_Q())
    assert np.array_equal(s.download_Q_p(), o.get_Q())
    gp, op = s.download_prims(), o.get_prims()
    for k in ("rho", "u", "v", "w", "p", "T"):
        np.testing.assert_allclose(gp[k], op[k], rtol=1e-15, atol=1e-15, err_msg=k)


def test_calc_dt(golden_dir):
    g = load(golden_dir, "tgv16.npz")
    s = solver_from(g["Q0"], tgv_params(16))
    assert abs(s.calc_dt() - g["dt"][0]) <= 1e-14 * g["dt"][0]


def test_stage1(golden_dir):
    g = load(golden_dir, "tgv16.npz")
    s = solver_from(g["Q0"], tgv_params(16))
    s.stage(g["dt"][0], 1)
    assert_close(interior(s.download_Q_p()), g["Qp_stage1"], 1e-11, "stage 1", tight=1e-14)


def test_three_steps(golden_dir):
    g = load(golden_dir, "tgv16.npz")
    s = solver_from(g["Q0"], tgv_params(16))
    for n in range(3):
        dt, t = s.step()
        assert abs(dt - g["dt"][n]) <= 1e-14 * g["dt"][n]
        assert abs(t - g["t"][n]) <= 1e-14 * g["t"][n]
    assert_close(interior(s.download_Q()), g["Q3"], 1e-11, "16^3 step 3", tight=1e-13)


@pytest.mark.parametrize("name,steps,key", [("tgv_odd.npz", 2, "Q2"), ("tgv_min.npz", 2, "Q2"),
                                            ("tgv_pert.npz", 3, "Q3")])
def test_cases(golden_dir, name, steps, key):
    g = load(golden_dir, name)
    IM, JM, KM = (int(x) for x in g["N"])
    kw = dict(Re=float(g["Re"]), Mach=float(g["Mach"])) if "Re" in g.files else {}
    s = solver_from(g["Q0"], tgv_params(IM, JM=JM, KM=KM, **kw))
    for n in range(steps):
        dt, t = s.step()
        assert abs(dt - g["dt"][n]) <= 1e-14 * g["dt"][n]
    assert_close(interior(s.download_Q()), g[key], 1e-11, name, tight=1e-13)


def test_ghosts_after_step_are_periodic_images(golden_dir):
    g = load(golden_dir, "tgv_odd.npz")
    IM, JM, KM = (int(x) for x in g["N"])
    s = solver_from(g["Q0"], tgv_params(IM, JM=JM, KM=KM))
    s.step()
    Q = s.download_Q()
    Qi = interior(Q)
    ix = np.arange(-NG, IM + NG) % IM
    jx = np.arange(-NG, JM + NG) % JM
    kx = np.arange(-NG, KM + NG) % KM
    assert np.array_equal(Q, Qi[np.ix_(kx, jx, ix)])


def test_history_64_100_steps(golden_dir):
    """Parity bar: 64^3 TGV, 100 RK3 steps, against the reference's own
    history and the oracle's full state; KE and enstrophy every 10 steps."""
    from oracle.oracle import OracleBlock
    from cbns3d_cart_mpi_gb300.solver import initial_condition
    g = load(golden_dir, "tgv64_hist.npz")
    p = tgv_params(64)
    from cbns3d_cart_mpi_gb300.solver import Solver
    s = Solver(p)
    s.upload_Q(initial_condition(p), 0.0)
    o = OracleBlock(p)
    o.initial_condition()
    ke0, en0 = s.diagnostics()
    assert abs(ke0 - g["ke"][0]) <= 1e-12 * g["ke"][0]
    assert abs(en0 - g["enstrophy"][0]) <= 1e-12 * g["enstrophy"][0]
    worst_dt = worst_ke = worst_en = 0.0
    for n in range(1, 101):
        dt, t = s.step()
        o.step()
        worst_dt = max(worst_dt, abs(dt - g["dt"][n - 1]) / g["dt"][n - 1])
        assert abs(dt - g["dt"][n - 1]) <= 1e-12 * g["dt"][n - 1], n
        if n % 10 == 0:
            m = n // 10
            ke, en = s.diagnostics()
            worst_ke = max(worst_ke, abs(ke - g["ke"][m]) / g["ke"][m])
            worst_en = max(worst_en, abs(en - g["enstrophy"][m]) / g["enstrophy"][m])
            assert abs(ke - g["ke"][m]) <= 1e-10 * g["ke"][m], (n, ke, g["ke"][m])
            assert abs(en - g["enstrophy"][m]) <= 1e-10 * g["enstrophy"][m], (n, en, g["enstrophy"][m])
    Qg = s.download_Q()
    Qo = o.get_Q()
    # The measured margins (shown with pytest -s).
    print("64^3 x 100 steps vs oracle: rel Linf per field", dict(zip(FIELDS, rel_linf(interior(Qg), interior(Qo)))),
          "; dt", worst_dt, "; KE", worst_ke, "; enstrophy", worst_en)
    assert_close(interior(Qg), interior(Qo), 1e-11, "64^3 step 100 vs oracle")
    assert_close(interior(Qg)[::4, ::4, ::4], g["Q100_sub"], 1e-11, "64^3 step 100 vs reference")
    sums = interior(Qg).reshape(-1, 5).sum(axis=0)
    np.testing.assert_allclose(sums, g["sums"][10], rtol=1e-11, atol=1e-9)


def test_run_graph_matches_step_loop_and_stops_at_t_end():
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition
    p = tgv_params(16, t_end=0.03)
    Q0 = initial_condition(p)
    a, b = Solver(p), Solver(p)
    a.upload_Q(Q0, 0.0)
    b.upload_Q(Q0, 0.0)
    n = 0
    while a.step() is not None:
        n += 1
    done = b.run(50)
    assert done == n
    ta, _ = a.time()
    tb, _ = b.time()
    assert ta == tb and abs(ta - 0.03) < 1e-5 + 1e-15
    assert np.array_equal(a.download_Q(), b.download_Q())


def test_free_stream_is_preserved():
    """A uniform state has an exactly zero right-hand side: every face sees the
    same stencil, so every flux difference is 0.  Stage 1 (Q - dt*0) is then
    bitwise Q; full steps keep Q to within the rounding of the RK3 weights."""
    from cbns3d_cart_mpi_gb300.solver import Solver
    p = tgv_params(12, JM=8, KM=10)
    Q = np.zeros((10 + 2 * NG, 8 + 2 * NG, 12 + 2 * NG, 5))
    rho, u, v, w, pr = 1.1, 0.3, -0.2, 0.15, p.p_inf
    Q[...] = [rho, rho * u, rho * v, rho * w, pr / p.gam1 + 0.5 * rho * (u * u + v * v + w * w)]
    s = Solver(p)
    s.upload_Q(Q, 0.0)
    s.stage(1e-3, 1)
    assert np.array_equal(s.download_Q_p(), Q)
    s.upload_Q(Q, 0.0)
    s.step()
    s.step()
    np.testing.assert_allclose(s.download_Q(), Q, rtol=1e-15, atol=0)


def test_nonphysical_state_is_reported():
    """A host-injected negative density gives a status, not a fault."""
    from cbns3d_cart_mpi_gb300.solver import CbnsError, Solver, initial_condition
    p = tgv_params(8)
    Q = initial_condition(p)
    Q[NG + 3, NG + 3, NG + 3, 0] = -1.0
    s = Solver(p)
    s.upload_Q(Q, 0.0)
    with pytest.raises(CbnsError) as ei:
        s.step()
    assert ei.value.status == CBNS_ERR_NONPHYSICAL


def test_bad_dims_rejected():
    from cbns3d_cart_mpi_gb300.solver import CbnsError, Solver
    with pytest.raises(CbnsError) as ei:
        Solver(tgv_params(3, JM=8, KM=8))
    assert ei.value.status == CBNS_ERR_BAD_DIMS


def test_diagnostics_match_oracle():
    from oracle.oracle import OracleBlock
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition_perturbed
    p = tgv_params(24, JM=20, KM=16, Re=500.0, Mach=0.2)
    Q0 = initial_condition_perturbed(p, seed=3, amp=1e-2)
    s = Solver(p)
    s.upload_Q(Q0, 0.0)
    o = OracleBlock(p)
    o.set_Q(Q0, 0.0)
    ke, en = s.diagnostics()
    ko, eo = o.diagnostics()
    assert abs(ke - ko) <= 1e-13 * ko and abs(en - eo) <= 1e-13 * eo


@pytest.mark.parametrize("precision", ["fp64", "fp64_ff"])
@pytest.mark.parametrize("Re,Mach,shape,seed", [(400.0, 0.3, (24, 20, 16), 11), (3200.0, 0.05, (20, 28, 12), 12),
                                                (900.0, 0.15, (33, 17, 9), 13)])
def test_parameter_corners_vs_oracle(Re, Mach, shape, seed, precision):
    """The ensemble and serving workloads draw Re in [400, 3200] and Ma in
    [0.05, 0.3] with perturbed initial data: corners of that range on odd block
    shapes, 20 steps against the oracle at the parity bar and the binary64
    run's absolute bound (float-float, in its perturbation form, is as close to
    the oracle as binary64); float-float's time step, from float-float
    primitives, gets ten times binary64's bound."""
    from oracle.oracle import OracleBlock
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition_perturbed
    IM, JM, KM = shape
    p = tgv_params(IM, JM=JM, KM=KM, Re=Re, Mach=Mach)
    Q0 = initial_condition_perturbed(p, seed=seed, amp=1e-3, nmodes=16, kmax=4)
    s = Solver(p, precision=precision)
    s.upload_Q(Q0, 0.0)
    o = OracleBlock(p)
    o.set_Q(Q0, 0.0)
    dt_tol = 1e-13 if precision == "fp64" else 1e-12
    for n in range(20):
        dt, t = s.step()
        dto, to = o.step()
        assert abs(dt - dto) <= dt_tol * dto, n
    Qg, Qo = interior(s.download_Q()), interior(o.get_Q())
    print(precision, "Re %g Ma %g rel Linf" % (Re, Mach), dict(zip(FIELDS, rel_linf(Qg, Qo))))
    assert_close(Qg, Qo, 1e-11, "%s Re %g Ma %g" % (precision, Re, Mach), tight=1e-13)


def test_fp64_ff_history_64_100_steps(golden_dir):
    """CBNS_FP64_FF (float-float faces) at the binary64 parity bar: 64^3 TGV,
    100 RK3 steps, against the reference's own state (every 4th cell) and its
    KE and enstrophy history, and against the binary64 GPU run's full state."""
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition
    g = load(golden_dir, "tgv64_hist.npz")
    p = tgv_params(64)
    states = {}
    for prec in ("fp64", "fp64_ff"):
        s = Solver(p, precision=prec)
        s.upload_Q(initial_condition(p), 0.0)
        worst_ke = worst_en = 0.0
        for n in range(1, 101):
            dt, t = s.step()
            assert abs(dt - g["dt"][n - 1]) <= 1e-12 * g["dt"][n - 1], (prec, n)
            if n % 10 == 0:
                m = n // 10
                ke, en = s.diagnostics()
                worst_ke = max(worst_ke, abs(ke - g["ke"][m]) / g["ke"][m])
                worst_en = max(worst_en, abs(en - g["enstrophy"][m]) / g["enstrophy"][m])
        assert worst_ke <= 1e-10 and worst_en <= 1e-10, (prec, worst_ke, worst_en)
        states[prec] = interior(s.download_Q())
        s.close()
        print(prec, "64^3 x 100 steps vs reference (every 4th cell): rel Linf",
              dict(zip(FIELDS, rel_linf(states[prec][::4, ::4, ::4], g["Q100_sub"]))), "; KE", worst_ke,
              "; enstrophy", worst_en)
    assert_close(states["fp64_ff"][::4, ::4, ::4], g["Q100_sub"], 1e-11, "fp64_ff step 100 vs reference")
    print("fp64_ff vs fp64 full state: rel Linf", dict(zip(FIELDS, rel_linf(states["fp64_ff"], states["fp64"]))))
    assert_close(states["fp64_ff"], states["fp64"], 1e-11, "fp64_ff vs fp64 step 100")


def test_face_reciprocal_within_one_ulp_of_ieee_division():
    """The face kernel's reciprocal (the hardware estimate and one third-order
    correction, csrc/cbns_device.cuh rcp64) against CUDA's IEEE 1.0/x on the GPU: at most one
    ulp apart, over values log-uniform in [1e-150, 1e150] (the range the WENO
    normalisation's product is admitted to) and uniform in [0.1, 10] (densities,
    sums of sqrt(rho))."""
    import ctypes

    import torch

    from cbns3d_cart_mpi_gb300 import _lib
    rng = np.random.default_rng(7)
    x = np.concatenate([10.0 ** rng.uniform(-150, 150, 1 << 20), rng.uniform(0.1, 10.0, 1 << 20)])
    dev = torch.device("cuda", torch.cuda.current_device())
    xd = torch.from_numpy(x).to(dev)
    y = torch.empty_like(xd)
    ref = torch.empty_like(xd)
    st = _lib.probe().cbns_probe_rcp64(ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                       ctypes.c_void_p(ref.data_ptr()), x.size)
    assert st == 0
    yb = y.cpu().numpy().view(np.int64)
    rb = ref.cpu().numpy().view(np.int64)
    ulps = np.abs(yb - rb)
    print("rcp64 vs 1.0/x: max %d ulp, %.3g of values differ" % (ulps.max(), (ulps > 0).mean()))
    assert ulps.max() <= 1


def test_float_float_building_blocks_against_binary64():
    """The float-float arithmetic of CBNS_FP64_FF faces (csrc/cbns_ff.cuh) on the
    GPU against numpy's binary64: the split of a binary64 value into two binary32
    parts keeps 47 bits (relative error below 2^-46); reciprocal, reciprocal
    square root and product within 2^-44 relative; sum and x*y + x within 2^-44
    of the operands' magnitudes.  Below binary32's normal range a split is 0 (an
    absolute error under 2^-126), and a value beyond it splits to NaN."""
    import ctypes

    import torch

    from cbns3d_cart_mpi_gb300 import _lib
    rng = np.random.default_rng(11)
    m = 1 << 18
    # Float-float shares binary32's exponent range: the split is tried over
    # [1e-30, 1e30], the arithmetic where results and their low parts stay normal.
    x = np.concatenate([10.0 ** rng.uniform(-30, 30, m), 10.0 ** rng.uniform(-9, 9, m), rng.uniform(0.1, 10.0, m)])
    y = np.concatenate([np.ones(m), 10.0 ** rng.uniform(-9, 9, m), rng.uniform(-10.0, 10.0, m)])
    x[m:m + m // 2] *= np.where(rng.random(m // 2) < 0.5, -1.0, 1.0)  # signed values for the split and sum
    special = np.array([0.0, -0.0, 1e-35, -1e-35, 1e-40, 3e38, 1e39, -1e300])
    dev = torch.device("cuda", torch.cuda.current_device())
    xs = np.concatenate([x, special])
    ys = np.concatenate([y, np.ones(special.size)])
    xd, yd = torch.from_numpy(xs).to(dev), torch.from_numpy(ys).to(dev)
    out = torch.empty(6 * xs.size, dtype=torch.float64, device=dev)
    st = _lib.probe().cbns_probe_ff(ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(yd.data_ptr()),
                                    ctypes.c_void_p(out.data_ptr()), xs.size)
    assert st == 0
    o = out.cpu().numpy().reshape(-1, 6)
    r, sp = o[:x.size], o[x.size:]
    a = slice(m, x.size)  # the arithmetic's operands
    xa, ya, ra = x[a], y[a], r[a]
    pos = xa > 0
    errs = {
        "split": np.abs(r[:, 0] - x) / np.abs(x),
        "rcp": np.abs(ra[pos, 1] * xa[pos] - 1.0),
        "rsqrt": np.abs(ra[pos, 2] * np.sqrt(xa[pos]) - 1.0),
        "mul": np.abs(ra[:, 3] - xa * ya) / np.abs(xa * ya),
        "add": np.abs(ra[:, 4] - (xa + ya)) / (np.abs(xa) + np.abs(ya)),
        "fma": np.abs(ra[:, 5] - (xa * ya + xa)) / (np.abs(xa * ya) + np.abs(xa)),
    }
    print("float-float max relative errors (log2):", {k: round(float(np.log2(v.max())), 2) for k, v in errs.items()})
    assert errs["split"].max() < 2.0 ** -46
    for k in ("rcp", "rsqrt", "mul", "add", "fma"):
        assert errs[k].max() < 2.0 ** -44, k
    # specials: signed zeros, below the normal range, beyond it
    assert sp[0, 0] == 0.0 and sp[1, 0] == 0.0 and np.signbit(sp[1, 0])
    assert abs(sp[2, 0] - 1e-35) <= 2.0 ** -23 * 1e-35 and abs(sp[3, 0] + 1e-35) <= 2.0 ** -23 * 1e-35
    assert sp[4, 0] == 0.0
    assert abs(sp[5, 0] - 3e38) <= 2.0 ** -46 * 3e38
    assert np.isnan(sp[6, 0]) and np.isnan(sp[7, 0])


@pytest.mark.parametrize("precision", ["fp64", "fp64_ff"])
def test_low_mach_vs_oracle(precision):
    """Below the workloads' Mach range: Ma 0.02 (energy about 2e3 times the
    velocity scale, the stiffest ratio for float-float's fixed 47 bits), 20
    steps on an odd block against the oracle at the parity bar."""
    from oracle.oracle import OracleBlock
    from cbns3d_cart_mpi_gb300.solver import Solver, initial_condition_perturbed
    p = tgv_params(18, JM=14, KM=10, Re=1600.0, Mach=0.02)
    Q0 = initial_condition_perturbed(p, seed=21, amp=1e-3, nmodes=16, kmax=4)
    s = Solver(p, precision=precision)
    s.upload_Q(Q0, 0.0)
    o = OracleBlock(p)
    o.set_Q(Q0, 0.0)
    for n in range(20):
        dt, _ = s.step()
        dto, _ = o.step()
        assert abs(dt - dto) <= (1e-13 if precision == "fp64" else 1e-12) * dto, n
    Qg, Qo = interior(s.download_Q()), interior(o.get_Q())
    print(precision, "Ma 0.02 rel Linf", dict(zip(FIELDS, rel_linf(Qg, Qo))))
    assert_close(Qg, Qo, 1e-11, "%s Ma 0.02" % precision, tight=1e-13)
