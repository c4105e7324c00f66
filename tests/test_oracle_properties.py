"""Consistency properties of the reference's numerics, on the oracle's restatement
(bitwise equal to the reference, see test_oracle_golden.py): the Roe eigenvector
matrices are inverse to each other, WENO5 reproduces constant and linear data,
and the Lax-Friedrichs flux of two equal states is the physical flux."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.usefixtures("built")


def lib():
    from oracle.oracle import lib as L
    lb = L()
    dp = ctypes.POINTER(ctypes.c_double)
    lb.oracle_eigenvectors.argtypes = [ctypes.c_double, dp, dp, dp, dp, dp]
    lb.oracle_weno5.argtypes = [dp]
    lb.oracle_weno5.restype = ctypes.c_double
    lb.oracle_lf_flux.argtypes = [ctypes.c_double, dp, dp, dp, dp]
    return lb


def ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


NORMALS = [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0)]


def states(rng, n):
    rho = rng.uniform(0.5, 2.0, n)
    vel = rng.uniform(-1.0, 1.0, (n, 3))
    p = rng.uniform(20.0, 120.0, n)
    return np.column_stack([rho, vel, p])


def test_left_and_right_eigenvectors_are_inverse():
    lb = lib()
    rng = np.random.default_rng(1)
    for sL, sR in zip(states(rng, 50), states(rng, 50)):
        for n in NORMALS:
            R = np.zeros(25)
            L = np.zeros(25)
            lb.oracle_eigenvectors(1.4, ptr(np.ascontiguousarray(sL)), ptr(np.ascontiguousarray(sR)),
                                   ptr(np.array(n)), ptr(R), ptr(L))
            np.testing.assert_allclose(L.reshape(5, 5) @ R.reshape(5, 5), np.eye(5), atol=1e-13)


def test_weno5_reproduces_constant_and_linear_data():
    lb = lib()
    rng = np.random.default_rng(2)
    for _ in range(200):
        c, g = rng.uniform(-100, 100), rng.uniform(-10, 10)
        v = np.full(5, c)
        assert abs(lb.oracle_weno5(ptr(v)) - c) <= 4 * np.spacing(abs(c))
        # cells -2..+2 of a linear function; the interface is at +1/2
        lin = c + g * np.arange(-2, 3, dtype=float)
        assert abs(lb.oracle_weno5(ptr(lin)) - (c + 0.5 * g)) <= 1e-12 * (abs(c) + abs(g))


def test_lf_flux_of_equal_states_is_the_physical_flux():
    lb = lib()
    rng = np.random.default_rng(3)
    gamma = 1.4
    for s in states(rng, 50):
        rho, u, v, w, p = s
        E = p / (gamma - 1) + 0.5 * rho * (u * u + v * v + w * w)
        for n in NORMALS:
            f = np.zeros(5)
            lb.oracle_lf_flux(gamma, ptr(np.ascontiguousarray(s)), ptr(np.ascontiguousarray(s)), ptr(np.array(n)),
                              ptr(f))
            qn = u * n[0] + v * n[1] + w * n[2]
            phys = np.array([rho * qn, rho * qn * u + p * n[0], rho * qn * v + p * n[1], rho * qn * w + p * n[2],
                             qn * (E + p)])
            np.testing.assert_allclose(f, phys, rtol=1e-13, atol=1e-12)
