"""The error-free additions of the float-float arithmetic (csrc/cbns_ff.cuh),
restated in numpy binary32 on the host, where every operation rounds to nearest
as the device's __fadd_rn/__fsub_rn do.

ff_two_sum_nonneg replaces Knuth's TwoSum by Dekker's Fast2Sum on the larger and
the smaller operand wherever both operands are known to be >= 0 (the WENO
indicators and weight denominators, squared speeds).  The kernels rely on the
two giving the same pair (s, e) with s + e = a + b exactly; this checks it over
random pairs across the binary32 exponent range, equal and near-equal values,
exponent gaps beyond 24 bits, subnormals and zeros.  No GPU needed.
"""
import numpy as np

F = np.float32


def two_sum(a, b):
    s = a + b
    v = s - a
    return s, (a - (s - v)) + (b - v)


def two_sum_nonneg(a, b):
    s = a + b
    return s, np.minimum(a, b) - (s - np.maximum(a, b))


def operands(rng, n):
    mant = rng.uniform(1.0, 2.0, n)
    a = np.ldexp(mant, rng.integers(-140, 120, n)).astype(F)
    gap = rng.integers(-40, 40, n)
    b = np.ldexp(rng.uniform(1.0, 2.0, n), np.clip(np.frexp(a)[1] + gap, -149, 120)).astype(F)
    near = (a * (F(1) + F(2.0 ** -23) * rng.integers(-4, 5, n).astype(F))).astype(F)
    special = np.array([0.0, 0.0, 1e-45, 1e-45, 1e-40, 3e-39, 1.0, 1.0, 2.0 ** -24, 1.0,
                        3.4e38, 1.0], dtype=F)
    xs = np.concatenate([a, a, special[0::2]])
    ys = np.concatenate([b, near, special[1::2]])
    return xs, ys


def test_fast2sum_on_max_min_equals_two_sum_for_nonnegative_pairs():
    rng = np.random.default_rng(5)
    a, b = operands(rng, 1 << 20)
    s1, e1 = two_sum(a, b)
    s2, e2 = two_sum_nonneg(a, b)
    s3, e3 = two_sum_nonneg(b, a)  # operand order does not matter
    assert np.isfinite(s1).all()
    assert np.array_equal(s1, s2) and np.array_equal(s1, s3)
    assert np.array_equal(e1, e2) and np.array_equal(e1, e3)
    # and the pair is exact: s + e = a + b, compared in binary64 (exact up to a
    # 29-bit exponent gap; beyond it binary64 rounds both sides alike)
    exact = a.astype(np.float64) + b.astype(np.float64)
    assert np.array_equal(s1.astype(np.float64) + e1.astype(np.float64), exact)


def test_two_sum_nonneg_propagates_nan():
    a = np.array([np.nan, 1.0, np.nan], dtype=F)
    b = np.array([1.0, np.nan, np.nan], dtype=F)
    s, e = two_sum_nonneg(a, b)
    assert np.isnan(s).all() and np.isnan(e).all()
