"""The pair ("double-float") arithmetic of the pair precision mode on the GPU
(cns_selftest_pair) against exact rational arithmetic: the split of a double into its
nearest pair, the sum, the product, the fused multiply-add and the compensated accumulation,
within the double-word error bounds (Joldes, Muller and Popescu, ACM TOMS 2017; u = 2^-24),
and the packed two-lane forms bit for bit equal to the scalar ones."""
import ctypes
from fractions import Fraction

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U2 = Fraction(1, 2 ** 48)   # u^2


def _inputs(n, seed=5):
    rng = np.random.default_rng(seed)

    def draw():
        m = rng.uniform(1.0, 2.0, n) * rng.choice([-1.0, 1.0], n)
        return np.ldexp(m, rng.integers(-30, 31, n))
    a, b, c = draw(), draw(), draw()
    q = n // 4
    # cancellation: b ~ -a (the sum) and c ~ -a b (the multiply-add)
    b[:q] = -a[:q] * (1.0 + rng.uniform(-1e-9, 1e-9, q))
    c[q:2 * q] = -(a[q:2 * q] * b[q:2 * q]) * (1.0 + rng.uniform(-1e-9, 1e-9, q))
    return a, b, c


def _run(gpu_lib, a, b, c):
    out = np.zeros(a.size * 30, dtype=np.float32)
    p = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    assert gpu_lib.cns_selftest_pair(0, p(a), p(b), p(c), a.size, p(out)) == 0
    return out.reshape(a.size, 15, 2)


def _val(hl):
    return Fraction(float(hl[0])) + Fraction(float(hl[1]))


def test_pair_operations_within_bounds(gpu_lib):
    a, b, c = _inputs(4000)
    r = _run(gpu_lib, a, b, c)
    for t in range(a.size):
        x, y, z = _val(r[t, 0]), _val(r[t, 1]), _val(r[t, 2])
        # nearest pair: |pair - a| <= ~2^-48 |a| (h rounded, then the remainder), normalised tail
        for q, v in enumerate((a[t], b[t], c[t])):
            assert abs(_val(r[t, q]) - Fraction(float(v))) <= Fraction(1, 2 ** 47) * abs(Fraction(float(v)))
            assert abs(float(r[t, q, 1])) <= 2.0 ** -24 * abs(float(r[t, q, 0]))
        # scalar results 3..6 on (a, b, c); packed lane 1, results 11..14, on (b, c, a)
        for base, (p, q, s) in ((3, (x, y, z)), (11, (y, z, x))):
            add, mul, fm, acc = (_val(r[t, base + k]) for k in range(4))
            assert abs(add - (p + q)) <= 4 * U2 * (abs(p) + abs(q)), (t, base, "add")
            assert abs(mul - p * q) <= 8 * U2 * abs(p * q), (t, base, "mul")
            bound = 16 * U2 * (abs(p * q) + abs(s))
            assert abs(fm - (p * q + s)) <= bound, (t, base, "fma")
            assert abs(acc - (p * q + s)) <= bound, (t, base, "acc")


def test_packed_lane_equals_scalar(gpu_lib):
    a, b, c = _inputs(20000, seed=9)
    r = _run(gpu_lib, a, b, c)
    # lane 0 of the packed sum, product, multiply-add and accumulation (results 7..10) is
    # the scalar path's result (3..6), float for float
    np.testing.assert_array_equal(r[:, 7:11, :], r[:, 3:7, :])
