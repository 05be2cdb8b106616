"""A model of the pair ("double-float") algorithms of the pair precision mode in exact
rational arithmetic with IEEE single-precision rounding (round to nearest even), checked on
the CPU: 2Sum and the FMA-based product error are exact, and the sum, product, fused
multiply-add and compensated accumulation stay within the double-word bounds that the GPU
self test (tests/test_pair_arith_gpu.py) asserts for the device code (Joldes, Muller and
Popescu, ACM TOMS 2017; u = 2^-24). The model follows the operation sequences of the
device code step for step; it checks the algorithms and the bounds, the GPU test the code."""
from fractions import Fraction

import numpy as np

U2 = Fraction(1, 2 ** 48)


def rn32(q: Fraction) -> Fraction:
    """q rounded to the nearest binary32 value, ties to even (normal range only)."""
    if q == 0:
        return Fraction(0)
    s = -1 if q < 0 else 1
    a = abs(q)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    m = a * Fraction(2) ** (23 - e)          # in [2^23, 2^24)
    M = m.numerator // m.denominator
    r = m - M
    if r > Fraction(1, 2) or (r == Fraction(1, 2) and M % 2 == 1):
        M += 1
    return s * Fraction(M) * Fraction(2) ** (e - 23)


def add(a, b): return rn32(a + b)
def sub(a, b): return rn32(a - b)
def mul(a, b): return rn32(a * b)
def fma(a, b, c): return rn32(a * b + c)


def two_sum(a, b):
    s = add(a, b)
    bb = sub(s, a)
    return s, add(sub(a, sub(s, bb)), sub(b, bb))


def fast_two_sum(a, b):
    s = add(a, b)
    return s, sub(b, sub(s, a))


def pair_add(x, y):
    sh, sl = two_sum(x[0], y[0])
    return fast_two_sum(sh, add(sl, add(x[1], y[1])))


def mul_parts(x, y):
    ch = mul(x[0], y[0])
    cl1 = fma(x[0], y[0], -ch)
    return ch, add(cl1, fma(x[1], y[0], mul(x[0], y[1])))


def pair_mul(x, y):
    return fast_two_sum(*mul_parts(x, y))


def pair_fma(a, b, c):
    ph, pl = mul_parts(a, b)
    sh, sl = two_sum(ph, c[0])
    return fast_two_sum(sh, add(sl, add(pl, c[1])))


def acc_fma(c, a, b):
    """ffacc initialised with c, one add_prod(a, b), value()."""
    h, l = c
    ph, pl = mul_parts(a, b)
    sh, sl = two_sum(h, ph)
    l = add(l, add(sl, pl))
    return two_sum(sh, l)


def split(x: float):
    """d_to_ff: the head rounded, then the remainder rounded."""
    h = rn32(Fraction(x))
    return h, rn32(Fraction(x) - h)


def _draws(n, seed):
    rng = np.random.default_rng(seed)

    def draw():
        m = rng.uniform(1.0, 2.0, n) * rng.choice([-1.0, 1.0], n)
        return np.ldexp(m, rng.integers(-30, 31, n))
    a, b, c = draw(), draw(), draw()
    q = n // 4
    b[:q] = -a[:q] * (1.0 + rng.uniform(-1e-9, 1e-9, q))
    c[q:2 * q] = -(a[q:2 * q] * b[q:2 * q]) * (1.0 + rng.uniform(-1e-9, 1e-9, q))
    return a, b, c


def test_rounding_model():
    # ties to even at 1 + 2^-24 and 1 + 3 2^-24; the nearest float to 1/3
    assert rn32(1 + Fraction(1, 2 ** 24)) == 1
    assert rn32(1 + Fraction(3, 2 ** 24)) == 1 + Fraction(4, 2 ** 24)
    assert rn32(Fraction(1, 3)) == Fraction(float(np.float32(1.0) / np.float32(3.0)))


def test_error_free_transforms_and_bounds():
    a, b, c = _draws(1500, seed=11)
    for t in range(a.size):
        x, y, z = split(a[t]), split(b[t]), split(c[t])
        X, Y, Z = (p[0] + p[1] for p in (x, y, z))
        for v, (h, l) in zip((a[t], b[t], c[t]), (x, y, z)):
            assert abs(h + l - Fraction(v)) <= Fraction(1, 2 ** 47) * abs(Fraction(v))
            assert abs(l) <= Fraction(1, 2 ** 24) * abs(h)
        s, e = two_sum(x[0], y[0])
        assert s + e == x[0] + y[0]                        # 2Sum is exact
        ch = mul(x[0], y[0])
        assert ch + fma(x[0], y[0], -ch) == x[0] * y[0]    # the FMA recovers the product's error
        r = pair_add(x, y)
        assert abs(r[0] + r[1] - (X + Y)) <= 4 * U2 * (abs(X) + abs(Y))
        r = pair_mul(x, y)
        assert abs(r[0] + r[1] - X * Y) <= 8 * U2 * abs(X * Y)
        bound = 16 * U2 * (abs(X * Y) + abs(Z))
        r = pair_fma(x, y, z)
        assert abs(r[0] + r[1] - (X * Y + Z)) <= bound
        r = acc_fma(z, x, y)
        assert abs(r[0] + r[1] - (X * Y + Z)) <= bound
