"""The FP64 <-> FP32 conversions the FP32-RHS kernels run on the integer units against
the hardware conversions, over random bit patterns, values next to the FP32 rounding
midpoints, and the edges of the FP32 range (zero, subnormal, overflow, infinity, NaN):
bitwise equal, except that magnitudes below 2^-126 (the FP32 subnormal range) become a
zero of the same sign and NaN stays NaN."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(seed=7):
    rng = np.random.default_rng(seed)
    x = [rng.integers(0, 2**64, 400_000, dtype=np.uint64).view(np.float64),
         rng.standard_normal(400_000) * 10.0 ** rng.uniform(-40, 40, 400_000)]
    f = (rng.standard_normal(100_000) * 10.0 ** rng.uniform(-30, 30, 100_000)).astype(np.float32)
    lo = f.astype(np.float64)
    hi = np.nextafter(f, np.float32(np.inf)).astype(np.float64)
    mid = 0.5 * (lo + hi)
    x += [mid, np.nextafter(mid, np.inf), np.nextafter(mid, -np.inf)]
    fmax = float(np.finfo(np.float32).max)
    tiny = float(np.finfo(np.float32).tiny)
    edge = [0.0, -0.0, np.inf, -np.inf, np.nan, fmax, -fmax, fmax * (1 + 2.0**-25), fmax * (1 + 2.0**-24),
            tiny, -tiny, tiny * (1 - 2.0**-30), tiny * 0.5, 5e-324, 1.0, -1.0, 3.0, 1.0 / 3.0]
    x.append(np.array(edge))
    x = np.ascontiguousarray(np.concatenate(x))
    y = np.ascontiguousarray(rng.integers(0, 2**32, x.size, dtype=np.uint64).astype(np.uint32).view(np.float32))
    y[:8] = [0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, np.finfo(np.float32).tiny, np.finfo(np.float32).max]
    return x, y


def test_alu_conversions_match_hardware(gpu_lib):
    x, y = _inputs()
    n = x.size
    fa, fh = np.empty(n, np.float32), np.empty(n, np.float32)
    da, dh = np.empty(n, np.float64), np.empty(n, np.float64)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert gpu_lib.cns_selftest_convert(0, p(x), p(y), n, p(fa), p(fh), p(da), p(dh)) == 0
    tiny = float(np.finfo(np.float32).tiny)
    nan_x, small_x = np.isnan(x), np.abs(x) < tiny
    reg = ~nan_x & ~small_x
    assert np.array_equal(fa[reg].view(np.uint32), fh[reg].view(np.uint32))
    assert np.all(np.isnan(fa[nan_x]))
    assert np.all(fa[small_x] == 0) and np.array_equal(np.signbit(fa[small_x]), np.signbit(x[small_x]))
    nan_y, small_y = np.isnan(y), np.abs(y) < tiny
    reg = ~nan_y & ~small_y
    assert np.array_equal(da[reg].view(np.uint64), dh[reg].view(np.uint64))
    assert np.all(np.isnan(da[nan_y]))
    assert np.all(da[small_y] == 0) and np.array_equal(np.signbit(da[small_y]), np.signbit(y[small_y]))
    # and the hardware conversion is the IEEE one numpy computes (finite, normal results)
    with np.errstate(over="ignore", invalid="ignore"):
        ref = x.astype(np.float32)
    ok = np.isfinite(ref) & (np.abs(ref) >= tiny)
    assert np.array_equal(fh[ok].view(np.uint32), ref[ok].view(np.uint32))
