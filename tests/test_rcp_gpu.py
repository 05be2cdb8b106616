"""The FP64 reciprocal used for 1/rho (an FP32 seed refined by two Newton steps, with the
IEEE division outside the seed's range) against the IEEE division 1.0 / x: within one ulp
over densities from 1e-30 to 1e30, at the edges of the FP32 seed's range, and equal on the
special values."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(gpu_lib, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    fast, lib = np.empty_like(x), np.empty_like(x)
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    assert gpu_lib.cns_selftest_rcp(0, p(x), x.size, p(fast), p(lib)) == 0
    return x, fast, lib


def test_rcp_within_one_ulp(gpu_lib):
    rng = np.random.default_rng(23)
    mag = np.exp(rng.uniform(np.log(1e-30), np.log(1e30), 1_000_000))
    near_one = 1.0 + rng.uniform(-0.5, 0.5, 200_000)
    edges = []
    for k in (-128, -127, -126, -125, -124, -1, 0, 1, 124, 125, 126, 127, 128):
        b = 2.0 ** k
        edges.append(b * (1.0 + rng.uniform(-1e-6, 1e-6, 2000)))
        edges.append(np.array([b, np.nextafter(b, 0.0), np.nextafter(b, np.inf)]))
    f32 = np.finfo(np.float32)
    edges.append(np.array([float(f32.tiny), float(f32.max), float(f32.smallest_subnormal), 1e-300, 1e300,
                           1e-310, 3.0, 7.0, 1.0 / 3.0]))
    x = np.concatenate([mag, near_one] + edges)
    x = np.concatenate([x, -x])
    x, fast, lib = _run(gpu_lib, x)
    fin = np.isfinite(lib)            # 1 / 1e-310 overflows: those must match exactly
    np.testing.assert_array_equal(fast[~fin], lib[~fin])
    err = np.abs(fast[fin] - lib[fin]) / np.spacing(np.abs(lib[fin]))
    assert err.max() <= 1.0, (err.max(), x[fin][np.argmax(err)])
    assert np.mean(fast == lib) > 0.9


def test_rcp_special_values(gpu_lib):
    x, fast, lib = _run(gpu_lib, np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 1.7e308]))
    np.testing.assert_array_equal(fast, lib)
