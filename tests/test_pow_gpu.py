"""The FP64 power used for the viscosity law mu ~ T^viscexp (exp(a ln T) with series and
Cody-Waite reduction) against the CUDA library pow: within 4 ulp over temperatures far
beyond the flows' range, for the exponents the configurations use."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("a", [0.7, 0.76, 2.0 / 3.0, 0.5, 1.5, -0.3])
def test_pow_visc_matches_library_pow(gpu_lib, a):
    rng = np.random.default_rng(17)
    x = np.concatenate([np.exp(rng.uniform(np.log(1e-3), np.log(1e3), 500_000)),
                        1.0 + rng.uniform(-1e-6, 1e-6, 100_000),
                        np.array([1.0, 2.0, 0.5, np.sqrt(2.0), np.sqrt(0.5), 1e-200, 1e200])])
    x = np.ascontiguousarray(x)
    fast, lib = np.empty_like(x), np.empty_like(x)
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    assert gpu_lib.cns_selftest_pow(0, p(x), x.size, ctypes.c_double(a), p(fast), p(lib)) == 0
    ulp = np.spacing(np.abs(lib))
    err = np.abs(fast - lib) / ulp
    assert err.max() <= 4.0, (a, err.max(), x[np.argmax(err)])
    assert np.all(fast[x == 1.0] == 1.0)


def test_pow_visc_special_arguments(gpu_lib):
    x = np.ascontiguousarray(np.array([0.0, -1.0, np.inf, np.nan, 1e-310, 1e305]))
    fast, lib = np.empty_like(x), np.empty_like(x)
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    assert gpu_lib.cns_selftest_pow(0, p(x), x.size, ctypes.c_double(0.7), p(fast), p(lib)) == 0
    np.testing.assert_array_equal(fast, lib)
