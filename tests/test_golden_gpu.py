"""The GB300 library against the golden vectors of the unmodified reference GPU code, on
the small golden cases and on the benchmark workloads themselves (64^3 Taylor-Green box,
128x160x192 isothermal channel, 10 steps)."""
import numpy as np
import pytest

from cudanavierstokes_gb300 import Solver
from tests import golden_cases
from tests._util import state_errors

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("name", golden_cases.names())
def test_library_matches_reference(gpu_lib, oracle_mod, name):
    c = golden_cases.load(name)
    p = c["params"]
    s = Solver(p)
    np.testing.assert_allclose(s.grid()["x"], c["x"], rtol=0, atol=1e-14)
    if c["kind"] == "bl":
        s.set_sponge(*golden_cases.sponge_from_ic(c, oracle_mod.Oracle(p).sponge_strengths()))
    s.copy_field_in(*c["ic"])
    s.run(c["nsteps"])
    errs = state_errors(s.copy_field_out(), c["out"])
    assert max(errs) <= TOL, errs


def _benchmark_case(name):
    c = golden_cases.load_large(name)
    s = Solver(c["params"])
    x = s.grid()["x"]
    np.testing.assert_allclose(x, c["x"], rtol=0, atol=1e-14)
    ic = golden_cases.initial_fields(c, x)
    sub = c["sub"]
    for a, b in zip(ic, c["ic_sub"]):
        np.testing.assert_allclose(a[::sub, ::sub, ::sub], b, rtol=0, atol=1e-14 * max(1.0, float(np.abs(b).max())))
    s.copy_field_in(*ic)
    return c, s, ic


@pytest.mark.parametrize("name", golden_cases.large_names())
def test_library_matches_reference_at_benchmark_size(gpu_lib, name):
    """Whole benchmark grid, 10 steps: the reference's subsample and plane sums within 1e-12
    of the field scale, and the reference's printed time step."""
    c, s, _ = _benchmark_case(name)
    logs = s.run(c["nsteps"])
    errs = golden_cases.large_errors(s.copy_field_out(), c)
    assert max(errs) <= TOL, errs
    dts = np.diff(np.concatenate([[0.0], logs["time"]]))
    for step, dt, _ in c["steplog"]:
        assert abs(dts[int(step)] - dt) <= 5e-7 * dt


@pytest.mark.parametrize("name", golden_cases.large_names())
def test_library_matches_oracle_at_benchmark_size(gpu_lib, oracle_mod, name):
    """Every point of the benchmark grid after 10 steps, against the oracle (which the test
    above and the CPU suite pin to the reference at this size): fields, time, dt and body
    force."""
    c, s, ic = _benchmark_case(name)
    o = oracle_mod.Oracle(c["params"])
    o.set_state(*ic)
    lo = o.run(c["nsteps"])
    lg = s.run(c["nsteps"])
    errs = state_errors(s.copy_field_out(), o.get_state())
    assert max(errs) <= TOL, errs
    np.testing.assert_allclose(lg["time"], lo["time"], rtol=1e-13)
    so, sg = o.scalars(), s.scalars()
    assert abs(sg["dt"] - so["dt"]) <= 1e-13 * abs(so["dt"])
    assert abs(sg["dpdz"] - so["dpdz"]) <= 1e-12 * max(1.0, abs(so["dpdz"]))
