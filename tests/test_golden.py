"""Pin the CPU oracle to the reference: run every golden case (initial state, parameters
and step count recorded from a run of the unmodified CudaNavierStokes GPU code) and compare
the final state, the grid and the printed dt sequence."""
import numpy as np
import pytest

from tests import golden_cases
from tests._util import state_errors

TOL = 1e-12


def test_golden_cases_present():
    assert len(golden_cases.names()) >= 5


@pytest.mark.parametrize("name", golden_cases.names())
def test_oracle_matches_reference(oracle_mod, name):
    c = golden_cases.load(name)
    p = c["params"]
    o = oracle_mod.Oracle(p)
    np.testing.assert_allclose(o.grid()["x"], c["x"], rtol=0, atol=1e-14)
    if c["kind"] == "bl":
        o.set_sponge(*golden_cases.sponge_from_ic(c, o.sponge_strengths()))
    o.set_state(*c["ic"])
    logs = o.run(c["nsteps"])
    errs = state_errors(o.get_state(), c["out"])
    assert max(errs) <= TOL, errs
    # the reference prints dt with 7 significant digits at every dt update
    for step, dt, _ in c["steplog"]:
        assert abs(logs["dt"][int(step)] - dt) <= 5e-7 * dt


@pytest.mark.parametrize("name", golden_cases.names())
def test_oracle_statistics_match_reference(oracle_mod, name):
    """calcAvgChan's prof.txt (final fields) and printRes's friction Reynolds number
    (initial fields) as printed by the reference (%lf: 6 decimals)."""
    case = golden_cases.load(name)
    o = oracle_mod.Oracle(case["params"])
    o.set_state(*case["ic"])
    assert abs(o.friction_reynolds() - case["ret"]) <= 5.01e-7
    o.set_state(*case["out"])
    prof = o.plane_stats().T
    assert prof.shape == case["prof"].shape
    assert np.abs(prof - case["prof"]).max() <= 5.01e-7


@pytest.mark.parametrize("name", golden_cases.large_names())
def test_oracle_matches_reference_at_benchmark_size(oracle_mod, name):
    """The benchmark workloads themselves (64^3 Taylor-Green, 128x160x192 channel), 10 steps
    of the unmodified reference: the oracle's final fields against the reference's
    subsample and whole-grid plane sums, and the printed dt sequence."""
    c = golden_cases.load_large(name)
    p = c["params"]
    o = oracle_mod.Oracle(p)
    x = o.grid()["x"]
    np.testing.assert_allclose(x, c["x"], rtol=0, atol=1e-14)
    ic = golden_cases.initial_fields(c, x)
    s = c["sub"]
    for a, b in zip(ic, c["ic_sub"]):
        np.testing.assert_allclose(a[::s, ::s, ::s], b, rtol=0, atol=1e-14 * max(1.0, float(np.abs(b).max())))
    o.set_state(*ic)
    logs = o.run(c["nsteps"])
    errs = golden_cases.large_errors(o.get_state(), c)
    assert max(errs) <= TOL, errs
    for step, dt, _ in c["steplog"]:
        assert abs(logs["dt"][int(step)] - dt) <= 5e-7 * dt
