"""Flow statistics on the device against the oracle (itself pinned to the reference's
printed prof.txt and friction Reynolds number): calcAvgChan plane profiles and printRes
Re_tau, on the golden cases and on a perturbed stretched channel."""
import numpy as np
import pytest

from cudanavierstokes_gb300 import Solver
from cudanavierstokes_gb300.params import PREC_FP32_RHS, PREC_FP64, channel_params, tgv_params
from tests import golden_cases
from tests._util import smooth_random_state, wall_state

pytestmark = pytest.mark.gpu


def _col_err(a, b, uscale):
    """Per column max|a - b| / scale: each column's own max, except that the Favre mean
    velocities (columns 2-4) are measured against the flow's velocity scale U, the
    velocity variances (7-9) against U^2 (a plane-mean velocity of a symmetric flow is
    rounding noise around zero) and the rho / rhoE variances against 1e-6 of the squared
    plane mean (zero up to rounding for a uniform field)."""
    def scale(q):
        if q in (2, 3, 4):
            return max(np.abs(b[2:5]).max(), uscale)
        if q in (7, 8, 9):
            return max(np.abs(b[7:10]).max(), uscale ** 2)
        if q in (6, 10):   # variance of rho / rhoE: a uniform field's is rounding noise
            return max(np.abs(b[q]).max(), 1e-6 * np.abs(b[q - 5]).max() ** 2)
        return max(np.abs(b[q]).max(), 1e-300)
    return [float(np.abs(a[q] - b[q]).max() / scale(q)) for q in range(b.shape[0])]


def _uscale(fields):
    return max(float(np.abs(f).max()) for f in fields[1:4])


@pytest.mark.parametrize("name", golden_cases.names())
def test_statistics_match_oracle(gpu_lib, oracle_mod, name):
    case = golden_cases.load(name)
    p = case["params"]
    o = oracle_mod.Oracle(p)
    s = Solver(p)
    for fields in (case["ic"], case["out"]):
        o.set_state(*fields)
        s.copy_field_in(*fields)
        assert abs(s.friction_reynolds() - o.friction_reynolds()) <= 1e-12 * max(abs(o.friction_reynolds()), 1.0)
        assert max(_col_err(s.plane_stats(), o.plane_stats(), _uscale(fields))) <= 1e-12


def test_statistics_on_a_perturbed_channel(gpu_lib, oracle_mod):
    p = channel_params(40, 20, 24)
    o = oracle_mod.Oracle(p)
    f = wall_state(p, o.grid()["x"])
    o.set_state(*f)
    s = Solver(p)
    s.copy_field_in(*f)
    ret = s.friction_reynolds()
    assert ret > 0 and abs(ret - o.friction_reynolds()) <= 1e-12 * ret
    st = s.plane_stats()
    assert max(_col_err(st, o.plane_stats(), _uscale(f))) <= 1e-12
    np.testing.assert_array_equal(st[0], o.grid()["x"])


def _diss_close(a, b):
    return all(abs(a[k] - b[k]) <= 1e-12 * abs(b[k]) for k in ("eps", "enstrophy"))


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_FP32_RHS])
@pytest.mark.parametrize("name", golden_cases.names())
def test_dissipation_matches_oracle(gpu_lib, oracle_mod, name, prec):
    """Viscous dissipation and enstrophy of the golden cases' start and end fields (periodic
    box, stretched walls, boundary layer with its perturbed wall ghosts): the FP64
    diagnostic in either precision mode against the oracle."""
    case = golden_cases.load(name)
    p = case["params"]
    o = oracle_mod.Oracle(p)
    s = Solver(p.copy(precision=prec))
    for fields in (case["ic"], case["out"]):
        o.set_state(*fields)
        s.copy_field_in(*fields)
        d, do = s.dissipation(), o.dissipation()
        assert do["eps"] > 0 and do["enstrophy"] > 0
        assert _diss_close(d, do), (d, do)


def test_dissipation_of_an_evolved_fp32_state(gpu_lib, oracle_mod):
    """After FP32-RHS steps the diagnostic reads the FP64 state: the oracle on the copied-out
    state gives the same values."""
    p = tgv_params(24).copy(my=20, mz=16)
    s = Solver(p.copy(precision=PREC_FP32_RHS))
    s.copy_field_in(*smooth_random_state(p, seed=4))
    s.run(5)
    o = oracle_mod.Oracle(p)
    o.set_state(*s.copy_field_out())
    assert _diss_close(s.dissipation(), o.dissipation())
