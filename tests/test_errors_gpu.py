"""Error reporting of the device checks (no GPU fault involved: non-finite and
non-physical values only flow through arithmetic): a state with negative temperature is
rejected when it is copied in, and a run made unstable by a CFL number far above the
explicit scheme's limit stops with CNS_ERR_NONFINITE instead of returning garbage."""
import numpy as np
import pytest

from cudanavierstokes_gb300 import Solver
from cudanavierstokes_gb300.initial import tgv_fields
from cudanavierstokes_gb300.native import CnsError
from cudanavierstokes_gb300.params import PREC_FP32_RHS, PREC_FP64, tgv_params

pytestmark = pytest.mark.gpu

CNS_ERR_NONFINITE = 4


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_FP32_RHS])
def test_negative_temperature_is_rejected_at_copy_in(gpu_lib, prec):
    p = tgv_params(16, precision=prec)
    r, u, v, w, e = tgv_fields(p)
    e = e.copy()
    e[3, 4, 5] = -1.0                        # rhoE < kinetic energy: T < 0
    s = Solver(p)
    with pytest.raises(CnsError) as ei:
        s.copy_field_in(r, u, v, w, e)
    assert ei.value.code == CNS_ERR_NONFINITE


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_FP32_RHS])
@pytest.mark.parametrize("bad", [0.0, -0.0, -1.0, float("nan"), float("-nan")])
def test_non_positive_density_is_rejected_at_copy_in(gpu_lib, prec, bad):
    """The positivity test of the recovered state (on the bit patterns in FP64 mode) flags
    zero of either sign, negative and NaN densities."""
    p = tgv_params(16, precision=prec)
    r, u, v, w, e = tgv_fields(p)
    r = r.copy()
    r[2, 7, 1] = bad
    s = Solver(p)
    with pytest.raises(CnsError) as ei:
        s.copy_field_in(r, u, v, w, e)
    assert ei.value.code == CNS_ERR_NONFINITE


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_FP32_RHS])
def test_unstable_run_reports_nonfinite_state(gpu_lib, prec):
    p = tgv_params(16, precision=prec).copy(cfl=50.0)
    s = Solver(p)
    s.copy_field_in(*tgv_fields(p))
    with pytest.raises(CnsError) as ei:
        s.run(20)
    assert ei.value.code == CNS_ERR_NONFINITE
    # a stable run of the same start is fine
    q = Solver(tgv_params(16, precision=prec))
    q.copy_field_in(*tgv_fields(q.p))
    q.run(3)
    assert all(np.isfinite(f).all() for f in q.copy_field_out())


def test_statistics_need_a_state(gpu_lib):
    """The device statistics on a handle with no field copied in return CNS_ERR_STATE."""
    s = Solver(tgv_params(16))
    for call in (s.dissipation, s.friction_reynolds, s.plane_stats):
        with pytest.raises(CnsError) as e:
            call()
        assert e.value.code == 6   # CNS_ERR_STATE
