"""The GB300 library against the golden vectors of the unmodified reference GPU code."""
import numpy as np
import pytest

from cudanavierstokes_gb300 import Solver
from tests import golden_cases
from tests._util import state_errors

pytestmark = pytest.mark.gpu


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
    assert max(errs) <= 1e-12, errs
