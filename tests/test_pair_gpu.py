"""GPU parity of the pair mode (CNS_PREC_PAIR_RHS): the RHS in FP32-pair arithmetic
(~48 significant bits, ff.cuh), the state, the RK accumulation, the state recovery and the
reductions in FP64.

Bars: the FP64 path's. A single RHS evaluation and the state after multi-step runs within
1e-12 per field (norm-wise) of the FP64 oracle, and on the benchmark workloads (64^3
Taylor-Green box, 128x160x192 channel, 10 steps) within 1e-12 of the reference's own output.
The pair arithmetic rounds at ~2^-48 per operation against FP64's 2^-53; the RHS (a small
difference of large fluxes) carries that with the cancellation's amplification, and a stage
moves the state by dt times the RHS.
"""
import numpy as np
import pytest

from cudanavierstokes_gb300 import Solver
from cudanavierstokes_gb300.initial import channel_fields, tgv_fields
from cudanavierstokes_gb300.params import (PREC_PAIR_RHS, RK3_CLASSIC, RK4_CLASSIC, boundary_layer_params,
                                           channel_params, tgv_params)
from tests import golden_cases
from tests._util import field_errors, smooth_random_state, state_errors, wall_state

pytestmark = pytest.mark.gpu

TOL_STATE = 1e-12
TOL_RHS = 1e-12

SV = [(1, 1), (2, 1), (2, 2), (3, 1), (3, 2), (3, 3), (4, 1), (4, 2), (4, 3), (4, 4)]


def _pair(oracle_mod, p, fields):
    o = oracle_mod.Oracle(p)
    s = Solver(p.copy(precision=PREC_PAIR_RHS))
    o.set_state(*fields)
    s.copy_field_in(*fields)
    return o, s


@pytest.mark.parametrize("S,V", SV)
def test_pair_rhs_all_orders_odd_edges(gpu_lib, oracle_mod, S, V):
    p = tgv_params(17).copy(my=13, mz=11, stencil_size=S, stencil_visc=V)
    o, s = _pair(oracle_mod, p, smooth_random_state(p, seed=300 + S * 10 + V))
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= TOL_RHS, errs


@pytest.mark.parametrize("S,V", [(4, 4), (3, 2)])
def test_pair_rhs_channel_walls(gpu_lib, oracle_mod, S, V):
    """Stretched x (the non-uniform second-derivative tables as pairs) and wall ghosts."""
    p = channel_params(24, 16, 20).copy(stencil_size=S, stencil_visc=V)
    o = oracle_mod.Oracle(p)
    o, s = _pair(oracle_mod, p, wall_state(p, o.grid()["x"]))
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= TOL_RHS, errs


@pytest.mark.parametrize("quirk", [0, 1])
def test_pair_rhs_quirk_switch(gpu_lib, oracle_mod, quirk):
    p = tgv_params(16).copy(quirk_dissipation_y=quirk)
    o, s = _pair(oracle_mod, p, smooth_random_state(p, seed=7))
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= TOL_RHS, errs


@pytest.mark.parametrize("case", ["tgv_s4v4", "tgv_classic_s2v1", "tgv_rk4", "channel_s3v2", "channel_s4v4"])
def test_pair_run_parity(gpu_lib, oracle_mod, case):
    if case == "tgv_s4v4":
        p, n = tgv_params(16).copy(my=20, mz=24), 10
        f = tgv_fields(p)
    elif case == "tgv_classic_s2v1":
        p, n = tgv_params(16).copy(stencil_size=2, stencil_visc=1, scheme=RK3_CLASSIC, check_cfl=4, check_bulk=3), 6
        f = smooth_random_state(p, seed=3)
    elif case == "tgv_rk4":
        p, n = tgv_params(16).copy(scheme=RK4_CLASSIC, check_cfl=2), 5
        f = smooth_random_state(p, seed=4)
    else:
        S, V = (3, 2) if case == "channel_s3v2" else (4, 4)
        p, n = channel_params(16, 12, 20).copy(stencil_size=S, stencil_visc=V, check_cfl=3, check_bulk=2), 8
        f = channel_fields(p, oracle_mod.Oracle(p).grid()["x"], seed=0)
    o, s = _pair(oracle_mod, p, f)
    lo = o.run(n)
    lg = s.run(n)
    errs = state_errors(s.copy_field_out(), o.get_state())
    assert max(errs) <= TOL_STATE, errs
    np.testing.assert_allclose(lg["time"], lo["time"], rtol=1e-13)
    so, sg = o.scalars(), s.scalars()
    assert abs(sg["dt"] - so["dt"]) <= 1e-13 * abs(so["dt"])
    assert abs(sg["dpdz"] - so["dpdz"]) <= 1e-12 * max(1.0, abs(so["dpdz"]))


def test_pair_boundary_layer(gpu_lib, oracle_mod):
    """Sponge, boundary-layer extrapolation and the wall ghosts computed in FP64 from pairs."""
    from oracle.ref_harness import blasius_like_profile
    p = boundary_layer_params(16, 8, 160).copy(check_cfl=2)
    o = oracle_mod.Oracle(p)
    spx, spz = o.sponge_strengths()
    rref, uref, wref, eref = o.sponge_refs(*blasius_like_profile())
    fields = [np.broadcast_to(a[:, None, :], p.shape).copy() for a in (rref, uref, np.zeros_like(rref), wref, eref)]
    o.set_sponge(spx, spz, rref, uref, wref, eref)
    s = Solver(p.copy(precision=PREC_PAIR_RHS))
    s.set_sponge(spx, spz, rref, uref, wref, eref)
    o.set_state(*fields)
    s.copy_field_in(*fields)
    o.run(6)
    s.run(6)
    assert max(state_errors(s.copy_field_out(), o.get_state())) <= TOL_STATE


@pytest.mark.parametrize("name", golden_cases.large_names())
def test_pair_matches_reference_at_benchmark_size(gpu_lib, name):
    """The FP64 path's acceptance bar on the benchmark workloads: after 10 steps, the
    reference's subsample and plane sums within 1e-12 of the field scale."""
    c = golden_cases.load_large(name)
    s = Solver(c["params"].copy(precision=PREC_PAIR_RHS))
    s.copy_field_in(*golden_cases.initial_fields(c, s.grid()["x"]))
    s.run(c["nsteps"])
    errs = golden_cases.large_errors(s.copy_field_out(), c)
    assert max(errs) <= TOL_STATE, errs


def test_pair_is_deterministic(gpu_lib):
    p = channel_params(24, 16, 20, precision=PREC_PAIR_RHS)
    outs = []
    for _ in range(2):
        s = Solver(p)
        s.copy_field_in(*channel_fields(p, s.grid()["x"], seed=1))
        s.run(3)
        outs.append(s.copy_field_out())
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
