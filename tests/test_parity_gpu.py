"""GPU parity: the GB300 library (through its C ABI) against the CPU oracle.

Bar (FP64 path): norm-wise relative error max|a-b|/max|b| <= 1e-12 per field, for a single
RHS evaluation and after multi-step runs. FP32-RHS path: <= 2e-5 against the FP64 oracle.
"""
import numpy as np
import pytest

from cudanavierstokes_gb300 import Solver
from cudanavierstokes_gb300.initial import channel_fields, tgv_fields
from cudanavierstokes_gb300.params import (PREC_FP32_RHS, PREC_FP64, RK3_CLASSIC, RK4_CLASSIC, boundary_layer_params,
                                           channel_params, tgv_params)
from tests._util import field_errors, rel_err, smooth_random_state, state_errors, wall_state

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _pair(oracle_mod, p, fields):
    o = oracle_mod.Oracle(p)
    s = Solver(p)
    o.set_state(*fields)
    s.copy_field_in(*fields)
    return o, s


SV = [(1, 1), (2, 1), (2, 2), (3, 1), (3, 2), (3, 3), (4, 1), (4, 2), (4, 3), (4, 4)]


@pytest.mark.parametrize("S,V", SV)
def test_rhs_periodic_all_orders(gpu_lib, oracle_mod, S, V):
    p = tgv_params(16).copy(my=20, mz=24, stencil_size=S, stencil_visc=V)
    o, s = _pair(oracle_mod, p, smooth_random_state(p, seed=S * 10 + V))
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= TOL64, errs


@pytest.mark.parametrize("S,V", SV)
def test_rhs_all_orders_odd_edges(gpu_lib, oracle_mod, S, V):
    """Odd, unequal edges (partial blocks in x and y) at every stencil order, FP64."""
    p = tgv_params(17).copy(my=13, mz=11, stencil_size=S, stencil_visc=V)
    o, s = _pair(oracle_mod, p, smooth_random_state(p, seed=100 + S * 10 + V))
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= TOL64, errs


@pytest.mark.parametrize("S,V", [(4, 4), (3, 2), (2, 1)])
def test_rhs_channel_walls(gpu_lib, oracle_mod, S, V):
    p = channel_params(24, 16, 20).copy(stencil_size=S, stencil_visc=V)
    o = oracle_mod.Oracle(p)
    f = wall_state(p, o.grid()["x"])
    o, s = _pair(oracle_mod, p, f)
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= TOL64, errs


@pytest.mark.parametrize("quirk", [0, 1])
def test_rhs_quirk_switch(gpu_lib, oracle_mod, quirk):
    p = tgv_params(16).copy(quirk_dissipation_y=quirk)
    o, s = _pair(oracle_mod, p, smooth_random_state(p, seed=7))
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= TOL64, errs


def test_quirk_changes_energy_only(gpu_lib):
    p = tgv_params(16)
    f = smooth_random_state(p, seed=7)
    a = Solver(p.copy(quirk_dissipation_y=1))
    b = Solver(p.copy(quirk_dissipation_y=0))
    a.copy_field_in(*f)
    b.copy_field_in(*f)
    ra, rb = a.calc_rhs(), b.calc_rhs()
    for q in range(4):
        assert np.array_equal(ra[q], rb[q])
    assert rel_err(ra[4], rb[4]) > 1e-9


def _bl_setup(oracle_mod, p):
    from oracle.ref_harness import blasius_like_profile
    o = oracle_mod.Oracle(p)
    spx, spz = o.sponge_strengths()
    rref, uref, wref, eref = o.sponge_refs(*blasius_like_profile())
    N = (p.my,)
    fields = [np.broadcast_to(a[:, None, :], p.shape).copy() for a in (rref, uref, np.zeros_like(rref), wref, eref)]
    o.set_sponge(spx, spz, rref, uref, wref, eref)
    s = Solver(p)
    s.set_sponge(spx, spz, rref, uref, wref, eref)
    o.set_state(*fields)
    s.copy_field_in(*fields)
    del N
    return o, s


def test_rhs_boundary_layer(gpu_lib, oracle_mod):
    """The boundary-layer start is near equilibrium (its net RHS is a small difference of
    large terms), so the single-RHS comparison uses it plus 1 % smooth perturbations; the
    unperturbed start is covered at state level by test_run_parity[bl_s3v2]."""
    p = boundary_layer_params(16, 8, 160)
    o, s = _bl_setup(oracle_mod, p)
    base = o.get_state()
    noise = smooth_random_state(p, seed=21, amp=0.01)
    f = [base[0] * noise[0], base[1] + 0.01 * noise[1], base[2] + 0.01 * noise[2], base[3] + 0.01 * noise[3],
         base[4] * noise[0]]
    o.set_state(*f)
    s.copy_field_in(*f)
    t = 0.37
    o.set_scalars(0.0, 0.0, t)
    s.set_scalars(0.0, 0.0, t)
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= TOL64, errs


def test_sponge_profile_interpolation(gpu_lib, oracle_mod):
    from oracle.ref_harness import blasius_like_profile
    p = boundary_layer_params(16, 8, 160)
    o = oracle_mod.Oracle(p)
    rref, uref, wref, eref = o.sponge_refs(*blasius_like_profile())
    s = Solver(p)
    s.set_sponge_profiles(*blasius_like_profile(), init_fields=True)
    r, u, v, w, e = s.copy_field_out()
    for a, b in ((r, rref), (u, uref), (w, wref), (e, eref)):
        assert rel_err(a, np.broadcast_to(b[:, None, :], p.shape)) <= 1e-14
    assert np.all(v == 0)


def test_boundary_layer_from_generated_inflow(gpu_lib, oracle_mod):
    """The self-similar inflow profiles of cudanavierstokes_gb300.blasius through the sponge
    spline into the reference fields, then three steps, against the oracle."""
    pytest.importorskip("scipy")
    from cudanavierstokes_gb300.blasius import self_similar_profiles
    p = boundary_layer_params(16, 8, 160)
    prof = self_similar_profiles(p.gam, p.Ma, p.Pr)
    args = [prof[k] for k in ("x", "r", "u", "w", "e")]
    o = oracle_mod.Oracle(p)
    spx, spz = o.sponge_strengths()
    rref, uref, wref, eref = o.sponge_refs(*args)
    o.set_sponge(spx, spz, rref, uref, wref, eref)
    o.set_state(*[np.broadcast_to(a[:, None, :], p.shape).copy()
                  for a in (rref, uref, np.zeros_like(rref), wref, eref)])
    s = Solver(p)
    s.set_sponge_profiles(*args, init_fields=True)
    for a, b in zip(s.copy_field_out(), o.get_state()):
        assert rel_err(a, b) <= 1e-14
    o.run(3)
    s.run(3)
    assert max(state_errors(s.copy_field_out(), o.get_state())) <= TOL64


@pytest.mark.parametrize("case", ["tgv_s4v4", "tgv_classic_s2v1", "channel_s3v2", "channel_s4v4", "bl_s3v2",
                                  "tgv_rk4"])
def test_run_parity(gpu_lib, oracle_mod, case):
    if case == "tgv_s4v4":
        p, n = tgv_params(16).copy(my=20, mz=24), 10
        f = tgv_fields(p)
    elif case == "tgv_classic_s2v1":
        p, n = tgv_params(16).copy(stencil_size=2, stencil_visc=1, scheme=RK3_CLASSIC, check_cfl=4, check_bulk=3), 6
        f = smooth_random_state(p, seed=3)
    elif case == "tgv_rk4":
        p, n = tgv_params(16).copy(scheme=RK4_CLASSIC, check_cfl=2), 5
        f = smooth_random_state(p, seed=4)
    elif case.startswith("channel"):
        S, V = (3, 2) if case == "channel_s3v2" else (4, 4)
        p, n = channel_params(16, 12, 20).copy(stencil_size=S, stencil_visc=V, check_cfl=3, check_bulk=2), 8
        f = channel_fields(p, oracle_mod.Oracle(p).grid()["x"], seed=0)
    else:
        p, n = boundary_layer_params(16, 8, 160).copy(check_cfl=2), 6
    if case == "bl_s3v2":
        o, s = _bl_setup(oracle_mod, p)
    else:
        o, s = _pair(oracle_mod, p, f)
    lo = o.run(n)
    lg = s.run(n)
    errs = state_errors(s.copy_field_out(), o.get_state())
    assert max(errs) <= TOL64, errs
    np.testing.assert_allclose(lg["time"], lo["time"], rtol=1e-13)
    so, sg = o.scalars(), s.scalars()
    assert abs(sg["dt"] - so["dt"]) <= 1e-13 * abs(so["dt"])
    assert abs(sg["dpdz"] - so["dpdz"]) <= 1e-12 * max(1.0, abs(so["dpdz"]))
    has = ~np.isnan(lo["par1"])
    assert np.array_equal(has, ~np.isnan(lg["par1"]))
    np.testing.assert_allclose(lg["par1"][has], lo["par1"][has], rtol=1e-12)


def test_fp32_rhs_against_fp64_oracle(gpu_lib, oracle_mod):
    p = tgv_params(24)
    f = smooth_random_state(p, seed=11)
    o = oracle_mod.Oracle(p)
    o.set_state(*f)
    s = Solver(p.copy(precision=PREC_FP32_RHS))
    s.copy_field_in(*f)
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= 2e-5, errs
    o.run(5)
    s.run(5)
    errs = field_errors(s.copy_field_out(), o.get_state())
    assert max(errs) <= 2e-6, errs


def test_fp32_rhs_channel(gpu_lib, oracle_mod):
    p = channel_params(24, 16, 20)
    o = oracle_mod.Oracle(p)
    f = wall_state(p, o.grid()["x"])
    o.set_state(*f)
    s = Solver(p.copy(precision=PREC_FP32_RHS))
    s.copy_field_in(*f)
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= 1e-4, errs


def test_fp32_rhs_larger_channel(gpu_lib, oracle_mod):
    """A larger stretched channel with walls (many blocks per plane) against the FP64
    oracle: one RHS and five steps."""
    p = channel_params(64, 64, 48)
    o = oracle_mod.Oracle(p)
    f = wall_state(p, o.grid()["x"])
    o.set_state(*f)
    s = Solver(p.copy(precision=PREC_FP32_RHS))
    s.copy_field_in(*f)
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= 1e-4, errs
    o.run(5)
    s.run(5)
    assert max(state_errors(s.copy_field_out(), o.get_state())) <= 2e-6


@pytest.mark.parametrize("S,V", SV)
def test_fp32_rhs_all_orders_odd_edges(gpu_lib, oracle_mod, S, V):
    """The FP32 RHS at every stencil order on a periodic box with odd, unequal edges (a
    partial last block in x and y) against the FP64 oracle."""
    p = tgv_params(17).copy(my=12, mz=10, stencil_size=S, stencil_visc=V)
    f = smooth_random_state(p, seed=S * 10 + V)
    o = oracle_mod.Oracle(p)
    o.set_state(*f)
    s = Solver(p.copy(precision=PREC_FP32_RHS))
    s.copy_field_in(*f)
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= 2e-5, errs


def test_fp32_classic_rk3_against_fp64_oracle(gpu_lib, oracle_mod):
    """The classic RK3 stages (k1, k2 registers in FP32, the state in FP64) with dt
    recomputed during the run, FP32-RHS against the FP64 oracle."""
    p = tgv_params(16).copy(my=20, mz=24, scheme=RK3_CLASSIC, check_cfl=2)
    f = smooth_random_state(p, seed=12)
    o = oracle_mod.Oracle(p)
    o.set_state(*f)
    s = Solver(p.copy(precision=PREC_FP32_RHS))
    s.copy_field_in(*f)
    o.run(5)
    s.run(5)
    assert max(state_errors(s.copy_field_out(), o.get_state())) <= 2e-6


def test_fp32_boundary_layer_against_fp64_oracle(gpu_lib, oracle_mod):
    """Boundary layer (sponge, perturbed wall, extrapolated ghosts) in FP32-RHS mode: four
    steps against the FP64 oracle."""
    p = boundary_layer_params(16, 8, 160)
    o, s64 = _bl_setup(oracle_mod, p)
    f = o.get_state()
    s = Solver(p.copy(precision=PREC_FP32_RHS))
    spx, spz = o.sponge_strengths()
    from oracle.ref_harness import blasius_like_profile
    rref, uref, wref, eref = o.sponge_refs(*blasius_like_profile())
    s.set_sponge(spx, spz, rref, uref, wref, eref)
    s.copy_field_in(*f)
    o.run(4)
    s.run(4)
    assert max(state_errors(s.copy_field_out(), o.get_state())) <= 2e-6
    del s64


def test_fp32_channel_odd_mx(gpu_lib, oracle_mod):
    """Stretched channel with walls and an odd wall-normal size (non-uniform x tables):
    RHS and three steps against the FP64 oracle."""
    p = channel_params(25, 16, 20)
    o = oracle_mod.Oracle(p)
    f = wall_state(p, o.grid()["x"])
    o.set_state(*f)
    s = Solver(p.copy(precision=PREC_FP32_RHS))
    s.copy_field_in(*f)
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= 1e-4, errs
    o.run(3)
    s.run(3)
    assert max(state_errors(s.copy_field_out(), o.get_state())) <= 2e-6


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_FP32_RHS])
def test_rhs_in_band_groups(gpu_lib, oracle_mod, prec):
    """A plane wide enough (mx = 512) for the RHS kernel to be launched over groups of
    4-row bands (9 of the 16 bands, then 7): the RHS and two steps against the oracle."""
    p = channel_params(512, 64, 12)
    o = oracle_mod.Oracle(p)
    f = wall_state(p, o.grid()["x"])
    o.set_state(*f)
    s = Solver(p.copy(precision=prec))
    s.copy_field_in(*f)
    errs = field_errors(s.calc_rhs(), o.rhs())
    assert max(errs) <= (TOL64 if prec == PREC_FP64 else 1e-4), errs
    o.run(2)
    s.run(2)
    assert max(state_errors(s.copy_field_out(), o.get_state())) <= (TOL64 if prec == PREC_FP64 else 2e-6)


def test_rk4_third_order_or_better(gpu_lib):
    """RK4 (no counterpart in the reference): halving dt cuts the error against a fine
    reference run by at least 2^3."""
    base = tgv_params(16).copy(scheme=RK4_CLASSIC)
    f = smooth_random_state(base, seed=5)
    T = None
    res = {}
    for cfl in (0.4, 0.2, 0.05):
        s = Solver(base.copy(cfl=cfl, check_cfl=10**6))
        s.copy_field_in(*f)
        s.run(1)
        dt = s.scalars()["dt"]
        if T is None:
            T = 8 * dt
        s.copy_field_in(*f)
        nsteps = int(round(T / dt))
        s.run(nsteps)
        res[cfl] = s.copy_field_out()
    e1 = rel_err(res[0.4][1], res[0.05][1])
    e2 = rel_err(res[0.2][1], res[0.05][1])
    assert e1 / e2 > 8.0, (e1, e2)


def test_determinism(gpu_lib):
    p = channel_params(24, 16, 20)
    f = channel_fields(p, Solver(p).grid()["x"], seed=1)
    outs = []
    for _ in range(2):
        s = Solver(p)
        s.copy_field_in(*f)
        s.run(4)
        outs.append(s.copy_field_out())
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_grid_matches_oracle(gpu_lib, oracle_mod):
    for p in (channel_params(24, 16, 20), boundary_layer_params(16, 8, 160), tgv_params(16)):
        g = Solver(p).grid()
        go = oracle_mod.Oracle(p).grid()
        for k in ("x", "xp", "xpp", "y", "z"):
            np.testing.assert_array_equal(g[k], go[k])


def test_graph_replay_matches_direct_launches(gpu_lib):
    p = channel_params(24, 16, 20).copy(check_cfl=3, check_bulk=2)
    f = channel_fields(p, Solver(p).grid()["x"], seed=2)
    outs, logs = [], []
    for graphs in (True, False):
        s = Solver(p)
        s.set_graphs(graphs)
        s.copy_field_in(*f)
        logs.append(s.run(7))
        logs.append(s.run(4))      # a second run restarts the step counter and the schedule
        outs.append(s.copy_field_out())
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    for k in ("par1", "time"):
        np.testing.assert_array_equal(logs[0][k], logs[2][k])
        np.testing.assert_array_equal(logs[1][k], logs[3][k])


def test_fp32_rhs_stage_kinds_run_alike(gpu_lib):
    """Performance guard: a Wray stage that reads the previous RHS (a != 0) must not be much
    slower than the first stage (interleaved register loads and stores once made the
    kernel 3.7x slower for those stages)."""
    p = channel_params(128, 160, 48, precision=PREC_FP32_RHS)
    s = Solver(p)
    s.copy_field_in(*channel_fields(p, s.grid()["x"], seed=0))
    s.time_phases(3)
    first = min(s.time_phases(1)["rhs_ms"] for _ in range(3))
    avg = min(s.time_phases(3)["rhs_ms"] for _ in range(3))
    assert avg <= 1.5 * first, (first, avg)


def test_gpu_rhs_mirror_and_shift(gpu_lib):
    """Independent of the oracle: the channel RHS of a state mirrored in x (wall-normal
    velocity reversed) is the mirrored RHS, and a periodic shift by one cell in y shifts
    the RHS bit for bit."""
    p = channel_params(24, 12, 16)
    s = Solver(p)
    x = s.grid()["x"]
    f = wall_state(p, x, seed=5)
    s.copy_field_in(*f)
    a = s.calc_rhs()
    m = [g[:, :, ::-1].copy() for g in f]
    m[1] = -m[1]
    s.copy_field_in(*m)
    b = s.calc_rhs()
    for q in range(5):
        ref = -a[q][:, :, ::-1] if q == 1 else a[q][:, :, ::-1]
        assert np.max(np.abs(b[q] - ref)) <= 1e-13 * np.max(np.abs(a[q])), q
    s.copy_field_in(*[np.roll(g, 1, axis=1) for g in f])
    c = s.calc_rhs()
    for q in range(5):
        assert np.array_equal(c[q], np.roll(a[q], 1, axis=1)), q
