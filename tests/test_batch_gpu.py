"""Batched ensemble, in both execution modes (one persistent launch per RK stage for all
members; members' own step graphs on concurrent streams): members of uneven size and
physics against standalone solvers; a member's result is identical alone and in a mix;
membership changes between steps; the autotuner; the bounded barrier's give-up path."""
import ctypes

import numpy as np
import pytest

from cudanavierstokes_gb300 import Solver
from cudanavierstokes_gb300.batch import Batch
from cudanavierstokes_gb300.initial import channel_fields, tgv_fields
from cudanavierstokes_gb300.params import (PREC_FP32_RHS, PREC_FP64, boundary_layer_params, channel_params,
                                           tgv_params)
from tests._util import smooth_random_state, state_errors

pytestmark = pytest.mark.gpu


def members(prec):
    a = tgv_params(16, precision=prec, Re=800.0)
    b = tgv_params(24, precision=prec, my=20, mz=28, Ma=0.3, check_cfl=2)
    c = channel_params(24, 16, 20, precision=prec, check_cfl=3, check_bulk=2)
    fa = tgv_fields(a)
    fb = smooth_random_state(b, seed=3)
    fc = channel_fields(c, Solver(c).grid()["x"], seed=0)
    return [(a, fa), (b, fb), (c, fc)]


MODES = (0, 1)   # persistent, concurrent


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("prec", [PREC_FP64, PREC_FP32_RHS])
def test_batch_matches_standalone_solvers(gpu_lib, prec, mode):
    ms = members(prec)
    n = 5
    bt = Batch(precision=prec)
    bt.set_mode(mode)
    ids = [bt.add(p, f, max_steps=16) for p, f in ms]
    bt.step(n)
    tol = 1e-12 if prec == PREC_FP64 else 1e-6
    for mid, (p, f) in zip(ids, ms):
        s = Solver(p)
        s.copy_field_in(*f)
        lg = s.run(n)
        errs = state_errors(bt.fields(mid), s.copy_field_out())
        assert max(errs) <= tol, (mid, errs)
        lb = bt.logs(mid, n)
        # FP32 RHS: the persistent kernel scales compile-time stencil weights by the spacing,
        # the standalone kernel uses premultiplied weights, so they agree to FP32 rounding
        # and the time steps (from the state) to well within the state tolerance
        np.testing.assert_allclose(lb["time"], lg["time"], rtol=1e-12 if prec == PREC_FP64 else tol)
        has = ~np.isnan(lg["par1"])
        np.testing.assert_allclose(lb["par1"][has], lg["par1"][has], rtol=1e-10 if prec == PREC_FP64 else tol)
        assert bt.steps_done(mid) == n


@pytest.mark.parametrize("mode", MODES)
def test_member_alone_equals_member_in_mix(gpu_lib, mode):
    ms = members(PREC_FP32_RHS)
    alone = Batch(precision=PREC_FP32_RHS)
    alone.set_mode(mode)
    i0 = alone.add(*ms[1], max_steps=8)
    alone.step(4)
    mix = Batch(precision=PREC_FP32_RHS)
    mix.set_mode(mode)
    ids = [mix.add(p, f, max_steps=8) for p, f in ms]
    mix.step(4)
    for a, b in zip(alone.fields(i0), mix.fields(ids[1])):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("mode", MODES)
def test_membership_changes_between_steps(gpu_lib, mode):
    ms = members(PREC_FP64)
    bt = Batch(precision=PREC_FP64)
    bt.set_mode(mode)
    i0 = bt.add(*ms[0], max_steps=20)
    bt.step(2)
    i1 = bt.add(*ms[1], max_steps=20)     # joins later (other ping-pong parity)
    bt.step(3)
    bt.remove(i0)
    i2 = bt.add(*ms[2], max_steps=20)
    bt.step(2)
    assert bt.info()["count"] == 2
    assert bt.steps_done(i1) == 5 and bt.steps_done(i2) == 2
    # the late members equal standalone runs of the same length
    for mid, (p, f), n in ((i1, ms[1], 5), (i2, ms[2], 2)):
        s = Solver(p)
        s.copy_field_in(*f)
        s.run(n)
        assert max(state_errors(bt.fields(mid), s.copy_field_out())) <= 1e-12


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("prec", [PREC_FP64, PREC_FP32_RHS])
def test_boundary_layer_member(gpu_lib, oracle_mod, prec, mode):
    """A boundary-layer member (sponge, perturbed wall, extrapolated ghosts, time-dependent
    wall ghosts) next to a periodic one equals its standalone solver."""
    from oracle.ref_harness import blasius_like_profile
    p = boundary_layer_params(16, 8, 160, precision=prec, stencil_size=4, stencil_visc=4)   # the batch's orders
    o = oracle_mod.Oracle(p)
    spx, spz = o.sponge_strengths()
    refs = o.sponge_refs(*blasius_like_profile())
    rref, uref, wref, eref = refs
    noise = smooth_random_state(p, seed=8, amp=0.01)
    f = [np.broadcast_to(a[:, None, :], p.shape) * (1.0 + 0.01 * noise[0]) if q in (0, 4) else
         np.broadcast_to(a[:, None, :], p.shape) + 0.01 * noise[q]
         for q, a in enumerate((rref, uref, np.zeros_like(rref), wref, eref))]
    other = members(prec)[0]
    bt = Batch(precision=prec)
    bt.set_mode(mode)
    i0 = bt.add(*other, max_steps=8)
    ib = bt.add(p, f, max_steps=8)
    bt.set_member_sponge(ib, spx, spz, rref, uref, wref, eref)
    bt.step(4)
    s = Solver(p)
    s.set_sponge(spx, spz, rref, uref, wref, eref)
    s.copy_field_in(*f)
    s.run(4)
    tol = 1e-12 if prec == PREC_FP64 else 1e-6
    assert max(state_errors(bt.fields(ib), s.copy_field_out())) <= tol
    assert bt.steps_done(i0) == 4


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("S,V", [(1, 1), (2, 2), (3, 2), (4, 1)])
def test_other_stencil_orders(gpu_lib, S, V, mode):
    """Batches of other stencil orders (their own kernel instantiations): a periodic box and
    a channel against standalone solvers, FP64."""
    ms = [(p.copy(stencil_size=S, stencil_visc=V), f) for p, f in members(PREC_FP64)[1:]]
    bt = Batch(precision=PREC_FP64, stencil_size=S, stencil_visc=V)
    bt.set_mode(mode)
    ids = [bt.add(p, f, max_steps=8) for p, f in ms]
    bt.step(3)
    for mid, (p, f) in zip(ids, ms):
        s = Solver(p)
        s.copy_field_in(*f)
        s.run(3)
        assert max(state_errors(bt.fields(mid), s.copy_field_out())) <= 1e-12


def test_budget_admission(gpu_lib):
    p, f = members(PREC_FP64)[0]
    bt = Batch(precision=PREC_FP64, hbm_budget_bytes=1)
    with pytest.raises(Exception):
        bt.add(p, f, max_steps=4)
    assert bt.info()["count"] == 0


def test_autotune_and_shapes(gpu_lib):
    ms = members(PREC_FP32_RHS)
    bt = Batch(precision=PREC_FP32_RHS)
    for p, f in ms:
        bt.add(p, f, max_steps=64)
    ms_best = bt.tune(2)
    t, b = bt.shape()
    assert t in (128, 256) and b >= 1
    assert bt.mode() in MODES
    assert ms_best > 0 or ms_best == -1.0
    bt.step(1)


def test_bounded_barrier_gives_up(gpu_lib):
    flag = ctypes.c_int(-1)
    assert gpu_lib.cns_selftest_barrier_timeout(0, 2000, ctypes.byref(flag)) == 0
    assert flag.value == 1


def test_persistent_fp32_batch_beyond_the_member_table(gpu_lib):
    """An FP32 batch of more members than the persistent kernel's argument table holds (64)
    runs its RHS phase with the members' parameters staged in shared memory: members of
    uneven size and physics still equal their standalone solvers."""
    n = 66
    ms = []
    for q in range(n):
        p = tgv_params(10 + (q % 4) * 2, precision=PREC_FP32_RHS, my=9 + q % 3, mz=10 + q % 5,
                       Re=400.0 + 37.0 * q, Ma=0.1 + 0.005 * q)
        ms.append((p, smooth_random_state(p, seed=100 + q)))
    bt = Batch(precision=PREC_FP32_RHS)
    bt.set_mode(0)
    ids = [bt.add(p, f, max_steps=8) for p, f in ms]
    bt.step(3)
    for q in (0, 1, 31, 64, 65):
        p, f = ms[q]
        s = Solver(p)
        s.copy_field_in(*f)
        s.run(3)
        assert max(state_errors(bt.fields(ids[q]), s.copy_field_out())) <= 1e-6, q
