"""CPU tests of the oracle (the CPU restatement used as the parity reference and CPU baseline):
grid, stencil order, conservation, dt formula, time order, boundary images."""
import math

import numpy as np
import pytest

from cudanavierstokes_gb300.initial import tgv_fields
from cudanavierstokes_gb300.params import (Derived, RK3_CLASSIC, RK4_CLASSIC, boundary_layer_params,
                                           channel_params, tgv_params)
from tests._util import rel_err, smooth_random_state


def test_uniform_grid_and_cell_widths(oracle_mod):
    p = tgv_params(16)
    g = oracle_mod.Oracle(p).grid()
    np.testing.assert_allclose(g["x"], p.Lx * (np.arange(16) + 0.5) / 16, rtol=0, atol=1e-15)
    np.testing.assert_allclose(g["dxv"], p.Lx / 16, rtol=1e-14)


def test_channel_grid_symmetric_and_stretched(oracle_mod):
    p = channel_params(32, 8, 8)
    g = oracle_mod.Oracle(p).grid()
    x = g["x"]
    assert np.all(np.diff(x) > 0) and 0 < x[0] and x[-1] < p.Lx
    np.testing.assert_allclose(x + x[::-1], p.Lx, atol=1e-13)
    assert (x[1] - x[0]) < (x[16] - x[15])          # clustered at the walls
    np.testing.assert_allclose(g["dxv"].sum(), p.Lx, rtol=1e-13)


@pytest.mark.parametrize("V", [1, 2, 3, 4])
def test_gradient_order_of_accuracy(oracle_mod, V):
    errs = []
    for n in (16, 32):
        p = tgv_params(n).copy(stencil_size=4, stencil_visc=V)
        o = oracle_mod.Oracle(p)
        xs = 2 * math.pi * (np.arange(n) + 0.5) / n
        Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
        u = np.sin(X) * np.cos(Y)
        d = Derived.of(p)
        rho = np.ones(p.shape)
        e = d.Rgas / (p.gam - 1) + 0.5 * u * u
        o.set_state(rho, u, np.zeros(p.shape), np.zeros(p.shape), e)
        g, _ = o.gradients()
        errs.append(np.max(np.abs(g[0] - np.cos(X) * np.cos(Y))))
    order = math.log2(errs[0] / errs[1])
    assert order > 2 * V - 0.3, (V, errs, order)


def test_mass_conservation_periodic(oracle_mod):
    p = tgv_params(16).copy(my=20, mz=24)
    o = oracle_mod.Oracle(p)
    o.set_state(*smooth_random_state(p, seed=3))
    R = o.rhs()
    assert abs(R[0].sum()) <= 1e-12 * np.abs(R[0]).sum()


def test_inviscid_momentum_conservation(oracle_mod):
    p = tgv_params(16).copy(Re=1e12)
    o = oracle_mod.Oracle(p)
    o.set_state(*smooth_random_state(p, seed=4))
    R = o.rhs()
    for q in (1, 2, 3):
        assert abs(R[q].sum()) <= 1e-11 * np.abs(R[q]).sum()


def test_dt_formula(oracle_mod):
    p = channel_params(24, 8, 12)
    o = oracle_mod.Oracle(p)
    g = o.grid()
    r, u, v, w, e = smooth_random_state(p, seed=5)
    o.set_state(r, u, v, w, e)
    d = Derived.of(p)
    ien = e / r - 0.5 * (u * u + v * v + w * w)
    sos = np.sqrt(p.gam * (p.gam - 1) * ien)
    T = (p.gam - 1.0) / d.Rgas * ien
    mu = T ** p.viscexp / p.Re
    dx = g["dxv"][None, None, :]
    dy, dz = p.Ly / p.my, p.Lz / p.mz
    conv = np.maximum((np.abs(u) + sos) / dx, np.maximum((np.abs(v) + sos) / dy, (np.abs(w) + sos) / dz))
    visc = np.maximum(mu / dx ** 2, np.maximum(mu / dy ** 2, mu / dz ** 2))
    ref = np.min(p.cfl / np.maximum(conv, visc))
    assert abs(o.calc_dt() - ref) <= 1e-12 * ref


def test_low_storage_rk3_third_order(oracle_mod):
    base = tgv_params(16)
    f = smooth_random_state(base, seed=6)
    res = {}
    T = None
    for cfl in (0.4, 0.2, 0.05):
        o = oracle_mod.Oracle(base.copy(cfl=cfl, check_cfl=10**6))
        o.set_state(*f)
        dt = o.calc_dt()
        T = T or 8 * dt
        o.run(int(round(T / dt)))
        res[cfl] = o.get_state()
    e1 = rel_err(res[0.4][1], res[0.05][1])
    e2 = rel_err(res[0.2][1], res[0.05][1])
    assert e1 / e2 > 6.0, (e1, e2)


def test_classic_rk3_third_order(oracle_mod):
    base = tgv_params(16).copy(scheme=RK3_CLASSIC)
    f = smooth_random_state(base, seed=6)
    res = {}
    T = None
    for cfl in (0.4, 0.2, 0.05):
        o = oracle_mod.Oracle(base.copy(cfl=cfl, check_cfl=10**6))
        o.set_state(*f)
        dt = o.calc_dt()
        T = T or 8 * dt
        o.run(int(round(T / dt)))
        res[cfl] = o.get_state()
    e1 = rel_err(res[0.4][1], res[0.05][1])
    e2 = rel_err(res[0.2][1], res[0.05][1])
    assert e1 / e2 > 6.0, (e1, e2)


def test_classic_rk4_fourth_order(oracle_mod):
    """The oracle's RK4 (a textbook restatement; the reference has no RK4): halving dt cuts
    the time-integration error by ~16."""
    base = tgv_params(16).copy(scheme=RK4_CLASSIC)
    f = smooth_random_state(base, seed=6)
    res = {}
    T = None
    for cfl in (0.4, 0.2, 0.05):
        o = oracle_mod.Oracle(base.copy(cfl=cfl, check_cfl=10**6))
        o.set_state(*f)
        dt = o.calc_dt()
        T = T or 8 * dt
        o.run(int(round(T / dt)))
        res[cfl] = o.get_state()
    e1 = rel_err(res[0.4][1], res[0.05][1])
    e2 = rel_err(res[0.2][1], res[0.05][1])
    assert e1 / e2 > 12.0, (e1, e2)


def test_tgv_kinetic_energy_decays(oracle_mod):
    p = tgv_params(16)
    o = oracle_mod.Oracle(p)
    o.set_state(*tgv_fields(p))
    logs = o.run(10)
    k0 = logs["par1"][0]
    assert abs(k0 - 0.25) < 1e-3        # <u.u> of the Taylor-Green start is 1/4
    ke1, _ = o.bulk()
    assert ke1 < k0


def test_tgv_initial_dissipation_and_enstrophy(oracle_mod):
    """Taylor-Green start u = sin x cos y cos z, v = -cos x sin y cos z, w = 0: the mean
    squared vorticity is 1/8 + 1/8 + 4/8 = 3/4 and, being divergence-free, the viscous
    dissipation is mu <|curl u|^2> = 3/4 mu with mu = T/Re, T = 1 up to the O(Ma^2)
    pressure field; the decay rate of K = <rho |u|^2>/2 over the first steps matches it."""
    p = tgv_params(32)
    o = oracle_mod.Oracle(p)
    o.set_state(*tgv_fields(p))
    d = o.dissipation()
    assert abs(d["enstrophy"] - 0.75) <= 1e-7
    assert abs(d["eps"] * p.Re / 0.75 - 1.0) <= 3e-3
    ke0, _ = o.bulk()                      # <u.u>
    o.run(20)
    ke1, _ = o.bulk()
    t1 = o.scalars()["time"]
    d1 = o.dissipation()
    rate = 0.5 * (ke0 - ke1) / t1          # -d(<u.u>/2)/dt over the first steps
    assert abs(rate / (0.5 * (d["eps"] + d1["eps"])) - 1.0) <= 2e-2


def test_quirk_only_affects_energy(oracle_mod):
    p = tgv_params(16)
    f = smooth_random_state(p, seed=8)
    a = oracle_mod.Oracle(p.copy(quirk_dissipation_y=1))
    b = oracle_mod.Oracle(p.copy(quirk_dissipation_y=0))
    a.set_state(*f)
    b.set_state(*f)
    ra, rb = a.rhs(), b.rhs()
    for q in range(4):
        assert np.array_equal(ra[q], rb[q])
    assert not np.array_equal(ra[4], rb[4])


def test_channel_forcing_controller(oracle_mod):
    p = channel_params(16, 8, 8)
    o = oracle_mod.Oracle(p)
    g = o.grid()
    from cudanavierstokes_gb300.initial import channel_fields
    o.set_state(*channel_fields(p, g["x"], seed=0))
    logs = o.run(1)
    r, u, v, w, e = o.get_state()
    # dpdz after step 0 follows 0.99*dpdz0 - 0.5*(bulk(rho w)/bulk(rho) - 1) of the step-0 state
    assert logs["dpdz"][0] != p.dpdz_init


def test_threads_do_not_change_results(oracle_mod):
    p = tgv_params(16)
    f = smooth_random_state(p, seed=9)
    outs = []
    for nt in (1, 3):
        oracle_mod.set_threads(nt)
        o = oracle_mod.Oracle(p)
        o.set_state(*f)
        o.run(2)
        outs.append(o.get_state())
    oracle_mod.set_threads(oracle_mod.max_threads())
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_boundary_layer_runs(oracle_mod):
    from oracle.ref_harness import blasius_like_profile
    p = boundary_layer_params(16, 8, 160)
    o = oracle_mod.Oracle(p)
    spx, spz = o.sponge_strengths()
    assert spz[0] > 0 and spz[-1] > 0 and np.all(spx >= 0) and spx[0] == 0
    refs = o.sponge_refs(*blasius_like_profile())
    o.set_sponge(spx, spz, *refs)
    rref, uref, wref, eref = refs
    o.set_state(*[np.broadcast_to(a[:, None, :], p.shape).copy()
                  for a in (rref, uref, np.zeros_like(rref), wref, eref)])
    logs = o.run(3)
    assert np.all(np.isfinite(o.get_state()[0])) and logs["dt"][0] > 0


def test_rejects_bad_parameters(oracle_mod):
    with pytest.raises(ValueError):
        oracle_mod.Oracle(tgv_params(16).copy(stencil_visc=5))
    with pytest.raises(ValueError):
        oracle_mod.Oracle(tgv_params(4))


def test_channel_rhs_mirror_symmetry(oracle_mod):
    """The stretched channel is symmetric about its mid-plane: a state mirrored in x with
    the wall-normal velocity reversed has the mirrored RHS, with the wall-normal momentum
    term reversed (walls, stretched-grid metrics and fluxes treat both halves alike)."""
    from tests._util import wall_state
    p = channel_params(24, 12, 16)
    o = oracle_mod.Oracle(p)
    x = o.grid()["x"]
    assert np.allclose(x + x[::-1], p.Lx, atol=1e-13)
    f = wall_state(p, x, seed=5)
    o.set_state(*f)
    a = o.rhs()
    m = [g[:, :, ::-1].copy() for g in f]
    m[1] = -m[1]
    o.set_state(*m)
    b = o.rhs()
    for q in range(5):
        ref = -a[q][:, :, ::-1] if q == 1 else a[q][:, :, ::-1]
        assert np.max(np.abs(b[q] - ref)) <= 1e-13 * np.max(np.abs(a[q])), q


def test_periodic_shift_invariance(oracle_mod):
    """Shifting a periodic state by one cell in y (and in z) shifts its RHS bit for bit."""
    p = tgv_params(12).copy(my=10, mz=14)
    o = oracle_mod.Oracle(p)
    f = smooth_random_state(p, seed=9)
    o.set_state(*f)
    a = o.rhs()
    for axis in (1, 0):   # y, then z ([k][j][i] arrays)
        o.set_state(*[np.roll(g, 1, axis=axis) for g in f])
        b = o.rhs()
        for q in range(5):
            assert np.array_equal(b[q], np.roll(a[q], 1, axis=axis)), (axis, q)
