"""Boundary-layer inflow generator: the reference's own selfSimilarSol output (golden
vectors made by tests/golden/make_blasius_golden.py), the incompressible Blasius limit,
the adiabatic-wall recovery temperature and the files the driver reads."""
import math
import os

import numpy as np
import pytest

pytest.importorskip("scipy")
from cudanavierstokes_gb300.blasius import self_similar_profiles, write_profiles  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "blasius_ref_profiles.npz")


def test_matches_reference_generator():
    g = np.load(GOLDEN)
    p = self_similar_profiles(float(g["gam"]), float(g["Ma"]), float(g["Pr"]))
    for name in "xruwe":
        assert p[name].shape == g[name].shape
        assert np.abs(p[name] - g[name]).max() <= 1e-10 * np.abs(g[name]).max(), name


def test_incompressible_blasius_limit():
    p = self_similar_profiles(Ma=1e-3)
    assert abs(p["shear_wall"] - 0.469600) < 2e-4        # f''(0) of f''' + f f'' = 0
    assert abs(p["t_wall"] - 1.0) < 1e-6
    assert np.allclose(p["r"], 1.0, atol=1e-6)


def test_adiabatic_wall_recovery_temperature():
    gam, Ma, Pr = 1.4, 2.0, 0.72
    p = self_similar_profiles(gam, Ma, Pr)
    recovery = (p["t_wall"] - 1.0) / (0.5 * (gam - 1.0) * Ma * Ma)
    assert abs(recovery - math.sqrt(Pr)) < 0.02            # laminar recovery factor ~ sqrt(Pr)
    w = p["w"]
    assert abs(w[0]) < 1e-12 and np.all(np.diff(w[:600]) >= -1e-5) and abs(w[-1] - 1.0) < 1e-5   # solver tolerance


def test_writes_driver_files(tmp_path):
    p = self_similar_profiles()
    write_profiles(str(tmp_path), p)
    for name in "xruwe":
        a = np.fromfile(tmp_path / "blasius1D" / f"{name}Prof.bin")
        np.testing.assert_array_equal(a, p[name])
