"""CPU tests of bench.py's host-side pieces: argument defaults (one GPU, a run that ends
within minutes), the cubic evaluation at t_end of the precision study, and the roofline's
DRAM traffic taken from the committed ncu summaries."""
import sys

import numpy as np
import pytest

import bench


def test_defaults(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse_args()
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1
    assert a.impl == "gb300" and a.workload == "channel" and a.precision == "fp64"
    assert a.batch_members == 48 and a.batch_mode == "tuned"


def test_at_time_recovers_a_cubic():
    t = np.linspace(0.0, 2.0, 41)
    y = 1.0 - 0.3 * t + 0.2 * t ** 2 - 0.05 * t ** 3
    v, d = bench.at_time(t, y, 1.23)
    assert v == pytest.approx(1.0 - 0.3 * 1.23 + 0.2 * 1.23 ** 2 - 0.05 * 1.23 ** 3, rel=1e-12)
    assert d == pytest.approx(-0.3 + 0.4 * 1.23 - 0.15 * 1.23 ** 2, rel=1e-10)


def test_traffic_scales_with_points():
    """Each precision's summary gives bytes per launch on its capture; the roofline scales
    them to the benchmark grid by points."""
    for fp32 in (False, True):
        kv = bench.read_profile_summary(bench.TRAFFIC_FILE_FP32 if fp32 else bench.TRAFFIC_FILE)
        per_point = float(kv["dram_bytes_per_launch"]) / float(kv["points"])
        assert 100.0 < per_point < 400.0
        assert bench.read_traffic(2 * int(kv["points"]), fp32=fp32) == pytest.approx(
            2 * float(kv["dram_bytes_per_launch"]))
    assert bench.read_traffic(1000, fp32=True) < bench.read_traffic(1000)


def test_fp32_roofline_object():
    """The FP32-RHS leg's roofline: algorithmic bytes against the measured HBM bandwidth, the
    FP32 flop rate against the given FMA peak, the ncu traffic and the executed counters of
    the committed summary."""
    from cudanavierstokes_gb300 import roofline as rf
    N = 3932160
    ph = {"ghost_ms": 0.0135, "grad_ms": 0.0361, "rhs_ms": 0.25}
    r = bench.fp32_roofline(N, 4, 4, ph, 70.0)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(rf.RHS_KERNEL_BYTES * N / 0.25e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["fp32"]["frac"] == pytest.approx(r["fp32"]["achieved"] / 70.0)
    assert r["traffic"] == pytest.approx(bench.read_traffic(N, fp32=True))
    assert r["executed"]["global_ld_per_point"] > 0 and 0 < r["executed"]["fp64_pipe_active_pct"] <= 100


def test_reference_arm_times_the_full_grid(monkeypatch):
    """--impl reference measures the configured channel grid itself (no extrapolation from a
    sample): the oracle is set up on the workload's own parameters."""
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    a = bench.parse_args()
    p, _ = bench.workload(a.workload, "fp64", a.grid)
    assert (p.mx, p.my, p.mz) == (128, 160, 192)


def test_reference_arm_line(monkeypatch, capsys, oracle_mod):
    """The reference arm end to end on a small channel: one JSON line with the arm's tag, the
    metric and its own cpu_baseline and e2e (no host-device copies)."""
    import json
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--grid", "16,12,20", "--steps", "2",
                                      "--warmup", "1"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["steps"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["grid"] == [16, 12, 20]


def test_precision_flag_maps_to_the_solver_modes(monkeypatch):
    """--precision fp64 | fp32 | pair selects the solver's precision for the workload."""
    from cudanavierstokes_gb300.params import PREC_FP32_RHS, PREC_FP64, PREC_PAIR_RHS
    for flag, prec in (("fp64", PREC_FP64), ("fp32", PREC_FP32_RHS), ("pair", PREC_PAIR_RHS)):
        monkeypatch.setattr(sys, "argv", ["bench.py", "--precision", flag])
        a = bench.parse_args()
        p, _ = bench.workload(a.workload, a.precision, a.grid)
        assert p.precision == prec and (p.mx, p.my, p.mz) == (128, 160, 192)
