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
