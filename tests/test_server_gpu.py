"""Serving loop: requests that arrive while others run join the batch between steps; every
result is bitwise identical to the same request served alone."""
import time

import numpy as np
import pytest

from cudanavierstokes_gb300.initial import tgv_fields
from cudanavierstokes_gb300.params import PREC_FP32_RHS, channel_params, tgv_params
from cudanavierstokes_gb300.server import Server
from tests._util import smooth_random_state

pytestmark = pytest.mark.gpu


def requests():
    out = []
    for n, (edge, steps) in enumerate(((16, 6), (24, 9), (20, 4))):
        p = tgv_params(edge, precision=PREC_FP32_RHS, Re=400.0 + 200 * n, Ma=0.1 + 0.1 * n)
        out.append((p, tgv_fields(p, phases=(0.3 * n, 0.1 * n, 0.0)), steps))
    c = channel_params(24, 16, 20, precision=PREC_FP32_RHS)
    out.append((c, smooth_random_state(c, seed=9, amp=0.02), 5))
    return out


def test_continuous_batching_and_isolation(gpu_lib):
    reqs = requests()
    srv = Server(precision=PREC_FP32_RHS)
    ids = []
    for p, f, n in reqs:               # staggered arrivals while earlier requests run
        ids.append(srv.submit(p, f, n))
        time.sleep(0.02)
    mixed = [srv.wait(i, timeout_s=120) for i in ids]
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["p99_s"] >= st["p50_s"] > 0
    assert st["point_steps"] == sum(p.npoints * n for p, _, n in reqs)
    srv.close()
    for (p, f, n), res in zip(reqs, mixed):
        alone = Server(precision=PREC_FP32_RHS)
        rid = alone.submit(p, f, n)
        ref = alone.wait(rid, timeout_s=120)
        alone.close()
        for a, b in zip(res, ref):
            assert np.array_equal(a, b)


def test_admission_waits_for_budget(gpu_lib):
    p = tgv_params(16, precision=PREC_FP32_RHS)
    f = tgv_fields(p)
    # room for about one member at a time: the second request waits for the first to retire
    srv = Server(precision=PREC_FP32_RHS, hbm_budget_bytes=7 * 1024 * 1024)
    a = srv.submit(p, f, 5)
    b = srv.submit(p, f, 5)
    ra = srv.wait(a, timeout_s=120)
    rb = srv.wait(b, timeout_s=120)
    for x, y in zip(ra, rb):
        assert np.array_equal(x, y)
    srv.close()


def test_invalid_request_is_rejected(gpu_lib):
    srv = Server(precision=PREC_FP32_RHS)
    p = tgv_params(16, precision=PREC_FP32_RHS, stencil_size=5)
    with pytest.raises(Exception):
        srv.submit(p, tgv_fields(tgv_params(16)), 3)
    srv.close()
