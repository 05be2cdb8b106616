"""Seeded synthetic workloads: the batched Taylor-Green ensemble and the serving request
stream (no public dataset is involved; inputs are analytic fields and seeded draws)."""
from __future__ import annotations

import math

import numpy as np

from .initial import channel_fields, tgv_fields
from .params import PREC_FP32_RHS, CnsParams, channel_params, tgv_params

ENSEMBLE_EDGES = (32, 48, 64, 96, 128)


def ensemble(n: int = 48, seed: int = 0, precision: int = PREC_FP32_RHS):
    """n Taylor-Green boxes: edge uniform over {32, 48, 64, 96, 128}, Re log-uniform in
    [400, 3200], Ma uniform in [0.1, 0.8], per-axis phase offsets uniform in [0, 2 pi)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        edge = int(rng.choice(ENSEMBLE_EDGES))
        re = float(math.exp(rng.uniform(math.log(400.0), math.log(3200.0))))
        ma = float(rng.uniform(0.1, 0.8))
        ph = tuple(float(x) for x in rng.uniform(0.0, 2 * math.pi, size=3))
        p = tgv_params(edge, precision=precision, Re=re, Ma=ma)
        out.append((p, ph))
    return out


def ensemble_fields(p: CnsParams, phases):
    return tgv_fields(p, phases=phases)


SERVE_EDGES = (32, 48, 64, 96, 128, 160, 192)


def serving_requests(n: int, rate: float, seed: int = 0, precision: int = PREC_FP32_RHS, channel_frac: float = 0.25):
    """Poisson arrivals at `rate` per second of "advance N steps" requests, N uniform in
    [50, 500]: Taylor-Green boxes with edges 32..192 (parameters drawn as the ensemble) and
    stretched channels 64 x 48 x 64 (channel parameters). Returns (t_arrival, params, kind,
    nsteps, seed) tuples; fields are generated by request_fields."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for q in range(n):
        t += float(rng.exponential(1.0 / rate))
        nsteps = int(rng.integers(50, 501))
        if rng.uniform() < channel_frac:
            p = channel_params(64, 48, 64, precision=precision)
            out.append((t, p, "channel", nsteps, int(rng.integers(1 << 30))))
        else:
            edge = int(rng.choice(SERVE_EDGES))
            re = float(math.exp(rng.uniform(math.log(400.0), math.log(3200.0))))
            ma = float(rng.uniform(0.1, 0.8))
            p = tgv_params(edge, precision=precision, Re=re, Ma=ma)
            out.append((t, p, "tgv", nsteps, int(rng.integers(1 << 30))))
    return out


def request_fields(p: CnsParams, kind: str, seed: int):
    if kind == "channel":
        from .solver import host_grid
        return channel_fields(p, host_grid(p)["x"], seed=seed)
    rng = np.random.default_rng(seed)
    return tgv_fields(p, phases=tuple(float(v) for v in rng.uniform(0.0, 2 * math.pi, size=3)))
