"""Shared helpers for the tests: comparison norms and seeded test states."""
from __future__ import annotations

import math

import numpy as np

from cudanavierstokes_gb300.params import Derived


def rel_err(a, b) -> float:
    """Norm-wise relative error max|a-b| / max|b| (pointwise relative error is undefined
    where a field is zero, e.g. w in the Taylor-Green start)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = float(np.max(np.abs(b)))
    if den == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b))) / den


def field_errors(A, B):
    return [rel_err(a, b) for a, b in zip(A, B)]


def state_errors(A, B):
    """Per-field errors of a (rho, u, v, w, rhoE) state: rho and rhoE relative to their own
    maximum; the velocity components relative to the largest velocity component of B (a
    component that stays near zero, e.g. the spanwise velocity of a boundary layer, has no
    meaningful scale of its own)."""
    vscale = max(float(np.max(np.abs(b))) for b in B[1:4])
    out = []
    for q, (a, b) in enumerate(zip(A, B)):
        if q in (1, 2, 3):
            out.append(float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) / vscale)
        else:
            out.append(rel_err(a, b))
    return out


def smooth_random_state(p, seed: int = 1, amp: float = 0.05):
    """A smooth, fully three-dimensional state with O(1) variation of every field: a few
    seeded periodic Fourier modes on top of a uniform flow at rest (rho ~ 1, T ~ 1)."""
    rng = np.random.default_rng(seed)
    d = Derived.of(p)
    z, y, x = np.meshgrid(*(2 * math.pi * (np.arange(n) + 0.5) / n for n in (p.mz, p.my, p.mx)), indexing="ij")

    def modes():
        f = np.zeros(p.shape)
        for _ in range(4):
            kx, ky, kz = rng.integers(1, 3, size=3)
            ph = rng.uniform(0, 2 * math.pi, size=3)
            f += rng.uniform(-1, 1) * np.sin(kx * x + ph[0]) * np.cos(ky * y + ph[1]) * np.cos(kz * z + ph[2])
        return f

    rho = 1.0 + amp * modes()
    u, v, w = modes() * 0.5, modes() * 0.5, modes() * 0.5
    T = 1.0 + amp * modes()
    press = rho * d.Rgas * T
    e = press / (p.gam - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return [rho, u, v, w, e]


def wall_state(p, x, seed: int = 2, amp: float = 0.05):
    """Smooth channel-like state with u = v = w = 0 and T = 1 at the walls x = 0, Lx."""
    rng = np.random.default_rng(seed)
    d = Derived.of(p)
    z, y, xx = np.meshgrid(2 * math.pi * (np.arange(p.mz) + 0.5) / p.mz,
                           2 * math.pi * (np.arange(p.my) + 0.5) / p.my, np.asarray(x), indexing="ij")
    s = np.sin(math.pi * xx / p.Lx)

    def modes():
        f = np.zeros(p.shape)
        for _ in range(3):
            ky, kz = rng.integers(1, 3, size=2)
            ph = rng.uniform(0, 2 * math.pi, size=2)
            f += rng.uniform(-1, 1) * np.cos(ky * y + ph[0]) * np.cos(kz * z + ph[1])
        return f

    u = 0.2 * s * s * modes()
    v = 0.2 * s * s * modes()
    w = 1.5 * s + 0.2 * s * s * modes()
    rho = 1.0 + amp * s * modes()
    T = 1.0 + 0.3 * s + amp * s * s * modes()
    press = rho * d.Rgas * T
    e = press / (p.gam - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return [rho, u, v, w, e]
