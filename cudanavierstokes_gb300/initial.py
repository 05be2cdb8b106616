"""Initial conditions and the reference's field file format.

Fields are numpy arrays of shape (mz, my, mx) (C order [k][j][i], x fastest), the
layout of the reference's host arrays and of its raw FP64 field files
(CudaNavierStokes src/comm.cpp:205-279, src/init.cpp:13-30).
"""
from __future__ import annotations

import math
import os

import numpy as np

from .params import CnsParams, Derived


def cell_centres(n: int, L: float) -> np.ndarray:
    """Uniform cell-centred coordinates L*(0.5+i)/n (src/init.cpp:57-69)."""
    return L * (0.5 + np.arange(n, dtype=np.float64)) / n


def _energy(p: CnsParams, rho, u, v, w, press):
    return press / (p.gam - 1.0) + 0.5 * rho * (u * u + v * v + w * w)


def tgv_fields(p: CnsParams, phases=(0.0, 0.0, 0.0)):
    """Taylor-Green vortex with rho = 1:
    u = sin x cos y cos z, v = -cos x sin y cos z, w = 0,
    p = 1/(gam Ma^2) + (cos 2x + cos 2y)(cos 2z + 2)/16, rho E = p/(gam-1) + rho|u|^2/2,
    on the cell-centred grid, with optional per-axis phase offsets."""
    x = 2.0 * math.pi * cell_centres(p.mx, p.Lx) / p.Lx + phases[0]
    y = 2.0 * math.pi * cell_centres(p.my, p.Ly) / p.Ly + phases[1]
    z = 2.0 * math.pi * cell_centres(p.mz, p.Lz) / p.Lz + phases[2]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(u)
    press = 1.0 / (p.gam * p.Ma * p.Ma) + (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0
    rho = np.ones_like(u)
    return [rho, u, v, w, _energy(p, rho, u, v, w, press)]


def tgv_reference_fields(p: CnsParams):
    """The reference's own initCHIT (src/init.cpp:126-148): rho = p/(R T0), T0 = 1."""
    d = Derived.of(p)
    x = cell_centres(p.mx, p.Lx)
    y = cell_centres(p.my, p.Ly)
    z = cell_centres(p.mz, p.Lz)
    fx, fy, fz = 2 * math.pi * x / p.Lx, 2 * math.pi * y / p.Ly, 2 * math.pi * z / p.Lz
    Z, Y, X = np.meshgrid(fz, fy, fx, indexing="ij")
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(u)
    P0 = 1.0 * d.Rgas
    press = P0 + 1.0 / 16.0 * (np.cos(2.0 * X) + np.cos(2.0 * Y)) * (np.cos(2.0 * Z) + 2.0)
    rho = press / d.Rgas / 1.0
    return [rho, u, v, w, _energy(p, rho, u, v, w, press)]


def channel_fields(p: CnsParams, x: np.ndarray, seed: int = 0, amplitude: float = 0.1):
    """Isothermal channel start: rho = 1, T = 1 (p = rho R T), laminar Poiseuille
    w = 1.5 (1 - (x - 1)^2) in the streamwise (z) direction with bulk 1 for x in [0, 2],
    plus a seeded uniform perturbation in [-amplitude, amplitude] on u, v, w
    (numpy PCG64, drawn in [k][j][i] order)."""
    d = Derived.of(p)
    shape = p.shape
    xc = np.asarray(x, dtype=np.float64)
    rng = np.random.default_rng(seed)
    pu = rng.uniform(-amplitude, amplitude, size=shape)
    pv = rng.uniform(-amplitude, amplitude, size=shape)
    pw = rng.uniform(-amplitude, amplitude, size=shape)
    half = 0.5 * p.Lx
    wmean = 1.5 * (1.0 - ((xc - half) / half) ** 2)
    u = pu
    v = pv
    w = np.broadcast_to(wmean[None, None, :], shape) + pw
    rho = np.ones(shape)
    press = rho * d.Rgas * 1.0
    return [rho, u, v, np.ascontiguousarray(w), _energy(p, rho, u, v, w, press)]


FIELD_NAMES = ("r", "u", "v", "w", "e")


def field_path(directory: str, name: str, step: int) -> str:
    """fields/%c.%07d.bin (src/comm.cpp:218, :264)."""
    return os.path.join(directory, f"{name}.{step:07d}.bin")


def write_fields(directory: str, step: int, fields) -> None:
    """Raw native-endian FP64, C order [k][j][i] (saveFileMPI, src/comm.cpp:205-254)."""
    os.makedirs(directory, exist_ok=True)
    for name, f in zip(FIELD_NAMES, fields):
        np.ascontiguousarray(f, dtype=np.float64).tofile(field_path(directory, name, step))


def read_fields(directory: str, step: int, shape):
    """Inverse of write_fields (readFileMPI, src/comm.cpp:256-279)."""
    out = []
    for name in FIELD_NAMES:
        a = np.fromfile(field_path(directory, name, step), dtype=np.float64)
        if a.size != int(np.prod(shape)):
            raise ValueError(f"{field_path(directory, name, step)}: {a.size} values, expected {np.prod(shape)}")
        out.append(a.reshape(shape))
    return out
