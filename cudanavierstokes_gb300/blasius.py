"""Inflow profiles for the boundary-layer configuration: the compressible self-similar
(Blasius) boundary layer, written as blasius1D/{x,r,u,w,e}Prof.bin for the sponge
reference fields (the reference's python-utils/selfSimilarSol.py, which needs matplotlib).

Similarity variables (Howarth-Dorodnitsyn form): with F the stream function, U = F', T the
temperature scaled by its free-stream value, C = T^(a-1) the Chapman-Rubesin factor of the
viscosity law mu ~ T^a, Ec = (gamma - 1) Ma^2 and Pr the Prandtl number,

    (C F'')' = -F F''                     momentum
    (C T' / Pr)' = -F T' - Ec C F''^2     energy (written for T with C T'/Pr as unknown)
    Y' = sqrt(2) T                        physical wall distance

on eta in [0, eta_max], no slip F(0) = U(0) = 0, adiabatic wall T'(0) = 0, Y(0) = 0, free
stream U = T = 1. The solution is a first-order system solved with scipy's collocation BVP
solver from the guess U = sqrt(eta / eta_max), T = 1, Y = eta_max; profiles are then
expressed in the wall distance scaled by the 99 % thickness: rho = 1/T, the streamwise
velocity U, the wall-normal velocity (U Y / 2 - F T / sqrt(2)) / delta99 and the internal
energy T R / (gamma - 1), R = 1 / (gamma Ma^2), and continued to `n_out` points at a spacing
of 0.15 with the free-stream values.
"""
from __future__ import annotations

import math
import os

import numpy as np


def self_similar_profiles(gam: float = 1.4, Ma: float = 0.3, Pr: float = 0.72, visc_exp: float = 1.5,
                          n_eta: int = 600, eta_max: float = 10.0, n_out: int = 1000) -> dict:
    """Profiles (arrays of n_out values): x (wall distance / delta99), r, u (wall-normal
    velocity), w (streamwise velocity), e (internal energy); plus the wall temperature,
    the wall shear C F''(0) and delta99 in similarity units. The reference fixes the
    viscosity exponent at 1.5 whatever its argument, hence the default."""
    from scipy.integrate import solve_bvp

    Ec = (gam - 1.0) * Ma * Ma
    Rgas = 1.0 / (gam * Ma * Ma)

    # unknowns z = [F, U, C U', T, C T' / Pr ... scaled as below, Y]
    def rhs(eta, z):
        F, U, Q, T, H, Y = z
        C = T ** (visc_exp - 1.0)
        dU = Q / C
        return np.vstack((U,
                          dU,
                          -F * dU,
                          H * Pr / C,
                          -F * H * Pr / C - Ec * Q * Q / C,
                          math.sqrt(2.0) * T))

    def bc(z0, zi):
        return np.array([z0[0], z0[1], z0[4], z0[5], zi[1] - 1.0, zi[3] - 1.0])

    eta = np.linspace(0.0, eta_max, n_eta)
    guess = np.zeros((6, n_eta))
    guess[1] = np.sqrt(eta / eta[-1])
    guess[3] = 1.0
    guess[5] = eta[-1]
    sol = solve_bvp(rhs, bc, eta, guess)
    if not sol.success:
        raise RuntimeError(f"self-similar boundary layer did not converge: {sol.message}")
    F, U, Q, T, _, Y = sol.sol(eta)

    k99 = int(np.argmax(U > 0.99))
    delta = Y[k99]
    r = 1.0 / T
    V = (U * Y / 2.0 - F / (r * math.sqrt(2.0))) / delta
    y = Y / delta

    out = {name: np.zeros(n_out) for name in ("x", "r", "u", "w", "e")}
    m = y.size
    out["x"][:m] = y
    out["r"][:m] = r
    out["w"][:m] = U
    out["u"][:m] = V
    out["e"][:m] = T * Rgas / (gam - 1.0)
    for i in range(m, n_out):
        out["x"][i] = out["x"][i - 1] + 0.15
    for name in ("r", "u", "w", "e"):
        out[name][m:] = out[name][m - 1]
    out["t_wall"] = float(T[0])
    out["shear_wall"] = float(Q[0])   # C F''(0), 0.4696 for the incompressible Blasius layer
    out["delta99"] = float(delta)
    return out


def write_profiles(run_dir: str, prof: dict) -> None:
    """blasius1D/{x,r,u,w,e}Prof.bin (raw FP64), the files the boundary-layer driver reads."""
    d = os.path.join(run_dir, "blasius1D")
    os.makedirs(d, exist_ok=True)
    for name in ("x", "r", "u", "w", "e"):
        np.asarray(prof[name], dtype=np.float64).tofile(os.path.join(d, f"{name}Prof.bin"))


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="write blasius1D/*Prof.bin for a boundary-layer run")
    ap.add_argument("run_dir", nargs="?", default=".")
    ap.add_argument("--gam", type=float, default=1.4)
    ap.add_argument("--Ma", type=float, default=0.3)
    ap.add_argument("--Pr", type=float, default=0.72)
    a = ap.parse_args()
    write_profiles(a.run_dir, self_similar_profiles(a.gam, a.Ma, a.Pr))
