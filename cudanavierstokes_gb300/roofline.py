"""Algorithmic work per grid point, defined once for the roofline figures.

FLOP counts (FMA = 2) follow the per-direction operation count of the split-form RHS with
one interface flux per point: 3 velocity gradients 3(3V+1), 4 first derivatives
(mu, lambda, T, theta) 4(3V+1), 4 second derivatives (u, v, w, T) 4(3V+2), the pressure
gradient 3S+1, the five split-form fluxes 16.5 S(S+1) + 10 and about 45 pointwise
operations; plus the state recovery (14, one pow and one division), the dilatation (2)
and the Runge-Kutta update (26, three divisions). At S = V = 4 this is about 1.68 kflop
per point and stage, 5.0 kflop per point and RK3 step.

Compulsory HBM traffic per point and stage: read the 5 conserved FP64 values and the 5
values of the Runge-Kutta register, write both back: 20 words = 160 B (both precision
modes keep state and accumulation in FP64), 480 B per RK3 step.
"""
from __future__ import annotations


def rhs_kernel_flops(S: int, V: int) -> float:
    """Per point and stage, the RHS + stage-update kernel (no gradients, no state)."""
    per_dir = 4 * (3 * V + 1) + 4 * (3 * V + 2) + (3 * S + 1) + 16.5 * S * (S + 1) + 10 + 45
    return 3 * per_dir + 26


def grad_kernel_flops(V: int) -> float:
    return 9 * (3 * V + 1) + 2


def fused_rhs_kernel_flops(S: int, V: int) -> float:
    """The RHS kernel also recovers the next stage's state (calcState's arithmetic)."""
    return rhs_kernel_flops(S, V) + state_kernel_flops()


def state_kernel_flops() -> float:
    return 14.0


def stage_flops(S: int, V: int) -> float:
    return rhs_kernel_flops(S, V) + grad_kernel_flops(V) + state_kernel_flops()


def step_flops(S: int, V: int, stages: int = 3) -> float:
    return stages * stage_flops(S, V)


STAGE_BYTES = 160.0      # compulsory HBM bytes per point and stage
RHS_KERNEL_BYTES = 160.0  # the stage-update kernel reads/writes the state and the RK register


def step_bytes(stages: int = 3) -> float:
    return stages * STAGE_BYTES
