"""Runtime parameter surface and workload presets.

`CnsParams` is the ctypes mirror of `cns_params` in include/cns.h, which itself
mirrors the reference's compile-time macros (CudaNavierStokes src/globals.h:14-58,
src/sponge.h:4-17, src/perturbation.h:14-22).

Axis convention is the reference's: x is the only wall-normal / stretched /
non-periodic direction, y is periodic, z is periodic (or extrapolated for the
boundary layer) and carries the channel body force.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

RK3_LOWSTORAGE = 0
RK3_CLASSIC = 1
RK4_CLASSIC = 2

PREC_FP64 = 0
PREC_FP32_RHS = 1
PREC_PAIR_RHS = 2   # RHS in FP32-pair (~48-bit) arithmetic, FP64 state

# status codes (include/cns.h)
CNS_OK = 0
CNS_ERR_INVALID = 1
CNS_ERR_CUDA = 2
CNS_ERR_OOM = 3
CNS_ERR_NONFINITE = 4
CNS_ERR_TIMEOUT = 5
CNS_ERR_STATE = 6


class CnsParams(ctypes.Structure):
    """ctypes layout of `cns_params` (include/cns.h)."""

    _fields_ = [
        ("mx", ctypes.c_int32), ("my", ctypes.c_int32), ("mz", ctypes.c_int32),
        ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("Lz", ctypes.c_double),
        ("stencil_size", ctypes.c_int32), ("stencil_visc", ctypes.c_int32),
        ("Re", ctypes.c_double), ("Pr", ctypes.c_double), ("Ma", ctypes.c_double),
        ("gam", ctypes.c_double), ("viscexp", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("scheme", ctypes.c_int32), ("boundary_layer", ctypes.c_int32),
        ("perturbed", ctypes.c_int32), ("forcing", ctypes.c_int32),
        ("periodic_x", ctypes.c_int32), ("nonuniform_x", ctypes.c_int32),
        ("stretch", ctypes.c_double), ("twall_top", ctypes.c_double),
        ("twall_bot", ctypes.c_double),
        ("check_cfl", ctypes.c_int32), ("check_bulk", ctypes.c_int32),
        ("quirk_dissipation_y", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("ndivz", ctypes.c_int32),
        ("dpdz_init", ctypes.c_double),
        ("sp_top_str", ctypes.c_double), ("sp_top_len", ctypes.c_double), ("sp_top_exp", ctypes.c_double),
        ("sp_inl_str", ctypes.c_double), ("sp_inl_len", ctypes.c_double), ("sp_inl_exp", ctypes.c_double),
        ("sp_out_str", ctypes.c_double), ("sp_out_len", ctypes.c_double), ("sp_out_exp", ctypes.c_double),
        ("pert_kc", ctypes.c_int32), ("pert_lp", ctypes.c_int32),
        ("pert_amp1", ctypes.c_double), ("pert_amp2", ctypes.c_double),
        ("pert_omega1_per_re", ctypes.c_double), ("pert_omega2", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}

    def copy(self, **overrides) -> "CnsParams":
        p = CnsParams()
        ctypes.pointer(p)[0] = self
        for k, v in overrides.items():
            if not hasattr(p, k):
                raise AttributeError(f"cns_params has no field {k!r}")
            setattr(p, k, v)
        return p

    @property
    def npoints(self) -> int:
        return int(self.mx) * int(self.my) * int(self.mz)

    @property
    def shape(self) -> tuple[int, int, int]:
        """numpy shape of a field: C order [k][j][i] (x fastest)."""
        return (int(self.mz), int(self.my), int(self.mx))


def default_params() -> CnsParams:
    """Reference defaults for every constant that is not a workload choice
    (src/globals.h, src/sponge.h:4-17, src/perturbation.h:14-22, src/cuda_utils.cu:69),
    on a 64^3 periodic box."""
    p = CnsParams()
    p.mx = p.my = p.mz = 64
    p.Lx = p.Ly = p.Lz = 2.0 * math.pi
    p.stencil_size = 4
    p.stencil_visc = 4
    p.Re, p.Pr, p.Ma, p.gam, p.viscexp = 1600.0, 0.71, 0.1, 1.4, 1.0
    p.cfl = 0.5
    p.scheme = RK3_LOWSTORAGE
    p.boundary_layer = 0
    p.perturbed = 0
    p.forcing = 0
    p.periodic_x = 1
    p.nonuniform_x = 0
    p.stretch = 5.0
    p.twall_top = 1.0
    p.twall_bot = 1.0
    p.check_cfl = 100
    p.check_bulk = 100
    p.quirk_dissipation_y = 1
    p.precision = PREC_FP64
    p.ndivz = 1
    p.dpdz_init = 0.00372
    p.sp_top_str, p.sp_top_len, p.sp_top_exp = 1.0, 1.0, 2.0
    p.sp_inl_str, p.sp_inl_len, p.sp_inl_exp = 0.5, 20.0, 2.0
    p.sp_out_str, p.sp_out_len, p.sp_out_exp = 0.5, 20.0, 2.0
    p.pert_kc, p.pert_lp = 110, 40
    p.pert_amp1, p.pert_amp2 = 2e-4, 3e-5
    p.pert_omega1_per_re, p.pert_omega2 = 121.0e-6, 10.0
    return p


def tgv_params(n: int = 64, **kw) -> CnsParams:
    """Taylor-Green vortex, periodic [0, 2pi)^3, gamma 1.4, Ma 0.1, Re 1600, Pr 0.71,
    8th-order stencils (S = V = 4), Wray RK3, CFL 0.5, mu = T^1."""
    p = default_params()
    p.mx = p.my = p.mz = n
    return p.copy(**kw)


def channel_params(mx: int = 128, my: int = 160, mz: int = 192, **kw) -> CnsParams:
    """Supersonic isothermal-wall channel in reference axes: x wall-normal in [0, 2]
    (tanh stretching 1.5), y spanwise (4pi/3), z streamwise (4pi, body force), bulk
    Ma 1.5, Re 3000, Pr 0.72, mu = T^0.7, T_wall = 1, 8th order, Wray RK3, CFL 0.5."""
    p = default_params()
    p.mx, p.my, p.mz = mx, my, mz
    p.Lx, p.Ly, p.Lz = 2.0, 4.0 * math.pi / 3.0, 4.0 * math.pi
    p.Re, p.Pr, p.Ma, p.viscexp = 3000.0, 0.72, 1.5, 0.7
    p.periodic_x = 0
    p.nonuniform_x = 1
    p.forcing = 1
    p.stretch = 1.5
    return p.copy(**kw)


def boundary_layer_params(mx: int = 32, my: int = 16, mz: int = 160, **kw) -> CnsParams:
    """Laminar compressible boundary layer (reference src/globals.h defaults scaled
    down): x wall-normal with extrapolated top, z streamwise with extrapolated
    inflow/outflow, sponge and wall perturbation."""
    p = default_params()
    p.mx, p.my, p.mz = mx, my, mz
    p.Lx, p.Ly, p.Lz = 20.0, 7.0, 100.0
    p.stencil_size, p.stencil_visc = 3, 2
    p.Re, p.Pr, p.Ma, p.viscexp = 1500.0, 0.75, 0.35, 1.5
    p.cfl = 0.75
    p.boundary_layer = 1
    p.perturbed = 1
    p.periodic_x = 0
    p.nonuniform_x = 1
    p.stretch = 5.0
    return p.copy(**kw)


@dataclass(frozen=True)
class Derived:
    """Constants derived exactly as the reference's macros (src/globals.h:47-48)."""

    Ec: float
    Rgas: float

    @staticmethod
    def of(p: CnsParams) -> "Derived":
        # (gam - 1.f)*Ma*Ma and 1.f/(gam*Ma*Ma): the float literal 1.f is exact in double
        return Derived(Ec=((p.gam - 1.0) * p.Ma) * p.Ma, Rgas=1.0 / ((p.gam * p.Ma) * p.Ma))
