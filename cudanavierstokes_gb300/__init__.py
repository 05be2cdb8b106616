"""GB300-native (sm_103a) time-advance path of the CudaNavierStokes compressible
Navier-Stokes solver: split-form RHS + Runge-Kutta stages behind a C ABI
(include/cns.h), with a thin Python host layer."""
from .params import (CnsParams, PREC_FP32_RHS, PREC_FP64, PREC_PAIR_RHS, RK3_CLASSIC, RK3_LOWSTORAGE, RK4_CLASSIC,
                     boundary_layer_params, channel_params, default_params, tgv_params)
from .solver import Solver

__all__ = ["CnsParams", "Solver", "default_params", "tgv_params", "channel_params", "boundary_layer_params",
           "PREC_FP64", "PREC_FP32_RHS", "PREC_PAIR_RHS", "RK3_LOWSTORAGE", "RK3_CLASSIC", "RK4_CLASSIC"]
