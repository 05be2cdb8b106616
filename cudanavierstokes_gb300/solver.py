"""Host-side mirror of the reference's init / step / output sequence over the C ABI.

    reference (CudaNavierStokes)                  Solver
    setGPUParameters + initSolver                 Solver(params, device)
    initGrid outputs x, xp, xpp, y, z             Solver.grid()
    calculateSponge                               Solver.set_sponge_profiles / set_sponge
    copyField(0) / copyField(1)                   Solver.copy_field_in / copy_field_out
    runSimulationLowStorage / runSimulation       Solver.run(nsteps)
    calcRHS                                       Solver.calc_rhs()
    clearSolver                                   Solver.close()

Fields are numpy float64 arrays of shape (mz, my, mx) (x fastest), the reference's
host layout. Arrays in page-locked memory (e.g. torch pin_memory buffers exposed through
numpy) are transferred asynchronously by the CUDA runtime.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .params import CnsParams

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise ValueError("arrays must be C-contiguous float64")
    return a.ctypes.data_as(_dp)


def host_grid(params: CnsParams) -> dict:
    """Grid of these parameters computed on the host (initGrid / derivGrid), no device."""
    p = params.copy()
    x, xp, xpp = np.zeros(p.mx), np.zeros(p.mx), np.zeros(p.mx)
    y, z = np.zeros(p.my), np.zeros(p.mz)
    native.check(native.lib().cns_host_grid(ctypes.byref(p), _ptr(x), _ptr(xp), _ptr(xpp), _ptr(y), _ptr(z)))
    return dict(x=x, xp=xp, xpp=xpp, y=y, z=z)


class Solver:
    def __init__(self, params: CnsParams, device: int = 0):
        self.p = params.copy()
        self.shape = self.p.shape
        self._h = ctypes.c_void_p()
        native.check(native.lib().cns_create(ctypes.byref(self.p), int(device), ctypes.byref(self._h)))

    # -- lifecycle -------------------------------------------------------------------
    def close(self) -> None:
        if self._h:
            native.lib().cns_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None) -> None:
        native.check(native.lib().cns_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    # -- set-up ----------------------------------------------------------------------
    def grid(self) -> dict:
        p = self.p
        x, xp, xpp = np.zeros(p.mx), np.zeros(p.mx), np.zeros(p.mx)
        y, z = np.zeros(p.my), np.zeros(p.mz)
        native.check(native.lib().cns_get_grid(self._h, _ptr(x), _ptr(xp), _ptr(xpp), _ptr(y), _ptr(z)))
        return dict(x=x, xp=xp, xpp=xpp, y=y, z=z)

    def set_sponge(self, sponge_x, sponge_z, rref, uref, wref, eref) -> None:
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (sponge_x, sponge_z, rref, uref, wref, eref)]
        native.check(native.lib().cns_set_sponge(self._h, *[_ptr(v) for v in a]))

    def set_sponge_profiles(self, xin, rin, uin, win, ein, init_fields: bool = True) -> None:
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (xin, rin, uin, win, ein)]
        native.check(native.lib().cns_set_sponge_profiles(self._h, len(a[0]), *[_ptr(v) for v in a],
                                                          int(bool(init_fields))))

    # -- fields ----------------------------------------------------------------------
    def copy_field_in(self, r, u, v, w, e) -> None:
        a = [np.ascontiguousarray(f, dtype=np.float64).reshape(self.shape) for f in (r, u, v, w, e)]
        native.check(native.lib().cns_copy_field(self._h, 0, *[_ptr(f) for f in a]))

    def copy_field_out(self, out=None):
        out = out if out is not None else [np.empty(self.shape) for _ in range(5)]
        native.check(native.lib().cns_copy_field(self._h, 1, *[_ptr(f) for f in out]))
        return out

    # -- time advance ------------------------------------------------------------------
    def run(self, nsteps: int, logs: bool = True) -> dict:
        if not logs:
            native.check(native.lib().cns_run(self._h, int(nsteps), None, None, None))
            return {}
        out = {k: np.zeros(nsteps) for k in ("par1", "par2", "time")}
        native.check(native.lib().cns_run(self._h, int(nsteps), _ptr(out["par1"]), _ptr(out["par2"]),
                                          _ptr(out["time"])))
        return out

    def set_graphs(self, enable: bool) -> None:
        native.check(native.lib().cns_set_graphs(self._h, int(bool(enable))))

    def calc_rhs(self):
        out = [np.empty(self.shape) for _ in range(5)]
        native.check(native.lib().cns_calc_rhs(self._h, *[_ptr(f) for f in out]))
        return out

    def plane_stats(self) -> np.ndarray:
        """(11, mx): the columns of the reference's prof.txt (calcAvgChan), on the device."""
        out = np.zeros((11, self.p.mx))
        native.check(native.lib().cns_plane_stats(self._h, _ptr(out)))
        return out

    def friction_reynolds(self) -> float:
        """The reference's printRes friction Reynolds number at the x = 0 wall, on the device."""
        r = np.zeros(1)
        native.check(native.lib().cns_friction_reynolds(self._h, _ptr(r)))
        return float(r[0])

    def dissipation(self) -> dict:
        """Volume-averaged viscous dissipation <tau_ij du_i/dx_j> (`eps`) and enstrophy
        <|curl u|^2> (`enstrophy`) of the current state, FP64, on the device."""
        r = np.zeros(2)
        native.check(native.lib().cns_dissipation(self._h, _ptr(r)))
        return dict(eps=float(r[0]), enstrophy=float(r[1]))

    def scalars(self) -> dict:
        a, b, c = (ctypes.c_double() for _ in range(3))
        native.check(native.lib().cns_get_scalars(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return dict(dt=a.value, dpdz=b.value, time=c.value)

    def set_scalars(self, dt: float, dpdz: float, time: float, step: int = -1) -> None:
        native.check(native.lib().cns_set_scalars(self._h, float(dt), float(dpdz), float(time), int(step)))

    def time_phases(self, nstages: int = 3) -> dict:
        """Per-phase device time (ms) averaged over nstages low-storage stages."""
        ms = np.zeros(3)
        native.check(native.lib().cns_time_phases(self._h, int(nstages), _ptr(ms)))
        return dict(ghost_ms=float(ms[0]), grad_ms=float(ms[1]), rhs_ms=float(ms[2]))

    @property
    def kernel_launches(self) -> int:
        return int(native.lib().cns_kernel_launches(self._h))

    @property
    def device_bytes(self) -> int:
        return int(native.lib().cns_device_bytes(self._h))
