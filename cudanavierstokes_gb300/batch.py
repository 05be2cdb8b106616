"""Batched ensemble over the C ABI (cns_batch_*): many simulations of uneven grid sizes
advanced together, one persistent launch per Runge-Kutta stage, CUDA-graph replay."""
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


class Batch:
    def __init__(self, precision: int = 0, stencil_size: int = 4, stencil_visc: int = 4, device: int = 0,
                 hbm_budget_bytes: int = 0):
        self._b = ctypes.c_void_p()
        native.check(native.lib().cns_batch_create(int(device), int(precision), int(stencil_size), int(stencil_visc),
                                                   int(hbm_budget_bytes), ctypes.byref(self._b)))
        self.shapes = {}
        self.params = {}

    def close(self):
        if self._b:
            native.lib().cns_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        native.check(native.lib().cns_batch_set_stream(self._b, ctypes.c_void_p(stream_ptr or 0)))

    def add(self, params: CnsParams, fields, max_steps: int) -> int:
        p = params.copy()
        a = [np.ascontiguousarray(f, dtype=np.float64).reshape(p.shape) for f in fields]
        i = ctypes.c_int()
        native.check(native.lib().cns_batch_add(self._b, ctypes.byref(p), *[_ptr(f) for f in a], int(max_steps),
                                                ctypes.byref(i)))
        self.shapes[i.value] = p.shape
        self.params[i.value] = p
        return i.value

    def set_member_sponge(self, mid: int, sponge_x, sponge_z, rref, uref, wref, eref) -> None:
        """The sponge of a member (boundary layer): strengths on x and z, reference fields on
        the (x, z) plane, as Solver.set_sponge."""
        h = native.lib().cns_batch_member(self._b, int(mid))
        if not h:
            raise native.CnsError(1, "no batch member with this id")
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (sponge_x, sponge_z, rref, uref, wref, eref)]
        native.check(native.lib().cns_set_sponge(h, *[_ptr(v) for v in a]))

    def remove(self, mid: int) -> None:
        native.check(native.lib().cns_batch_remove(self._b, int(mid)))
        self.shapes.pop(mid, None)
        self.params.pop(mid, None)

    def fields(self, mid: int):
        out = [np.empty(self.shapes[mid]) for _ in range(5)]
        native.check(native.lib().cns_batch_get_fields(self._b, int(mid), *[_ptr(f) for f in out]))
        return out

    def logs(self, mid: int, n: int) -> dict:
        out = {k: np.zeros(n) for k in ("par1", "par2", "time")}
        dt = ctypes.c_double()
        native.check(native.lib().cns_batch_get_logs(self._b, int(mid), int(n), _ptr(out["par1"]), _ptr(out["par2"]),
                                                     _ptr(out["time"]), ctypes.byref(dt)))
        out["dt"] = dt.value
        return out

    def steps_done(self, mid: int) -> int:
        s = ctypes.c_int64()
        native.check(native.lib().cns_batch_member_steps(self._b, int(mid), ctypes.byref(s)))
        return s.value

    def info(self) -> dict:
        c, p, b, l = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        native.check(native.lib().cns_batch_info(self._b, ctypes.byref(c), ctypes.byref(p), ctypes.byref(b),
                                                 ctypes.byref(l)))
        return dict(count=c.value, points=p.value, bytes=b.value, launches=l.value)

    def step(self, nsteps: int = 1) -> None:
        native.check(native.lib().cns_batch_step(self._b, int(nsteps)))

    def set_shape(self, threads: int, blocks_per_sm: int) -> None:
        native.check(native.lib().cns_batch_set_shape(self._b, int(threads), int(blocks_per_sm)))

    def shape(self):
        t, b = ctypes.c_int(), ctypes.c_int()
        native.check(native.lib().cns_batch_get_shape(self._b, ctypes.byref(t), ctypes.byref(b)))
        return t.value, b.value

    def set_mode(self, mode: int) -> None:
        """0: one persistent launch per RK stage over all members; 1: members' own step
        graphs on concurrent streams."""
        native.check(native.lib().cns_batch_set_mode(self._b, int(mode)))

    def mode(self) -> int:
        m = ctypes.c_int()
        native.check(native.lib().cns_batch_get_mode(self._b, ctypes.byref(m)))
        return m.value

    def tune(self, steps: int = 2) -> float:
        ms = ctypes.c_double()
        native.check(native.lib().cns_batch_tune(self._b, int(steps), ctypes.byref(ms)))
        return ms.value
