"""Serving over the C ABI (cns_server_*): "advance N steps" requests with continuous
batching on one GPU; the native worker thread does admission, stepping and retirement."""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .params import CnsParams

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


class Server:
    def __init__(self, precision: int = 1, stencil_size: int = 4, stencil_visc: int = 4, device: int = 0,
                 hbm_budget_bytes: int = 0, max_batch: int = 0):
        self._s = ctypes.c_void_p()
        native.check(native.lib().cns_server_create(int(device), int(precision), int(stencil_size), int(stencil_visc),
                                                    int(hbm_budget_bytes), int(max_batch), ctypes.byref(self._s)))
        self._shapes = {}

    def close(self):
        if self._s:
            native.lib().cns_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, params: CnsParams, fields, nsteps: int) -> int:
        p = params.copy()
        a = [np.ascontiguousarray(f, dtype=np.float64).reshape(p.shape) for f in fields]
        rid = ctypes.c_int64()
        native.check(native.lib().cns_server_submit(self._s, ctypes.byref(p), *[_ptr(f) for f in a], int(nsteps),
                                                    ctypes.byref(rid)))
        self._shapes[rid.value] = p.shape
        return rid.value

    def poll(self, rid: int):
        st, lat = ctypes.c_int(), ctypes.c_double()
        native.check(native.lib().cns_server_poll(self._s, int(rid), ctypes.byref(st), ctypes.byref(lat)))
        return st.value, lat.value

    def wait(self, rid: int, timeout_s: float = 600.0, fetch: bool = True):
        out = [np.empty(self._shapes[rid]) for _ in range(5)] if fetch else [None] * 5
        native.check(native.lib().cns_server_wait(self._s, int(rid), float(timeout_s), *[_ptr(f) for f in out]))
        self._shapes.pop(rid, None)
        return out if fetch else None

    def stats(self) -> dict:
        st = native.ServerStats()
        native.check(native.lib().cns_server_stats(self._s, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in st._fields_}
