"""ctypes binding of libcns_gb300.so (include/cns.h).

The library is built in-tree by cudanavierstokes_gb300.build. There is no fallback:
if the shared library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from .params import CnsParams

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libcns_gb300.so")

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

# every symbol include/cns.h declares, with (restype, argtypes)
SIGNATURES = {
    "cns_default_params": (None, [ctypes.POINTER(CnsParams)]),
    "cns_check_params": (ctypes.c_int, [ctypes.POINTER(CnsParams)]),
    "cns_last_error": (ctypes.c_char_p, []),
    "cns_version": (ctypes.c_char_p, []),
    "cns_create": (ctypes.c_int, [ctypes.POINTER(CnsParams), ctypes.c_int, ctypes.POINTER(_vp)]),
    "cns_destroy": (ctypes.c_int, [_vp]),
    "cns_set_stream": (ctypes.c_int, [_vp, _vp]),
    "cns_get_grid": (ctypes.c_int, [_vp] + [_dp] * 5),
    "cns_host_grid": (ctypes.c_int, [ctypes.POINTER(CnsParams)] + [_dp] * 5),
    "cns_set_sponge_profiles": (ctypes.c_int, [_vp, ctypes.c_int] + [_dp] * 5 + [ctypes.c_int]),
    "cns_set_sponge": (ctypes.c_int, [_vp] + [_dp] * 6),
    "cns_copy_field": (ctypes.c_int, [_vp, ctypes.c_int] + [_dp] * 5),
    "cns_run": (ctypes.c_int, [_vp, ctypes.c_int] + [_dp] * 3),
    "cns_calc_rhs": (ctypes.c_int, [_vp] + [_dp] * 5),
    "cns_set_graphs": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cns_get_scalars": (ctypes.c_int, [_vp] + [_dp] * 3),
    "cns_set_scalars": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int64]),
    "cns_time_phases": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "cns_kernel_launches": (ctypes.c_int64, [_vp]),
    "cns_device_bytes": (ctypes.c_int64, [_vp]),
    "cns_reduce_state": (ctypes.c_int, [ctypes.c_int] * 3 + [_vp] * 7 + [ctypes.c_double] * 4 + [_vp, _vp]),
    "cns_reduce_state_noalloc": (ctypes.c_int, [ctypes.c_int] * 3 + [_vp] * 7 + [ctypes.c_double] * 4 + [_vp, _vp]),
    "cns_batch_create": (ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.c_int64, ctypes.POINTER(_vp)]),
    "cns_batch_destroy": (ctypes.c_int, [_vp]),
    "cns_batch_set_stream": (ctypes.c_int, [_vp, _vp]),
    "cns_batch_add": (ctypes.c_int, [_vp, ctypes.POINTER(CnsParams)] + [_dp] * 5 +
                      [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "cns_batch_remove": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cns_batch_member": (_vp, [_vp, ctypes.c_int]),
    "cns_batch_get_fields": (ctypes.c_int, [_vp, ctypes.c_int] + [_dp] * 5),
    "cns_batch_get_logs": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int] + [_dp] * 4),
    "cns_batch_member_steps": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]),
    "cns_batch_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)] + [ctypes.POINTER(ctypes.c_int64)] * 3),
    "cns_batch_step": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cns_batch_set_shape": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "cns_batch_get_shape": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "cns_batch_set_mode": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cns_batch_get_mode": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "cns_batch_tune": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "cns_selftest_barrier_timeout": (ctypes.c_int, [ctypes.c_int, ctypes.c_longlong, ctypes.POINTER(ctypes.c_int)]),
    "cns_probe_fma_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]),
    "cns_plane_stats": (ctypes.c_int, [_vp, _dp]),
    "cns_friction_reynolds": (ctypes.c_int, [_vp, _dp]),
    "cns_dissipation": (ctypes.c_int, [_vp, _dp]),
    "cns_selftest_pow": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_longlong, ctypes.c_double, _vp, _vp]),
    "cns_selftest_rcp": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_longlong, _vp, _vp]),
    "cns_selftest_pair": (ctypes.c_int, [ctypes.c_int, _vp, _vp, _vp, ctypes.c_longlong, _vp]),
    "cns_selftest_convert": (ctypes.c_int, [ctypes.c_int, _vp, _vp, ctypes.c_longlong, _vp, _vp, _vp, _vp]),
}


class ServerStats(ctypes.Structure):
    """ctypes layout of cns_server_stats_t."""

    _fields_ = [("completed", ctypes.c_int64), ("queued", ctypes.c_int64), ("running", ctypes.c_int64),
                ("batch_steps", ctypes.c_int64), ("point_steps", ctypes.c_int64), ("busy_seconds", ctypes.c_double),
                ("p50_s", ctypes.c_double), ("p99_s", ctypes.c_double), ("max_s", ctypes.c_double)]


SIGNATURES.update({
    "cns_server_create": (ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.c_int64, ctypes.c_int, ctypes.POINTER(_vp)]),
    "cns_server_destroy": (ctypes.c_int, [_vp]),
    "cns_server_submit": (ctypes.c_int, [_vp, ctypes.POINTER(CnsParams)] + [_dp] * 5 +
                          [ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]),
    "cns_server_poll": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int), _dp]),
    "cns_server_wait": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_double] + [_dp] * 5),
    "cns_server_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
})


class CnsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cns error {code}: {msg}")
        self.code = code


def lib():
    """Load the GB300 library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(the solver has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != 0:
        raise CnsError(rc, lib().cns_last_error().decode(errors="replace"))
