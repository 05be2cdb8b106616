"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU oracle (oracle/cns_oracle.cpp).

The oracle is a CPU restatement of the CudaNavierStokes time-advance path used as the
parity reference and as the timed CPU baseline. Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg may import this module; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from cudanavierstokes_gb300.params import CnsParams  # noqa: E402

BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libcns_oracle.so")
SRC = os.path.join(HERE, "cns_oracle.cpp")

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    """Compile the oracle with the host compiler (no architecture-specific flags, so the
    same source builds on x86_64 and aarch64)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    # -fno-ipa-modref: GCC 13.3 on aarch64 at -O1/-O2 drops the ghost-cell stores of the
    # line extrapolation helpers (boundary-layer top boundary) under its interprocedural
    # mod/ref analysis; bisected on the Grace host (x86_64 builds are unaffected).
    cmd = ["g++", "-O2", "-fno-ipa-modref", "-fopenmp", "-fPIC", "-shared", "-std=c++17", "-o", tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(CnsParams)
        v = ctypes.c_void_p
        L.cnso_create.argtypes = [P]
        L.cnso_create.restype = v
        L.cnso_destroy.argtypes = [v]
        L.cnso_last_error.restype = ctypes.c_char_p
        L.cnso_set_threads.argtypes = [ctypes.c_int]
        L.cnso_max_threads.restype = ctypes.c_int
        L.cnso_get_grid.argtypes = [v] + [_dp] * 6
        L.cnso_set_state.argtypes = [v] + [_dp] * 5
        L.cnso_get_state.argtypes = [v] + [_dp] * 5
        L.cnso_get_derived.argtypes = [v] + [_dp] * 5
        L.cnso_gradients.argtypes = [v, _dp, _dp]
        L.cnso_set_sponge.argtypes = [v] + [_dp] * 6
        L.cnso_sponge_strengths.argtypes = [v, _dp, _dp]
        L.cnso_sponge_refs.argtypes = [v, ctypes.c_int] + [_dp] * 9
        L.cnso_rhs.argtypes = [v] + [_dp] * 5
        L.cnso_calc_dt.argtypes = [v, _dp]
        L.cnso_bulk.argtypes = [v, _dp, _dp]
        L.cnso_run.argtypes = [v, ctypes.c_int] + [_dp] * 5
        L.cnso_get_scalars.argtypes = [v, _dp, _dp, _dp]
        L.cnso_set_scalars.argtypes = [v, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.cnso_plane_stats.argtypes = [v, _dp]
        L.cnso_friction_reynolds.argtypes = [v, _dp]
        L.cnso_dissipation.argtypes = [v, _dp]
        _lib = L
    return _lib


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def set_threads(n: int) -> None:
    lib().cnso_set_threads(int(n))


def max_threads() -> int:
    return int(lib().cnso_max_threads())


class Oracle:
    """One CPU solver instance (mirrors the reference's global solver state)."""

    def __init__(self, params: CnsParams):
        self.p = params.copy()
        self.h = lib().cnso_create(ctypes.byref(self.p))
        if not self.h:
            raise ValueError("oracle rejected parameters: " + lib().cnso_last_error().decode())
        self.shape = self.p.shape

    def close(self):
        if self.h:
            lib().cnso_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid(self):
        p = self.p
        x, xp, xpp, dxv = (np.zeros(p.mx) for _ in range(4))
        y, z = np.zeros(p.my), np.zeros(p.mz)
        lib().cnso_get_grid(self.h, _ptr(x), _ptr(xp), _ptr(xpp), _ptr(y), _ptr(z), _ptr(dxv))
        return dict(x=x, xp=xp, xpp=xpp, y=y, z=z, dxv=dxv)

    def set_state(self, r, u, v, w, e):
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(self.shape) for a in (r, u, v, w, e)]
        lib().cnso_set_state(self.h, *[_ptr(a) for a in arrs])

    def get_state(self):
        out = [np.zeros(self.shape) for _ in range(5)]
        lib().cnso_get_state(self.h, *[_ptr(a) for a in out])
        return out

    def derived(self):
        out = [np.zeros(self.shape) for _ in range(5)]
        lib().cnso_get_derived(self.h, *[_ptr(a) for a in out])
        return dict(zip(("h", "t", "p", "m", "l"), out))

    def gradients(self):
        g = np.zeros((9,) + self.shape)
        dil = np.zeros(self.shape)
        lib().cnso_gradients(self.h, _ptr(g), _ptr(dil))
        return g, dil

    def set_sponge(self, spx, spz, rref, uref, wref, eref):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (spx, spz, rref, uref, wref, eref)]
        lib().cnso_set_sponge(self.h, *[_ptr(a) for a in arrs])

    def sponge_strengths(self):
        spx, spz = np.zeros(self.p.mx), np.zeros(self.p.mz)
        lib().cnso_sponge_strengths(self.h, _ptr(spx), _ptr(spz))
        return spx, spz

    def sponge_refs(self, xin, rin, uin, win, ein):
        n = len(xin)
        ins = [np.ascontiguousarray(a, dtype=np.float64) for a in (xin, rin, uin, win, ein)]
        outs = [np.zeros((self.p.mz, self.p.mx)) for _ in range(4)]
        lib().cnso_sponge_refs(self.h, n, *[_ptr(a) for a in ins], *[_ptr(a) for a in outs])
        return outs

    def rhs(self):
        out = [np.zeros(self.shape) for _ in range(5)]
        lib().cnso_rhs(self.h, *[_ptr(a) for a in out])
        return out

    def calc_dt(self) -> float:
        d = np.zeros(1)
        lib().cnso_calc_dt(self.h, _ptr(d))
        return float(d[0])

    def plane_stats(self):
        """calcAvgChan (src/init.cpp:150-208): (11, mx) = the columns of prof.txt."""
        out = np.zeros((11, self.p.mx))
        lib().cnso_plane_stats(self.h, _ptr(out))
        return out

    def friction_reynolds(self):
        """printRes (src/init.cpp:210-256): the average friction Reynolds number."""
        r = np.zeros(1)
        lib().cnso_friction_reynolds(self.h, _ptr(r))
        return float(r[0])

    def dissipation(self):
        """Volume-averaged viscous dissipation and enstrophy (cnso_dissipation)."""
        r = np.zeros(2)
        lib().cnso_dissipation(self.h, _ptr(r))
        return dict(eps=float(r[0]), enstrophy=float(r[1]))

    def bulk(self):
        a, b = np.zeros(1), np.zeros(1)
        lib().cnso_bulk(self.h, _ptr(a), _ptr(b))
        return float(a[0]), float(b[0])

    def run(self, nsteps: int):
        """Advance nsteps (runSimulation[LowStorage]); returns per-step logs."""
        logs = {k: np.zeros(nsteps) for k in ("par1", "par2", "time", "dt", "dpdz")}
        lib().cnso_run(self.h, int(nsteps), _ptr(logs["par1"]), _ptr(logs["par2"]), _ptr(logs["time"]),
                       _ptr(logs["dt"]), _ptr(logs["dpdz"]))
        return logs

    def scalars(self):
        a, b, c = np.zeros(1), np.zeros(1), np.zeros(1)
        lib().cnso_get_scalars(self.h, _ptr(a), _ptr(b), _ptr(c))
        return dict(dt=float(a[0]), dpdz=float(b[0]), time=float(c[0]))

    def set_scalars(self, dt: float, dpdz: float, time: float):
        lib().cnso_set_scalars(self.h, float(dt), float(dpdz), float(time))
