"""Loader for the golden vectors produced by running the unmodified reference GPU code
(oracle/ref_harness.py: staged on the reference checkout, run on a GB300 with
CUDA_LAUNCH_BLOCKING=1, collected into tests/golden/ref_*.npz)."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

from cudanavierstokes_gb300.params import CnsParams

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(f)[4:-4] for f in glob.glob(os.path.join(GOLDEN, "ref_*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    meta = json.loads(str(z["meta"]))
    p = CnsParams()
    for k, v in meta["params"].items():
        setattr(p, k, v)
    return dict(params=p, nsteps=int(meta["nsteps"]), ic=[a.copy() for a in z["ic"]],
                out=[a.copy() for a in z["out"]], x=z["x"].copy(), steplog=z["steplog"].copy(), kind=meta["ic"],
                ret=float(z["ret"][0]) if "ret" in z else None, prof=z["prof"].copy() if "prof" in z else None)


def large_names():
    """Golden cases at the benchmark sizes (tests/golden/refsub_*.npz)."""
    return sorted(os.path.basename(f)[7:-4] for f in glob.glob(os.path.join(GOLDEN, "refsub_*.npz")))


def load_large(name):
    """A benchmark-size golden case: parameters, step count, the strided subsample of the
    initial and final fields (stride `sub` per axis from 0), and per final field the
    maximum magnitude and the plane sums along z, y, x over the whole grid. Its initial
    fields are regenerated with initial_fields()."""
    z = np.load(os.path.join(GOLDEN, f"refsub_{name}.npz"))
    meta = json.loads(str(z["meta"]))
    p = CnsParams()
    for k, v in meta["params"].items():
        setattr(p, k, v)
    return dict(params=p, nsteps=int(meta["nsteps"]), kind=meta["ic"], sub=int(meta["sub"]), x=z["x"].copy(),
                steplog=z["steplog"].copy(), ic_sub=z["ic_sub"].copy(), out_sub=z["out_sub"].copy(),
                absmax=z["out_absmax"].copy(), sums=[z["out_sum_k"].copy(), z["out_sum_j"].copy(),
                                                     z["out_sum_i"].copy()])


def initial_fields(case, x):
    """The initial fields of a benchmark-size case (the generators the harness ran on the
    GPU host before the reference: analytic Taylor-Green, seeded channel on grid x)."""
    from cudanavierstokes_gb300 import initial
    p = case["params"]
    if case["kind"] == "tgv":
        return initial.tgv_fields(p)
    return initial.channel_fields(p, x, seed=0)


def large_errors(fields, case):
    """Errors of full final fields against a benchmark-size golden, per field: the largest of
    (a) the subsample's max |a - b| and (b) the plane sums' max |sum a - sum b| divided by the
    plane's point count, both over the field's scale (its maximum magnitude; the velocity
    components share the largest velocity maximum, as state_errors does)."""
    sub = case["sub"]
    vscale = float(max(case["absmax"][1:4]))
    a = np.stack([np.asarray(f) for f in fields])
    errs = []
    for q in range(5):
        scale = vscale if q in (1, 2, 3) else float(case["absmax"][q])
        e_sub = float(np.max(np.abs(a[q][::sub, ::sub, ::sub] - case["out_sub"][q])))
        e_sum = 0.0
        for kept, ref in enumerate(case["sums"]):      # plane sums along z (kept axis 0), y, x
            ax = tuple(d for d in range(3) if d != kept)
            n = a[q].size // a[q].shape[kept]
            e_sum = max(e_sum, float(np.max(np.abs(a[q].sum(axis=ax) - ref[q]))) / n)
        errs.append(max(e_sub, e_sum) / scale)
    return errs


def sponge_from_ic(case, strengths):
    """Boundary-layer cases start from the reference fields, which are uniform in y: the
    sponge references are the j = 0 plane of the step-0 state (rho, u, w, rhoE)."""
    r, u, v, w, e = case["ic"]
    spx, spz = strengths
    return spx, spz, r[:, 0, :], u[:, 0, :], w[:, 0, :], e[:, 0, :]
