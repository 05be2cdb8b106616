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


def sponge_from_ic(case, strengths):
    """Boundary-layer cases start from the reference fields, which are uniform in y: the
    sponge references are the j = 0 plane of the step-0 state (rho, u, w, rhoE)."""
    r, u, v, w, e = case["ic"]
    spx, spz = strengths
    return spx, spz, r[:, 0, :], u[:, 0, :], w[:, 0, :], e[:, 0, :]
