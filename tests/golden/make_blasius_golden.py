"""Golden vectors for the boundary-layer inflow generator: run the reference's own
python-utils/selfSimilarSol.py (unmodified; its plotting imports are satisfied by inert
stand-in modules, since matplotlib is not installed and the function draws nothing) in a
scratch directory and store the blasius1D/*Prof.bin it writes in
tests/golden/blasius_ref_profiles.npz.

Run in a checkout next to the reference (its location: $CNS_REFERENCE_ROOT, else the
default checkout location the parity harness uses):
    python tests/golden/make_blasius_golden.py
"""
import importlib.util
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "blasius_ref_profiles.npz")


def main():
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.ref_harness import reference_root
    root = reference_root()
    if root is None:
        raise SystemExit("reference checkout not found: set CNS_REFERENCE_ROOT")
    ref = os.path.join(root, "python-utils", "selfSimilarSol.py")
    mpl = types.ModuleType("matplotlib")
    mpl.rc = lambda *a, **k: None
    mpl.rcParams = {}
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)
    spec = importlib.util.spec_from_file_location("ref_self_similar", ref)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        os.makedirs("blasius1D")
        try:
            mod.selfSimilarSol()          # the reference's defaults: gam 1.4, Ma 0.3, Pr 0.72
        finally:
            os.chdir(cwd)
        prof = {n: np.fromfile(os.path.join(d, "blasius1D", f"{n}Prof.bin")) for n in "xruwe"}
    np.savez_compressed(OUT, gam=1.4, Ma=0.3, Pr=0.72, **prof)
    print("wrote", OUT, {k: v.shape for k, v in prof.items()})


if __name__ == "__main__":
    main()
