"""TEST INFRASTRUCTURE ONLY: build and run the unmodified CudaNavierStokes GPU code to
produce golden vectors that pin the CPU oracle (and, through it, the GB300 library).

The reference has no CPU path and no tests, so parity is pinned by running the
reference itself. Steps:

  stage   (on a machine with the reference checkout)
          For every case below: copy the reference's src/ into oracle/_ref/<case>/src
          (git-ignored, never committed), write a generated parameter header in place of
          its compile-time src/globals.h, add oracle/ref_mpi_stub.h as mpi.h, wrap the
          dead device-side-launch helpers of src/cuda_math.cu (device cudaDeviceSynchronize,
          which CUDA >= 12 rejects) in `#if 0`, write the initial fields as restart
          files fields/*.0000000.bin (or, for the boundary layer, synthetic self-similar
          profiles blasius1D/*.bin) and a Makefile.
          Cases at the benchmark sizes (the 64^3 Taylor-Green box and the 128x160x192
          channel) stage no field files: their initial fields are written on the run
          host, from the same seeded generators, just before the reference runs.
  run     (on a GB300 host) `make` each case for sm_103a and run ./ns with
          CUDA_LAUNCH_BLOCKING=1 (program order: the reference's streams race otherwise),
          then pack initial and final fields, the dt/dpdz log, the friction Reynolds
          number the reference prints for the initial field (printRes) and its prof.txt
          plane profiles of the final field (calcAvgChan) into <out>/<case>.npz. For the
          benchmark-size cases the fields are packed as a strided subsample plus, per
          field, the maximum magnitude and the plane sums along each axis over the whole
          grid (tests/golden stays a few MB).
  collect (back on the machine with the checkout) copy the packed results from <out>
          to tests/golden/ (ref_<case>.npz; benchmark-size cases refsub_<case>.npz).

  time    (on a GB300 host) build and run the staged timing cases (the benchmark
          channel at two run lengths) and write the reference's per-step time to
          <out>/ref_timing.json.

The reference checkout is taken from $CNS_REFERENCE_ROOT, else from the default checkout
location below; <out> is the --out directory the caller names.

Usage: python oracle/ref_harness.py stage [case ...]
       python oracle/ref_harness.py {run|time|collect} --out DIR [case ...]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)

from cudanavierstokes_gb300.params import (  # noqa: E402
    RK3_CLASSIC, RK3_LOWSTORAGE, CnsParams, boundary_layer_params, channel_params, tgv_params)
from cudanavierstokes_gb300 import initial  # noqa: E402

DEFAULT_REFERENCE_ROOT = "/root/reference"
STAGE_ROOT = os.path.join(HERE, "_ref")
GOLDEN = os.path.join(REPO, "tests", "golden")


def reference_root():
    """The reference checkout ($CNS_REFERENCE_ROOT, else the default location), or None
    when it is absent (a GPU host only has the staged copies under oracle/_ref)."""
    root = os.environ.get("CNS_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT)
    return root if os.path.isdir(os.path.join(root, "src")) else None


def cases():
    """Golden cases (reference axes). Sizes respect the reference's own launch-geometry
    checks (src/cuda_utils.cu:233-297): even edges, lPencils = 1 for edges <= 32."""
    return {
        # periodic TGV, 8th order, Wray RK3, non-cubic box to catch axis mix-ups
        "tgv_16x20x24_s4v4": dict(params=tgv_params(16).copy(my=20, mz=24), nsteps=10, ic="tgv"),
        # classic RK3, low order, dt recomputed during the run (checkCFL=4)
        "tgv_16_s2v1_rk3classic": dict(params=tgv_params(16).copy(stencil_size=2, stencil_visc=1,
                                                                   scheme=RK3_CLASSIC, check_cfl=4,
                                                                   check_bulk=3),
                                       nsteps=6, ic="tgv_ref"),
        # isothermal channel: stretched x, walls, body force; dt/dpdz recomputed at 0,3,6
        "channel_16x12x20_s3v2": dict(params=channel_params(16, 12, 20).copy(stencil_size=3, stencil_visc=2,
                                                                             check_cfl=3, check_bulk=2),
                                      nsteps=8, ic="channel"),
        # channel at 8th order
        "channel_24x16x16_s4v4": dict(params=channel_params(24, 16, 16), nsteps=5, ic="channel"),
        # boundary layer: extrapolated x top / z ends, sponge, wall perturbation
        "bl_16x8x160_s3v2": dict(params=boundary_layer_params(16, 8, 160), nsteps=6, ic="bl"),
    }


def large_cases():
    """Golden cases at the benchmark sizes, 10 steps each: the 64^3 Taylor-Green box (the
    analytic start with rho = 1) and the 128x160x192 isothermal channel (seeded start), as
    the benchmark configures them. Their fields are packed as a subsample with stride `sub`
    plus whole-grid maxima and plane sums."""
    return {
        "tgv_64_s4v4": dict(params=tgv_params(64), nsteps=10, ic="tgv", sub=2),
        "channel_128x160x192_s4v4": dict(params=channel_params(128, 160, 192), nsteps=10, ic="channel", sub=4),
    }


def timing_cases():
    """Throughput of the reference's own GPU code (S = V = 4, Wray RK3, FP64) on the
    benchmark channel (reference axes mx=128 wall-normal, my=160 span, mz=192 stream) and on
    the 64^3 Taylor-Green box, each started from the reference's own initialisation
    (restartFile = -1). Two runs of different length per case family: the per-step time is
    their difference quotient, which cancels the set-up, the initial-field generation and
    the file output inside the reference's own total time (src/main.cpp:71-75)."""
    fam = {"channel_128x160x192": (channel_params(128, 160, 192), (20, 200)),
           "tgv_64": (tgv_params(64), (100, 1000))}
    return {f"time_{f}_n{n}": dict(params=p, nsteps=n, ic="ref_init", family=f)
            for f, (p, ns) in fam.items() for n in ns}


def _lit(x: float) -> str:
    return repr(float(x))


COEFF_TEXT = {
    1: ("{-1.0/2.0}", "{1.0, -2.0}"),
    2: ("{ 1.0/12.0, -2.0/3.0}", "{-1.0/12.0,  4.0/3.0, -5.0/2.0}"),
    3: ("{-1.0/60.0,  3.0/20.0, -3.0/4.0}", "{ 1.0/90.0, -3.0/20.0,  3.0/2.0, -49.0/18.0}"),
    4: ("{ 1.0/280.0, -4.0/105.0,  1.0/5.0, -4.0/5.0}",
        "{-1.0/560.0,  8.0/315.0, -1.0/5.0,  8.0/5.0,  -205.0/72.0}"),
}


def parameter_header(p, nsteps: int, restart: int) -> str:
    """The reference's compile-time parameter surface, generated from a cns_params."""
    b = lambda v: "(true)" if v else "(false)"  # noqa: E731
    F, Sx = COEFF_TEXT[p.stencil_size]
    VF, VS = COEFF_TEXT[p.stencil_visc]
    return f"""/* generated by oracle/ref_harness.py */
#ifndef GLOBALS_H_
#define GLOBALS_H_
#define myprec double
#define MPI_myprec MPI_DOUBLE
#include "math.h"
#include "main.h"
#include <stdlib.h>
#include <stdio.h>
#define pRow 1
#define pCol 1
#define stencilSize {p.stencil_size}
#define stencilVisc {p.stencil_visc}
#define Lx ({_lit(p.Lx)})
#define Ly ({_lit(p.Ly)})
#define Lz ({_lit(p.Lz)})
#define mx_tot {p.mx}
#define my_tot {p.my}
#define mz_tot {p.mz}
#define nsteps {nsteps}
#define nfiles 1
#define CFL {_lit(p.cfl)}
#define restartFile {restart}
#define lowStorage {b(p.scheme == RK3_LOWSTORAGE)}
#define boundaryLayer {b(p.boundary_layer)}
#define perturbed {b(p.perturbed)}
#define forcing {b(p.forcing)}
#define periodicX {b(p.periodic_x)}
#define nonUniformX {b(p.nonuniform_x)}
#define checkCFLcondition {p.check_cfl}
#define checkBulk {p.check_bulk}
#define Re {_lit(p.Re)}
#define Pr {_lit(p.Pr)}
#define Ma {_lit(p.Ma)}
#define viscexp {_lit(p.viscexp)}
#define gam {_lit(p.gam)}
#define Ec ((gam - 1.f)*Ma*Ma)
#define Rgas (1.f/(gam*Ma*Ma))
const double stretch = {_lit(p.stretch)};
const myprec TwallTop = {_lit(p.twall_top)};
const myprec TwallBot = {_lit(p.twall_bot)};
#define mx (mx_tot)
#define my (my_tot/pRow)
#define mz (mz_tot/pCol)
#define nDivZ (1)
#define idx(i,j,k) ({{ ( k )*mx*my +( j )*mx + ( i ); }})
const int multiGPU = 0;
const double coeffF[] = {F};
const double coeffS[] = {Sx};
const double coeffVF[] = {VF};
const double coeffVS[] = {VS};
extern double dt, h_dpdz;
extern double dx,x[mx],xp[mx],xpp[mx],y[my_tot],z[mz_tot];
extern double r[mx*my*mz];
extern double u[mx*my*mz];
extern double v[mx*my*mz];
extern double w[mx*my*mz];
extern double e[mx*my*mz];
#endif
"""


MAKEFILE = r"""# generated by oracle/ref_harness.py: builds the staged reference for sm_103a
NVCC ?= nvcc
CXX ?= g++
CUDA_HOME ?= /usr/local/cuda
ARCH = -gencode arch=compute_103a,code=sm_103a
NVFLAGS = -O3 -rdc=true --use_fast_math $(ARCH) -Isrc
CXXFLAGS = -O3 -std=c++14 -Isrc -I$(CUDA_HOME)/include
CU = cuda_utils cuda_math cuda_main cuda_rhs calc_stress sponge
CC = main comm init
CUO = $(addprefix obj/,$(addsuffix .o,$(CU)))
CCO = $(addprefix obj/,$(addsuffix .o,$(CC)))
ns: $(CUO) $(CCO)
	$(NVCC) $(ARCH) -dlink $(CUO) -o obj/link.o
	$(CXX) -o ns $(CCO) $(CUO) obj/link.o -L$(CUDA_HOME)/lib64 -lcudadevrt -lcudart -lm
obj/%.o: src/%.cu
	@mkdir -p obj
	$(NVCC) $(NVFLAGS) -c $< -o $@
obj/%.o: src/%.cpp
	@mkdir -p obj
	$(CXX) $(CXXFLAGS) -c $< -o $@
"""


def _disable_dead_helpers(text: str) -> str:
    """Wrap reduceToMax .. reduceToOne (device functions that call cudaDeviceSynchronize
    from device code; nothing on the solver path calls them) in #if 0."""
    start = text.index("__device__ void reduceToMax")
    end = text.index("__global__ void integrateThreads")
    return text[:start] + "#if 0\n" + text[start:end] + "#endif\n" + text[end:]


def blasius_like_profile(n: int = 601, xmax: float = 60.0):
    """Smooth synthetic self-similar profile standing in for the missing blasius1D/*.bin
    (bLayerInit.py needs matplotlib). x is the similarity coordinate; w the streamwise
    velocity 0 -> 1, u a small wall-normal velocity, r from a Crocco-like temperature."""
    x = np.linspace(0.0, xmax, n)
    w = np.tanh(x / 3.0)
    u = 0.8 * (x * w - 3.0 * np.log(np.cosh(x / 3.0))) / 3.0
    T = 1.0 + 0.15 * (1.0 - w * w)
    r = 1.0 / T
    e = np.zeros_like(x)
    return x, r, u, w, e


def initial_fields(ic: str, p):
    """The initial fields of a staged case (written as restart files fields/*.0000000.bin)."""
    if ic == "tgv":
        return initial.tgv_fields(p)
    if ic == "tgv_ref":
        return initial.tgv_reference_fields(p)
    from oracle.oracle import Oracle  # grid of the stretched channel
    return initial.channel_fields(p, Oracle(p).grid()["x"], seed=0)


def stage(names):
    root = reference_root()
    if root is None:
        raise SystemExit("reference checkout not found: set CNS_REFERENCE_ROOT")
    ref_src = os.path.join(root, "src")
    allc = dict(cases(), **large_cases(), **timing_cases())
    for name in names or cases():
        c = allc[name]
        p, nsteps = c["params"], c["nsteps"]
        d = os.path.join(STAGE_ROOT, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(os.path.join(d, "src"))
        os.makedirs(os.path.join(d, "fields"))
        for fn in os.listdir(ref_src):
            if fn.endswith((".cu", ".cpp", ".h")) and fn != "globals.h" and fn != "cuda_derivs.cu":
                shutil.copy(os.path.join(ref_src, fn), os.path.join(d, "src", fn))
        cm = os.path.join(d, "src", "cuda_math.cu")
        with open(cm) as f:
            txt = f.read()
        with open(cm, "w") as f:
            f.write(_disable_dead_helpers(txt))
        shutil.copy(os.path.join(HERE, "ref_mpi_stub.h"), os.path.join(d, "src", "mpi.h"))
        restart = -1 if c["ic"] in ("bl", "ref_init") else 0
        with open(os.path.join(d, "src", "globals.h"), "w") as f:
            f.write(parameter_header(p, nsteps, restart))
        with open(os.path.join(d, "Makefile"), "w") as f:
            f.write(MAKEFILE)
        deferred = "sub" in c
        if c["ic"] == "ref_init" or deferred:
            pass
        elif c["ic"] == "bl":
            os.makedirs(os.path.join(d, "blasius1D"))
            for nm, arr in zip("xruwe", blasius_like_profile()):
                arr.astype(np.float64).tofile(os.path.join(d, "blasius1D", f"{nm}Prof.bin"))
        else:
            initial.write_fields(os.path.join(d, "fields"), 0, initial_fields(c["ic"], p))
        with open(os.path.join(d, "case.json"), "w") as f:
            json.dump(dict(name=name, nsteps=nsteps, ic=c["ic"], params=p.as_dict(), sub=c.get("sub", 0)),
                      f, indent=1)
        print("staged", d)


def pack_large(out, sub: int) -> dict:
    """A strided subsample of the fields (every `sub`-th point per axis, from 0) and, per
    field over the whole grid, the maximum magnitude and the plane sums along z, y and x."""
    a = np.stack(out)
    return dict(out_sub=np.ascontiguousarray(a[:, ::sub, ::sub, ::sub]), out_absmax=np.abs(a).max(axis=(1, 2, 3)),
                out_sum_k=a.sum(axis=(2, 3)), out_sum_j=a.sum(axis=(1, 3)), out_sum_i=a.sum(axis=(1, 2)))


def run(names, out_root):
    os.makedirs(out_root, exist_ok=True)
    known = dict(cases(), **large_cases())
    dirs = sorted(n for n in os.listdir(STAGE_ROOT) if os.path.isdir(os.path.join(STAGE_ROOT, n)) and n in known)
    ok = True
    for name in dirs:
        if names and name not in names:
            continue
        d = os.path.join(STAGE_ROOT, name)
        with open(os.path.join(d, "case.json")) as f:
            meta = json.load(f)
        nproc = str(os.cpu_count() or 4)
        # objects compiled elsewhere (another host architecture) are discarded first
        shutil.rmtree(os.path.join(d, "obj"), ignore_errors=True)
        if os.path.exists(os.path.join(d, "ns")):
            os.remove(os.path.join(d, "ns"))
        b = subprocess.run(["make", "-j", nproc], cwd=d, capture_output=True, text=True)
        if b.returncode != 0:
            print(f"[{name}] build failed:\n{b.stdout[-3000:]}\n{b.stderr[-3000:]}")
            ok = False
            continue
        sub = int(meta.get("sub", 0))
        pr = CnsParams()
        for k, v in meta["params"].items():
            setattr(pr, k, v)
        if sub:   # benchmark-size case: the initial fields are written here
            initial.write_fields(os.path.join(d, "fields"), 0, initial_fields(meta["ic"], pr))
        env = dict(os.environ, CUDA_LAUNCH_BLOCKING="1")
        r = subprocess.run(["./ns"], cwd=d, capture_output=True, text=True, env=env, timeout=600)
        log = r.stdout + r.stderr
        with open(os.path.join(out_root, name + ".log"), "w") as f:
            f.write(log)
        if r.returncode != 0:
            print(f"[{name}] run failed rc={r.returncode}\n{log[-2000:]}")
            ok = False
            continue
        p = meta["params"]
        shape = (p["mz"], p["my"], p["mx"])
        ic = initial.read_fields(os.path.join(d, "fields"), 0, shape)
        out = initial.read_fields(os.path.join(d, "fields"), 1, shape)
        steps = [(int(m.group(1)), float(m.group(2)), float(m.group(3)))
                 for m in re.finditer(r"step number (\d+) with (\S+) (\S+)", log)]
        m = re.search(r"friction Reynolds number is:\s+(\S+)", log)
        ret = np.array([float(m.group(1)) if m else np.nan])
        prof_path = os.path.join(d, "prof.txt")
        prof = np.loadtxt(prof_path) if os.path.exists(prof_path) else np.zeros((0, 11))
        common = dict(x=np.fromfile(os.path.join(d, "fields", "x.bin")),
                      steplog=np.array(steps, dtype=np.float64).reshape(-1, 3), ret=ret, prof=prof,
                      meta=json.dumps(meta))
        if sub:
            np.savez_compressed(os.path.join(out_root, name + ".npz"),
                                ic_sub=np.ascontiguousarray(np.stack(ic)[:, ::sub, ::sub, ::sub]),
                                **pack_large(out, sub), **common)
        else:
            np.savez_compressed(os.path.join(out_root, name + ".npz"), ic=np.stack(ic), out=np.stack(out), **common)
        print(f"[{name}] ok: {len(steps)} dt lines, rho range {out[0].min():.6f}..{out[0].max():.6f}")
    return ok


def time_runs(names, out_root):
    """Build and run the staged timing cases twice each: in the reference's native stream
    order (its default, unsynchronised) and with CUDA_LAUNCH_BLOCKING=1 (program order),
    and write the per-step times and Mpoint-steps/s to <out>/ref_timing.json."""
    tc = timing_cases()
    os.makedirs(out_root, exist_ok=True)
    res = {}
    for name in sorted(tc):
        if names and name not in names:
            continue
        d = os.path.join(STAGE_ROOT, name)
        shutil.rmtree(os.path.join(d, "obj"), ignore_errors=True)
        if os.path.exists(os.path.join(d, "ns")):
            os.remove(os.path.join(d, "ns"))
        b = subprocess.run(["make", "-j", str(os.cpu_count() or 4)], cwd=d, capture_output=True, text=True)
        if b.returncode != 0:
            print(f"[{name}] build failed:\n{b.stderr[-3000:]}")
            return False
        for mode, extra in (("native", {}), ("blocking", {"CUDA_LAUNCH_BLOCKING": "1"})):
            totals = []
            for rep in range(2):   # the shorter of two runs (the file output's time varies)
                r = subprocess.run(["./ns"], cwd=d, capture_output=True, text=True,
                                   env=dict(os.environ, **extra), timeout=900)
                log = r.stdout + r.stderr
                with open(os.path.join(out_root, f"{name}_{mode}.log"), "w") as f:
                    f.write(log)
                m = re.search(r"The total time is:\s+(\S+)", log)
                if r.returncode != 0 or not m:
                    print(f"[{name}/{mode}] run failed rc={r.returncode}\n{log[-2000:]}")
                    return False
                totals.append(float(m.group(1)))
            steps = re.findall(r"step number (\d+) with (\S+) (\S+)", log)
            res[f"{name}/{mode}"] = dict(total_s=min(totals), totals=totals, nsteps=tc[name]["nsteps"],
                                         last_dt=float(steps[-1][1]) if steps else None)
            print(f"[{name}/{mode}] total {min(totals):.3f} s")
    out = {"runs": res}
    for fam in sorted({c["family"] for c in tc.values()}):
        names_f = sorted((n for n in tc if tc[n]["family"] == fam), key=lambda n: tc[n]["nsteps"])
        p = tc[names_f[0]]["params"]
        pts = p.mx * p.my * p.mz
        for mode in ("native", "blocking"):
            a, b = (res.get(f"{n}/{mode}") for n in (names_f[0], names_f[-1]))
            if a and b:
                per = (b["total_s"] - a["total_s"]) / (b["nsteps"] - a["nsteps"])
                out.setdefault(fam, {})[mode] = dict(s_per_step=per, mpoint_steps_per_s=pts / per / 1e6)
    with open(os.path.join(out_root, "ref_timing.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))
    return True


def collect(names, out_root):
    os.makedirs(GOLDEN, exist_ok=True)
    large = large_cases()
    for fn in sorted(os.listdir(out_root)):
        if fn.endswith(".npz") and (not names or fn[:-4] in names):
            prefix = "refsub_" if fn[:-4] in large else "ref_"
            shutil.copy(os.path.join(out_root, fn), os.path.join(GOLDEN, prefix + fn))
            print("collected", fn)


def main(argv):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("cmd", choices=["stage", "run", "time", "collect"])
    ap.add_argument("cases", nargs="*")
    ap.add_argument("--out", help="directory of the packed results (run, time, collect)")
    a = ap.parse_intermixed_args(argv)
    if a.cmd == "stage":
        stage(a.cases)
        return 0
    if not a.out:
        ap.error(f"{a.cmd} needs --out DIR")
    if a.cmd == "run":
        return 0 if run(a.cases, a.out) else 1
    if a.cmd == "time":
        return 0 if time_runs(a.cases, a.out) else 1
    collect(a.cases, a.out)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
