"""In-tree build of the GB300 library (libcns_gb300.so) with nvcc for sm_103a.

Translation units are compiled in parallel; the RHS kernel instantiations for FP64 and
FP32 are separate units so the slowest compiles overlap. Output goes to
cudanavierstokes_gb300/_lib/ (git-ignored). No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libcns_gb300.so")
DRIVER = os.path.join(LIBDIR, "cns")
DRIVER_SRC = os.path.join(PKG, "csrc", "cns_main.cpp")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
           "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def sources():
    """Library translation units (the driver's main() is linked separately)."""
    return sorted(f for f in glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp"))
                  if f != DRIVER_SRC)


def headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + headers()):
        return obj
    cmd = [nvcc()] + ARCH + NVFLAGS + ["-c", src, "-o", obj + ".tmp"]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu"] + cmd[1:]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr[-6000:]}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile every CUDA/C++ source for sm_103a and link the shared library."""
    os.makedirs(OBJDIR, exist_ok=True)
    if force:
        for f in glob.glob(os.path.join(OBJDIR, "*.o")):
            os.remove(f)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC", "-lcudart_static", "-lrt",
                                                                  "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, LIB)
    if _stale(DRIVER, [LIB, DRIVER_SRC] + headers()):
        cmd = ["g++", "-O2", "-std=c++17", "-I" + INCLUDE, "-o", DRIVER + ".tmp", DRIVER_SRC, "-L" + LIBDIR,
               "-lcns_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stderr[-4000:]}")
        os.replace(DRIVER + ".tmp", DRIVER)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
