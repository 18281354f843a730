"""Builds librecon_track.so (sm_103a) in-tree with nvcc.

Eight translation units (kernels.cu, host.cu, refshim.cu, initnet.cu, selftest.cu, tsdf.cu, trajio.cu,
kinect.cu) compiled in parallel and linked
into recon_gb300/librecon_track.so.  -fmad=false keeps every floating-point
multiply and add separately rounded (the bit-exactness contract of the
kernels); -lineinfo keeps source lines for profiling.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "librecon_track.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
UNITS = ["kernels.cu", "host.cu", "refshim.cu", "initnet.cu", "selftest.cu", "tsdf.cu", "trajio.cu", "kinect.cu"]
HEADERS = ["scene.h", "fx.cuh", "solve.cuh", "track_kernels.cuh", "track_math.cuh", "exact_arith.cuh"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librecon_track.so")


def _sources():
    srcs = [os.path.join(CSRC, u) for u in UNITS] + [os.path.join(CSRC, h) for h in HEADERS]
    srcs.append(os.path.join(ROOT, "include", "recon_track.h"))
    srcs.append(os.path.join(ROOT, "include", "recon_ref_shim.h"))
    srcs.append(os.path.join(ROOT, "include", "recon_initnet.h"))
    srcs.append(os.path.join(ROOT, "include", "recon_tsdf.h"))
    srcs.append(os.path.join(ROOT, "include", "recon_kinect.h"))
    srcs.append(os.path.abspath(__file__))
    return srcs


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = [ARCH, "-O3", "-std=c++17", "-fmad=false", "-lineinfo", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-diag-suppress", "550"]
    # extra nvcc options (e.g. -DRECON_ITER_MIN_BLOCKS=3) for tuning builds
    flags += os.environ.get("RECON_NVCC_EXTRA", "").split()

    def compile_unit(u):
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        cmd = [cc, *flags, "-c", os.path.join(CSRC, u), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [cc, ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
