"""Builds libfm3dt_gpu.so in-tree with nvcc for sm_103a (GB300).

Translation units compile in parallel, all without automatic FMA
contraction: the gridder, boundary frames, receivers and rays round like the
reference's left-to-right Fortran arithmetic, and the solver's explicit FMAs
make every kernel instantiation compute the same bits.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shlex
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(ROOT, "libfm3dt_gpu.so")
DRIVER_DIR = os.path.join(ROOT, "driver")
DRIVER = os.path.join(ROOT, "fm3dt_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (a function that can end without its return value is an error: the host
# compiler may otherwise treat that end as unreachable)
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Werror=return-type",
          "--expt-relaxed-constexpr"]
SOURCES = {
    "model.cu": ["-fmad=false"],
    "boundary.cu": ["-fmad=false"],
    "receivers.cu": ["-fmad=false"],
    "rays.cu": ["-fmad=false"],
    "point.cu": ["-fmad=false"],
    "solver_f32.cu": ["-fmad=false"],
    "solver_f64.cu": ["-fmad=false"],
    "capi.cu": [],
}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _deps_mtime(dirs=(CSRC,)) -> float:
    m = 0.0
    for d in dirs:
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    hdr = os.path.join(os.path.dirname(ROOT), "include", "fm3dt_gpu.h")
    if os.path.exists(hdr):
        m = max(m, os.path.getmtime(hdr))
    return m


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def one(item):
        src, extra = item
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        # FM3DT_NVCC_FLAGS: extra flags for tuning builds (e.g. -DFM_ROUND_MINB_F32=8)
        cmd = [nv, *ARCH, *COMMON, *extra, *shlex.split(os.environ.get("FM3DT_NVCC_FLAGS", "")),
               "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(one, SOURCES.items()))
    if verbose:
        for _, log in results:
            if log:
                print(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    r = subprocess.run([nv, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_driver(force: bool = False) -> str:
    """Builds the host driver fm3dt_run (the reference's file contract over
    the C ABI) with g++, linked to libfm3dt_gpu.so in the same directory."""
    lib = build(force=force)
    if not force and os.path.exists(DRIVER) and \
            os.path.getmtime(DRIVER) >= max(_deps_mtime((DRIVER_DIR,)), os.path.getmtime(lib)):
        return DRIVER
    cxx = shutil.which("g++") or "g++"
    tmp = DRIVER + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", os.path.join(DRIVER_DIR, "fm3dt_run.cpp"),
           os.path.join(DRIVER_DIR, "fm3dt_files.cpp"), "-o", tmp, "-L" + ROOT, "-lfm3dt_gpu",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DRIVER)
    return DRIVER


SUBINV_DIR = os.path.join(ROOT, "subinv")
SUBINV_LIB = os.path.join(ROOT, "libfm3dt_subinv.so")
SUBINV = os.path.join(ROOT, "fm3dt_subinv")
HOST_FLAGS = ["-O2", "-std=c++17", "-Wall", "-ffp-contract=off", "-pthread"]


def build_subinv(force: bool = False) -> str:
    """Builds the host-side subspace inversion (libfm3dt_subinv.so and the
    fm3dt_subinv program) with g++; no CUDA involved."""
    deps = max(_deps_mtime((SUBINV_DIR, DRIVER_DIR)), os.path.getmtime(
        os.path.join(os.path.dirname(ROOT), "include", "fm3dt_subinv.h")))
    if not force and all(os.path.exists(p) and os.path.getmtime(p) >= deps for p in (SUBINV_LIB, SUBINV)):
        return SUBINV_LIB
    cxx = shutil.which("g++") or "g++"
    steps = [
        [cxx, *HOST_FLAGS, "-fPIC", "-shared", os.path.join(SUBINV_DIR, "subinv.cpp"), "-o", SUBINV_LIB + ".tmp"],
        [cxx, *HOST_FLAGS, os.path.join(SUBINV_DIR, "subinv_main.cpp"), os.path.join(DRIVER_DIR, "fm3dt_files.cpp"),
         "-o", SUBINV + ".tmp", "-L" + ROOT, "-lfm3dt_subinv", "-Wl,-rpath,$ORIGIN"],
    ]
    for i, cmd in enumerate(steps):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"subinv build failed:\n{r.stdout}\n{r.stderr}")
        if i == 0:
            os.replace(SUBINV_LIB + ".tmp", SUBINV_LIB)
    os.replace(SUBINV + ".tmp", SUBINV)
    return SUBINV_LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose=True, ptxas_info="-v" in sys.argv))
