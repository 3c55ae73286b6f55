"""Builds the CUDA trial engine, libugrowth.so, in-tree for sm_103a.

nvcc compiles the translation units in parallel: the double-precision
kernels (without multiply-add contraction, so they keep the reference's
rounding sequence), the single-precision kernels, the host side with the
C ABI of include/ugrowth.h, the pipe calibration, the reference's file
formats, and the topology generator (also without contraction); then the
command-line programs.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.environ.get("UG_BUILD_DIR", os.path.join(HERE, "_lib"))
LIB = os.path.join(OUT_DIR, "libugrowth.so")
CLI = os.path.join(OUT_DIR, "ug_growth")   # the command-line programs (csrc/ug_cli.cpp)
# extra nvcc flags, e.g. -DUG_RA_MIN_BLOCKS=4 to build a tuning variant into UG_BUILD_DIR
EXTRA = os.environ.get("UG_NVCC_EXTRA", "").split()
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
CLI_SRC = "ug_cli.cpp"
UNITS = [("ug_kernels_f64.cu", ["-fmad=false"]), ("ug_kernels_f32.cu", []), ("ug_host.cu", []), ("ug_calib.cu", []),
         ("ug_files.cpp", []), ("ug_topology.cu", ["-fmad=false"])]


def nvcc() -> str:
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    return "nvcc"


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".cpp"))] + [
        os.path.join(ROOT, "include", "ugrowth.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = []

    def compile_unit(unit):
        src, extra = unit
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc()] + ARCH + COMMON + EXTRA + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS) + 1) as ex:
        cli = ex.submit(compile_unit, (CLI_SRC, []))
        objs = list(ex.map(compile_unit, UNITS))
        cli_obj = cli.result()
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    # the command-line programs, linked against the library next to them
    cmd = [nvcc(), cli_obj, "-o", CLI + ".tmp", "-L" + OUT_DIR, "-lugrowth", "-Xlinker", "-rpath=$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of {CLI} failed:\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
