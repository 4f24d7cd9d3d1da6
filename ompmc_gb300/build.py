"""In-tree build of the native library and the command-line front end.

Produces
  ompmc_gb300/lib/libompmc_gb300.so   host library + CUDA engine (C ABI)
  ompmc_gb300/bin/omc_dosxyz          command-line front end (omc_dosxyz CLI)

with g++ for host code and nvcc for the device code, compiled for sm_103a
only.  Translation units are compiled in parallel; nothing here needs
cmake.  Re-running is incremental on source timestamps.
"""

from __future__ import annotations

import glob
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
CSRC = os.path.join(HERE, "csrc")
# Outputs are per host architecture: a tree copied between an x86-64 and an
# aarch64 machine never loads the other's binaries.
MACHINE = platform.machine()
OBJ = os.path.join(HERE, "_build", MACHINE)
LIB = os.path.join(HERE, "lib", MACHINE, "libompmc_gb300.so")
BIN = os.path.join(HERE, "bin", MACHINE, "omc_dosxyz")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: the host table builders must round exactly like the
# reference on every host architecture (no fused multiply-adds).
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function", f"-I{INCLUDE}"]
# --use_fast_math changes single-precision arithmetic only (approximate division, square root and
# transcendental intrinsics, denormals flushed): the FP32 transport path.  The FP64 path, and with it the
# serial lane that reproduces the reference's serial build, is unchanged.  Measured on the 6 MV slab: FP32
# 5.17e7 -> 7.21e7 histories/s, with the FP32-vs-FP64 dose error unchanged (bench.py fp32_dose_error).
NVCCFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}",
                    "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr", "--use_fast_math"]
# Extra -D definitions for tuning builds (e.g. OMC_NVCC_DEFINES="OMC_MIN_BLOCKS_FP32=5").
NVCCFLAGS += [f"-D{d}" for d in os.environ.get("OMC_NVCC_DEFINES", "").split() if d]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return (glob.glob(os.path.join(CSRC, "**", "*.h"), recursive=True)
            + glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
            + glob.glob(os.path.join(CSRC, "**", "*.inc"), recursive=True)
            + [os.path.join(INCLUDE, "omc_gpu.h")])


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "host", "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++", *CXXFLAGS, "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "engine", "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nvcc, *NVCCFLAGS, "-c", src, "-o", obj])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for j in jobs]
    failed = []
    for j, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out)
        if p.returncode != 0:
            failed.append(" ".join(j))
    if failed:
        raise RuntimeError("compilation failed:\n" + "\n".join(failed))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], check=True)
        os.replace(tmp, LIB)
    cli = os.path.join(CSRC, "frontend", "omc_dosxyz.c")
    if os.path.exists(cli) and (force or _stale(BIN, [cli, LIB, os.path.join(INCLUDE, "omc_gpu.h")])):
        subprocess.run(["gcc", "-O2", "-std=gnu11", f"-I{INCLUDE}", cli, "-o", BIN, f"-L{os.path.dirname(LIB)}",
                        "-lompmc_gb300", "-Wl,-rpath,$ORIGIN/../../lib/" + MACHINE, "-lm"], check=True)
    return LIB


if __name__ == "__main__":  # pragma: no cover
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
