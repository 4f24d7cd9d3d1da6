"""Python access to the test oracle (TEST INFRASTRUCTURE ONLY).

Loaded only by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py.  ``run`` drives oracle/liboracle.so (the C restatement of the
reference's transport) on tables built by the product's host library;
``ref_*`` drive the unmodified reference built by oracle/Makefile into
oracle/_ref/ (present only where the reference tree was available).
"""

from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", platform.machine(), "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


class Result(C.Structure):
    _fields_ = [("ensrc", C.c_double), ("seconds", C.c_double), ("histories", C.c_longlong),
                ("nthreads", C.c_int), ("status", C.c_int)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True, capture_output=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        L.omc_oracle_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_longlong,
                                     C.c_int, C.c_int, C.c_int, C.c_int, dp, dp, C.POINTER(Result)]
        L.omc_oracle_run.restype = C.c_int
        L.omc_oracle_ranmar.argtypes = [C.c_int, C.c_int, C.c_longlong, C.POINTER(C.c_int)]
        L.omc_oracle_ranmar.restype = None
        _lib = L
    return _lib


def run(problem, nperbatch=None, nbatch=None, seeds=None, nsplit=None, nthreads=1):
    """Oracle transport of an ompmc_gb300.api.Problem; returns
    (accum_endep, accum_endep2, Result)."""
    nreg = problem.nreg
    a = np.zeros(nreg)
    a2 = np.zeros(nreg)
    res = Result()
    seeds = problem.seeds if seeds is None else seeds
    st = lib().omc_oracle_run(problem.tables, C.cast(problem.phantom._p, C.c_void_p),
                              C.cast(problem.regions, C.c_void_p), C.cast(problem.source, C.c_void_p),
                              problem.nsplit if nsplit is None else nsplit,
                              problem.nperbatch if nperbatch is None else nperbatch,
                              problem.nbatch if nbatch is None else nbatch, seeds[0], seeds[1], nthreads,
                              a.ctypes.data_as(C.POINTER(C.c_double)), a2.ctypes.data_as(C.POINTER(C.c_double)),
                              C.byref(res))
    if st != 0:
        raise RuntimeError(f"oracle run failed with status {st}")
    return a, a2, res


def ranmar(ixx, jxx, n):
    out = np.zeros(n, dtype=np.int32)
    lib().omc_oracle_ranmar(ixx, jxx, n, out.ctypes.data_as(C.POINTER(C.c_int)))
    return out


# ---- the unmodified reference (only where oracle/_ref was built) ----------

def ref_available():
    return os.path.exists(os.path.join(REF_DIR, "ref_harness"))


def read_omct(path):
    """Reader of the 'OMCT' dump format written by the harness and by
    omc_tables_dump."""
    with open(path, "rb") as f:
        b = f.read()
    if b[:4] != b"OMCT":
        raise ValueError(f"{path}: not an OMCT dump")
    o, out = 4, {}
    while o < len(b):
        n = int.from_bytes(b[o:o + 4], "little")
        o += 4
        name = b[o:o + n].decode()
        o += n
        t = chr(b[o])
        o += 1
        cnt = int.from_bytes(b[o:o + 8], "little")
        o += 8
        dt, sz = (np.float64, 8) if t == "d" else (np.int32, 4)
        out[name] = np.frombuffer(b[o:o + cnt * sz], dtype=dt).copy()
        o += cnt * sz
    return out


def ref_run(cmd, *args, omp=False, timeout=600):
    exe = os.path.join(REF_DIR, "ref_harness_omp" if omp else "ref_harness")
    subprocess.run([exe, cmd, *map(str, args)], check=True, capture_output=True, timeout=timeout)


def ref_dose(inp_without_ext, out_path, nthreads=0, omp=False):
    ref_run("dose", inp_without_ext, out_path, nthreads, omp=omp)
    return read_omct(out_path)


def ref_tables(inp_without_ext, out_path):
    ref_run("tables", inp_without_ext, out_path)
    return read_omct(out_path)


def ref_ranmar(ixx, jxx, n, out_path):
    ref_run("rng", ixx, jxx, n, out_path)
    return read_omct(out_path)["rng"]
