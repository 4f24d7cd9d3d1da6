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
        L.omc_oracle_batch_totals.argtypes = [dp, C.c_int]
        L.omc_oracle_batch_totals.restype = C.c_int
        L.omc_oracle_ranmar.argtypes = [C.c_int, C.c_int, C.c_longlong, C.POINTER(C.c_int)]
        L.omc_oracle_ranmar.restype = None
        from ompmc_gb300._native import Beamlets_t, Dij_t

        L.omc_oracle_run_dij.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Beamlets_t),
                                         C.c_int, C.POINTER(C.c_longlong), C.c_longlong, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_double, C.POINTER(Dij_t), C.POINTER(Result)]
        L.omc_oracle_run_dij.restype = C.c_int
        L.omc_oracle_dij_free.argtypes = [C.POINTER(Dij_t)]
        L.omc_oracle_dij_free.restype = None
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


def batch_totals():
    """Energy deposited inside the phantom by each batch of the last run."""
    out = np.zeros(65536)
    n = lib().omc_oracle_batch_totals(out.ctypes.data_as(C.POINTER(C.c_double)), len(out))
    return out[:n].copy()


def _beamlets_struct(b):
    from ompmc_gb300._native import Beamlets_t

    keep = [np.ascontiguousarray(b.ibeam, dtype=np.int32)]
    cols = []
    for arr in (b.source[:, 0], b.source[:, 1], b.source[:, 2], b.corner[:, 0], b.corner[:, 1], b.corner[:, 2],
                b.side1[:, 0], b.side1[:, 1], b.side1[:, 2], b.side2[:, 0], b.side2[:, 1], b.side2[:, 2]):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        keep.append(a)
        cols.append(a.ctypes.data_as(C.POINTER(C.c_double)))
    return Beamlets_t(len(b.ibeam), len(b.source), keep[0].ctypes.data_as(C.POINTER(C.c_int)), *cols), keep


def run_dij(problem, beamlets, rel_threshold=1e-4, nhist=None, nperbatch=None, nbatch=None, seeds=None,
            nthreads=1):
    """Oracle of the omc_matrad beamlet loop; returns (col_ptr, row_idx,
    values, Result)."""
    from ompmc_gb300._native import Dij_t

    st, keep = _beamlets_struct(beamlets)
    nh = None if nhist is None else np.ascontiguousarray(nhist, dtype=np.int64)
    seeds = problem.seeds if seeds is None else seeds
    out = Dij_t()
    res = Result()
    rc = lib().omc_oracle_run_dij(problem.tables, C.cast(problem.phantom._p, C.c_void_p),
                                  C.cast(problem.regions, C.c_void_p), C.cast(problem.source, C.c_void_p),
                                  C.byref(st), problem.nsplit,
                                  nh.ctypes.data_as(C.POINTER(C.c_longlong)) if nh is not None else None,
                                  problem.nperbatch if nperbatch is None else nperbatch,
                                  problem.nbatch if nbatch is None else nbatch, seeds[0], seeds[1], nthreads,
                                  float(rel_threshold), C.byref(out), C.byref(res))
    try:
        if rc != 0:
            raise RuntimeError(f"oracle dij failed with status {rc}")
        col = np.ctypeslib.as_array(out.col_ptr, shape=(out.ncols + 1,)).copy()
        if out.nnz:
            rows = np.ctypeslib.as_array(out.row_idx, shape=(out.nnz,)).copy()
            vals = np.ctypeslib.as_array(out.values, shape=(out.nnz,)).copy()
        else:
            rows, vals = np.zeros(0, np.int32), np.zeros(0)
    finally:
        lib().omc_oracle_dij_free(C.byref(out))
    del keep
    return col, rows, vals, res


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


def ref_matrad_available():
    return os.path.exists(os.path.join(REF_DIR, "matrad_serial"))


def ref_matrad(workdir, phantom, beamlets, opts, timeout=1200):
    """Run the reference's omc_matrad front end (mexFunction, serial build)
    through oracle/matrad_harness.c.  phantom: ompmc_gb300.workloads.Phantom;
    beamlets: workloads.Beamlets; opts: the mcOpt fields (nHistories,
    nBatches, nSplit, spectrumFile, monoEnergy, charge, global_ecut,
    global_pcut, randomSeeds, pegsFile, pgs4formFile, dataFolder,
    outputFolder, relDoseThreshold, verbose).  Returns (col_ptr, row_idx,
    values) of the sparse dij."""
    os.makedirs(workdir, exist_ok=True)
    nz, ny, nx = phantom.shape
    with open(os.path.join(workdir, "geo.txt"), "w") as f:
        f.write(f"{nx} {ny} {nz}\n{len(phantom.media)}\n")
        for m in phantom.media:
            f.write(m + "\n")
        for b in (phantom.xb, phantom.yb, phantom.zb):
            f.write(" ".join(repr(float(v)) for v in b) + "\n")
    np.ascontiguousarray(phantom.rho, dtype=np.float64).tofile(os.path.join(workdir, "rho.f64"))
    np.ascontiguousarray(phantom.med, dtype=np.int32).tofile(os.path.join(workdir, "matix.i32"))
    b = beamlets
    with open(os.path.join(workdir, "src.txt"), "w") as f:
        f.write(f"{b.n} {len(b.source)}\n")
        rows = [b.ibeam + 1.0] + [b.source[:, k] for k in range(3)] + [b.corner[:, k] for k in range(3)] + \
               [b.side1[:, k] for k in range(3)] + [b.side2[:, k] for k in range(3)]
        for r in rows:
            f.write(" ".join(repr(float(v)) for v in r) + "\n")
    strings = {"spectrumFile", "pegsFile", "pgs4formFile", "dataFolder", "outputFolder"}
    with open(os.path.join(workdir, "opt.txt"), "w") as f:
        for k, v in opts.items():
            if k in strings:
                f.write(f"{k}\ts\t{v}\n")
            elif k == "verbose":
                f.write(f"{k}\tb\t{int(bool(v))}\n")
            else:
                vals = v if isinstance(v, (list, tuple)) else [v]
                f.write(f"{k}\td\t" + " ".join(repr(float(x)) for x in vals) + "\n")
    subprocess.run([os.path.join(REF_DIR, "matrad_serial"), workdir], check=True, capture_output=True,
                   timeout=timeout)
    with open(os.path.join(workdir, "dij.bin"), "rb") as f:
        raw = f.read()
    nrows, ncols, nnz = np.frombuffer(raw[:24], dtype=np.int64)
    o = 24
    jc = np.frombuffer(raw[o:o + 8 * (ncols + 1)], dtype=np.int64).copy()
    o += 8 * (ncols + 1)
    ir = np.frombuffer(raw[o:o + 8 * nnz], dtype=np.int64).copy()
    o += 8 * nnz
    pr = np.frombuffer(raw[o:o + 8 * nnz], dtype=np.float64).copy()
    return jc, ir, pr
