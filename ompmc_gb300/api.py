"""Python mirror of the omc_dosxyz front end over the C ABI.

``Problem`` runs the reference's initialisation chain (parseInputFile,
initPhantom, initMediaData, initSource, initRegions, initVrt;
ucodes/omc_dosxyz/omc_dosxyz.c:1155-1179) through the native host library.
``Engine`` is the GPU transport that replaces the batch/history loop
(omc_dosxyz.c:1237-1263).  ``Problem.dose()`` and ``write_3ddose`` are
accumulateResults/outputResults (:719-886).
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _native as N
from ._native import check

FP64, FP32 = 0, 1
AUTO, LANES, WAVEFRONT = 0, 1, 2


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Input:
    def __init__(self, path_without_ext: str | None = None, text: str | None = None):
        L = N.lib()
        self._h = C.c_void_p()
        if text is not None:
            check(L.omc_input_from_string(text.encode(), C.byref(self._h)))
        else:
            check(L.omc_input_parse(path_without_ext.encode(), C.byref(self._h)))

    def get(self, key: str):
        buf = C.create_string_buffer(1024)
        if N.lib().omc_input_get(self._h, key.encode(), buf, 1024):
            return buf.value.decode()
        return None

    def __del__(self):
        if getattr(self, "_h", None):
            N.lib().omc_input_free(self._h)
            self._h = None


class Phantom:
    def __init__(self, ptr):
        self._p = ptr

    @classmethod
    def read(cls, path: str):
        p = C.POINTER(N.Phantom_t)()
        check(N.lib().omc_phantom_read(path.encode(), C.byref(p)))
        return cls(p)

    @classmethod
    def from_arrays(cls, media, xb, yb, zb, med, rho):
        """med: [nz,ny,nx] 1-based medium numbers; rho: densities."""
        med = np.ascontiguousarray(med, dtype=np.int32)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        nz, ny, nx = med.shape
        names = (C.c_char_p * len(media))(*[m.encode() for m in media])
        xb, yb, zb = (np.ascontiguousarray(b, dtype=np.float64) for b in (xb, yb, zb))
        p = C.POINTER(N.Phantom_t)()
        check(N.lib().omc_phantom_create(len(media), names, nx, ny, nz, _dptr(xb), _dptr(yb), _dptr(zb),
                                          med.ctypes.data_as(C.POINTER(C.c_int)), _dptr(rho), C.byref(p)))
        return cls(p)

    @property
    def s(self):
        return self._p.contents

    @property
    def shape(self):
        s = self.s
        return (s.nz, s.ny, s.nx)

    @property
    def nreg(self):
        s = self.s
        return s.nx * s.ny * s.nz + 1

    @property
    def media(self):
        s = self.s
        return [s.med_names[i].value.decode() for i in range(s.nmed)]

    def density(self):
        s = self.s
        return np.ctypeslib.as_array(s.density, shape=(s.nz * s.ny * s.nx,)).reshape(self.shape).copy()

    def write(self, path):
        check(N.lib().omc_phantom_write(self._p, path.encode()))

    def __del__(self):
        if getattr(self, "_p", None):
            N.lib().omc_phantom_free(self._p)
            self._p = None


def build_source(inp: "Input", phantom: "Phantom"):
    """omc_source_build (initSource) alone: POINTER(Source_t), free with
    free_source."""
    src = C.POINTER(N.Source_t)()
    check(N.lib().omc_source_build(inp._h, phantom._p, C.byref(src)))
    return src


def free_source(src):
    N.lib().omc_source_free(src)


class Problem:
    """Host-side state of one dose job, built from a .inp file."""

    def __init__(self, inp: Input, phantom: Phantom | None = None):
        L = N.lib()
        self.input = inp
        if phantom is None:
            path = inp.get("phantom file")
            if path is None:
                raise N.OmcError(3, "Can not find 'phantom file' key on input file.")
            phantom = Phantom.read("".join(path.split()))
        self.phantom = phantom
        ps = phantom.s
        self.tables = C.c_void_p()
        check(L.omc_tables_build(inp._h, ps.nmed, C.cast(C.pointer(ps.med_names), C.c_void_p),
                                 C.byref(self.tables)))
        self.regions = C.POINTER(N.Regions_t)()
        check(L.omc_regions_build(inp._h, phantom._p, self.tables, C.byref(self.regions)))
        self.source = C.POINTER(N.Source_t)()
        check(L.omc_source_build(inp._h, phantom._p, C.byref(self.source)))
        g = lambda k, d: int(inp.get(k)) if inp.get(k) is not None else d
        self.nsplit = g("nsplit", 1)
        ncase, nbatch = g("ncase", 0), g("nbatch", 1)
        if nbatch > 0 and ncase // nbatch == 0:
            ncase = nbatch
        self.nbatch = nbatch
        self.nperbatch = ncase // nbatch if nbatch > 0 else 0
        seeds = (inp.get("rng seeds") or "97 33").split()
        self.seeds = (int(seeds[0]), int(seeds[1]))

    @classmethod
    def from_file(cls, path_without_ext: str):
        return cls(Input(path_without_ext))

    @property
    def nreg(self):
        return self.phantom.nreg

    def tables_head(self):
        return C.cast(self.tables, C.POINTER(N.TablesHead_t)).contents

    def dump_tables(self, path):
        check(N.lib().omc_tables_dump(self.tables, path.encode()))

    def dose(self, accum_endep, accum_endep2, nperbatch=None, nbatch=None, iout=1):
        """Batch mean dose (Gy per history) and relative uncertainty."""
        nperbatch = self.nperbatch if nperbatch is None else nperbatch
        nbatch = self.nbatch if nbatch is None else nbatch
        a = np.ascontiguousarray(accum_endep, dtype=np.float64)
        a2 = np.ascontiguousarray(accum_endep2, dtype=np.float64)
        dose = np.zeros(self.nreg)
        unc = np.zeros(self.nreg)
        check(N.lib().omc_accumulate_results(self.phantom._p, _dptr(a), _dptr(a2), iout, nperbatch, nbatch,
                                             _dptr(dose), _dptr(unc)))
        return dose, unc

    def write_3ddose(self, path, dose, unc):
        check(N.lib().omc_write_3ddose(path.encode(), self.phantom._p, _dptr(dose), _dptr(unc)))

    def __del__(self):
        L = N.lib()
        if getattr(self, "source", None):
            L.omc_source_free(self.source)
            self.source = None
        if getattr(self, "regions", None):
            L.omc_regions_free(self.regions)
            self.regions = None
        if getattr(self, "tables", None):
            L.omc_tables_free(self.tables)
            self.tables = None


class Engine:
    """GB300 transport engine (omc_engine_*)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        check(N.lib().omc_engine_create(device, C.byref(self._h)))
        self._problem = None

    def load(self, problem: Problem):
        L = N.lib()
        check(L.omc_engine_set_tables(self._h, problem.tables))
        self.set_geometry(problem)
        check(L.omc_engine_set_source(self._h, problem.source))
        self._problem = problem
        return self

    def set_geometry(self, problem: Problem):
        check(N.lib().omc_engine_set_geometry(self._h, problem.phantom._p, problem.regions))

    @staticmethod
    def config(nperbatch, nbatch, seeds=(97, 33), nsplit=1, precision=FP64, nlanes=0, stack_depth=0, serial=0,
               continue_streams=0, schedule=AUTO, inflight=0, chunk_events=0, drain_per_warp=0, history_stats=0):
        return N.RunConfig_t(int(nperbatch), int(nbatch), int(seeds[0]), int(seeds[1]), int(nsplit),
                             int(precision), int(nlanes), int(stack_depth), int(serial), int(continue_streams),
                             int(schedule), int(inflight), int(chunk_events), int(drain_per_warp),
                             int(history_stats))

    def run(self, nperbatch=None, nbatch=None, seeds=None, nsplit=None, precision=FP64, nlanes=0,
            stack_depth=0, serial=0, continue_streams=0, schedule=AUTO, inflight=0, chunk_events=0,
            drain_per_warp=0, history_stats=0):
        p = self._problem
        cfg = self.config(p.nperbatch if nperbatch is None else nperbatch, p.nbatch if nbatch is None else nbatch,
                          p.seeds if seeds is None else seeds, p.nsplit if nsplit is None else nsplit,
                          precision, nlanes, stack_depth, serial, continue_streams, schedule, inflight,
                          chunk_events, drain_per_warp, history_stats)
        a = np.zeros(p.nreg)
        a2 = np.zeros(p.nreg)
        st = N.RunStats_t()
        check(N.lib().omc_engine_run(self._h, C.byref(cfg), _dptr(a), _dptr(a2), C.byref(st)))
        return a, a2, st

    def run_resident(self, cfg):
        d1, d2 = C.c_void_p(), C.c_void_p()
        st = N.RunStats_t()
        check(N.lib().omc_engine_run_resident(self._h, C.byref(cfg), C.byref(d1), C.byref(d2), C.byref(st)))
        return d1.value, d2.value, st

    def history_sums(self):
        """(sum, sum2, histories, split) of the last run made with
        history_stats=1 (omc_engine_history_sums)."""
        n = self._problem.nreg
        a, a2 = np.zeros(n), np.zeros(n)
        h, sp = C.c_longlong(), C.c_longlong()
        check(N.lib().omc_engine_history_sums(self._h, _dptr(a), _dptr(a2), C.byref(h), C.byref(sp)))
        return a, a2, h.value, sp.value

    def batch_sums(self, weights):
        """Per-batch weighted sums of the last run's batch tallies
        (omc_engine_batch_sums): out[b] = sum_r weights[r] * E_b[r]."""
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if w.shape != (self._problem.nreg,):
            raise ValueError(f"weights must have {self._problem.nreg} entries")
        out = np.zeros(65536)
        nb = C.c_int()
        check(N.lib().omc_engine_batch_sums(self._h, _dptr(w), _dptr(out), C.byref(nb)))
        return out[:nb.value].copy()

    def set_beamlets(self, beamlets):
        """Upload a :class:`ompmc_gb300.workloads.Beamlets` set (the
        matRad mcSrc fields)."""
        st, keep = _beamlets_t(beamlets)
        check(N.lib().omc_engine_set_beamlets(self._h, C.byref(st)))
        self._beamlets = beamlets
        return self

    def run_dij(self, rel_threshold=1e-4, nhist=None, nperbatch=None, nbatch=None, seeds=None, nsplit=None,
                precision=FP64, serial=0, schedule=AUTO, fp32_values=False, tally_bytes=0, nlanes=0,
                continue_streams=0):
        """Dose-influence matrix of the uploaded beamlets; returns
        (col_ptr, row_idx, values, stats) with values per history
        (omc_engine_run_dij)."""
        p = self._problem
        cfg = self.config(p.nperbatch if nperbatch is None else nperbatch, p.nbatch if nbatch is None else nbatch,
                          p.seeds if seeds is None else seeds, p.nsplit if nsplit is None else nsplit,
                          precision, nlanes, 0, serial, continue_streams, schedule, 0)
        nh = None
        if nhist is not None:
            nh = np.ascontiguousarray(nhist, dtype=np.int64)
        dc = N.DijConfig_t(float(rel_threshold), nh.ctypes.data_as(C.POINTER(C.c_longlong)) if nh is not None
                           else None, 1 if fp32_values else 0, int(tally_bytes))
        out = C.POINTER(N.Dij_t)()
        st = N.RunStats_t()
        check(N.lib().omc_engine_run_dij(self._h, C.byref(cfg), C.byref(dc), C.byref(out), C.byref(st)))
        col_ptr, rows, vals = _take_dij(out, fp32_values)
        return col_ptr, rows, vals, st

    def tune(self, precision=FP32, sample_histories=2_000_000, nsplit=None, seeds=None):
        """omc_engine_tune: (inflight, chunk_events, rates of the 8
        candidates) fastest for the loaded geometry and source."""
        p = self._problem
        cfg = self.config(2, 2, p.seeds if seeds is None else seeds, p.nsplit if nsplit is None else nsplit,
                          precision)
        best = N.RunConfig_t()
        rates = (C.c_double * 8)()
        check(N.lib().omc_engine_tune(self._h, C.byref(cfg), int(sample_histories), C.byref(best), rates))
        return int(best.inflight), int(best.chunk_events), list(rates)

    def trace(self, iterations):
        """Record per-iteration device time and queue sizes of the next
        wavefront launches (0 = off)."""
        check(N.lib().omc_engine_trace(self._h, int(iterations)))

    def trace_read(self, cap=1 << 16):
        """[n, 4] int64: ns, photons, electrons, histories injected, per
        iteration of the last wavefront launch."""
        out = np.zeros((cap, 4), np.int64)
        n = C.c_int()
        check(N.lib().omc_engine_trace_read(self._h, out.ctypes.data_as(C.POINTER(C.c_longlong)), cap, C.byref(n)))
        return out[:n.value]

    def close(self):
        if getattr(self, "_h", None):
            N.lib().omc_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Server:
    """Dose server (omc_server_*): continuous batching of dose jobs on one
    GPU.  `media` are the server's pegs4 media; `data_text` is .inp text
    with the "pegs file", "pgs4form file" and "data folder" keys."""

    SHORTEST_FIRST, EQUAL_SHARES = 0, 1

    def __init__(self, media, data_text, precision=FP32, hbm_budget=0, max_jobs=0, round_histories=0, nsplit=1,
                 seeds=(97, 33), device=0, policy=0):
        self._inp = Input(text=data_text)
        cfg = N.ServerConfig_t(device, precision, int(hbm_budget), int(max_jobs), int(round_histories),
                               int(nsplit), int(seeds[0]), int(seeds[1]), int(policy))
        names = (C.c_char_p * len(media))(*[m.encode() for m in media])
        self._h = C.c_void_p()
        check(N.lib().omc_server_create(C.byref(cfg), self._inp._h, len(media), names, C.byref(self._h)))
        self._nreg = {}  # field jobs: regions
        self._dij = {}  # beamlet jobs: FP32 values

    def submit(self, phantom, source, ecut, pcut, nperbatch, nbatch):
        """phantom: :class:`Phantom`; source: a POINTER(Source_t) (e.g.
        Problem.source).  Returns the job id."""
        job = N.ServerJob_t(phantom._p, source, float(ecut), float(pcut), int(nperbatch), int(nbatch))
        jid = C.c_longlong()
        check(N.lib().omc_server_submit(self._h, C.byref(job), C.byref(jid)))
        self._nreg[jid.value] = phantom.nreg
        return jid.value

    def submit_problem(self, prob, nperbatch=None, nbatch=None):
        g = lambda k: float(prob.input.get(k))
        return self.submit(prob.phantom, prob.source, g("global ecut"), g("global pcut"),
                           prob.nperbatch if nperbatch is None else nperbatch,
                           prob.nbatch if nbatch is None else nbatch)

    def submit_dij(self, phantom, source, ecut, pcut, beamlets, nperbatch, nbatch, nhist=None, rel_threshold=1e-4,
                   fp32_values=False):
        """A beamlet job (omc_server_submit_dij): the dose-influence matrix of
        `beamlets` (:class:`ompmc_gb300.workloads.Beamlets`) on `phantom`,
        nhist[i] histories for beamlet i (default nperbatch * nbatch each).
        Returns the job id; collect it with :meth:`wait_dij`."""
        job = N.ServerJob_t(phantom._p, source, float(ecut), float(pcut), int(nperbatch), int(nbatch))
        bl, keep = _beamlets_t(beamlets)
        nh = None if nhist is None else np.ascontiguousarray(nhist, dtype=np.int64)
        jid = C.c_longlong()
        check(N.lib().omc_server_submit_dij(self._h, C.byref(job), C.byref(bl),
                                            None if nh is None else nh.ctypes.data_as(C.POINTER(C.c_longlong)),
                                            float(rel_threshold), 1 if fp32_values else 0, C.byref(jid)))
        del keep
        self._dij[jid.value] = bool(fp32_values)
        return jid.value

    def wait_dij(self, jid, timeout=-1.0):
        """(col_ptr, row_idx, values, ServerResult_t) of a beamlet job."""
        fp32 = self._dij.get(jid, False)
        out = C.POINTER(N.Dij_t)()
        r = N.ServerResult_t()
        check(N.lib().omc_server_wait_dij(self._h, jid, float(timeout), C.byref(out), C.byref(r)))
        del self._dij[jid]
        return (*_take_dij(out, fp32), r)

    def wait(self, jid, timeout=-1.0):
        """(accum_endep, accum_endep2, ServerResult_t) of a finished job."""
        nreg = self._nreg.get(jid, 0)  # 0: not a field job of this wrapper; the library says why
        a = np.zeros(nreg)
        a2 = np.zeros(nreg)
        r = N.ServerResult_t()
        check(N.lib().omc_server_wait(self._h, jid, float(timeout), _dptr(a) if nreg else None,
                                      _dptr(a2) if nreg else None, C.byref(r)))
        del self._nreg[jid]
        return a, a2, r

    def stats(self):
        st = N.ServerStats_t()
        check(N.lib().omc_server_get_stats(self._h, C.byref(st)))
        return st

    def close(self):
        if getattr(self, "_h", None):
            N.lib().omc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def _beamlets_t(b):
    keep = [np.ascontiguousarray(b.ibeam, dtype=np.int32)]
    cols = []
    for arr in (b.source[:, 0], b.source[:, 1], b.source[:, 2], b.corner[:, 0], b.corner[:, 1], b.corner[:, 2],
                b.side1[:, 0], b.side1[:, 1], b.side1[:, 2], b.side2[:, 0], b.side2[:, 1], b.side2[:, 2]):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        keep.append(a)
        cols.append(_dptr(a))
    return N.Beamlets_t(len(b.ibeam), len(b.source), keep[0].ctypes.data_as(C.POINTER(C.c_int)), *cols), keep


def _take_dij(out, fp32=False):
    try:
        d = out.contents
        col = np.ctypeslib.as_array(d.col_ptr, shape=(d.ncols + 1,)).copy()
        if d.nnz:
            rows = np.ctypeslib.as_array(d.row_idx, shape=(d.nnz,)).copy()
            vals = np.ctypeslib.as_array(d.values_f32 if fp32 else d.values, shape=(d.nnz,)).copy()
        else:
            rows, vals = np.zeros(0, np.int32), np.zeros(0, np.float32 if fp32 else np.float64)
    finally:
        N.lib().omc_dij_free(out)
    return col, rows, vals


def matrad_dij(phantom, beamlets, opts, precision=FP64, serial=0, device=0):
    """omc_matrad_dij: matRad's five inputs (cube from a
    :class:`ompmc_gb300.workloads.Phantom`, mcSrc from a
    :class:`ompmc_gb300.workloads.Beamlets`, mcOpt fields as a dict with
    matRad's names) in, (col_ptr, row_idx, values) out."""
    nz, ny, nx = phantom.shape
    rho = np.ascontiguousarray(phantom.rho, dtype=np.float64)
    mix = np.ascontiguousarray(phantom.med, dtype=np.int32)
    names = (C.c_char_p * len(phantom.media))(*[m.encode() for m in phantom.media])
    xb, yb, zb = (np.ascontiguousarray(b, dtype=np.float64) for b in (phantom.xb, phantom.yb, phantom.zb))
    geo = N.MatradGeo_t(nx, ny, nz, _dptr(rho), mix.ctypes.data_as(C.POINTER(C.c_int)), len(phantom.media), names,
                        _dptr(xb), _dptr(yb), _dptr(zb))
    enc = lambda k: opts[k].encode() if opts.get(k) else None
    seeds = (C.c_int * 2)(*[int(x) for x in opts.get("randomSeeds", (97, 33))])
    opt = N.MatradOpt_t(int(opts["nHistories"]), int(opts["nBatches"]), int(opts.get("nSplit", 1)),
                        enc("spectrumFile"), float(opts.get("monoEnergy", 0.0)), int(opts.get("charge", 0)),
                        float(opts["global_ecut"]), float(opts["global_pcut"]), seeds, enc("pegsFile"),
                        enc("pgs4formFile"), enc("dataFolder"), enc("outputFolder"),
                        float(opts["relDoseThreshold"]), int(bool(opts.get("verbose", 0))))
    bl, keep = _beamlets_t(beamlets)
    out = C.POINTER(N.Dij_t)()
    check(N.lib().omc_matrad_dij(device, C.byref(geo), C.byref(bl), C.byref(opt), precision, serial,
                                 C.byref(out)))
    del keep
    return _take_dij(out)


def gpu_ranmar(ixx, jxx, nstreams, n, device=0):
    out = np.zeros((nstreams, n), dtype=np.int32)
    check(N.lib().omc_gpu_ranmar(device, ixx, jxx, nstreams, n, out.ctypes.data_as(C.POINTER(C.c_int32))))
    return out


def atomic_rate(nreg, device=0):
    """Scattered FP64 atomicAdd throughput over nreg doubles (atomics/s,
    omc_measure_atomic_rate)."""
    r = C.c_double()
    check(N.lib().omc_measure_atomic_rate(device, int(nreg), C.byref(r)))
    return r.value


def stream_seeds(ixx, jxx, k):
    a, b = C.c_int(), C.c_int()
    N.lib().omc_stream_seeds(ixx, jxx, k, C.byref(a), C.byref(b))
    return a.value, b.value
