"""ctypes binding of the C ABI declared in include/omc_gpu.h.

The shared library ``ompmc_gb300/lib/libompmc_gb300.so`` holds the host
library (input, phantom, tables, regions, source, scoring) and the CUDA
transport engine.  It is built in-tree by :mod:`ompmc_gb300.build`.  There
is no fallback: if the library is missing, importing a symbol raises.
"""

from __future__ import annotations

import ctypes as C
import os
import platform

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", platform.machine(), "libompmc_gb300.so")

MXMED = 9
NAME_LEN = 64
INVDIM = 1000


class OmcError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


class Phantom_t(C.Structure):
    _fields_ = [("nmed", C.c_int), ("med_names", (C.c_char * NAME_LEN) * MXMED),
                ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("xbounds", C.POINTER(C.c_double)), ("ybounds", C.POINTER(C.c_double)),
                ("zbounds", C.POINTER(C.c_double)), ("med_index", C.POINTER(C.c_int)),
                ("density", C.POINTER(C.c_double))]


class Regions_t(C.Structure):
    _fields_ = [("nreg", C.c_int), ("med", C.POINTER(C.c_int)), ("rhof", C.POINTER(C.c_double)),
                ("pcut", C.POINTER(C.c_double)), ("ecut", C.POINTER(C.c_double))]


class Source_t(C.Structure):
    _fields_ = [("spectrum", C.c_int), ("charge", C.c_int), ("energy", C.c_double),
                ("deltak", C.c_double), ("cdfinv1", C.c_double * INVDIM),
                ("cdfinv2", C.c_double * INVDIM), ("ssd", C.c_double),
                ("xinl", C.c_double), ("xinu", C.c_double), ("yinl", C.c_double),
                ("yinu", C.c_double), ("xsize", C.c_double), ("ysize", C.c_double),
                ("ixinl", C.c_int), ("ixinu", C.c_int), ("iyinl", C.c_int), ("iyinu", C.c_int)]


class TablesHead_t(C.Structure):
    """Leading fields of omc_tables (the rest is only used natively)."""
    _fields_ = [("nmed", C.c_int), ("names", (C.c_char * NAME_LEN) * MXMED),
                ("ne", C.c_int * MXMED), ("meke", C.c_int * MXMED),
                ("rho", C.c_double * MXMED), ("rlc", C.c_double * MXMED),
                ("ae", C.c_double * MXMED), ("ap", C.c_double * MXMED),
                ("ue", C.c_double * MXMED), ("up", C.c_double * MXMED),
                ("te", C.c_double * MXMED), ("thmoll", C.c_double * MXMED)]


class RunConfig_t(C.Structure):
    _fields_ = [("nperbatch", C.c_longlong), ("nbatch", C.c_int), ("ixx", C.c_int), ("jxx", C.c_int),
                ("nsplit", C.c_int), ("precision", C.c_int), ("nlanes", C.c_int),
                ("stack_depth", C.c_int), ("serial", C.c_int), ("continue_streams", C.c_int),
                ("schedule", C.c_int), ("inflight", C.c_longlong), ("chunk_events", C.c_int),
                ("drain_per_warp", C.c_int), ("history_stats", C.c_int)]


class RunStats_t(C.Structure):
    _fields_ = [("ensrc", C.c_double), ("transport_ms", C.c_double), ("histories", C.c_longlong),
                ("steps", C.c_longlong), ("max_stack", C.c_int), ("error_flags", C.c_int),
                ("voxel_steps", C.c_longlong), ("deposits", C.c_longlong), ("kernel_ms", C.c_double),
                ("warnings", C.c_int)]


class Beamlets_t(C.Structure):
    _fields_ = [("nbeamlets", C.c_int), ("nbeams", C.c_int), ("ibeam", C.POINTER(C.c_int))] + [
        (n, C.POINTER(C.c_double)) for n in ("xsource", "ysource", "zsource", "xcorner", "ycorner", "zcorner",
                                             "xside1", "yside1", "zside1", "xside2", "yside2", "zside2")]


class Dij_t(C.Structure):
    _fields_ = [("nrows", C.c_int), ("ncols", C.c_int), ("nnz", C.c_longlong),
                ("col_ptr", C.POINTER(C.c_longlong)), ("row_idx", C.POINTER(C.c_int)),
                ("values", C.POINTER(C.c_double)), ("values_f32", C.POINTER(C.c_float))]


class DijConfig_t(C.Structure):
    _fields_ = [("rel_threshold", C.c_double), ("nhist", C.POINTER(C.c_longlong)), ("fp32_values", C.c_int),
                ("tally_bytes", C.c_longlong)]


class MatradGeo_t(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("cube_rho", C.POINTER(C.c_double)),
                ("cube_mat_ix", C.POINTER(C.c_int)), ("nmaterials", C.c_int), ("materials", C.POINTER(C.c_char_p)),
                ("xbounds", C.POINTER(C.c_double)), ("ybounds", C.POINTER(C.c_double)),
                ("zbounds", C.POINTER(C.c_double))]


class MatradOpt_t(C.Structure):
    _fields_ = [("n_histories", C.c_longlong), ("n_batches", C.c_int), ("n_split", C.c_int),
                ("spectrum_file", C.c_char_p), ("mono_energy", C.c_double), ("charge", C.c_int),
                ("global_ecut", C.c_double), ("global_pcut", C.c_double), ("random_seeds", C.c_int * 2),
                ("pegs_file", C.c_char_p), ("pgs4form_file", C.c_char_p), ("data_folder", C.c_char_p),
                ("output_folder", C.c_char_p), ("rel_dose_threshold", C.c_double), ("verbose", C.c_int)]


class ServerConfig_t(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("hbm_budget", C.c_longlong), ("max_jobs", C.c_int),
                ("round_histories", C.c_longlong), ("nsplit", C.c_int), ("ixx", C.c_int), ("jxx", C.c_int),
                ("policy", C.c_int)]


class ServerJob_t(C.Structure):
    _fields_ = [("phantom", C.POINTER(Phantom_t)), ("source", C.POINTER(Source_t)), ("ecut", C.c_double),
                ("pcut", C.c_double), ("nperbatch", C.c_longlong), ("nbatch", C.c_int)]


class ServerResult_t(C.Structure):
    _fields_ = [("ensrc", C.c_double), ("histories", C.c_longlong), ("submit_s", C.c_double),
                ("admit_s", C.c_double), ("finish_s", C.c_double), ("rounds", C.c_int), ("status", C.c_int)]


class ServerStats_t(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("finished", C.c_longlong), ("rounds", C.c_longlong),
                ("histories", C.c_longlong), ("max_resident", C.c_int), ("max_round_jobs", C.c_int),
                ("max_resident_bytes", C.c_longlong), ("transport_s", C.c_double)]


_lib = None


def lib(path: str | None = None):
    """Load (once) and return the native library."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("OMC_LIB", LIB_PATH)
    if not os.path.exists(path):
        raise OmcError(-1, f"native library not built: {path} (run ompmc_gb300.build.build())")
    L = C.CDLL(path)
    vp, pp = C.c_void_p, C.POINTER
    sig = {
        "omc_last_error": ([], C.c_char_p),
        "omc_status_string": ([C.c_int], C.c_char_p),
        "omc_input_parse": ([C.c_char_p, pp(vp)], C.c_int),
        "omc_input_from_string": ([C.c_char_p, pp(vp)], C.c_int),
        "omc_input_get": ([vp, C.c_char_p, C.c_char_p, C.c_size_t], C.c_int),
        "omc_input_free": ([vp], None),
        "omc_phantom_read": ([C.c_char_p, pp(pp(Phantom_t))], C.c_int),
        "omc_phantom_create": ([C.c_int, pp(C.c_char_p), C.c_int, C.c_int, C.c_int, pp(C.c_double),
                                pp(C.c_double), pp(C.c_double), pp(C.c_int), pp(C.c_double),
                                pp(pp(Phantom_t))], C.c_int),
        "omc_phantom_write": ([pp(Phantom_t), C.c_char_p], C.c_int),
        "omc_phantom_free": ([pp(Phantom_t)], None),
        "omc_tables_build": ([vp, C.c_int, vp, pp(vp)], C.c_int),
        "omc_tables_free": ([vp], None),
        "omc_tables_dump": ([vp, C.c_char_p], C.c_int),
        "omc_regions_build": ([vp, pp(Phantom_t), vp, pp(pp(Regions_t))], C.c_int),
        "omc_regions_free": ([pp(Regions_t)], None),
        "omc_source_build": ([vp, pp(Phantom_t), pp(pp(Source_t))], C.c_int),
        "omc_source_free": ([pp(Source_t)], None),
        "omc_accumulate_results": ([pp(Phantom_t), pp(C.c_double), pp(C.c_double), C.c_int, C.c_longlong,
                                    C.c_int, pp(C.c_double), pp(C.c_double)], C.c_int),
        "omc_write_3ddose": ([C.c_char_p, pp(Phantom_t), pp(C.c_double), pp(C.c_double)], C.c_int),
        "omc_engine_create": ([C.c_int, pp(vp)], C.c_int),
        "omc_engine_destroy": ([vp], None),
        "omc_engine_set_tables": ([vp, vp], C.c_int),
        "omc_engine_set_geometry": ([vp, pp(Phantom_t), pp(Regions_t)], C.c_int),
        "omc_engine_set_source": ([vp, pp(Source_t)], C.c_int),
        "omc_engine_run": ([vp, pp(RunConfig_t), pp(C.c_double), pp(C.c_double), pp(RunStats_t)], C.c_int),
        "omc_engine_run_resident": ([vp, pp(RunConfig_t), pp(vp), pp(vp), pp(RunStats_t)], C.c_int),
        "omc_engine_history_sums": ([vp, pp(C.c_double), pp(C.c_double), pp(C.c_longlong), pp(C.c_longlong)],
                                    C.c_int),
        "omc_engine_batch_sums": ([vp, pp(C.c_double), pp(C.c_double), pp(C.c_int)], C.c_int),
        "omc_engine_run_noalloc": ([vp, pp(RunConfig_t), C.c_void_p, C.c_void_p, pp(RunStats_t)], C.c_int),
        "omc_engine_set_beamlets": ([vp, pp(Beamlets_t)], C.c_int),
        "omc_engine_run_dij": ([vp, pp(RunConfig_t), pp(DijConfig_t), pp(pp(Dij_t)), pp(RunStats_t)], C.c_int),
        "omc_dij_free": ([pp(Dij_t)], None),
        "omc_matrad_dij": ([C.c_int, pp(MatradGeo_t), pp(Beamlets_t), pp(MatradOpt_t), C.c_int, C.c_int,
                            pp(pp(Dij_t))], C.c_int),
        "omc_job_device_bytes": ([pp(Phantom_t), C.c_int, C.c_int], C.c_size_t),
        "omc_engine_job_add": ([vp, pp(Phantom_t), pp(Regions_t), pp(Source_t), C.c_longlong, C.c_int, C.c_int,
                                pp(vp)], C.c_int),
        "omc_job_done": ([vp], C.c_longlong),
        "omc_job_histories": ([vp], C.c_longlong),
        "omc_engine_job_round": ([vp, pp(vp), pp(C.c_longlong), C.c_int, pp(RunConfig_t), pp(RunStats_t)],
                                 C.c_int),
        "omc_engine_job_result": ([vp, vp, pp(C.c_double), pp(C.c_double), pp(C.c_double)], C.c_int),
        "omc_engine_job_add_dij": ([vp, pp(Phantom_t), pp(Regions_t), pp(Source_t), pp(Beamlets_t),
                                    pp(C.c_longlong), C.c_longlong, C.c_int, C.c_int, pp(vp)], C.c_int),
        "omc_engine_job_dij": ([vp, vp, C.c_double, C.c_int, pp(pp(Dij_t))], C.c_int),
        "omc_job_dij_device_bytes": ([pp(Phantom_t), C.c_int, C.c_int], C.c_size_t),
        "omc_engine_job_remove": ([vp, vp], None),
        "omc_server_create": ([pp(ServerConfig_t), vp, C.c_int, pp(C.c_char_p), pp(vp)], C.c_int),
        "omc_server_submit": ([vp, pp(ServerJob_t), pp(C.c_longlong)], C.c_int),
        "omc_server_wait": ([vp, C.c_longlong, C.c_double, pp(C.c_double), pp(C.c_double), pp(ServerResult_t)],
                            C.c_int),
        "omc_server_submit_dij": ([vp, pp(ServerJob_t), pp(Beamlets_t), pp(C.c_longlong), C.c_double, C.c_int,
                                   pp(C.c_longlong)], C.c_int),
        "omc_server_wait_dij": ([vp, C.c_longlong, C.c_double, pp(pp(Dij_t)), pp(ServerResult_t)], C.c_int),
        "omc_server_get_stats": ([vp, pp(ServerStats_t)], C.c_int),
        "omc_server_destroy": ([vp], None),
        "omc_server_round_histories": ([C.c_longlong, C.c_longlong, C.c_longlong, C.c_int], C.c_longlong),
        "omc_engine_tune": ([vp, pp(RunConfig_t), C.c_longlong, pp(RunConfig_t), pp(C.c_double)], C.c_int),
        "omc_engine_trace": ([vp, C.c_int], C.c_int),
        "omc_engine_trace_read": ([vp, pp(C.c_longlong), C.c_int, pp(C.c_int)], C.c_int),
        "omc_device_memory": ([C.c_int, pp(C.c_size_t), pp(C.c_size_t)], C.c_int),
        "omc_measure_atomic_rate": ([C.c_int, C.c_longlong, pp(C.c_double)], C.c_int),
        "omc_gpu_ranmar": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_longlong, pp(C.c_int32)], C.c_int),
        "omc_stream_seeds": ([C.c_int, C.c_int, C.c_longlong, pp(C.c_int), pp(C.c_int)], None),
    }
    for name, (args, res) in sig.items():
        if not hasattr(L, name):
            continue
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(status: int):
    if status != 0:
        L = lib()
        raise OmcError(status, L.omc_last_error().decode(errors="replace"))
