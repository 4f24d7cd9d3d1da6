"""Benchmark of the GB300 transport on the 6 MV heterogeneous slab.

Workload (one "step" = one statistical batch of HISTORIES_PER_STEP
histories): the 150^3 slab phantom at 2 mm voxels (water 0-5 cm, lung
0.26 g/cm^3 5-15 cm, ICRP bone 1.85 g/cm^3 15-18 cm, water 18-30 cm), the
synthetic 24-bin 6 MV spectrum, a 10x10 cm^2 field from a point source at
SSD 100 cm, ECUT 0.700 / PCUT 0.010 MeV, 700icru media.  Ten steps are the
1e8-history job of that configuration.

Prints one JSON line: FP32-transport (FP64 tallies) histories/s as
`value`, the plain FP64 path beside it, the statistical efficiency
1/(s^2 T), the end-to-end rate through the C ABI with host buffers, the
roofline of the transport kernel, the CPU baseline (the oracle port on all
host cores) and the SM clocks seen during the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "6MV heterogeneous slab 150^3 @ 2 mm, 10x10 cm2 field, SSD 100 cm"
HISTORIES_PER_STEP = 10_000_000
FP64_HISTORIES = 20_000_000  # FP64 job: enough histories for the FP32 dose-error statement
NSPLIT16_HISTORIES = 10_000_000
LANES_PER_RANK_STRIDE = 1 << 21  # stream-index stride between ranks (> lanes of one GPU)
L2_FLUSH_BYTES = 256 << 20       # larger than the 129 MB L2


def build_problem(tmp):
    from ompmc_gb300 import api, data
    from ompmc_gb300 import workloads as W

    data.stage()
    P = data.paths()
    ph = W.slab(n=150, vox=0.2)
    phantom = api.Phantom.from_arrays(ph.media, ph.xb, ph.yb, ph.zb, ph.med, ph.rho)
    spec = W.write_spectrum(os.path.join(tmp, "6mv.spectrum"), "synthetic 6 MV", *W.spectrum_6mv())
    job = W.Job("(in memory)", P["pegs"], P["pgs4form"], P["data_folder"], tmp + os.sep, spectrum_file=spec,
                ncase=10 * HISTORIES_PER_STEP, nbatch=10, collimator=(-5.0, 5.0, -5.0, 5.0), ssd=100.0)
    return api.Problem(api.Input(text=job.text()), phantom=phantom)


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10:
                continue
            try:
                util = float(f[4])
                if util < 50:
                    continue
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[6:10]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per history of the transport kernel from the committed
    ncu summary (profiles/), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "wavefront_fp32_slab150.json")) as f:
            return float(json.load(f)["dram_bytes_per_history"])
    except (OSError, KeyError, ValueError):
        return None


def dose_factor(prob):
    """Per voxel in region order (region 0 left out), the dose that
    accumulateResults (omc_dosxyz.c:739-799) gives for a batch mean energy of
    1 MeV: 1.602e-10/(rho V N), and 0 where rho < 0.044.  Energy times it is
    the dose up to one constant, which is all that a "% of Dmax" selection
    needs; computed by the library's own accumulateResults."""
    n = prob.nreg
    d, _ = prob.dose(np.full(n, 2.0), np.full(n, 2.0), nperbatch=1, nbatch=2)
    return d[1:]


def max_rel_sigma(acc, acc2, nb, factor, frac=0.5):
    """max over voxels with dose > frac*Dmax of the batch relative
    uncertainty (accumulateResults, omc_dosxyz.c:739-751); `factor` is
    dose_factor(problem), so the selection is on dose, not energy."""
    m = acc[1:] / nb
    m2 = acc2[1:] / nb
    d = m * factor
    sel = d > frac * d.max()
    s = np.sqrt(np.maximum(m2[sel] - m[sel] ** 2, 0.0) / (nb - 1)) / m[sel]
    return float(s.max())


def cpu_oracle_sample(prob, target_seconds=8.0, cap=5_000_000):
    """The oracle port on every host core, on a sample of the workload sized
    to about target_seconds of wall time."""
    from oracle import binding as oracle

    oracle.build()
    probe = 20000
    _, _, r = oracle.run(prob, nperbatch=probe // 2, nbatch=2, nthreads=0)
    rate = probe / max(r.seconds, 1e-6)
    n = int(min(cap, max(probe, rate * target_seconds)))
    n -= n % 2
    _, _, r = oracle.run(prob, nperbatch=n // 2, nbatch=2, nthreads=0)
    return n / r.seconds, r.nthreads, n, r.seconds


REF_EXE = os.path.join(ROOT, "oracle", "_ref", os.uname().machine, "omc_dosxyz_omp")


def reference_sample(exe, tmp, phant, spec, n):
    """One run of the reference's own OpenMP build (omc_dosxyz, unmodified)
    on n histories of the workload in 2 batches; returns (transport seconds,
    threads).  The transport time is the difference of the two "Execution
    time up to this point" lines the reference prints before and after its
    batch loop (omc_dosxyz.c:1232-1267): table set-up, phantom parsing and
    the .3ddose output are outside it."""
    from ompmc_gb300 import data
    from ompmc_gb300 import workloads as W

    P = data.paths()
    job = W.Job(phant, P["pegs"], P["pgs4form"], P["data_folder"], tmp + os.sep, spectrum_file=spec, ncase=n,
                nbatch=2, collimator=(-5.0, 5.0, -5.0, 5.0), ssd=100.0)
    inp = job.write(os.path.join(tmp, "ref_job"))
    out = subprocess.run([exe, "-i", inp, "-o", "ref_job"], capture_output=True, text=True, timeout=600, cwd=tmp)
    if out.returncode != 0:
        raise RuntimeError(f"reference exited with {out.returncode}: {out.stdout[-500:]}")
    times = [float(ln.split(":")[1].split()[0]) for ln in out.stdout.splitlines()
             if ln.startswith("Execution time up to this point")]
    threads = [int(ln.split(":")[1]) for ln in out.stdout.splitlines() if ln.startswith("Number of OpenMP threads")]
    if len(times) < 2:
        raise RuntimeError("reference output without its timing lines")
    return times[1] - times[0], (threads[0] if threads else os.cpu_count())


def cpu_baseline_sample(prob, tmp, target_seconds=6.0):
    """The reference's CPU path on every host core, on a bounded sample of
    the workload: its own OpenMP build when it was built on this host, else
    the oracle port."""
    if os.path.exists(REF_EXE):
        from ompmc_gb300 import workloads as W

        phant = W.write_egsphant(W.slab(n=150, vox=0.2), os.path.join(tmp, "slab150_ref.egsphant"))
        spec = W.write_spectrum(os.path.join(tmp, "6mv_ref.spectrum"), "synthetic 6 MV", *W.spectrum_6mv())
        probe = 200_000
        secs, cores = reference_sample(REF_EXE, tmp, phant, spec, probe)
        n = int(min(20_000_000, max(probe, probe / max(secs, 1e-3) * target_seconds)))
        n -= n % 2
        secs, cores = reference_sample(REF_EXE, tmp, phant, spec, n)
        return {"value": n / secs, "unit": "histories/s", "cores": cores, "kind": "reference",
                "sample": f"{n} histories of the workload in 2 batches, the reference's own omc_dosxyz (OpenMP), "
                          f"{secs:.1f} s of transport"}
    rate, cores, n, secs = cpu_oracle_sample(prob, target_seconds)
    return {"value": rate, "unit": "histories/s", "cores": cores, "kind": "port",
            "sample": f"{n} histories of the workload (oracle port, OpenMP dynamic schedule), {secs:.1f} s"}


def run_reference_arm(args, rank):
    """The reference's CPU path on this host's cores: its own OpenMP build
    (oracle/_ref/<arch>/omc_dosxyz_omp, compiled by build() from the
    reference's sources), else the oracle port when that build is absent."""
    if rank != 0:
        return
    from ompmc_gb300 import data
    from ompmc_gb300 import workloads as W

    with tempfile.TemporaryDirectory() as tmp:
        data.stage()
        if os.path.exists(REF_EXE):
            ph = W.slab(n=150, vox=0.2)
            phant = W.write_egsphant(ph, os.path.join(tmp, "slab150.egsphant"))
            spec = W.write_spectrum(os.path.join(tmp, "6mv.spectrum"), "synthetic 6 MV", *W.spectrum_6mv())
            probe = 200_000
            secs, cores = reference_sample(REF_EXE, tmp, phant, spec, probe)
            n = int(min(20_000_000, max(probe, probe / max(secs, 1e-3) * 4.0)))
            n -= n % 2
            rates = []
            for step in range(args.warmup + args.steps):
                secs, cores = reference_sample(REF_EXE, tmp, phant, spec, n)
                if step >= args.warmup:
                    rates.append((n, secs))
            kind = "reference"
            note = ("the reference's own omc_dosxyz, unmodified, built from its sources with -O2 -fopenmp "
                    "(-fcommon) on this host; transport loop time from its own timing lines")
        else:
            prob = build_problem(tmp)
            rates, cores, n = [], 0, 0
            for step in range(args.warmup + args.steps):
                rate, cores, n, secs = cpu_oracle_sample(prob, target_seconds=4.0)
                if step >= args.warmup:
                    rates.append((n, secs))
            kind = "port"
            note = ("oracle port (C restatement of the reference, OpenMP, dynamic schedule, bit-exact with the "
                    "reference's serial build): the reference's own build is absent on this host")
        tot_n = sum(r[0] for r in rates)
        tot_s = sum(r[1] for r in rates)
        value = tot_n / tot_s
        line = {
            "impl": "reference", "metric": "histories/s", "value": value, "unit": "histories/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tot_s / len(rates), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "histories_per_step": n, "note": note},
            "cpu_baseline": {"value": value, "unit": "histories/s", "cores": cores, "kind": kind,
                             "sample": f"{n} histories per step of the workload, 2 batches"},
            "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)


def batch_ratio(a, b):
    """Relative difference of the batch means of a and b (per-batch values
    of two runs with the same histories per batch), and its standard error
    from the spread of the batches of each run."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    ma, mb = a.mean(), b.mean()
    va = a.var(ddof=1) / (len(a) * ma * ma)
    vb = b.var(ddof=1) / (len(b) * mb * mb)
    return float(ma / mb - 1.0), float((ma / mb) * np.sqrt(va + vb))


def fp32_dose_error(a32, b32, H32, K32, roi32, tot32, a64, b64, H64, K64, roi64, tot64, f, sel20):
    """FP32-transport dose error against the FP64 run: voxels above 20% of
    Dmax within 2 combined sigma (batch sigma per voxel; the Welch t mapped
    to a normal z), mean dose over the voxels above 50% of Dmax and total energy
    deposited in the phantom, each as a relative difference per history
    with its standard error from the batch spread of both runs."""
    from scipy import stats as S

    m32, m64 = a32[1:] / (K32 * H32), a64[1:] / (K64 * H64)  # energy per history
    v32 = np.maximum(b32[1:] / K32 / H32 ** 2 - m32 ** 2, 0) / (K32 - 1)
    v64 = np.maximum(b64[1:] / K64 / H64 ** 2 - m64 ** 2, 0) / (K64 - 1)
    va, vb = v32[sel20], v64[sel20]
    ok = (va + vb) > 0
    va, vb = va[ok], vb[ok]
    sig = np.sqrt(va + vb)
    t = (m32[sel20][ok] - m64[sel20][ok]) / sig
    # Welch-Satterthwaite degrees of freedom per voxel: the two runs have
    # different history counts, so their batch variances differ.
    dof = (va + vb) ** 2 / (va ** 2 / (K32 - 1) + vb ** 2 / (K64 - 1))
    z = S.norm.ppf(np.clip(S.t.cdf(t, dof), 1e-300, 1 - 1e-16))
    roi_d, roi_s = batch_ratio(np.asarray(roi32) / H32, np.asarray(roi64) / H64)
    tot_d, tot_s = batch_ratio(np.asarray(tot32) / H32, np.asarray(tot64) / H64)
    return {"voxels_above_20pct": int(sel20.sum()), "frac_within_2sigma": float(np.mean(np.abs(z) <= 2.0)),
            "mean_z2": float(np.mean(z * z)),
            "dose_rel_diff_above_50pct": roi_d, "dose_rel_diff_sigma": roi_s,
            "total_energy_rel_diff": tot_d, "total_energy_rel_diff_sigma": tot_s,
            "histories": {"fp32": K32 * H32, "fp64": K64 * H64}, "batches": {"fp32": K32, "fp64": K64},
            "sigma": "batch spread of the per-batch region sums of each run, so voxel correlations are included"}


def rel_sigmas(acc, acc2, nb, sel):
    m = acc[1:] / nb
    m2 = acc2[1:] / nb
    return np.sqrt(np.maximum(m2[sel] - m[sel] ** 2, 0.0) / (nb - 1)) / m[sel]


SERVE_SHORT = dict(jobs=16, rate=2.0, max_histories=2e7, beamlet_frac=0.25, seed=5)


def run_ours(args, rank, world, local_rank, dist_on):
    import torch

    from ompmc_gb300 import api
    from ompmc_gb300 import dist as D

    torch.cuda.set_device(local_rank)
    flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local_rank}")

    def flush_l2():
        flush_buf.zero_()
        torch.cuda.synchronize()

    def barrier():
        if dist_on:
            import torch.distributed as tdist

            tdist.barrier()
        torch.cuda.synchronize()

    with tempfile.TemporaryDirectory() as tmp:
        prob = build_problem(tmp)
        eng = api.Engine(local_rank).load(prob)
        seeds = D.rank_seeds(97, 33, rank, LANES_PER_RANK_STRIDE)
        H = args.histories_per_step
        K = args.steps
        f = dose_factor(prob)
        cfg32 = api.Engine.config(H, 1, seeds=seeds, precision=api.FP32, inflight=args.inflight)
        # warm-up: single batches of the same size; the last one (host
        # tallies) also fixes the voxels the dose-error statement uses, so
        # that they are not selected on the runs they compare
        for _ in range(args.warmup - 1):
            flush_l2()
            eng.run_resident(cfg32)  # seeds the streams the timed job continues
        sel_acc, _, _ = eng.run(nperbatch=H, nbatch=1, seeds=seeds, precision=api.FP32, continue_streams=1,
                                inflight=args.inflight)
        dsel = sel_acc[1:] * f
        sel20 = dsel > 0.2 * dsel.max()
        sel50 = dsel > 0.5 * dsel.max()
        w_roi = np.concatenate([[0.0], np.where(sel50, f, 0.0)])
        w_in = np.concatenate([[0.0], np.ones(prob.nreg - 1)])
        # timed region: the K-batch job of K*H histories, FP32 transport /
        # FP64 tallies.  The engine transports all batches of a job in one
        # launch (batch tallies side by side, > L2), so a step is one of its
        # batches.
        sampler = ClockSampler(local_rank)
        flush_l2()
        barrier()
        sampler.start()
        acc, acc2, st = eng.run(nperbatch=H, nbatch=K, seeds=seeds, precision=api.FP32, continue_streams=1,
                                inflight=args.inflight)
        barrier()
        clocks = sampler.stop()
        if st.error_flags:
            raise RuntimeError(f"device error flags {st.error_flags:#x}")
        roi32, tot32 = eng.batch_sums(w_roi), eng.batch_sums(w_in)
        dev_ms = float(st.kernel_ms)
        geo, dep, evs = st.voxel_steps, st.deposits, st.steps
        launches = 2  # wavefront transport of all batches, batch accumulation (streams continue: no seeding)
        if dist_on:
            import torch.distributed as tdist

            t = torch.tensor([dev_ms], dtype=torch.float64, device=f"cuda:{local_rank}")
            tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
            dev_ms = float(t.item())
        total_hist = world * K * H
        value = total_hist / (dev_ms / 1000.0)
        T = dev_ms / 1000.0
        s_all = rel_sigmas(acc, acc2, K, sel50) if K >= 2 else None
        s = float(s_all.max()) if s_all is not None else None
        efficiency = 1.0 / (s * s * T) if s else None
        # plain FP64 path, same workload and job structure; enough histories
        # for the FP32 dose-error statement below
        K64 = 10
        H64 = args.fp64_histories // K64
        eng.run(nperbatch=H64 // 8, nbatch=2, seeds=D.rank_seeds(1201, 77, rank, LANES_PER_RANK_STRIDE),
                precision=api.FP64)
        flush_l2()
        a64, b64, st64 = eng.run(nperbatch=H64, nbatch=K64, precision=api.FP64, continue_streams=1)
        roi64, tot64 = eng.batch_sums(w_roi), eng.batch_sums(w_in)
        fp64_value = H64 * K64 / (st64.kernel_ms / 1000.0)
        dose_err = fp32_dose_error(acc, acc2, H, K, roi32, tot32, a64, b64, H64, K64, roi64, tot64, f, sel20)
        # time to 1% in the voxels above 50% of Dmax: nsplit 1 (the job
        # above) and nsplit 16 (the best splitting number measured)
        K16, H16 = 10, args.nsplit16_histories // 10
        a16, b16, st16 = eng.run(nperbatch=H16, nbatch=K16, nsplit=16, precision=api.FP32,
                                 seeds=D.rank_seeds(2207, 91, rank, LANES_PER_RANK_STRIDE))
        T16 = st16.kernel_ms / 1000.0
        s16 = rel_sigmas(a16, b16, K16, sel50)
        s_mean = float(s_all.mean()) if s_all is not None else None
        t1 = {"unit": "s", "target": 0.01, "region": "voxels above 50% of Dmax (dose)",
              "nsplit1": {"histories": K * H, "T_s": T, "s_max": s, "s_mean": s_mean,
                          "by_max_s": T * (s / 0.01) ** 2 if s else None,
                          "by_mean_s": T * (s_mean / 0.01) ** 2 if s_mean else None},
              "nsplit16": {"histories": K16 * H16, "T_s": T16, "histories_per_s": K16 * H16 / T16,
                           "s_max": float(s16.max()), "s_mean": float(s16.mean()),
                           "by_max_s": T16 * (float(s16.max()) / 0.01) ** 2,
                           "by_mean_s": T16 * (float(s16.mean()) / 0.01) ** 2},
              "note": "T x (s/0.01)^2: s falls as 1/sqrt(histories); batch sigma (10 batches)"}
        # the same workload with history-by-history scoring: s by history
        # beside s by batch, over the same voxels
        Hh = args.hbh_histories
        ah, ah2, sth = eng.run(nperbatch=Hh // 10, nbatch=10, precision=api.FP32, history_stats=1,
                               seeds=D.rank_seeds(3307, 51, rank, LANES_PER_RANK_STRIDE))
        hs, hs2, h_merged, h_split = eng.history_sums()
        Th = sth.kernel_ms / 1000.0
        mh = hs[1:] / Hh
        rel_h = np.sqrt(np.maximum(hs2[1:] / Hh - mh * mh, 0.0) / (Hh - 1))[sel50] / mh[sel50]
        rel_b = rel_sigmas(ah, ah2, 10, sel50)
        hbh = {"histories": Hh, "T_s": Th, "histories_per_s": Hh / Th, "merged": h_merged, "split": h_split,
               "error_flags": int(sth.error_flags),
               "s_max": float(rel_h.max()), "s_mean": float(rel_h.mean()),
               "s_max_batch": float(rel_b.max()), "s_mean_batch": float(rel_b.mean()),
               "time_to_1pct_by_max_s": Th * (float(rel_h.max()) / 0.01) ** 2,
               "time_to_1pct_by_mean_s": Th * (float(rel_h.mean()) / 0.01) ** 2,
               "note": "history-by-history sums of x and x^2 per voxel (omc_engine_history_sums) on a run of its "
                       "own; s = relative sigma of the mean over the voxels above 50% of Dmax; the time to 1% "
                       "is that run's time scaled by (s/0.01)^2"}
        # end to end through the C ABI: phantom upload, the K-batch job,
        # batch sums back in host memory
        ph = prob.phantom
        regs = prob.regions
        h2d = prob.nreg * (1 + 4 + 8) + 8 * (sum(ph.shape) + 3) * 2
        d2h = 2 * prob.nreg * 8
        barrier()
        t0 = time.perf_counter()
        eng.set_geometry(prob)
        a, a2, st_e2e = eng.run(nperbatch=H, nbatch=K, seeds=seeds, precision=api.FP32)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        e2e_value = world * K * H / e2e_s
        # roofline of the transport kernel
        peak, peak_kind = measured_peaks()
        per_hist_bytes = (8.0 * geo + 8.0 * dep) / (K * H) + 16.0
        launch_s = dev_ms / 1000.0
        achieved = per_hist_bytes * K * H / launch_s / 1e9
        traffic_ph = profiled_traffic()
        # denominator of the tally atomics: scattered FP64 atomicAdd over
        # one batch tally (measured here, after the timed region)
        atomic_peak = api.atomic_rate(prob.nreg)
        eng.close()
        del regs
        line = None
        if rank == 0:
            serving = None
            if world == 1 and not args.no_serving:
                serving = run_serve_short(local_rank)
            cpu = None
            if world == 1 and not args.no_cpu_baseline:
                cpu = cpu_baseline_sample(prob, tmp)
            line = {
                "metric": "histories/s", "value": value, "unit": "histories/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": WORKLOAD, "histories_per_step": H, "global_histories": total_hist,
                           "transport": "FP32 arithmetic, FP64 tallies and energy balance",
                           "job": f"{K} batches of {H} histories in one launch (batches injected back to back)",
                           "l2": "flushed before the timed job (256 MB write); the job's batch tallies "
                                 f"({K * prob.nreg * 8 / 1e6:.0f} MB) exceed L2",
                           "parallelism": f"replicas x{world}"},
                "fp64": {"value": fp64_value, "unit": "histories/s", "histories": H64 * K64,
                         "job": f"{K64} batches of {H64} histories in one launch"},
                "fp32_over_fp64": value / world / fp64_value,
                "fp32_dose_error": dose_err,
                "efficiency": {"value": efficiency, "unit": "1/(s^2*T)", "s_max_rel_above_50pct": s,
                               "T_s": T},
                "time_to_1pct": t1,
                "history_by_history": hbh,
                "serving": serving,
                "job_ms": dev_ms,
                "per_history": {"events": evs / (K * H), "voxel_steps": geo / (K * H),
                                "deposits": dep / (K * H), "algorithmic_bytes": per_hist_bytes},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": peak_kind,
                             "traffic": (traffic_ph * K * H) if traffic_ph else None,
                             "kernel": "wavefront_kernel<float>",
                             "atomics_per_s": dep / (dev_ms / 1000.0),
                             "atomics": {"achieved": dep / (dev_ms / 1000.0), "peak": atomic_peak,
                                         "unit": "FP64 atomicAdd/s", "frac": dep / (dev_ms / 1000.0) / atomic_peak,
                                         "peak_kind": "measured live: scattered FP64 atomicAdd over one batch "
                                                      f"tally ({prob.nreg} doubles)"}},
                "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": "histories/s", "h2d_bytes_per_step": int(h2d // K),
                        "d2h_bytes_per_step": int(d2h // K),
                        "note": f"one job of {K} steps: the phantom ({int(h2d)} B) goes up and the batch sums "
                                f"({int(d2h)} B) come back once per job, shown here per step; the tables "
                                "(per medium set, resident across jobs) are uploaded before the timed region"},
                "gpu_launches": launches,
                "clocks": clocks,
            }
        return line


DIJ_WORKLOAD = ("matRad-style dij: CT-like blob phantom 256x256x128 @ 2 mm, 7 gantry angles x 5 mm beamlets "
                "within 3.5 cm of the axis, synthetic 6 MV, lognormal histories/beamlet (median 5e4, "
                "sigma_ln 1.0, clipped [1e4, 1e6])")


def run_dij_leg(args, local_rank):
    """One batched dij job (every beamlet in one persistent launch per tally
    group) on the CT-like phantom; histories/s of the transport and the
    wall time of the whole call (transport, device compaction into CSC,
    copy to host)."""
    import torch

    from ompmc_gb300 import api, data
    from ompmc_gb300 import workloads as W

    torch.cuda.set_device(local_rank)
    data.stage()
    P = data.paths()
    with tempfile.TemporaryDirectory() as tmp:
        ph = W.ct_like()
        phantom = api.Phantom.from_arrays(ph.media, ph.xb, ph.yb, ph.zb, ph.med, ph.rho)
        spec = W.write_spectrum(os.path.join(tmp, "6mv.spectrum"), "synthetic 6 MV", *W.spectrum_6mv())
        job = W.Job("(in memory)", P["pegs"], P["pgs4form"], P["data_folder"], tmp + os.sep, spectrum_file=spec,
                    ncase=50000, nbatch=1)
        prob = api.Problem(api.Input(text=job.text()), phantom=phantom)
        iso = (0.0, 0.0, 0.5 * (ph.zb[0] + ph.zb[-1]))
        gantry = tuple(360.0 * k / 7 for k in range(7))
        bl = W.beamlets(gantry_deg=gantry, iso=iso, sad=100.0, bixel=0.5, field=10.0, radius=3.5)
        nh = W.lognormal_histories(bl.n, median=5e4, sigma=1.0, lo=1e4, hi=1e6, seed=7)
        eng = api.Engine(local_rank).load(prob)
        eng.set_beamlets(bl)
        scale = args.dij_scale
        nh = np.maximum(1, (nh * scale).astype(np.int64))
        # warm-up on a 1/50 sample of every beamlet
        eng.run_dij(rel_threshold=1e-4, nhist=np.maximum(1, nh // 50), precision=api.FP32, fp32_values=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        col, rows, vals, st = eng.run_dij(rel_threshold=1e-4, nhist=nh, precision=api.FP32, fp32_values=True,
                                          seeds=(97, 33), continue_streams=1)
        wall = time.perf_counter() - t0
        if st.error_flags:
            raise RuntimeError(f"device error flags {st.error_flags:#x}")
        total = int(nh.sum())
        line = {
            "metric": "histories/s", "value": total / (st.kernel_ms / 1000.0), "unit": "histories/s", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": DIJ_WORKLOAD, "beamlets": bl.n, "histories": total,
                       "transport": "FP32 arithmetic, FP64 tallies, FP32 dij values",
                       "threshold": "1e-4 of each beamlet's max"},
            "transport_s": st.kernel_ms / 1000.0, "wall_s": wall, "wall_histories_per_s": total / wall,
            "nnz": int(len(vals)), "dij_bytes": int(len(vals) * 8 + len(col) * 8),
            "per_history": {"events": st.steps / total, "voxel_steps": st.voxel_steps / total,
                            "deposits": st.deposits / total},
        }
        eng.close()
        return line


def run_vrt_leg(args, local_rank):
    """Photon splitting (the reference's only variance reduction, "nsplit")
    on the benchmark workload: efficiency 1/(s^2 T) of a 10-batch FP32 job
    per splitting number, s from the job's own batches."""
    import torch

    from ompmc_gb300 import api

    torch.cuda.set_device(local_rank)
    H = args.vrt_histories
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        prob = build_problem(tmp)
        eng = api.Engine(local_rank).load(prob)
        eng.run(nperbatch=H // 10, nbatch=2, precision=api.FP32)
        f = dose_factor(prob)
        for ns in (1, 2, 4, 8, 16, 32):
            acc, acc2, st = eng.run(nperbatch=H, nbatch=10, nsplit=ns, precision=api.FP32, seeds=(97, 33 + ns))
            if st.error_flags:
                raise RuntimeError(f"device error flags {st.error_flags:#x} at nsplit {ns}")
            m, m2 = acc[1:] / 10, acc2[1:] / 10
            sel = m * f > 0.5 * (m * f).max()
            rel = np.sqrt(np.maximum(m2[sel] - m[sel] ** 2, 0.0) / 9) / m[sel]
            T = st.kernel_ms / 1e3
            out.append({"nsplit": ns, "histories_per_s": 10 * H / T, "T_s": T, "s_max": float(rel.max()),
                        "s_mean": float(rel.mean()), "efficiency_max": float(1 / (rel.max() ** 2 * T)),
                        "efficiency_mean": float(1 / (rel.mean() ** 2 * T))})
        eng.close()
    return {"metric": "efficiency 1/(s^2 T) vs photon splitting", "n_gpus": 1, "data": "synthetic",
            "config": {"workload": WORKLOAD, "histories": 10 * H, "batches": 10,
                       "s": "relative batch sigma over voxels above 50% of Dmax (max and mean)"},
            "results": out}


def run_queue_traffic_leg(args, local_rank):
    """Four one-launch FP32 jobs of 1e7 histories on the benchmark workload
    that separate the two large working sets of the wavefront kernel: one or
    ten batch tallies (27 or 270 MB) times 2e5 or 2e6 particles in flight
    (one queue generation of 7 or 72 MB).  Run under ncu with DRAM counters
    (-k regex:wavefront_kernel -s 1 -c 4) it gives the DRAM bytes of each;
    alone it prints the launch times."""
    import torch

    from ompmc_gb300 import api

    torch.cuda.set_device(local_rank)
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        prob = build_problem(tmp)
        eng = api.Engine(local_rank).load(prob)
        eng.run(nperbatch=1_000_000, nbatch=1, precision=api.FP32, inflight=200_000)  # warm-up launch
        for nb, inflight in ((1, 200_000), (1, 2_000_000), (10, 200_000), (10, 2_000_000)):
            a, a2, st = eng.run(nperbatch=10_000_000 // nb, nbatch=nb, precision=api.FP32, continue_streams=1,
                                inflight=inflight)
            if st.error_flags:
                raise RuntimeError(f"device error flags {st.error_flags:#x}")
            out.append({"nbatch": nb, "inflight": inflight, "kernel_ms": st.kernel_ms,
                        "histories_per_s": 1e7 / (st.kernel_ms / 1e3)})
        eng.close()
    return {"metric": "wavefront launch time by tally and queue working set", "n_gpus": 1, "data": "synthetic",
            "config": {"workload": WORKLOAD, "histories": 10_000_000}, "results": out}


CT_WORKLOAD = ("CT-like blob phantom 256x256x128 @ 2 mm (seed 2024), synthetic 6 MV, point source SSD 100 cm; "
               "fields 3x3 and 10x10 cm2 at gantry 0 (+z) and gantry 90 (phantom axes x and z exchanged so that "
               "the beam enters along +z)")


def run_ct_leg(args, local_rank):
    """FP32-transport dose error against an FP64 run of the same engine, per
    field, on the CT-like phantom: both precisions with the same histories in
    10 batches, on disjoint streams; the statement of fp32_dose_error (per
    voxel z over voxels above 20% of Dmax; mean dose over voxels above 50%
    of Dmax and total energy, each with a sigma from the per-batch sums of
    both runs, so voxel correlations are included).  The voxels are chosen on
    a separate FP32 run."""
    import torch

    from ompmc_gb300 import api, data
    from ompmc_gb300 import workloads as W

    torch.cuda.set_device(local_rank)
    data.stage()
    P = data.paths()
    H = args.ct_histories
    nb = 10
    ph0 = W.ct_like()
    # gantry 90: exchange x and z (arrays [z, y, x] -> [x, y, z])
    ph90 = W.Phantom(ph0.media, ph0.zb - ph0.zb.mean(), ph0.yb, ph0.xb - ph0.xb[0],
                     np.ascontiguousarray(ph0.med.transpose(2, 1, 0)),
                     np.ascontiguousarray(ph0.rho.transpose(2, 1, 0)))
    fields = []
    with tempfile.TemporaryDirectory() as tmp:
        spec = W.write_spectrum(os.path.join(tmp, "6mv.spectrum"), "synthetic 6 MV", *W.spectrum_6mv())
        for gname, ph in (("gantry0", ph0), ("gantry90", ph90)):
            phantom = api.Phantom.from_arrays(ph.media, ph.xb, ph.yb, ph.zb, ph.med, ph.rho)
            for half in (1.5, 5.0):
                job = W.Job("(in memory)", P["pegs"], P["pgs4form"], P["data_folder"], tmp + os.sep,
                            spectrum_file=spec, ncase=H, nbatch=nb, collimator=(-half, half, -half, half), ssd=100.0)
                prob = api.Problem(api.Input(text=job.text()), phantom=phantom)
                eng = api.Engine(local_rank).load(prob)
                f = dose_factor(prob)
                sel_acc, _, _ = eng.run(nperbatch=H // 2, nbatch=1, precision=api.FP32, seeds=(3001, 5))
                dsel = sel_acc[1:] * f
                sel20 = dsel > 0.2 * dsel.max()
                sel50 = dsel > 0.5 * dsel.max()
                w_roi = np.concatenate([[0.0], np.where(sel50, f, 0.0)])
                w_in = np.concatenate([[0.0], np.ones(prob.nreg - 1)])
                a32, b32, s32 = eng.run(precision=api.FP32, seeds=(97, 33))
                roi32, tot32 = eng.batch_sums(w_roi), eng.batch_sums(w_in)
                a64, b64, s64 = eng.run(precision=api.FP64, seeds=(12, 34))
                roi64, tot64 = eng.batch_sums(w_roi), eng.batch_sums(w_in)
                eng.close()
                err = fp32_dose_error(a32, b32, H // nb, nb, roi32, tot32, a64, b64, H // nb, nb, roi64, tot64, f,
                                      sel20)
                err.update({"field": f"{gname} {2 * half:g}x{2 * half:g} cm2", "histories": H,
                            "fp32_histories_per_s": H / (s32.kernel_ms / 1e3),
                            "fp64_histories_per_s": H / (s64.kernel_ms / 1e3)})
                fields.append(err)
    return {"metric": "FP32-transport dose error vs FP64, per field", "n_gpus": 1, "data": "synthetic",
            "config": {"workload": CT_WORKLOAD, "batches": nb}, "fields": fields}


SERVE_WORKLOAD = ("dose-server mix: Poisson arrivals; phantom homogeneous water / z-slab / seeded blob at 64^3, "
                  "128^3 or 256x256x160 (2-4.7 mm voxels over a 30-48 cm box); source 1.25 MeV, synthetic 6 MV or "
                  "synthetic 250 kVp, 10x10 cm2 field at SSD 100 cm; histories log-uniform over [1e5, 1e8]; "
                  "10 batches per job.  A fraction of the jobs are beamlet (dij) jobs instead: 50-500 bixels "
                  "(0.5 cm) drawn from 1-3 beams of 10x10 cm2 at SAD 100 cm about the phantom centre, synthetic "
                  "6 MV, the job's histories split evenly over its beamlets, relative threshold 1e-4, FP32 values")


def serve_library():
    """Phantoms of the serving mix (generated once) and the three sources."""
    from ompmc_gb300 import workloads as W

    sizes = [(64, 64, 64, 0.469), (128, 128, 128, 0.234), (256, 256, 160, 0.1875)]
    phantoms = []
    for nx, ny, nz, vox in sizes:
        phantoms.append(("water", W.homogeneous(vox=vox, nxyz=(nx, ny, nz))))
        layers = ((0.0, 5.0, W.WATER, 1.0), (5.0, 15.0, W.LUNG, 0.26), (15.0, 18.0, W.BONE, 1.85),
                  (18.0, nz * vox + 1.0, W.WATER, 1.0))
        sl = W.slab(vox=vox, layers=layers, nxyz=(nx, ny, nz))
        phantoms.append(("slab", sl))
        phantoms.append(("blob", W.ct_like(nx=nx, ny=ny, nz=nz, vox=vox, seed=11 + nx)))
    return phantoms


def run_serve_leg(args, local_rank):
    import torch

    from ompmc_gb300 import api, data
    from ompmc_gb300 import workloads as W

    torch.cuda.set_device(local_rank)
    data.stage()
    P = data.paths()
    rng = np.random.default_rng(args.serve_seed)
    with tempfile.TemporaryDirectory() as tmp:
        lib = serve_library()
        phs = [api.Phantom.from_arrays(p.media, p.xb, p.yb, p.zb, p.med, p.rho) for _, p in lib]
        spec6 = W.write_spectrum(os.path.join(tmp, "6mv.spectrum"), "synthetic 6 MV", *W.spectrum_6mv())
        spec250 = W.write_spectrum(os.path.join(tmp, "250.spectrum"), "synthetic 250 kVp", *W.spectrum_250kvp())
        texts = []
        for spec in (None, spec6, spec250):
            job = W.Job("(in memory)", P["pegs"], P["pgs4form"], P["data_folder"], tmp + os.sep,
                        spectrum_file=spec, mono_energy=1.25, collimator=(-5.0, 5.0, -5.0, 5.0), ssd=100.0)
            texts.append(job.text())
        inputs = [api.Input(text=t) for t in texts]
        sources = {}
        njobs = args.serve_jobs
        draws = []
        brng = np.random.default_rng(args.serve_seed + 1000)  # beamlet choices apart: field draws stay as they were
        for _ in range(njobs):
            ip = int(rng.integers(len(phs)))
            isrc = int(rng.integers(3))
            nh = int(10 ** rng.uniform(5.0, np.log10(args.serve_max_histories)))
            nh -= nh % 10
            bl = None
            if brng.uniform() < args.serve_beamlet_frac:
                isrc = 1
                p = lib[ip][1]
                iso = (0.5 * (p.xb[0] + p.xb[-1]), 0.5 * (p.yb[0] + p.yb[-1]), 0.5 * (p.zb[0] + p.zb[-1]))
                angles = tuple(float(a) for a in brng.choice([0.0, 40.0, 80.0, 280.0, 320.0],
                                                              size=int(brng.integers(1, 4)), replace=False))
                full = W.beamlets(gantry_deg=angles, iso=iso, sad=100.0, bixel=0.5, field=10.0)
                pick = np.sort(brng.choice(full.n, size=min(full.n, int(brng.integers(50, 501))), replace=False))
                bl = W.Beamlets(full.ibeam[pick], full.source, full.corner[pick], full.side1[pick], full.side2[pick])
                nh = max(nh - nh % (10 * bl.n), 10 * bl.n)
            draws.append((ip, isrc, max(nh, 10), bl))
            if (ip, isrc) not in sources:
                sources[(ip, isrc)] = api.build_source(inputs[isrc], phs[ip])
        mean_h = float(np.mean([d[2] for d in draws]))
        gaps = rng.exponential(1.0 / args.serve_rate, size=njobs)
        media = [W.AIR, W.LUNG, W.WATER, W.BONE]
        data_text = f"pegs file = {P['pegs']}\npgs4form file = {P['pgs4form']}\ndata folder = {P['data_folder']}\n"
        out = {}
        modes = (("continuous", 0, api.Server.SHORTEST_FIRST), ("continuous_equal_shares", 0, api.Server.EQUAL_SHARES),
                 ("one_at_a_time", 1, api.Server.SHORTEST_FIRST))
        wanted = getattr(args, "serve_modes", None)
        for mode, max_jobs, policy in modes:
            if wanted and mode not in wanted:
                continue
            srv = api.Server(media, data_text, precision=api.FP32, max_jobs=max_jobs, policy=policy,
                             round_histories=getattr(args, "serve_round_histories", 0))
            # warm-up job (tables, kernels)
            srv.wait(srv.submit(phs[0], sources.get((0, 0)) or api.build_source(inputs[0], phs[0]), 0.7, 0.01,
                                1000, 10))
            ids = []
            t0 = time.perf_counter()
            for (ip, isrc, nh, bl), gap in zip(draws, gaps):
                time.sleep(gap)
                if bl is None:
                    ids.append(srv.submit(phs[ip], sources[(ip, isrc)], 0.7, 0.01, nh // 10, 10))
                else:
                    ids.append(srv.submit_dij(phs[ip], sources[(ip, isrc)], 0.7, 0.01, bl, nh // (10 * bl.n), 10,
                                              rel_threshold=1e-4, fp32_values=True))
            res = [(srv.wait(i) if d[3] is None else srv.wait_dij(i))[-1] for i, d in zip(ids, draws)]
            makespan = time.perf_counter() - t0
            st = srv.stats()
            srv.close()
            lat = np.array([r.finish_s - r.submit_s for r in res])
            is_dij = np.array([d[3] is not None for d in draws])
            tot = sum(d[2] for d in draws)
            out[mode] = {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                         "beamlet_jobs_p50_s": float(np.percentile(lat[is_dij], 50)) if is_dij.any() else None,
                         "mean_s": float(lat.mean()), "histories_per_s": tot / makespan,
                         "gpu_transport_s": st.transport_s, "rounds": int(st.rounds),
                         "max_resident": int(st.max_resident), "max_round_jobs": int(st.max_round_jobs)}
        for src in sources.values():
            api.free_source(src)
        total = sum(d[2] for d in draws)
        return {"metric": "job latency p50/p99 (s) and histories/s", "n_gpus": 1, "data": "synthetic",
                "dtype": "f32", "config": {"workload": SERVE_WORKLOAD, "jobs": njobs, "rate_per_s": args.serve_rate,
                                           "mean_histories": mean_h, "total_histories": total,
                                           "beamlet_jobs": int(sum(d[3] is not None for d in draws)),
                                           "seed": args.serve_seed,
                                           "round_histories": getattr(args, "serve_round_histories", 0) or
                                           "adaptive: a quarter of the resident backlog, 4e6 to 3.2e7"},
                "continuous": out.get("continuous"), "continuous_equal_shares": out.get("continuous_equal_shares"),
                "one_at_a_time": out.get("one_at_a_time")}


def run_serve_short(local_rank):
    """A short Poisson serving run for the default line: job latency p50/p99
    and histories/s with continuous batching (the mix of the --serve leg,
    fewer and smaller jobs)."""
    ns = argparse.Namespace(serve_seed=SERVE_SHORT["seed"], serve_jobs=SERVE_SHORT["jobs"],
                            serve_rate=SERVE_SHORT["rate"], serve_max_histories=SERVE_SHORT["max_histories"],
                            serve_beamlet_frac=SERVE_SHORT["beamlet_frac"], serve_modes=("continuous",))
    r = run_serve_leg(ns, local_rank)
    c = r["continuous"]
    return {"p50_s": c["p50_s"], "p99_s": c["p99_s"], "histories_per_s": c["histories_per_s"],
            "beamlet_jobs_p50_s": c["beamlet_jobs_p50_s"], "jobs": SERVE_SHORT["jobs"],
            "rate_per_s": SERVE_SHORT["rate"], "total_histories": r["config"]["total_histories"],
            "beamlet_jobs": r["config"]["beamlet_jobs"],
            "workload": "the --serve mix: " + SERVE_WORKLOAD + f"; here {SERVE_SHORT['jobs']} jobs at "
                        f"{SERVE_SHORT['rate']}/s, histories log-uniform over [1e5, {SERVE_SHORT['max_histories']:.0e}]"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--histories-per-step", type=int, default=HISTORIES_PER_STEP,
                    help="smaller values only for profiler captures of the same code path")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="leave the short serving run out of the default line")
    ap.add_argument("--fp64-histories", type=int, default=FP64_HISTORIES)
    ap.add_argument("--nsplit16-histories", type=int, default=NSPLIT16_HISTORIES)
    ap.add_argument("--hbh-histories", type=int, default=20_000_000,
                    help="histories of the history-by-history run (10 batches)")
    ap.add_argument("--inflight", type=int, default=0,
                    help="particles in flight (0 = the engine's default); smaller values only to keep the device "
                         "memory of profiler captures small")
    ap.add_argument("--dij", action="store_true", help="measure the batched dij workload instead (one JSON line)")
    ap.add_argument("--dij-scale", type=float, default=1.0, help="scale of the dij history counts")
    ap.add_argument("--serve", action="store_true", help="measure the dose-server mix instead (one JSON line)")
    ap.add_argument("--ct", action="store_true", help="FP32-vs-FP64 dose error per field on the CT-like phantom")
    ap.add_argument("--vrt", action="store_true", help="efficiency 1/(s^2 T) against the photon splitting number")
    ap.add_argument("--queue-traffic", action="store_true",
                    help="four one-launch jobs that separate the tally and queue working sets (for a DRAM capture)")
    ap.add_argument("--vrt-histories", type=int, default=2_000_000, help="histories per batch (10 batches)")
    ap.add_argument("--ct-histories", type=int, default=20_000_000)
    ap.add_argument("--serve-jobs", type=int, default=40)
    ap.add_argument("--serve-rate", type=float, default=0.5, help="job arrivals per second")
    ap.add_argument("--serve-max-histories", type=float, default=1e8)
    ap.add_argument("--serve-seed", type=int, default=5)
    ap.add_argument("--serve-beamlet-frac", type=float, default=0.25, help="share of beamlet (dij) jobs in the mix")
    ap.add_argument("--serve-round-histories", type=int, default=0,
                    help="histories per server round (0: adaptive to the resident backlog)")
    ap.add_argument("--serve-modes", type=lambda v: tuple(v.split(",")), default=None,
                    help="comma list of continuous, continuous_equal_shares, one_at_a_time (default: all)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return
    if args.dij:
        if rank == 0:
            print(json.dumps(run_dij_leg(args, local_rank)), flush=True)
        return
    if args.vrt:
        if rank == 0:
            print(json.dumps(run_vrt_leg(args, local_rank)), flush=True)
        return
    if args.ct:
        if rank == 0:
            print(json.dumps(run_ct_leg(args, local_rank)), flush=True)
        return
    if args.queue_traffic:
        if rank == 0:
            print(json.dumps(run_queue_traffic_leg(args, local_rank)), flush=True)
        return
    if args.serve:
        if rank == 0:
            print(json.dumps(run_serve_leg(args, local_rank)), flush=True)
        return
    dist_on = world > 1
    if dist_on:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
    line = run_ours(args, rank, world, local_rank, dist_on)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if dist_on:
        import torch.distributed as tdist

        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
