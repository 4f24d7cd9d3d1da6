"""GPU transport against the OpenMP oracle at the benchmark configurations'
own sizes, on the stated acceptance bar:

- at least 95% of the voxels above 20% of Dmax agree within 2 combined
  sigma (batch sigma of each run; the Welch t statistic, with its
  Welch-Satterthwaite degrees of freedom, mapped to a normal z, so that
  exact agreement gives 95.45%);
- the total energy deposited in the phantom agrees within 0.1%, at a
  history count where 0.1% is at least 3 sigma of the difference (sigma
  from the spread of the per-batch totals of both runs, so the
  correlations between voxels are included).

Configurations: the plain small case (1.25 MeV parallel beam, 10x10 cm2,
on 60^3 water at 0.5 cm, FP64) and the 6 MV heterogeneous slab (150^3 at
2 mm: water, lung 0.26, ICRP bone 1.85, water; synthetic 24-bin spectrum,
10x10 cm2 at SSD 100 cm), FP64 and FP32 transport.  The reference's own
loop for these runs is omc_dosxyz.c:1237-1263, its scoring :696-799."""

import os

import numpy as np
import pytest
from cases import run_seeds
from scipy import stats as S

from ompmc_gb300 import api, data
from ompmc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NBATCH = 20


def _problem(tmp, ph, **job):
    P = data.paths()
    phantom = api.Phantom.from_arrays(ph.media, ph.xb, ph.yb, ph.zb, ph.med, ph.rho)
    j = W.Job("(in memory)", P["pegs"], P["pgs4form"], P["data_folder"], str(tmp) + os.sep, nbatch=NBATCH,
              collimator=(-5.0, 5.0, -5.0, 5.0), **job)
    return api.Problem(api.Input(text=j.text()), phantom=phantom)


def _judge(g, g2, gtot, o, o2, otot, nh, f):
    """Acceptance figures of run g (GPU) against run o (oracle), both NBATCH
    batches of nh histories; f = dose factor per voxel (voxel selection by
    dose, as accumulateResults defines it)."""
    mg, mo = g[1:] / NBATCH, o[1:] / NBATCH
    vg = np.maximum(g2[1:] / NBATCH - mg ** 2, 0) / (NBATCH - 1)
    vo = np.maximum(o2[1:] / NBATCH - mo ** 2, 0) / (NBATCH - 1)
    d = 0.5 * (mg + mo) * f
    sel = d > 0.2 * d.max()
    va, vb = vg[sel], vo[sel]
    t = (mg[sel] - mo[sel]) / np.sqrt(va + vb)
    dof = (va + vb) ** 2 / np.maximum((va ** 2 + vb ** 2) / (NBATCH - 1), 1e-300)  # Welch-Satterthwaite
    z = S.norm.ppf(np.clip(S.t.cdf(t, dof), 1e-300, 1 - 1e-16))
    gtot, otot = np.asarray(gtot) / nh, np.asarray(otot) / nh
    rel = gtot.mean() / otot.mean() - 1
    sig = (gtot.mean() / otot.mean()) * np.sqrt(gtot.var(ddof=1) / (NBATCH * gtot.mean() ** 2)
                                                 + otot.var(ddof=1) / (NBATCH * otot.mean() ** 2))
    return {"n": int(sel.sum()), "frac_2sigma": float(np.mean(np.abs(z) <= 2)), "mean_z": float(z.mean()),
            "mean_z2": float(np.mean(z * z)), "etot_rel": float(rel), "etot_sigma": float(sig)}


def _dose_factor(prob):
    n = prob.nreg
    d, _ = prob.dose(np.full(n, 2.0), np.full(n, 2.0), nperbatch=1, nbatch=2)
    return d[1:]


def _check(c):
    assert c["n"] > 1000, c
    assert c["frac_2sigma"] >= 0.95, c
    assert abs(c["mean_z"]) < 0.05 and c["mean_z2"] < 1.1, c
    assert 3 * c["etot_sigma"] <= 1e-3, c  # the run is large enough for the 0.1% test
    assert abs(c["etot_rel"]) < 1e-3, c


def _gpu(engine, prob, nh, precision, seed_index):
    w = np.zeros(prob.nreg)
    w[1:] = 1.0
    a, a2, st = engine.run(nperbatch=nh, nbatch=NBATCH, precision=precision, seeds=run_seeds(seed_index))
    assert st.error_flags == 0
    return a, a2, engine.batch_sums(w)


@pytest.fixture(scope="module")
def water60(tmp_path_factory, native, oracle):
    """1.25 MeV parallel beam (SSD 1e8: w = 1 within 1e-15), 10x10 cm2, on
    60^3 water at 0.5 cm; 12e6 histories of the oracle on every host core."""
    tmp = tmp_path_factory.mktemp("water60")
    prob = _problem(tmp, W.homogeneous(n=60, vox=0.5), mono_energy=1.25, ssd=1e8, ncase=1, seeds=(97, 33))
    nh = 600_000
    o, o2, res = oracle.run(prob, nperbatch=nh, nbatch=NBATCH, nthreads=0)
    return prob, nh, (o, o2, oracle.batch_totals())


@pytest.fixture(scope="module")
def slab150(tmp_path_factory, native, oracle):
    """The 6 MV heterogeneous slab at 150^3 x 2 mm, 52e6 histories of the
    oracle on every host core (at 16e6 and 36e6 the total-energy sigma of
    the difference was 0.049% and 0.035%, too large for a 3-sigma test of
    0.1%)."""
    tmp = tmp_path_factory.mktemp("slab150")
    spec = W.write_spectrum(os.path.join(str(tmp), "6mv.spectrum"), "synthetic 6 MV", *W.spectrum_6mv())
    prob = _problem(tmp, W.slab(n=150, vox=0.2), spectrum_file=spec, ssd=100.0, ncase=1, seeds=(97, 33))
    nh = 2_600_000
    o, o2, res = oracle.run(prob, nperbatch=nh, nbatch=NBATCH, nthreads=0)
    return prob, nh, (o, o2, oracle.batch_totals())


def test_config_water60_fp64(engine, water60):
    prob, nh, (o, o2, otot) = water60
    engine.load(prob)
    g, g2, gtot = _gpu(engine, prob, nh, api.FP64, 0)
    _check(_judge(g, g2, gtot, o, o2, otot, nh, _dose_factor(prob)))


@pytest.mark.parametrize("precision", [api.FP64, api.FP32])
def test_config_slab150(precision, engine, slab150):
    prob, nh, (o, o2, otot) = slab150
    engine.load(prob)
    g, g2, gtot = _gpu(engine, prob, nh, precision, 1 + precision)
    _check(_judge(g, g2, gtot, o, o2, otot, nh, _dose_factor(prob)))
