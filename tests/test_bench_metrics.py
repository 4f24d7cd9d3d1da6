"""The bench's statistics on the host: the "% of Dmax" selections are made
on dose, as accumulateResults (omc_dosxyz.c:739-799) defines it, not on
deposited energy."""

import os

import numpy as np

import bench
from ompmc_gb300 import api, data
from ompmc_gb300 import workloads as W


def _problem(tmp_path):
    # lung, bone, air and water voxels of unequal size
    ph = W.slab(n=6, vox=1.0)
    ph.rho.reshape(-1)[:6] = 0.01  # air: dose zeroed below 0.044
    ph.rho.reshape(-1)[6:40] = 0.26
    ph.xb = np.cumsum(np.r_[0.0, [0.5, 1.0, 1.5, 1.0, 2.0, 1.0]])
    phantom = api.Phantom.from_arrays(ph.media, ph.xb, ph.yb, ph.zb, ph.med, ph.rho)
    data.stage()
    P = data.paths()
    job = W.Job("(in memory)", P["pegs"], P["pgs4form"], P["data_folder"], str(tmp_path) + os.sep, ncase=20,
                nbatch=2, collimator=(-1.0, 1.0, -1.0, 1.0), ssd=100.0)
    prob = api.Problem(api.Input(text=job.text()), phantom=phantom)
    return ph, prob


def test_dose_factor_is_one_over_mass(native, tmp_path):
    ph, prob = _problem(tmp_path)
    f = bench.dose_factor(prob)
    dx, dy, dz = np.diff(ph.xb), np.diff(ph.yb), np.diff(ph.zb)
    vol = (dz[:, None, None] * dy[None, :, None] * dx[None, None, :]).reshape(-1)
    rho = ph.rho.reshape(-1)
    want = np.where(rho < 0.044, 0.0, 1.602e-10 / (rho * vol))
    np.testing.assert_allclose(f, want, rtol=1e-12, atol=0)


def test_max_rel_sigma_selects_on_dose(native, tmp_path):
    """A lung voxel whose energy is below half the maximum but whose dose is
    the maximum counts; air voxels with the largest energy do not."""
    ph, _ = _problem(tmp_path)
    rho = ph.rho.reshape(-1)
    rho[6:] = 1.0
    lung = 6  # x index 0: the thinnest column
    rho[lung] = 0.26
    phantom = api.Phantom.from_arrays(ph.media, ph.xb, ph.yb, ph.zb, ph.med, ph.rho)
    data.stage()
    P = data.paths()
    job = W.Job("(in memory)", P["pegs"], P["pgs4form"], P["data_folder"], str(tmp_path) + os.sep, ncase=20,
                nbatch=2, collimator=(-1.0, 1.0, -1.0, 1.0), ssd=100.0)
    prob = api.Problem(api.Input(text=job.text()), phantom=phantom)
    f = bench.dose_factor(prob)
    n = prob.nreg
    nb = 10
    mean = np.full(n - 1, 1.0)
    mean[:6] = 5.0  # air: most energy, zero dose
    mean[lung] = 0.4  # 8% of the largest energy, 1.5x the dose of the water beside it
    rel = np.full(n - 1, 0.01)
    rel[lung] = 0.07
    rel[:6] = 0.5
    var = (rel * mean) ** 2 * (nb - 1)  # batch variance giving that relative sigma
    acc = np.r_[0.0, mean * nb]
    acc2 = np.r_[0.0, (var + mean ** 2) * nb]
    assert abs(bench.max_rel_sigma(acc, acc2, nb, f) - 0.07) < 1e-9
    # the energy-based selection would have taken the air voxels and left the lung voxel out
    m = acc[1:] / nb
    assert m[lung] < 0.5 * m.max() and (m * f)[lung] > 0.5 * (m * f).max()
