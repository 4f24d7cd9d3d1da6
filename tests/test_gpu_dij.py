"""Dose-influence matrix (omc_matrad) on the GPU, through the C ABI:
trajectory parity of the serial lane with the reference's matRad front end
(golden fixtures), exact equality across tally-group sizes, and
statistical parity of the many-lane FP64/FP32 paths with the OpenMP oracle,
including uneven history counts per beamlet."""

import os

import numpy as np
import pytest
from cases import DIJ_CASES, dij_case, run_seeds
from conftest import GOLDEN
from stats import compare_runs, consistent

from ompmc_gb300 import _native as N
from ompmc_gb300 import api

pytestmark = pytest.mark.gpu


def dense(col, rows, vals, nrows):
    out = np.zeros((len(col) - 1, nrows))
    for j in range(len(col) - 1):
        out[j, rows[col[j]:col[j + 1]]] = vals[col[j]:col[j + 1]]
    return out


@pytest.fixture
def dij_problem(engine, tmp_path):
    def make(name, ncase=None, nbatch=None, seeds=(97, 33)):
        inp, ph, bl, opts, thr, nsplit = dij_case(name, str(tmp_path / name), ncase=ncase, nbatch=nbatch, seeds=seeds)
        prob = api.Problem.from_file(inp)
        engine.load(prob)
        engine.set_beamlets(bl)
        return prob, bl, thr

    return make


@pytest.mark.parametrize("name", sorted(DIJ_CASES))
def test_serial_dij_reproduces_reference(name, engine, dij_problem):
    """One lane, one stream, beamlets and histories in the reference's
    order: the FP64 dij equals the reference's matRad output up to the last
    bits of CUDA's math functions against the host libm."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    prob, bl, thr = dij_problem(name)
    col, rows, vals, st = engine.run_dij(rel_threshold=thr, precision=api.FP64, serial=1)
    assert st.error_flags == 0
    assert st.histories == bl.n * prob.nperbatch * prob.nbatch
    np.testing.assert_array_equal(col, g["jc"])
    np.testing.assert_array_equal(rows, g["ir"])
    np.testing.assert_allclose(vals, g["pr"], rtol=1e-7, atol=0)


def test_tally_groups_do_not_change_the_result(engine, dij_problem):
    """A tally budget of 4 beamlets (7 groups for 27 beamlets) gives the
    same serial dij bit for bit, and FP32 storage is the rounding of it."""
    prob, bl, thr = dij_problem("dij_slab")
    nreg = prob.nreg
    a = engine.run_dij(rel_threshold=thr, precision=api.FP64, serial=1)
    b = engine.run_dij(rel_threshold=thr, precision=api.FP64, serial=1, tally_bytes=4 * nreg * 8)
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)
    c = engine.run_dij(rel_threshold=thr, precision=api.FP64, serial=1, fp32_values=True)
    assert c[2].dtype == np.float32
    np.testing.assert_array_equal(c[0], a[0])
    np.testing.assert_array_equal(c[2], a[2].astype(np.float32))


@pytest.mark.parametrize("precision", [api.FP64, api.FP32])
@pytest.mark.parametrize("schedule", [api.WAVEFRONT, api.LANES])
def test_many_lanes_dij_statistically_identical(precision, schedule, engine, oracle, dij_problem):
    """K = 16 independent dij runs (different seeds) of the GPU and of the
    OpenMP oracle, threshold 0: the per (beamlet, voxel) Welch statistics
    over entries above 20% of the beamlet maximum are consistent with one
    distribution, and so are the totals (|t| < 4)."""
    prob, bl, _ = dij_problem("dij_slab", ncase=2000, nbatch=2)
    nrows = prob.nreg - 1
    k = 16

    def gpu(i):
        col, rows, vals, st = engine.run_dij(rel_threshold=0.0, precision=precision, schedule=schedule,
                                             seeds=run_seeds(i))
        assert st.error_flags == 0
        return dense(col, rows, vals, nrows)

    def cpu(i):
        col, rows, vals, _ = oracle.run_dij(prob, bl, rel_threshold=0.0, seeds=(211 + i, 7 + 5 * i), nthreads=0)
        return dense(col, rows, vals, nrows)

    c = compare_runs(np.stack([gpu(i) for i in range(k)]), np.stack([cpu(i) for i in range(k)]))
    assert c["n"] > 200, c
    assert consistent(c), c
    assert abs(c["t_total"]) < 4.0, c


def test_uneven_histories_per_beamlet(engine, oracle, dij_problem):
    """Histories per beamlet drawn lognormally: each column is normalised
    by its own count, so per-beamlet integral doses agree with the oracle's
    within their statistical spread."""
    from ompmc_gb300 import workloads as W

    prob, bl, _ = dij_problem("dij_slab", ncase=1000, nbatch=2)
    nh = W.lognormal_histories(bl.n, median=1500, sigma=0.8, lo=300, hi=8000, seed=3)
    nrows = prob.nreg - 1
    k = 6

    def gpu(i):
        col, rows, vals, st = engine.run_dij(rel_threshold=0.0, nhist=nh, precision=api.FP32, seeds=run_seeds(i))
        assert st.histories == nh.sum()
        return dense(col, rows, vals, nrows).sum(axis=1)

    def cpu(i):
        col, rows, vals, res = oracle.run_dij(prob, bl, rel_threshold=0.0, nhist=nh, seeds=(77 + i, 3), nthreads=0)
        return dense(col, rows, vals, nrows).sum(axis=1)

    g = np.stack([gpu(i) for i in range(k)])
    o = np.stack([cpu(i) for i in range(k)])
    z = (g.mean(0) - o.mean(0)) / np.sqrt(g.var(0, ddof=1) / k + o.var(0, ddof=1) / k)
    assert np.mean(np.abs(z) < 3) > 0.9, z
    assert abs(g.mean(0).sum() / o.mean(0).sum() - 1) < 0.02


def test_dij_errors(engine, dij_problem, problem_factory):
    fresh = api.Engine(0)
    fresh.load(problem_factory("slab_6mv"))
    with pytest.raises(N.OmcError) as e:
        fresh.run_dij()
    assert e.value.status == 10  # OMC_ERR_STATE: no beamlets
    fresh.close()
    prob, bl, _ = dij_problem("dij_slab")
    with pytest.raises(N.OmcError) as e:
        engine.run_dij(nhist=np.zeros(bl.n, np.int64))
    assert e.value.status == 1
    with pytest.raises(N.OmcError):
        engine.run_dij(rel_threshold=-1.0)
