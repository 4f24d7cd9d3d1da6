"""History-by-history scoring (cfg.history_stats) through the C ABI: the
per-region sums of x and x^2 over histories (x = energy a history deposits
in a region), the estimators of Walters, Kawrakow and Rogers (Med. Phys.
29 (2002) 2745), against the batch method the reference uses
(omc_dosxyz.c:696-755)."""

import numpy as np
import pytest
from cases import run_seeds
from stats import compare, consistent

from ompmc_gb300 import _native as N
from ompmc_gb300 import api

pytestmark = pytest.mark.gpu


def _sigma2_history(s, s2, n):
    m = s / n
    return np.maximum(s2 / n - m * m, 0.0) / (n - 1)


def _sigma2_batch(a, a2, nbatch, nperbatch):
    # variance of the per-history mean from nbatch batch totals
    m = a / nbatch
    v = np.maximum(a2 / nbatch - m * m, 0.0) / (nbatch - 1)
    return v / nperbatch ** 2


@pytest.mark.parametrize("precision", [api.FP32, api.FP64])
def test_history_sums_agree_with_the_batch_method(precision, engine, problem_factory):
    """Sum over histories = sum over batches (the same deposits), and the
    variance of the mean per voxel from history-by-history sums agrees with
    the 50-batch estimate (the median of their ratio over voxels above 20%
    of Dmax within 10% of 1; one batch variance has a relative spread of
    20%)."""
    prob = problem_factory("slab_6mv", ncase=400000, nbatch=50, seeds=(71, 73))
    engine.load(prob)
    a, a2, st = engine.run(precision=precision, history_stats=1)
    assert st.error_flags == 0
    s, s2, nh, split = engine.history_sums()
    n = prob.nperbatch * prob.nbatch
    assert nh == n and split == 0
    np.testing.assert_allclose(s, a, rtol=1e-9, atol=1e-12 * a.max())
    sel = a[1:] > 0.2 * a[1:].max()
    assert sel.sum() > 100
    vh = _sigma2_history(s[1:], s2[1:], n)[sel]
    vb = _sigma2_batch(a[1:], a2[1:], prob.nbatch, prob.nperbatch)[sel]
    r = vb / vh
    assert 0.9 < np.median(r) < 1.1, np.median(r)
    assert 0.95 < r.mean() < 1.05, r.mean()


def test_history_scoring_leaves_the_dose_unchanged(engine, problem_factory):
    """A run with history tracking gives the batch-tally distribution of a
    run without it (streams disjoint)."""
    prob = problem_factory("slab_6mv", ncase=400000, nbatch=50, seeds=(79, 83))
    engine.load(prob)
    a, a2, sa = engine.run(precision=api.FP32, history_stats=1)
    b, b2, sb = engine.run(precision=api.FP32, seeds=run_seeds(5))
    assert sa.error_flags == 0 and sb.error_flags == 0
    c = compare(a, a2, b, b2, prob.nbatch)
    assert consistent(c), c
    assert abs(c["etot_rel"]) < 6.0 / np.sqrt(400000), c


def test_history_scoring_electrons_and_one_batch(engine, problem_factory):
    """Electron pencil beam (long tracks, many regions per history) in one
    batch: every history is merged, none over the merge table."""
    prob = problem_factory("electron_pencil", ncase=20000, nbatch=2)
    engine.load(prob)
    a, a2, st = engine.run(nperbatch=20000, nbatch=1, precision=api.FP32, history_stats=1)
    assert st.error_flags == 0
    s, s2, nh, split = engine.history_sums()
    assert nh == 20000 and split == 0
    np.testing.assert_allclose(s, a, rtol=1e-9, atol=1e-12 * a.max())
    assert np.all(s2 >= 0) and np.all(s2 <= s * s + 1e-12 * a.max() ** 2)


def test_history_scoring_needs_the_wavefront(engine, problem_factory):
    prob = problem_factory("water_mono")
    engine.load(prob)
    with pytest.raises(N.OmcError) as e:
        engine.run(precision=api.FP64, serial=1, history_stats=1)
    assert e.value.status == 1
    engine.run(precision=api.FP32)
    with pytest.raises(N.OmcError) as e:
        engine.history_sums()
    assert e.value.status == 10
