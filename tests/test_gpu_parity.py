"""GPU transport against the reference: RANMAR bit-exactness, trajectory
parity of the serial lane with the reference's serial build (golden
fixtures), and statistical parity of the many-lane FP64 and FP32 paths with
the oracle.  All calls go through the C ABI."""

import os

import numpy as np
import pytest
from cases import CASES, RANMAR_N, RANMAR_SEEDS, run_seeds
from conftest import GOLDEN
from stats import compare, consistent

from ompmc_gb300 import _native as N
from ompmc_gb300 import api

pytestmark = pytest.mark.gpu


def test_ranmar_streams_bit_exact(native):
    g = np.load(os.path.join(GOLDEN, "ranmar.npz"))
    for a, b in RANMAR_SEEDS:
        out = api.gpu_ranmar(a, b, 1, RANMAR_N)
        np.testing.assert_array_equal(out[0], g[f"{a}_{b}"], err_msg=f"seeds {a} {b}")


def test_ranmar_lane_streams_follow_thread_seeding(native, oracle):
    # lane k = stream k of the seed pair (the reference's OpenMP thread k
    # while jxx + k <= 30081, then the next unused stream).
    out = api.gpu_ranmar(97, 31320, 20, 300)
    for k in range(20):
        ik, jk = api.stream_seeds(97, 31320, k)
        np.testing.assert_array_equal(out[k], oracle.ranmar(ik, jk, 300))


@pytest.mark.parametrize("name", sorted(CASES))
def test_serial_lane_reproduces_reference_trajectories(name, engine, problem_factory):
    """One lane, one stream, histories in order: the reference's serial
    build.  FP64 transport follows the same trajectories; only the last
    bits of CUDA's math functions against the host libm differ."""
    g = np.load(os.path.join(GOLDEN, f"dose_{name}.npz"))
    prob = problem_factory(name)
    engine.load(prob)
    a, a2, st = engine.run(precision=api.FP64, serial=1)
    assert st.error_flags == 0
    ref = g["accum_endep"]
    assert abs(st.ensrc - g["ensrc"][0]) <= 1e-9 * g["ensrc"][0]
    np.testing.assert_allclose(a[1:].sum(), ref[1:].sum(), rtol=1e-8)
    np.testing.assert_allclose(a, ref, rtol=1e-7, atol=1e-9 * ref.max())
    np.testing.assert_allclose(a2, g["accum_endep2"], rtol=1e-6, atol=1e-9 * g["accum_endep2"].max())


PARITY = [("water_mono", 400000), ("slab_6mv", 400000), ("slab_250kvp", 400000), ("electron_pencil", 40000),
          ("positron_field", 40000), ("slab_split10", 40000)]


@pytest.mark.parametrize("name,ncase", PARITY)
@pytest.mark.parametrize("precision", [api.FP64, api.FP32])
@pytest.mark.parametrize("schedule", [api.WAVEFRONT, api.LANES])
def test_many_lanes_statistically_identical(name, ncase, precision, schedule, engine, oracle, problem_factory):
    """Per-voxel z-scores of the GPU against the OpenMP-seeded oracle over
    voxels above 20% of Dmax (50 batches): the count outside 2 sigma and
    the sum of z^2 are what two samples of one distribution give, and the
    total energies agree within 6/sqrt(N)."""
    prob = problem_factory(name, ncase=ncase, nbatch=50, seeds=(33, 97))
    engine.load(prob)
    g, g2, st = engine.run(precision=precision, schedule=schedule)
    assert st.error_flags == 0
    o, o2, res = oracle.run(prob, nthreads=0)
    c = compare(g, g2, o, o2, prob.nbatch)
    assert c["n"] >= 10, c
    assert consistent(c), c
    # The total deposit of N histories scatters by roughly 1/sqrt(N).
    assert abs(c["etot_rel"]) < 6.0 / np.sqrt(ncase), c
    if prob.source.contents.spectrum == 0:
        assert st.ensrc == pytest.approx(res.ensrc, rel=1e-12)
    else:
        # Sampled spectrum energies: the relative spread of a single energy is
        # below 1, so two sums of N agree within 4/sqrt(N) at 4 sigma or more.
        assert st.ensrc == pytest.approx(res.ensrc, rel=4.0 / np.sqrt(ncase))


def test_fp32_against_fp64_on_the_gpu(engine, problem_factory):
    """The FP32-transport dose error, stated against an FP64 run of the same
    engine: statistically indistinguishable."""
    prob = problem_factory("slab_6mv", ncase=400000, nbatch=50, seeds=(7, 11))
    engine.load(prob)
    d, d2, _ = engine.run(precision=api.FP64)
    f, f2, _ = engine.run(precision=api.FP32, seeds=run_seeds(0))  # streams disjoint from the FP64 run's
    c = compare(f, f2, d, d2, prob.nbatch)
    assert consistent(c), c
    assert abs(c["etot_rel"]) < 0.01, c


@pytest.mark.parametrize("precision", [api.FP32, api.FP64])
def test_drain_mode_does_not_change_the_dose(precision, engine, problem_factory):
    """The end-of-run drain mode (inline electron interactions, whole
    tracks per take) only reschedules events.  Forced on from the first
    iteration (all 400k histories injected at once, threshold far above the
    in-flight count) it gives the distribution of a run without it."""
    prob = problem_factory("slab_6mv", ncase=400000, nbatch=50, seeds=(13, 17))
    engine.load(prob)
    a, a2, sa = engine.run(precision=precision, drain_per_warp=-1, seeds=(13, 17))
    b, b2, sb = engine.run(precision=precision, drain_per_warp=1 << 20, seeds=(19, 23))
    assert sa.error_flags == 0 and sb.error_flags == 0
    c = compare(a, a2, b, b2, prob.nbatch)
    assert c["n"] >= 10, c
    assert consistent(c), c
    assert abs(c["etot_rel"]) < 6.0 / np.sqrt(400000), c
    assert sb.ensrc == pytest.approx(sa.ensrc, rel=4.0 / np.sqrt(400000))


@pytest.mark.parametrize("schedule", [api.WAVEFRONT, api.LANES])
def test_energy_balance_closes(engine, problem_factory, schedule):
    """Electrons: all source energy is deposited inside the phantom or
    scored outside it (region 0) up to the energy carried away by escaping
    photons; nothing is created."""
    prob = problem_factory("electron_pencil", ncase=20000)
    engine.load(prob)
    for prec in (api.FP64, api.FP32):
        a, _, st = engine.run(precision=prec, schedule=schedule)
        assert a.sum() <= st.ensrc * (1 + 1e-6)
        assert a[1:].sum() > 0.5 * st.ensrc


def test_results_independent_of_lane_count(engine, problem_factory):
    prob = problem_factory("water_mono", ncase=200000, nbatch=50, seeds=(3, 4))
    engine.load(prob)
    a, a2, _ = engine.run(precision=api.FP32, nlanes=4096, schedule=api.LANES)
    b, b2, _ = engine.run(precision=api.FP32, schedule=api.WAVEFRONT, seeds=run_seeds(1))
    c = compare(a, a2, b, b2, prob.nbatch)
    assert consistent(c) and abs(c["etot_rel"]) < 0.01, c


def test_reproducible_for_fixed_seeds_and_lanes(engine, problem_factory):
    """Same seeds, same lane count: the same per-lane streams; the history
    hand-out order can differ between runs, so only statistics are fixed,
    but the serial lane is exactly reproducible."""
    prob = problem_factory("slab_6mv")
    engine.load(prob)
    a, _, _ = engine.run(precision=api.FP64, serial=1)
    b, _, _ = engine.run(precision=api.FP64, serial=1)
    np.testing.assert_array_equal(a, b)


def test_batch_sums_are_the_batch_tallies_weighted(engine, problem_factory):
    """omc_engine_batch_sums over the batches of one multi-batch launch: with
    unit weights inside the phantom they add up to the accumulated total, and
    the squares of per-region weights add up to the accumulated squares."""
    prob = problem_factory("slab_6mv", ncase=200000, nbatch=10, seeds=(41, 47))
    engine.load(prob)
    a, a2, _ = engine.run(precision=api.FP32)
    w = np.zeros(prob.nreg)
    w[1:] = 1.0
    tot = engine.batch_sums(w)
    assert len(tot) == prob.nbatch
    assert tot.sum() == pytest.approx(a[1:].sum(), rel=1e-12)
    r = int(np.argmax(a))
    one = np.zeros(prob.nreg)
    one[r] = 1.0
    per_batch = engine.batch_sums(one)
    assert per_batch.sum() == pytest.approx(a[r], rel=1e-12)
    assert (per_batch ** 2).sum() == pytest.approx(a2[r], rel=1e-12)
    # One-batch runs keep no batch tallies.
    engine.run(nbatch=1, precision=api.FP32)
    with pytest.raises(N.OmcError) as e:
        engine.batch_sums(w)
    assert e.value.status == 10
