"""omc_engine_tune: the run-option autotuner times its candidates on the
loaded workload and returns a configuration that runs cleanly.
omc_measure_atomic_rate: the tally-atomic denominator of the bench."""

import pytest

from ompmc_gb300 import api

pytestmark = pytest.mark.gpu


def test_tune_returns_the_fastest_working_options(engine, problem_factory):
    prob = problem_factory("slab_6mv", ncase=200000, nbatch=10, seeds=(31, 37))
    engine.load(prob)
    inflight, chunk, rates = engine.tune(api.FP32, sample_histories=200000)
    assert len(rates) == 8 and all(r > 0 for r in rates)
    assert chunk in (1, 2) and inflight > 0
    per_thread = (32, 64, 128, 192)
    k = rates.index(max(rates))
    assert chunk == 1 + k % 2
    a, _, st = engine.run(precision=api.FP32, inflight=inflight, chunk_events=chunk)
    assert st.error_flags == 0 and a[1:].sum() > 0
    assert inflight % per_thread[k // 2] == 0


def test_atomic_rate(native):
    """Scattered FP64 atomicAdd throughput: positive, and higher over an
    L2-resident array than the transport's measured tally rate on the 6 MV
    slab (1.97e9/s), which it bounds."""
    small = api.atomic_rate(150 ** 3 + 1)
    assert small > 2e9
    big = api.atomic_rate(1 << 28)  # 2 GB, well past L2
    assert 0 < big
    with pytest.raises(Exception):
        api.atomic_rate(0)
