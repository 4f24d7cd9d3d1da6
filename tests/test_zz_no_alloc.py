"""omc_engine_run_noalloc: the transport entry point that allocates no device
memory, for callers that cannot call cudaMalloc while a job runs (all
device memory handed out by their own pool or caching allocator, or a
fixed device-memory budget).  Its scratch is one fixed-size device array;
the caller passes the device tally and the stream the work runs on.
Checked through the C ABI against omc_engine_run on two calls in a row:
bit for bit with the single-lane schedule, and statistically with 4096
lanes, with and without photon splitting.

This file is collected last so that a run stopping at the first failure has
already run every other test."""

import ctypes as C

import numpy as np
import pytest
from cases import run_seeds
from stats import compare, consistent

from ompmc_gb300 import _native as N
from ompmc_gb300 import api

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(engine, cfg, d_endep):
    """One call on torch's current stream, the stream that cleared d_endep."""
    st = N.RunStats_t()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    N.check(N.lib().omc_engine_run_noalloc(engine._h, C.byref(cfg), C.c_void_p(d_endep.data_ptr()), stream,
                                           C.byref(st)))
    return st


def test_noalloc_matches_engine_run_serial_twice(engine, problem_factory):
    prob = problem_factory("slab_6mv")
    engine.load(prob)
    nh = prob.nperbatch * prob.nbatch
    ref, _, st_ref = engine.run(nperbatch=nh, nbatch=1, precision=api.FP64, serial=1)
    d_endep = torch.zeros(prob.nreg, dtype=torch.float64, device="cuda:0")
    cfg = api.Engine.config(nh, 1, seeds=prob.seeds, precision=api.FP64, serial=1)
    for call in range(2):
        d_endep.zero_()  # same stream as the call: ordered before its deposits
        st = _noalloc(engine, cfg, d_endep)
        got = d_endep.cpu().numpy()
        assert st.error_flags == 0 and st.histories == nh
        np.testing.assert_array_equal(got, ref, err_msg=f"call {call}")
        assert st.ensrc == st_ref.ensrc


@pytest.mark.parametrize("name,nsplit", [("water_mono", 1), ("slab_split10", 3)])
def test_noalloc_many_lanes_statistically_identical_twice(name, nsplit, engine, problem_factory):
    prob = problem_factory(name, ncase=200000 if nsplit == 1 else 40000, nbatch=20, seeds=(5, 6))
    engine.load(prob)
    ref, ref2, _ = engine.run(precision=api.FP32, schedule=api.LANES, nlanes=4096, nsplit=nsplit)
    d_endep = torch.zeros(prob.nreg, dtype=torch.float64, device="cuda:0")
    for call in range(2):
        acc = np.zeros(prob.nreg)
        acc2 = np.zeros(prob.nreg)
        for b in range(prob.nbatch):
            # Streams disjoint from the reference run's and from the other
            # call's: equal streams on equal lanes would replay histories.
            cfg = api.Engine.config(prob.nperbatch, 1, seeds=run_seeds(call), precision=api.FP32, nlanes=4096,
                                    nsplit=nsplit, continue_streams=1 if b else 0)
            d_endep.zero_()
            st = _noalloc(engine, cfg, d_endep)
            assert st.error_flags == 0 and st.histories == prob.nperbatch
            e = d_endep.cpu().numpy()
            acc += e
            acc2 += e * e
        c = compare(acc, acc2, ref, ref2, prob.nbatch)
        assert consistent(c) and abs(c["etot_rel"]) < 6.0 / np.sqrt(prob.nperbatch * prob.nbatch), (call, c)


def test_noalloc_limits_are_enforced(engine, problem_factory):
    prob = problem_factory("water_mono")
    engine.load(prob)
    d_endep = torch.zeros(prob.nreg, dtype=torch.float64, device="cuda:0")
    for bad in (dict(nlanes=4097), dict(stack_depth=65), dict(nsplit=5)):
        cfg = api.Engine.config(100, 1, precision=api.FP32, **bad)
        with pytest.raises(N.OmcError) as e:
            _noalloc(engine, cfg, d_endep)
        assert e.value.status == 1 and "maximum" in str(e.value)
    # An explicit depth within the maximum is accepted with any nsplit.
    cfg = api.Engine.config(100, 1, precision=api.FP32, nsplit=5, stack_depth=64, nlanes=64)
    d_endep.zero_()
    st = _noalloc(engine, cfg, d_endep)
    assert st.histories == 100
