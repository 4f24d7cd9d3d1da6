"""Failure handling on the GPU without faulting it: bounded device loops
report through error flags and status codes, and the context stays usable."""

import numpy as np
import pytest

from ompmc_gb300 import _native as N
from ompmc_gb300 import api

pytestmark = pytest.mark.gpu


def test_stack_overflow_is_reported_not_fatal(engine, problem_factory):
    # Photon splitting with nsplit = 10 needs more than 4 stack slots; the
    # device drops the overflowing histories, flags them and returns.
    prob = problem_factory("slab_split10", ncase=2000)
    engine.load(prob)
    with pytest.raises(N.OmcError) as e:
        engine.run(precision=api.FP32, stack_depth=4, schedule=api.LANES)
    assert e.value.status == 8  # OMC_ERR_STACK
    # The engine still works afterwards.
    a, _, st = engine.run(precision=api.FP32)
    assert st.error_flags == 0 and a[1:].sum() > 0


def test_run_before_load_is_refused(native):
    e = api.Engine(0)
    with pytest.raises(N.OmcError) as err:
        N.check(N.lib().omc_engine_run(e._h, None, None, None, None))
    assert err.value.status == 1
    cfg = api.Engine.config(10, 2)
    import ctypes as C

    with pytest.raises(N.OmcError) as err:
        N.check(N.lib().omc_engine_run(e._h, C.byref(cfg), None, None, None))
    assert err.value.status == 10  # OMC_ERR_STATE
    e.close()


def test_bad_configuration_rejected(engine, problem_factory):
    prob = problem_factory("water_mono")
    engine.load(prob)
    with pytest.raises(N.OmcError):
        engine.run(nbatch=0)
    with pytest.raises(N.OmcError):
        engine.run(precision=7)


def test_empty_run(engine, problem_factory):
    prob = problem_factory("water_mono")
    engine.load(prob)
    a, a2, st = engine.run(nperbatch=0, nbatch=3)
    assert st.histories == 0 and not a.any() and not a2.any()


def test_wavefront_small_inflight_target(engine, problem_factory):
    # An in-flight target far above what the queues can hold is impossible
    # by construction; a tiny target with photon splitting still works.
    prob = problem_factory("slab_split10", ncase=2000)
    engine.load(prob)
    a, _, st = engine.run(precision=api.FP32, schedule=api.WAVEFRONT, inflight=64)
    assert st.error_flags == 0 and a[1:].sum() > 0
