"""Resident jobs and the dose server (continuous batching), through the C
ABI: a job advanced in rounds of uneven size gives the batch sums
omc_engine_run gives; a job gives the same result alone and in a mix of
jobs with other phantoms, sources and particle kinds; admission respects
the device-memory budget; small jobs overtake large ones; beamlet (dij)
jobs queued among field jobs give the dij omc_engine_run_dij gives."""

import ctypes as C
import dataclasses
import time

import numpy as np
import pytest
from cases import SLAB4
from stats import compare, consistent

from ompmc_gb300 import _native as N
from ompmc_gb300 import api, data

pytestmark = pytest.mark.gpu

MEDIA = [m for _, _, m, _ in SLAB4]  # H2O, LUNG, ICRPBONE, AIR


def data_text():
    P = data.paths()
    return f"pegs file = {P['pegs']}\npgs4form file = {P['pgs4form']}\ndata folder = {P['data_folder']}\n"


def same_distribution(a, a2, b, b2, nbatch, n):
    c = compare(a, a2, b, b2, nbatch)
    assert c["n"] >= 10, c
    assert consistent(c), c
    assert abs(c["etot_rel"]) < 6.0 / np.sqrt(n), c


def test_job_rounds_match_engine_run(engine, problem_factory):
    prob = problem_factory("slab_6mv", ncase=200000, nbatch=20, seeds=(5, 7))
    engine.load(prob)
    ref, ref2, st = engine.run(precision=api.FP32)
    L = N.lib()
    job = C.c_void_p()
    g = lambda k: float(prob.input.get(k))
    N.check(L.omc_engine_job_add(engine._h, prob.phantom._p, prob.regions, prob.source, prob.nperbatch, prob.nbatch,
                                 api.FP32, C.byref(job)))
    try:
        cfg = api.Engine.config(1, 1, seeds=(41, 43), precision=api.FP32)
        total = prob.nperbatch * prob.nbatch
        for k, q in enumerate((3, 70001, 29996, 100000)):  # rounds cut across batch boundaries
            cfg.continue_streams = 1 if k else 0
            jobs = (C.c_void_p * 1)(job)
            quota = (C.c_longlong * 1)(q)
            N.check(L.omc_engine_job_round(engine._h, jobs, quota, 1, C.byref(cfg), None))
        assert L.omc_job_done(job) == total
        a = np.zeros(prob.nreg)
        a2 = np.zeros(prob.nreg)
        ens = C.c_double()
        N.check(L.omc_engine_job_result(engine._h, job, api._dptr(a), api._dptr(a2), C.byref(ens)))
    finally:
        L.omc_engine_job_remove(engine._h, job)
    same_distribution(a, a2, ref, ref2, prob.nbatch, total)
    assert ens.value == pytest.approx(st.ensrc, rel=4.0 / np.sqrt(total))


def test_job_same_alone_and_in_mix(native, problem_factory):
    a_prob = problem_factory("water_mono", ncase=200000, nbatch=20, seeds=(1, 2))
    others = [problem_factory("slab_6mv", ncase=400000, nbatch=10, seeds=(3, 4)),
              problem_factory("slab_250kvp", ncase=300000, nbatch=10, seeds=(5, 6)),
              problem_factory("electron_pencil", ncase=40000, nbatch=10, seeds=(7, 8)),
              problem_factory("positron_field", ncase=40000, nbatch=10, seeds=(9, 10))]
    srv = api.Server(MEDIA, data_text(), precision=api.FP32, round_histories=150000, policy=api.Server.EQUAL_SHARES)
    try:
        alone = srv.wait(srv.submit_problem(a_prob))
        ids = [srv.submit_problem(p) for p in others[:2]]
        mid = srv.submit_problem(a_prob)
        ids += [srv.submit_problem(p) for p in others[2:]]
        mixed = srv.wait(mid)
        rest = [srv.wait(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    n = a_prob.nperbatch * a_prob.nbatch
    assert st.max_round_jobs >= 3, st.max_round_jobs
    assert mixed[2].rounds > 1
    same_distribution(mixed[0], mixed[1], alone[0], alone[1], a_prob.nbatch, n)
    # every job of the mix against its own single-job run on an engine
    eng = api.Engine(0)
    try:
        for p, (a, a2, r) in zip(others, rest):
            eng.load(p)
            ref, ref2, rst = eng.run(precision=api.FP32, seeds=(17, 19))
            same_distribution(a, a2, ref, ref2, p.nbatch, p.nperbatch * p.nbatch)
            assert r.histories == p.nperbatch * p.nbatch
    finally:
        eng.close()


def test_admission_respects_budget(native, problem_factory):
    probs = [problem_factory("water_mono", ncase=20000, nbatch=4, seeds=(11, 12 + i)) for i in range(3)]
    srv = api.Server(MEDIA, data_text(), precision=api.FP32, hbm_budget=1)
    try:
        ids = [srv.submit_problem(p) for p in probs]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert st.max_resident == 1 and st.finished == 3
    assert all(r[2].status == 0 and r[0][1:].sum() > 0 for r in res)
    # arrival order: each job is admitted after the previous one finished
    for (_, _, r0), (_, _, r1) in zip(res, res[1:]):
        assert r1.admit_s >= r0.finish_s - 1e-3


@pytest.mark.parametrize("policy", [0, 1])
def test_small_job_overtakes_large_one(policy, native, problem_factory):
    big = problem_factory("slab_6mv", ncase=4000000, nbatch=10, seeds=(21, 22))
    small = problem_factory("water_mono", ncase=20000, nbatch=10, seeds=(23, 24))
    srv = api.Server(MEDIA, data_text(), precision=api.FP32, round_histories=400000, policy=policy)
    try:
        b = srv.submit_problem(big)
        s = srv.submit_problem(small)
        rs = srv.wait(s)[2]
        rb = srv.wait(b)[2]
    finally:
        srv.close()
    assert rs.finish_s < rb.finish_s
    assert rb.rounds >= 5 and rs.rounds <= 2


def test_unknown_medium_is_refused(native, tmp_path):
    from ompmc_gb300 import workloads as W

    srv = api.Server(["H2O700ICRU"], data_text(), precision=api.FP32)
    try:
        ph = W.slab(n=8, vox=1.0)
        phantom = api.Phantom.from_arrays(ph.media, ph.xb, ph.yb, ph.zb, ph.med, ph.rho)
        src = N.Source_t()
        src.energy = 1.0
        with pytest.raises(N.OmcError) as e:
            srv.submit(phantom, C.pointer(src), 0.7, 0.01, 10, 2)
        assert e.value.status == 4
    finally:
        srv.close()


def column_sums(col, vals):
    return np.array([vals[col[j]:col[j + 1]].sum() for j in range(len(col) - 1)])


def test_beamlet_jobs_beside_field_jobs(engine, problem_factory, tmp_path):
    """Beamlet jobs queued among a field job share its rounds (launches):
    each gives the dij that omc_engine_run_dij gives for the beamlets alone
    (per-beamlet integral doses over 16 jobs against 16 engine runs on
    disjoint streams, within their spread; the same CSC shape), and the
    field job, whose rounds carried the beamlet jobs' histories, gives the
    dose omc_engine_run gives."""
    from cases import dij_case, run_seeds

    inp, _, bl, _, _, _ = dij_case("dij_slab", str(tmp_path / "d"), ncase=1000, nbatch=2)
    prob = api.Problem.from_file(inp)
    field = problem_factory("slab_6mv", ncase=2000000, nbatch=10, seeds=(3, 4))
    g = lambda key: float(prob.input.get(key))
    k = 16
    srv = api.Server(MEDIA, data_text(), precision=api.FP32, round_histories=100000)
    try:
        fid = srv.submit_problem(field)
        t0 = time.perf_counter()
        while srv.stats().rounds < 1 and time.perf_counter() - t0 < 60:
            time.sleep(0.001)
        ids = [srv.submit_dij(prob.phantom, prob.source, g("global ecut"), g("global pcut"), bl, 1000, 2,
                              rel_threshold=0.0) for _ in range(k)]
        with pytest.raises(N.OmcError):
            srv.wait(ids[0])  # a beamlet job is collected with wait_dij
        outs = [srv.wait_dij(i) for i in ids]
        fa, fa2, fr = srv.wait(fid)
        st = srv.stats()
    finally:
        srv.close()
    for col, rows, vals, r in outs:
        assert r.status == 0 and r.rounds >= 1
        assert r.histories == bl.n * 2000
        assert len(col) == bl.n + 1 and col[-1] == len(rows) == len(vals)
        assert np.all(np.diff(col) > 0) and rows.max() < prob.nreg - 1
    assert fr.rounds > 10 and st.finished == k + 1
    assert st.max_round_jobs >= 2  # beamlet and field histories in one launch
    assert fr.finish_s > min(o[3].finish_s for o in outs)  # beamlet jobs finished while the field job ran
    srv_sums = np.stack([column_sums(o[0], o[2]) for o in outs])
    engine.load(prob)
    engine.set_beamlets(bl)
    eng_sums = []
    for i in range(k):
        col, rows, vals, est = engine.run_dij(rel_threshold=0.0, precision=api.FP32, seeds=run_seeds(i))
        eng_sums.append(column_sums(col, vals))
    eng_sums = np.stack(eng_sums)
    z = (srv_sums.mean(0) - eng_sums.mean(0)) / np.sqrt(srv_sums.var(0, ddof=1) / k + eng_sums.var(0, ddof=1) / k)
    assert np.mean(np.abs(z) < 3) > 0.9, z
    assert abs(srv_sums.mean(0).sum() / eng_sums.mean(0).sum() - 1) < 0.02
    # distinct beamlet jobs draw from distinct streams
    assert not np.array_equal(outs[0][2], outs[1][2])
    engine.load(field)
    ref, ref2, _ = engine.run(precision=api.FP32, seeds=(29, 31))
    same_distribution(fa, fa2, ref, ref2, field.nbatch, field.nperbatch * field.nbatch)


def test_beamlet_job_errors(native, tmp_path):
    from cases import dij_case

    inp, _, bl, _, _, _ = dij_case("dij_slab", str(tmp_path / "d"))
    prob = api.Problem.from_file(inp)
    srv = api.Server(MEDIA, data_text(), precision=api.FP32)
    try:
        args = (prob.phantom, prob.source, 0.7, 0.01)
        with pytest.raises(N.OmcError) as e:
            srv.submit_dij(*args, bl, 10, 1, rel_threshold=-1.0)
        assert e.value.status == 1
        with pytest.raises(N.OmcError) as e:
            srv.submit_dij(*args, bl, 10, 1, nhist=np.zeros(bl.n, np.int64))
        assert e.value.status == 1
        bad = dataclasses.replace(bl, ibeam=np.full(bl.n, 7, np.int32))
        with pytest.raises(N.OmcError) as e:
            srv.submit_dij(*args, bad, 10, 1)
        assert e.value.status == 1
    finally:
        srv.close()
