"""The oracle is pinned against the reference's own outputs (golden
fixtures made by tests/golden/make_golden.py from the unmodified reference),
and, where the reference was built here, against the live reference."""

import json
import os

import numpy as np
import pytest
from cases import CASES, DIJ_CASES, RANMAR_N, RANMAR_SEEDS, dij_case, write_case
from conftest import GOLDEN

from ompmc_gb300 import _native as N
from ompmc_gb300 import workloads as W


def test_ranmar_matches_reference_streams(oracle):
    g = np.load(os.path.join(GOLDEN, "ranmar.npz"))
    for a, b in RANMAR_SEEDS:
        np.testing.assert_array_equal(oracle.ranmar(a, b, RANMAR_N), g[f"{a}_{b}"], err_msg=f"seeds {a} {b}")


def test_ranmar_invalid_seeds_fall_back_like_reference(oracle):
    # omc_random.c:75-82: out-of-range seeds become Marsaglia's defaults.
    np.testing.assert_array_equal(oracle.ranmar(0, 99999, 50), oracle.ranmar(1802, 9373, 50))


@pytest.mark.parametrize("name", sorted(CASES))
def test_serial_dose_bit_exact_with_reference(name, oracle, problem_factory):
    """Serial oracle == reference serial build, bit for bit (same seeds,
    same history order, same libm on this host).  On another host
    architecture libm may round differently, so there the comparison is to
    the last few ulps."""
    g = np.load(os.path.join(GOLDEN, f"dose_{name}.npz"))
    prob = problem_factory(name)
    a, a2, res = oracle.run(prob, nthreads=1)
    import platform

    if platform.machine() == "x86_64":
        np.testing.assert_array_equal(a, g["accum_endep"])
        np.testing.assert_array_equal(a2, g["accum_endep2"])
        assert res.ensrc == g["ensrc"][0]
    else:
        np.testing.assert_allclose(a[1:].sum(), g["accum_endep"][1:].sum(), rtol=1e-6)
        np.testing.assert_allclose(res.ensrc, g["ensrc"][0], rtol=1e-9)


def test_tables_match_reference_digests(native, problem_factory):
    import hashlib

    from oracle.binding import read_omct

    prob = problem_factory("slab_6mv")
    import tempfile

    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "t.bin")
        prob.dump_tables(path)
        mine = read_omct(path)
    with open(os.path.join(GOLDEN, "tables.json")) as f:
        ref = json.load(f)
    checked = 0
    for k, digest in ref.items():
        if k not in mine:
            continue  # geometry/source entries of the harness dump
        v = mine[k]
        if k in ("rayleigh.b_array", "rayleigh.c_array"):
            v = v.reshape(-1, 100)[:, :99]  # the reference never sets entry 99
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == digest, k
        checked += 1
    assert checked >= 80


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "ref_harness")),
                    reason="reference not built on this machine")
def test_live_reference_tables_and_dose(oracle, problem_factory, tmp_path):
    """Against the live reference: every table and a fresh dose run with
    other seeds and history count."""
    from oracle.binding import read_omct

    inp = write_case("slab_6mv", str(tmp_path), ncase=3000, seeds=(12, 345))
    ref = oracle.ref_tables(inp, str(tmp_path / "ref.bin"))
    from ompmc_gb300 import api

    prob = api.Problem.from_file(inp)
    prob.dump_tables(str(tmp_path / "mine.bin"))
    mine = read_omct(str(tmp_path / "mine.bin"))
    for k, v in mine.items():
        r = ref[k]
        if k in ("rayleigh.b_array", "rayleigh.c_array"):
            r, v = r.reshape(-1, 100)[:, :99], v.reshape(-1, 100)[:, :99]
        np.testing.assert_array_equal(v, r, err_msg=k)
    # region / source arrays of initRegions / initSource
    rg = prob.regions.contents
    n = rg.nreg
    np.testing.assert_array_equal(np.ctypeslib.as_array(rg.med, (n,)), ref["region.med"])
    np.testing.assert_array_equal(np.ctypeslib.as_array(rg.rhof, (n,))[1:], ref["region.rhof"][1:])
    np.testing.assert_array_equal(np.ctypeslib.as_array(rg.ecut, (n,))[1:], ref["region.ecut"][1:])
    np.testing.assert_array_equal(np.ctypeslib.as_array(rg.pcut, (n,))[1:], ref["region.pcut"][1:])
    src = prob.source.contents
    np.testing.assert_array_equal(np.array(src.cdfinv1), ref["source.cdfinv1"])
    np.testing.assert_array_equal(np.array(src.cdfinv2), ref["source.cdfinv2"])
    d = oracle.ref_dose(inp, str(tmp_path / "dose.bin"))
    a, a2, res = oracle.run(prob, nthreads=1)
    np.testing.assert_array_equal(a, d["accum_endep"])
    np.testing.assert_array_equal(a2, d["accum_endep2"])


NINE_MEDIA = ((0.0, 3.0, W.WATER, 1.0), (3.0, 6.0, W.LUNG, 0.26), (6.0, 9.0, W.BONE, 1.85),
              (9.0, 12.0, W.AIR, 0.0012), (12.0, 15.0, "PMMA700ICRU", 1.19), (15.0, 18.0, "AL700ICRU", 2.7),
              (18.0, 21.0, "POLYSTY700ICRU", 1.06), (21.0, 24.0, "ICRUTISSUE700ICRU", 1.0),
              (24.0, 30.0, "TI700ICRU", 4.5))


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "ref_harness")),
                    reason="reference not built on this machine")
def test_live_reference_at_the_media_limit(oracle, tmp_path):
    """Nine media, the reference's MXMED (ompmc.h:358): every table of the
    host builders equals the reference's, and a serial oracle run equals
    the reference's batch sums bit for bit.  A tenth medium is refused."""
    from ompmc_gb300 import api, data
    from oracle.binding import read_omct

    ph = W.slab(n=12, vox=2.5, layers=NINE_MEDIA)
    assert len(ph.media) == 9
    W.write_egsphant(ph, str(tmp_path / "nine.egsphant"))
    P = data.paths()
    spec = W.write_spectrum(str(tmp_path / "nine.spectrum"), "synthetic 6 MV", *W.spectrum_6mv())
    job = W.Job(str(tmp_path / "nine.egsphant"), P["pegs"], P["pgs4form"], P["data_folder"], str(tmp_path) + os.sep,
                spectrum_file=spec, ncase=600, nbatch=3, seeds=(7, 8), ssd=100.0)
    inp = job.write(str(tmp_path / "nine"))
    ref = oracle.ref_tables(inp, str(tmp_path / "ref.bin"))
    prob = api.Problem.from_file(inp)
    prob.dump_tables(str(tmp_path / "mine.bin"))
    mine = read_omct(str(tmp_path / "mine.bin"))
    for k, v in mine.items():
        r = ref[k]
        if k in ("rayleigh.b_array", "rayleigh.c_array"):
            r, v = r.reshape(-1, 100)[:, :99], v.reshape(-1, 100)[:, :99]
        np.testing.assert_array_equal(v, r, err_msg=k)
    d = oracle.ref_dose(inp, str(tmp_path / "dose.bin"))
    a, a2, _ = oracle.run(prob, nthreads=1)
    np.testing.assert_array_equal(a, d["accum_endep"])
    np.testing.assert_array_equal(a2, d["accum_endep2"])
    ten = list(NINE_MEDIA) + [(30.0, 31.0, "CU700ICRU", 8.9)]
    ph10 = W.slab(n=12, vox=2.6, layers=tuple(ten))
    with pytest.raises(N.OmcError):
        api.Phantom.from_arrays(ph10.media, ph10.xb, ph10.yb, ph10.zb, ph10.med, ph10.rho)


def test_oracle_threads_statistically_consistent(oracle, problem_factory):
    """The multi-threaded oracle (the reference's OpenMP seeding) agrees with
    the serial one within statistics."""
    prob = problem_factory("water_mono", ncase=20000)
    a1, b1, _ = oracle.run(prob, nthreads=1)
    a4, b4, _ = oracle.run(prob, nthreads=4)
    n = prob.nbatch
    tot1, tot4 = a1[1:].sum(), a4[1:].sum()
    # batch estimate of the total's standard deviation
    assert abs(tot1 - tot4) < 0.03 * tot1


@pytest.mark.parametrize("name", sorted(DIJ_CASES))
def test_serial_dij_bit_exact_with_reference(name, oracle, native, tmp_path):
    """The oracle's beamlet loop == the reference's omc_matrad front end
    (serial build, run outside MATLAB): same columns, rows and values."""
    import platform

    from ompmc_gb300 import api

    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    inp, ph, bl, opts, thr, nsplit = dij_case(name, str(tmp_path / name))
    prob = api.Problem.from_file(inp)
    col, rows, vals, res = oracle.run_dij(prob, bl, rel_threshold=thr)
    if platform.machine() == "x86_64":
        np.testing.assert_array_equal(col, g["jc"])
        np.testing.assert_array_equal(rows, g["ir"])
        np.testing.assert_array_equal(vals, g["pr"])
    else:
        np.testing.assert_allclose(vals.sum(), g["pr"].sum(), rtol=1e-6)
    assert res.histories == bl.n * opts["nHistories"]


@pytest.mark.skipif(not __import__("oracle.binding", fromlist=["x"]).ref_matrad_available(),
                    reason="reference matRad front end not built here")
def test_live_reference_dij_with_uneven_options(oracle, native, tmp_path):
    """Where the reference was built: a third beamlet set with other seeds
    and a zero threshold, live against the reference."""
    from ompmc_gb300 import api

    inp, ph, bl, opts, thr, nsplit = dij_case("dij_slab", str(tmp_path / "live"), ncase=120, nbatch=4,
                                              seeds=(12, 345))
    opts["relDoseThreshold"] = 0.0
    jc, ir, pr = oracle.ref_matrad(str(tmp_path / "live" / "ref"), ph, bl, opts)
    prob = api.Problem.from_file(inp)
    col, rows, vals, _ = oracle.run_dij(prob, bl, rel_threshold=0.0)
    np.testing.assert_array_equal(col, jc)
    np.testing.assert_array_equal(rows, ir)
    np.testing.assert_array_equal(vals, pr)
