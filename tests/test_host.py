"""Host library (no GPU): input file semantics, phantom I/O, regions,
source, batch statistics and the .3ddose writer, each checked against the
reference behaviour it restates."""

import ctypes as C
import os

import numpy as np
import pytest

from ompmc_gb300 import _native as N
from ompmc_gb300 import api
from ompmc_gb300 import workloads as W


def test_input_substring_keys_and_comment_lines(native):
    # omc_utilities.c:79-123: lines containing '#' are skipped, keys match by
    # substring, the first match wins, values keep their spaces.
    text = "ncase  = 1000\n# nbatch = 99\nnbatch = 10 # trailing\nnbatch= 7\nrng seeds = 5 6\n\n   \n"
    inp = api.Input(text=text)
    assert inp.get("ncase").strip() == "1000"
    assert inp.get("nbatch").strip() == "7"  # the '#' line and the commented one are gone
    assert inp.get("seeds") == " 5 6"
    assert inp.get("case") is not None  # substring of "ncase"
    assert inp.get("missing") is None


def test_input_file_appends_extension(native, tmp_path):
    p = tmp_path / "job"
    (tmp_path / "job.inp").write_text("charge = -1\n")
    assert api.Input(str(p)).get("charge").strip() == "-1"
    with pytest.raises(N.OmcError) as e:
        api.Input(str(tmp_path / "absent"))
    assert e.value.status == 2  # OMC_ERR_IO


def test_egsphant_round_trip(native, tmp_path):
    ph = W.ct_like(nx=9, ny=7, nz=5, vox=0.4, nblobs=6, seed=3)
    path = str(tmp_path / "ct.egsphant")
    W.write_egsphant(ph, path)
    p = api.Phantom.read(path)
    assert p.shape == (5, 7, 9)
    assert p.media == ph.media
    np.testing.assert_array_equal(p.density(), ph.rho)
    s = p.s
    np.testing.assert_array_equal(np.ctypeslib.as_array(s.med_index, (ph.nvox,)), ph.med.reshape(-1))
    np.testing.assert_array_equal(np.ctypeslib.as_array(s.xbounds, (10,)), ph.xb)
    # native writer -> native reader
    p.write(str(tmp_path / "again.egsphant"))
    q = api.Phantom.read(str(tmp_path / "again.egsphant"))
    np.testing.assert_array_equal(q.density(), ph.rho)


def test_egsphant_errors(native, tmp_path):
    bad = tmp_path / "bad.egsphant"
    bad.write_text("1\nH2O700ICRU\n0.25\n2 2 2\n0 1 2\n")
    with pytest.raises(N.OmcError) as e:
        api.Phantom.read(str(bad))
    assert e.value.status == 5  # OMC_ERR_FORMAT
    bad.write_text("12\n")
    with pytest.raises(N.OmcError):
        api.Phantom.read(str(bad))


def _egsphant_text(nx, ny, nz, dens_tokens):
    rows = "\n".join("1" * nx for _ in range(ny))
    media = "\n".join(rows + "\n" for _ in range(nz))
    b = lambda n: " ".join(str(0.5 * i) for i in range(n + 1))
    return f"1\nH2O700ICRU\n0.25\n{nx} {ny} {nz}\n{b(nx)}\n{b(ny)}\n{b(nz)}\n{media}\n" + dens_tokens


def test_egsphant_density_block_parsed_in_pieces(native, tmp_path):
    """A density block of several MB is cut at whitespace into one piece per
    thread; the values equal the sequential strtod reading (Python's float
    is correctly rounded too), trailing text after the last voxel is ignored,
    and a block that is short, or holds a token that is not a number before
    its last voxel, is refused as before."""
    nx, ny, nz = 64, 64, 60
    nv = nx * ny * nz
    rng = np.random.default_rng(4)
    vals = rng.uniform(0.0005, 2.5, nv)
    toks = [repr(float(v)) if i % 3 else f"{v:.6e}" for i, v in enumerate(vals)]
    # mixed separators: spaces, tabs, newlines every 7 values
    body = "".join(t + ("\n" if i % 7 == 6 else (" \t" if i % 5 == 0 else " ")) for i, t in enumerate(toks))
    path = tmp_path / "big.egsphant"
    path.write_text(_egsphant_text(nx, ny, nz, body + "\ntrailing words 1.0 x\n"))
    assert path.stat().st_size > 3 << 20
    p = api.Phantom.read(str(path))
    np.testing.assert_array_equal(p.density(), np.array([float(t) for t in toks]).reshape(nz, ny, nx))
    short = tmp_path / "short.egsphant"
    short.write_text(_egsphant_text(nx, ny, nz, " ".join(toks[:-1]) + "\n"))
    with pytest.raises(N.OmcError) as e:
        api.Phantom.read(str(short))
    assert e.value.status == 5
    broken = tmp_path / "broken.egsphant"
    toks2 = list(toks)
    toks2[nv // 2] = "abc"
    broken.write_text(_egsphant_text(nx, ny, nz, " ".join(toks2) + " 1.0\n"))
    with pytest.raises(N.OmcError) as e:
        api.Phantom.read(str(broken))
    assert e.value.status == 5


def test_egsphant_density_tokens_as_fscanf(native, tmp_path):
    """Tokens read as fscanf %lf reads them: a leading '+', hex floats and
    exponents with a sign; a token that only starts with a number ends the
    block."""
    toks = ["+1.5", "0x1p-1", "2.5E+00", "1e-3", "7", "0.1", "3.25e0", "1E1"]
    want = [1.5, 0.5, 2.5, 1e-3, 7.0, 0.1, 3.25, 10.0]
    path = tmp_path / "tok.egsphant"
    path.write_text(_egsphant_text(2, 2, 2, "\n".join(toks) + "\n1.0x junk\n"))
    np.testing.assert_array_equal(api.Phantom.read(str(path)).density().reshape(-1), want)
    path.write_text(_egsphant_text(2, 2, 2, " ".join(toks[:7]) + " 1.0x\n"))
    a = api.Phantom.read(str(path)).density().reshape(-1)  # "1.0x": strtod reads 1.0
    np.testing.assert_array_equal(a, want[:7] + [1.0])
    path.write_text(_egsphant_text(2, 2, 2, " ".join(toks[:6]) + " x 1.0 2.0\n"))
    with pytest.raises(N.OmcError):
        api.Phantom.read(str(path))


def test_from_arrays_matches_file(native, tmp_path):
    ph = W.slab(n=6, vox=5.0)
    W.write_egsphant(ph, str(tmp_path / "s.egsphant"))
    a = api.Phantom.read(str(tmp_path / "s.egsphant"))
    b = api.Phantom.from_arrays(ph.media, ph.xb, ph.yb, ph.zb, ph.med, ph.rho)
    np.testing.assert_array_equal(a.density(), b.density())
    assert a.media == b.media


def _numpy_accumulate(ph, acc, acc2, nhist, nbatch):
    """accumulateResults (omc_dosxyz.c:719-799) in numpy."""
    nz, ny, nx = ph.shape
    e = acc[1:] / nbatch
    e2 = acc2[1:] / nbatch
    with np.errstate(invalid="ignore", divide="ignore"):
        unc = np.where(e != 0.0, np.sqrt((e2 - e * e) / (nbatch - 1)) / e, 0.9999999)
    vol = (np.diff(ph.zb)[:, None, None] * np.diff(ph.yb)[None, :, None] * np.diff(ph.xb)[None, None, :]).reshape(-1)
    dose = np.where(e != 0.0, e * (1.602e-10 / (vol * ph.rho.reshape(-1) * nhist)), 0.0)
    air = ph.rho.reshape(-1) < 0.044
    dose[air] = 0.0
    unc[air] = 0.9999999
    return dose, unc


def test_accumulate_results_matches_numpy(native, problem_factory):
    prob = problem_factory("slab_6mv")
    rng = np.random.default_rng(1)
    n = prob.nreg
    acc = rng.uniform(0, 1, n) * (rng.uniform(0, 1, n) > 0.2)
    acc2 = acc * acc / 10 + rng.uniform(0, 1e-3, n)
    dose, unc = prob.dose(acc, acc2)
    ph = W.slab(n=20, vox=1.5, layers=((0, 5, W.WATER, 1.0), (5, 15, W.LUNG, 0.26), (15, 18, W.BONE, 1.85),
                                       (18, 30, W.AIR, 0.0012)))
    d2, u2 = _numpy_accumulate(ph, acc, acc2, prob.nperbatch, prob.nbatch)
    np.testing.assert_allclose(dose[1:], d2, rtol=1e-14)
    np.testing.assert_allclose(unc[1:], u2, rtol=1e-12)


def test_3ddose_format(native, problem_factory, tmp_path):
    prob = problem_factory("water_mono")
    n = prob.nreg
    dose = np.linspace(0, 1e-12, n)
    unc = np.linspace(0, 0.5, n)
    path = str(tmp_path / "out.3ddose")
    prob.write_3ddose(path, dose, unc)
    lines = open(path).read().split("\n")
    assert lines[0] == "   12   12   12"  # "%5d%5d%5d"
    assert lines[1].split()[0] == "-15.000000"  # "%f " bounds
    vals = lines[4].split()
    assert len(vals) == n - 1 and vals[1] == f"{dose[2]:e}"
    assert lines[5].split()[3] == f"{unc[4]:f}"


def test_regions_and_cutoffs(native, problem_factory):
    prob = problem_factory("slab_6mv")
    rg = prob.regions.contents
    med = np.ctypeslib.as_array(rg.med, (rg.nreg,))
    ecut = np.ctypeslib.as_array(rg.ecut, (rg.nreg,))
    pcut = np.ctypeslib.as_array(rg.pcut, (rg.nreg,))
    assert med[0] == -1 and ecut[0] == 0.0
    assert set(np.unique(med[1:])) == {0, 1, 2, 3}
    np.testing.assert_array_equal(ecut[1:], 0.7)  # global ecut == pegs AE
    np.testing.assert_array_equal(pcut[1:], 0.01)


def test_source_spectrum_inverse_cdf(native, problem_factory):
    """initSource (omc_dosxyz.c:444-503): cdfinv1 holds the lower bin edge,
    cdfinv2 the bin width, on 1000 equal-probability cells."""
    prob = problem_factory("slab_6mv")
    s = prob.source.contents
    assert s.spectrum == 1 and s.deltak == 1000
    c1 = np.array(s.cdfinv1)
    c2 = np.array(s.cdfinv2)
    np.testing.assert_allclose(c2, 0.25)
    assert c1[0] == 0.0 and np.all(np.diff(c1) >= 0) and c1[-1] <= 5.75
    e, w = W.spectrum_6mv()[1:]
    cdf = np.cumsum(w) / w.sum()
    for k in (10, 400, 900):
        i = np.searchsorted(cdf, k / 1000.0)
        assert c1[k] == (e[i - 1] if i else 0.0)


def test_missing_medium_reported(native, tmp_path):
    from ompmc_gb300 import data

    P = data.paths()
    ph = W.homogeneous(n=3, vox=1.0, medium="NOSUCHMEDIUM")
    W.write_egsphant(ph, str(tmp_path / "p.egsphant"))
    job = W.Job(str(tmp_path / "p.egsphant"), P["pegs"], P["pgs4form"], P["data_folder"], str(tmp_path) + "/")
    with pytest.raises(N.OmcError) as e:
        api.Problem.from_file(job.write(str(tmp_path / "j")))
    assert e.value.status == 4 and "NOSUCHMEDIUM" in str(e.value)


def test_missing_data_file_reported(native, tmp_path):
    from ompmc_gb300 import data

    P = data.paths()
    ph = W.homogeneous(n=3, vox=1.0)
    W.write_egsphant(ph, str(tmp_path / "p.egsphant"))
    job = W.Job(str(tmp_path / "p.egsphant"), P["pegs"], P["pgs4form"], str(tmp_path) + "/", str(tmp_path) + "/")
    with pytest.raises(N.OmcError) as e:
        api.Problem.from_file(job.write(str(tmp_path / "j")))
    assert e.value.status == 2 and "xcom_photo.data" in str(e.value)


def test_stream_seed_rule(native):
    # Stream k uses (ixx, jxx + k) like the reference's OpenMP threads
    # (omc_random.c:72) while jxx + k <= 30081, and then continues with the
    # next unused stream: initRandom reads jxx through (jxx/169 % 178,
    # jxx % 169), so jxx = 30082 + r is the stream of jxx = r.
    assert api.stream_seeds(97, 33, 0) == (97, 33)
    assert api.stream_seeds(97, 33, 5) == (97, 38)
    assert api.stream_seeds(97, 30081, 1) == (98, 30082)
    assert api.stream_seeds(97, 30081, 2) == (98, 1)
    assert api.stream_seeds(97, 31328, 0) == (97, 31328)
    assert api.stream_seeds(97, 31328, 1) == (97, 1247)  # 31328 is the stream of 1246
    assert api.stream_seeds(31328, 30081, 2) == (1, 1)
    # Distinct streams, not only distinct pairs, over a whole device's lanes
    # and across jobs placed 2^20 streams apart.
    def stream(p):
        return (p[0], p[1] % 30082)
    ks = list(range(0, 400000, 3)) + [(1 << 20) * j + k for j in range(1, 4) for k in range(0, 100000, 11)]
    keys = {stream(api.stream_seeds(97, 33, k)) for k in ks}
    assert len(keys) == len(ks)
    # Composition: stream k of stream K's pair is stream K + k.
    for K in (0, 5, 30076, 31328, 1 << 20):
        for k in (0, 1, 7, 30082):
            assert stream(api.stream_seeds(*api.stream_seeds(97, 33, K), k)) == stream(api.stream_seeds(97, 33, K + k))


def test_ranmar_jxx_alias_is_the_reference_generator(oracle):
    # The reason for the rule above, on the oracle's generator (the
    # reference's initRandom): jxx = 30082 + r and jxx = r draw the same
    # numbers, and the rule's next stream does not.
    a = oracle.ranmar(97, 31328, 200)
    assert np.array_equal(a, oracle.ranmar(97, 1246, 200))
    assert not np.array_equal(oracle.ranmar(*api.stream_seeds(97, 31328, 1), 200), a)


def test_3ddose_text_is_printf_byte_for_byte(native, tmp_path, problem_factory):
    """The parallel .3ddose writer produces exactly the reference's
    fprintf("%e ") / fprintf("%f ") text (outputResults,
    omc_dosxyz.c:842-879), edge values included."""
    import numpy as np

    prob = problem_factory("slab_6mv")
    rng = np.random.default_rng(3)
    n = prob.nreg
    d = rng.random(n) * 10.0 ** rng.integers(-300, 300, n)
    u = rng.random(n) * 10.0 ** rng.integers(-9, 17, n)
    d[1:6] = [0.0, -0.0, 5e-324, 0.5e-6, 9.9999995e-5]
    u[1:4] = [0.9999999, 0.0000005, 1e17]
    path = str(tmp_path / "x.3ddose")
    prob.write_3ddose(path, d, u)
    lines = open(path).read().split("\n")
    s = prob.phantom.s
    assert lines[0] == "%5d%5d%5d" % (s.nx, s.ny, s.nz)
    assert lines[4] == "".join("%e " % x for x in d[1:])
    assert lines[5] == "".join("%f " % x for x in u[1:])


def test_server_round_size_rule(native):
    """The dose server's round size: a configured size as given; else 4e6
    while more than two jobs are resident, and with one or two a quarter of
    their histories left, at most four times the shortest job's, within
    [4e6, 3.2e7]."""
    from ompmc_gb300 import _native as N

    f = N.lib().omc_server_round_histories
    assert f(150000, 10**9, 10**5, 1) == 150000
    assert f(0, 10**9, 10**8, 3) == 4_000_000              # busy: short rounds
    assert f(0, 10**8, 10**8, 1) == 25_000_000             # one large job: a quarter of it
    assert f(0, 10**9, 10**9, 2) == 32_000_000             # capped
    assert f(0, 10**8 + 10**6, 10**6, 2) == 4_000_000      # a small job resident: 4x its rest, at least 4e6
    assert f(0, 6 * 10**7, 3 * 10**6, 2) == 12_000_000
    assert f(0, 10**5, 10**5, 1) == 4_000_000              # floor
    assert f(0, 0, -1, 0) == 4_000_000
