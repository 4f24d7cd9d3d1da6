"""The omc_dosxyz command-line front end: same command line, .inp keys and
.3ddose output as the reference's (ucodes/omc_dosxyz/omc_dosxyz.c:1075-1300,
outputResults :801-886), with the history loop on the GPU."""

import os
import subprocess

import numpy as np
import pytest
from cases import write_case
from conftest import GOLDEN

from ompmc_gb300 import api, build


def cli():
    return build.BIN


def read_3ddose(path):
    """Parse a .3ddose file: dims, bounds, dose and uncertainty (x fastest)."""
    tok = open(path).read().split()
    nx, ny, nz = (int(t) for t in tok[:3])
    pos = 3
    bounds = []
    for n in (nx, ny, nz):
        bounds.append(np.array([float(t) for t in tok[pos:pos + n + 1]]))
        pos += n + 1
    nv = nx * ny * nz
    dose = np.array([float(t) for t in tok[pos:pos + nv]])
    unc = np.array([float(t) for t in tok[pos + nv:pos + 2 * nv]])
    assert pos + 2 * nv == len(tok)
    return (nx, ny, nz), bounds, dose, unc


def test_usage_and_missing_input_fail_loudly(native, tmp_path):
    r = subprocess.run([cli()], capture_output=True, text=True)
    assert r.returncode != 0 and "usage" in r.stderr
    r = subprocess.run([cli(), "-i", str(tmp_path / "absent"), "-o", "x"], capture_output=True, text=True)
    assert r.returncode != 0 and "Unable to open file" in r.stderr


def test_missing_key_is_reported(native, tmp_path):
    (tmp_path / "bad.inp").write_text("ncase = 10\nnbatch = 2\n")
    r = subprocess.run([cli(), "-i", str(tmp_path / "bad"), "-o", "x"], capture_output=True, text=True)
    assert r.returncode != 0 and "phantom file" in r.stderr


def test_one_batch_is_refused_before_any_device_call(native, tmp_path):
    """accumulateResults divides by nbatch - 1; the command line refuses
    nbatch = 1 right after reading the input, before the engine exists."""
    inp = write_case("water_mono", str(tmp_path / "one"), ncase=100, nbatch=1)
    r = subprocess.run([cli(), "-i", inp, "-o", "x"], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "at least 2" in r.stderr, r.stderr


@pytest.mark.gpu
def test_serial_run_writes_the_reference_3ddose(native, tmp_path):
    """--serial --fp64 follows the reference's serial build: the .3ddose
    equals the one accumulateResults/outputResults make from the reference's
    own batch tallies (golden fixture), to the printed digits."""
    name = "slab_6mv"
    inp = write_case(name, str(tmp_path / name))
    r = subprocess.run([cli(), "-i", inp, "-o", "cli_out", "--serial", "--fp64", "--verbose"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Fraction of incident energy deposited in the phantom" in r.stdout
    dims, bounds, dose, unc = read_3ddose(str(tmp_path / name / "cli_out.3ddose"))

    prob = api.Problem.from_file(inp)
    g = np.load(os.path.join(GOLDEN, f"dose_{name}.npz"))
    d_ref, u_ref = prob.dose(g["accum_endep"], g["accum_endep2"])
    assert dims == (prob.phantom.s.nx, prob.phantom.s.ny, prob.phantom.s.nz)
    # %e prints 7 significant digits; the trajectories agree to ~1e-10.
    np.testing.assert_allclose(dose, d_ref[1:], rtol=2e-6, atol=1e-6 * d_ref.max())
    np.testing.assert_allclose(unc, u_ref[1:], rtol=1e-4, atol=2e-6)
    assert os.path.getsize(str(tmp_path / name / "cli_out.omct")) > 0


@pytest.mark.gpu
def test_fp32_run_is_statistically_the_fp64_run(native, tmp_path):
    name = "water_mono"
    inp = write_case(name, str(tmp_path / name), ncase=200000, nbatch=20)
    outs = {}
    for prec in ("--fp64", "--fp32"):
        r = subprocess.run([cli(), "-i", inp, "-o", "o" + prec[2:], prec], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        outs[prec] = read_3ddose(str(tmp_path / name / ("o" + prec[2:] + ".3ddose")))
    d64, u64 = outs["--fp64"][2:]
    d32, u32 = outs["--fp32"][2:]
    sel = d64 > 0.2 * d64.max()
    z = (d32[sel] - d64[sel]) / np.sqrt((u32[sel] * d32[sel]) ** 2 + (u64[sel] * d64[sel]) ** 2)
    assert np.mean(np.abs(z) <= 2) > 0.9
    assert abs(d32[sel].sum() / d64[sel].sum() - 1) < 0.01
