"""omc_matrad_dij, the C-ABI replacement of the matRad front end's
mexFunction (ucodes/omc_matrad/omc_matrad.c:1258-1530): matRad's inputs in,
the reference's sparse dij out."""

import os

import numpy as np
import pytest
from cases import dij_case
from conftest import GOLDEN

from ompmc_gb300 import _native as N
from ompmc_gb300 import api


def test_missing_inputs_are_refused(native, tmp_path):
    _, ph, bl, opts, _, _ = dij_case("dij_slab", str(tmp_path / "a"))
    bad = dict(opts)
    bad["pegsFile"] = ""
    with pytest.raises(N.OmcError) as e:
        api.matrad_dij(ph, bl, bad)
    assert e.value.status == 1
    bad = dict(opts)
    bad["nBatches"] = 0
    with pytest.raises(N.OmcError) as e:
        api.matrad_dij(ph, bl, bad)
    assert e.value.status == 1


def test_host_chain_runs_up_to_the_device(native, tmp_path):
    """On a machine without a GPU the tables, regions and source are built
    from matRad's inputs and the call stops at engine creation."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    _, ph, bl, opts, _, _ = dij_case("dij_slab", str(tmp_path / "b"))
    with pytest.raises(N.OmcError) as e:
        api.matrad_dij(ph, bl, opts)
    assert e.value.status == 7 and "CUDA" in str(e.value)
    bad = dict(opts)
    bad["spectrumFile"] = str(tmp_path / "nowhere.spectrum")
    with pytest.raises(N.OmcError) as e:
        api.matrad_dij(ph, bl, bad)
    assert e.value.status == 2


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["dij_slab", "dij_split"])
def test_matrad_entry_reproduces_reference(name, native, tmp_path):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    _, ph, bl, opts, _, _ = dij_case(name, str(tmp_path / name))
    col, rows, vals = api.matrad_dij(ph, bl, opts, precision=api.FP64, serial=1)
    np.testing.assert_array_equal(col, g["jc"])
    np.testing.assert_array_equal(rows, g["ir"])
    np.testing.assert_allclose(vals, g["pr"], rtol=1e-7, atol=0)


@pytest.mark.gpu
def test_matrad_entry_fp32_many_lanes(native, tmp_path):
    _, ph, bl, opts, _, _ = dij_case("dij_slab", str(tmp_path / "f"), ncase=4000, nbatch=2)
    col, rows, vals = api.matrad_dij(ph, bl, opts, precision=api.FP32)
    assert len(col) == bl.n + 1 and col[-1] == len(vals) > 0
    assert np.all(np.diff(col) > 0)
    for j in range(bl.n):
        r = rows[col[j]:col[j + 1]]
        assert np.all(np.diff(r) > 0)  # ascending rows within a column
