"""Host side of the dose server: on a machine without a GPU, creation
builds the tables and then fails loudly at the device; bad arguments are
refused before any device call."""

import pytest

from ompmc_gb300 import _native as N
from ompmc_gb300 import api, data


def _data_text():
    P = data.paths()
    return f"pegs file = {P['pegs']}\npgs4form file = {P['pgs4form']}\ndata folder = {P['data_folder']}\n"


def test_server_needs_a_device(native):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(N.OmcError) as e:
        api.Server(["H2O700ICRU"], _data_text())
    assert e.value.status == 7


def test_server_arguments_checked(native):
    with pytest.raises(N.OmcError) as e:
        api.Server(["H2O700ICRU"], _data_text(), precision=5)
    assert e.value.status == 1
    with pytest.raises(N.OmcError) as e:
        api.Server(["NOT_A_MEDIUM"], _data_text())
    assert e.value.status == 4
