"""Host side of the dose server: on a machine without a GPU, creation
builds the tables and then fails loudly at the device; bad arguments, null
handles included, are refused before any device call."""

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


def test_server_calls_refuse_null_arguments(native):
    """Field and beamlet submissions and waits check their arguments before
    touching a server, so a null server is an argument error, not a crash."""
    import ctypes as C

    L = N.lib()
    jid = C.c_longlong()
    assert L.omc_server_submit(None, None, C.byref(jid)) == 1
    assert L.omc_server_submit_dij(None, None, None, None, 0.0, 0, C.byref(jid)) == 1
    out = C.POINTER(N.Dij_t)()
    assert L.omc_server_wait_dij(None, 1, 0.0, C.byref(out), None) == 1
    r = C.c_double()
    assert L.omc_measure_atomic_rate(0, 0, C.byref(r)) == 1
