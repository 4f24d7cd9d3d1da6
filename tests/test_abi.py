"""The C-ABI library loads and exports every function include/omc_gpu.h
declares (no GPU calls)."""

import os
import re

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "omc_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(omc_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("omc_engine_run", "omc_engine_create", "omc_tables_build", "omc_phantom_read",
                 "omc_source_build", "omc_regions_build", "omc_write_3ddose", "omc_gpu_ranmar"):
        assert must in names


def test_library_exports_every_declared_symbol(native):
    missing = [n for n in declared_functions() if not hasattr(native, n)]
    assert not missing, missing


def test_library_is_the_in_tree_build(native):
    from ompmc_gb300 import _native

    assert os.path.exists(_native.LIB_PATH)
    assert _native.LIB_PATH.startswith(ROOT)
