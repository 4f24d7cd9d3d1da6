"""Location of the physics data files the engine reads.

The engine reads ompMC's data files in their own formats: a pegs4 medium
file, ``pgs4form.dat``, ``xcom_{photo,rayleigh,pair,triplet}.data``,
``msnew.data`` and ``spinms.data``.  A user points the ``.inp`` keys at their
own copies.  For tests and benchmarks the files are staged once into
``ompmc_gb300/data/staged/`` (not version controlled) from a reference tree
given by the ``OMC_REFERENCE_DATA`` environment variable, else a checkout
named ``reference`` beside this repository, and ``spinms.data`` is written
by :mod:`ompmc_gb300.spinms` because the reference does not ship it.
"""

from __future__ import annotations

import os
import shutil

from . import spinms

HERE = os.path.dirname(os.path.abspath(__file__))
STAGED = os.path.join(HERE, "data", "staged")
_DEFAULT_REF = os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

PEGS_FILES = ("700icru.pegs4dat", "pgs4form.dat")
DATA_FILES = ("xcom_photo.data", "xcom_rayleigh.data", "xcom_pair.data", "xcom_triplet.data",
              "msnew.data")


def reference_root():
    root = os.environ.get("OMC_REFERENCE_DATA", _DEFAULT_REF)
    return root if os.path.isdir(os.path.join(root, "pegs4")) else None


def stage(force: bool = False) -> str:
    """Stage the data files (copy from the reference tree when it is present,
    write spinms.data) and return the staged root."""
    os.makedirs(os.path.join(STAGED, "pegs4"), exist_ok=True)
    os.makedirs(os.path.join(STAGED, "data"), exist_ok=True)
    ref = reference_root()
    if ref is not None:
        for name in PEGS_FILES:
            dst = os.path.join(STAGED, "pegs4", name)
            if force or not os.path.exists(dst):
                shutil.copyfile(os.path.join(ref, "pegs4", name), dst)
        for name in DATA_FILES:
            dst = os.path.join(STAGED, "data", name)
            if force or not os.path.exists(dst):
                shutil.copyfile(os.path.join(ref, "data", name), dst)
    spin = os.path.join(STAGED, "data", "spinms.data")
    if force or not os.path.exists(spin):
        spinms.write_spin_neutral(spin)
    missing = [p for p in paths().values() if not os.path.exists(p)]
    if missing:
        raise FileNotFoundError("physics data missing (no reference tree to stage from): "
                                + ", ".join(missing))
    return STAGED


def paths():
    return {
        "pegs": os.path.join(STAGED, "pegs4", "700icru.pegs4dat"),
        "pgs4form": os.path.join(STAGED, "pegs4", "pgs4form.dat"),
        "data_folder": os.path.join(STAGED, "data") + os.sep,
        "spinms": os.path.join(STAGED, "data", "spinms.data"),
    }


def available() -> bool:
    return all(os.path.exists(p) for p in paths().values())
