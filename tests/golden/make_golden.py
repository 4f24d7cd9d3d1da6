"""Generate the golden fixtures of tests/golden/ from the UNMODIFIED reference.

Runs the reference built by oracle/Makefile (`make -C oracle ref`, which
needs the reference source tree) through oracle/ref_harness.c and stores:

  ranmar.npz        first RANMAR_N numbers (24-bit integers) of each seed pair
                    in tests.cases.RANMAR_SEEDS, from omc_random.c
  tables.json       SHA-256 of every interaction table the reference builds
                    for the four-medium slab case (initMediaData)
  dose_<case>.npz   raw batch sums accum_endep / accum_endep2 and the source
                    energy of the reference's serial build for each case in
                    tests.cases.CASES
  <dij case>.npz    the sparse dose-influence matrix (jc, ir, pr) the
                    reference's omc_matrad front end returns (serial build,
                    run outside MATLAB by oracle/matrad_harness.c) for each
                    case in tests.cases.DIJ_CASES

Usage:  python tests/golden/make_golden.py
"""

from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cases import CASES, DIJ_CASES, RANMAR_N, RANMAR_SEEDS, dij_case, write_case  # noqa: E402

from ompmc_gb300 import data  # noqa: E402
from oracle import binding as O  # noqa: E402

# Arrays the reference never initialises in full; compared only where set.
UNSET = {"rayleigh.b_array", "rayleigh.c_array"}


def table_digests(d):
    out = {}
    for k, v in sorted(d.items()):
        if k in UNSET:
            v = v.reshape(-1, 100)[:, :99]
        out[k] = hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()
    return out


def main():
    if not (O.ref_available() and O.ref_matrad_available()):
        raise SystemExit("reference not built: run `make -C oracle ref` where the reference tree is present")
    data.stage()
    with tempfile.TemporaryDirectory() as tmp:
        streams = {f"{a}_{b}": O.ref_ranmar(a, b, RANMAR_N, os.path.join(tmp, "r.bin")) for a, b in RANMAR_SEEDS}
        np.savez_compressed(os.path.join(HERE, "ranmar.npz"), **streams)
        inp = write_case("slab_6mv", tmp)
        tab = O.ref_tables(inp, os.path.join(tmp, "t.bin"))
        with open(os.path.join(HERE, "tables.json"), "w") as f:
            json.dump(table_digests(tab), f, indent=1, sort_keys=True)
        for name in CASES:
            inp = write_case(name, os.path.join(tmp, name))
            d = O.ref_dose(inp, os.path.join(tmp, name + ".bin"))
            np.savez_compressed(os.path.join(HERE, f"dose_{name}.npz"), accum_endep=d["accum_endep"],
                                accum_endep2=d["accum_endep2"], ensrc=d["ensrc"], nperbatch=d["nperbatch"],
                                nbatch=d["nbatch"])
            print(name, "ensrc", d["ensrc"][0], "edep", d["accum_endep"][1:].sum())
        for name in DIJ_CASES:
            d = os.path.join(tmp, name)
            _, ph, bl, opts, _, _ = dij_case(name, d)
            jc, ir, pr = O.ref_matrad(os.path.join(d, "ref"), ph, bl, opts)
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), jc=jc, ir=ir, pr=pr)
            print(name, "beamlets", bl.n, "nnz", len(pr))


if __name__ == "__main__":
    main()
