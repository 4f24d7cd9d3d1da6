"""Small dose jobs shared by the golden-fixture generator and the tests.

Every case is a complete omc_dosxyz input (phantom, source, cuts, seeds),
written from the seeded generators of ompmc_gb300.workloads, small enough
for the serial oracle to finish in well under a second.
"""

from __future__ import annotations

import os

from ompmc_gb300 import data
from ompmc_gb300 import workloads as W

SLAB4 = ((0.0, 5.0, W.WATER, 1.0), (5.0, 15.0, W.LUNG, 0.26), (15.0, 18.0, W.BONE, 1.85),
         (18.0, 30.0, W.AIR, 0.0012))

# name -> (phantom builder, job keyword arguments)
CASES = {
    # 1.25 MeV parallel beam on water (the plain small configuration, coarse).
    "water_mono": (lambda: W.homogeneous(n=12, vox=2.5),
                   dict(mono_energy=1.25, ncase=2000, ssd=1e8)),
    # Synthetic 6 MV point source on a four-medium slab.
    "slab_6mv": (lambda: W.slab(n=20, vox=1.5, layers=SLAB4),
                 dict(spectrum="6mv", ncase=2000, ssd=100.0)),
    # 5 MeV electron pencil beam.
    "electron_pencil": (lambda: W.homogeneous(n=12, vox=0.5),
                        dict(mono_energy=5.0, charge=-1, collimator=(0.0, 0.0, 0.0, 0.0), ncase=500, ssd=100.0)),
    # 5 MeV positrons, 2x2 cm field.
    "positron_field": (lambda: W.homogeneous(n=12, vox=0.5),
                       dict(mono_energy=5.0, charge=1, collimator=(-1.0, 1.0, -1.0, 1.0), ncase=500, ssd=100.0)),
    # Photon splitting (nsplit = 10) with the 6 MV slab.
    "slab_split10": (lambda: W.slab(n=20, vox=1.5, layers=SLAB4),
                     dict(spectrum="6mv", ncase=1000, ssd=100.0, nsplit=10)),
    # 250 kVp spectrum on the slab (photo-electric dominated).
    "slab_250kvp": (lambda: W.slab(n=20, vox=1.5, layers=SLAB4),
                    dict(spectrum="250kvp", ncase=2000, ssd=100.0)),
}


def write_case(name: str, directory: str, ncase: int | None = None, nbatch: int = 10, seeds=(97, 33),
               nsplit: int | None = None) -> str:
    """Write the case's .egsphant/.spectrum/.inp into directory; returns the
    input path without the .inp extension."""
    builder, kw = CASES[name]
    kw = dict(kw)
    os.makedirs(directory, exist_ok=True)
    P = data.paths()
    ph = builder()
    phant = os.path.join(directory, name + ".egsphant")
    W.write_egsphant(ph, phant)
    spec = kw.pop("spectrum", None)
    spectrum_file = None
    if spec == "6mv":
        spectrum_file = W.write_spectrum(os.path.join(directory, name + ".spectrum"), "synthetic 6 MV",
                                         *W.spectrum_6mv())
    elif spec == "250kvp":
        spectrum_file = W.write_spectrum(os.path.join(directory, name + ".spectrum"), "synthetic 250 kVp",
                                         *W.spectrum_250kvp())
    if ncase is not None:
        kw["ncase"] = ncase
    if nsplit is not None:
        kw["nsplit"] = nsplit
    job = W.Job(phant, P["pegs"], P["pgs4form"], P["data_folder"], directory + os.sep,
                spectrum_file=spectrum_file, nbatch=nbatch, seeds=seeds, **kw)
    return job.write(os.path.join(directory, name))


RANMAR_SEEDS = [(97, 33), (97, 34), (1802, 9373), (12, 31328), (31328, 1), (5, 17)]
RANMAR_N = 2000


# Beamlet (omc_matrad) cases: name -> (dose case, job keywords, beamlet
# keywords, relative dose threshold).  The reference's matRad front end
# always reads a spectrum file, so both use the synthetic 6 MV spectrum.
DIJ_CASES = {
    "dij_slab": ("slab_6mv", dict(ncase=300, nbatch=3, nsplit=1),
                 dict(gantry_deg=(0.0, 90.0, 51.43), bixel=1.0, field=3.0, radius=1.6), 1e-4),
    "dij_split": ("slab_6mv", dict(ncase=200, nbatch=2, nsplit=3),
                  dict(gantry_deg=(180.0, 308.57), bixel=1.0, field=3.0, radius=1.6), 1e-2),
}


def dij_case(name: str, directory: str, ncase: int | None = None, nbatch: int | None = None, seeds=(97, 33)):
    """Write the dose case behind a beamlet case; returns (input path
    without .inp, phantom, beamlets, mcOpt fields for the reference's
    matRad front end, relative threshold, nsplit)."""
    from ompmc_gb300 import workloads as W2

    base, job, bkw, thr = DIJ_CASES[name]
    ncase = job["ncase"] if ncase is None else ncase
    nbatch = job["nbatch"] if nbatch is None else nbatch
    inp = write_case(base, directory, ncase=ncase, nbatch=nbatch, seeds=seeds, nsplit=job["nsplit"])
    ph = CASES[base][0]()
    zc = 0.5 * (ph.zb[0] + ph.zb[-1])
    bl = W2.beamlets(iso=(0.3, -0.2, zc), sad=100.0, **bkw)
    P = data.paths()
    opts = dict(nHistories=ncase, nBatches=nbatch, nSplit=job["nsplit"],
                spectrumFile=os.path.join(directory, base + ".spectrum"), monoEnergy=1.25, charge=0,
                global_ecut=0.7, global_pcut=0.01, randomSeeds=list(seeds), pegsFile=P["pegs"],
                pgs4formFile=P["pgs4form"], dataFolder=P["data_folder"], outputFolder=directory + os.sep,
                relDoseThreshold=thr, verbose=0)
    return inp, ph, bl, opts, thr, job["nsplit"]


def run_seeds(i: int, base=(5003, 7)):
    """Seed pair of repeat i of a run: its lane streams start 2^20 streams
    after repeat i-1's, so repeats never share a stream (a launch seeds at
    most about 10^5 lanes).  Adjacent pairs such as (61 + i, 5) would not do:
    lane k of a run is stream k of its pair, so two such runs share most of
    their streams."""
    from ompmc_gb300 import api

    return api.stream_seeds(base[0], base[1], (i + 1) << 20)
