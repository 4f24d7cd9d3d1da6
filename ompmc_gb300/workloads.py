"""Synthetic inputs in ompMC's own formats (.egsphant, spectrum, .inp).

No phantom or spectrum file of the benchmark set is available, so every
workload is generated here from a stated, seeded recipe:

* ``homogeneous``: water box (the 1.25 MeV plain case, 60^3 at 0.5 cm);
* ``slab``: z-slabs water / lung (0.26) / ICRP bone (1.85) / water at 2 mm;
* ``ct_like``: density 1 + sum of Gaussian blobs, clipped, thresholded into
  air / lung / water / bone, from a numpy ``default_rng(seed)``;
* spectra: a synthetic 6 MV bremsstrahlung shape and a 250 kVp shape.

File layouts follow the reference readers: ``initPhantom``
(ucodes/omc_dosxyz/omc_dosxyz.c:62-175), ``initSource`` (:368-503) and
``parseInputFile`` (src/omc_utilities.c:63-105).
"""

from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

WATER, LUNG, BONE, AIR = "H2O700ICRU", "LUNG700ICRU", "ICRPBONE700ICRU", "AIR700ICRU"


@dataclass
class Phantom:
    """Voxel phantom; arrays are indexed [z, y, x] (region order)."""

    media: list
    xb: np.ndarray
    yb: np.ndarray
    zb: np.ndarray
    med: np.ndarray  # uint8, 1-based medium number, 0 = vacuum
    rho: np.ndarray  # float64 density

    @property
    def shape(self):
        return self.med.shape

    @property
    def nvox(self):
        return int(self.med.size)


def _bounds(n, vox, lo):
    return lo + vox * np.arange(n + 1, dtype=np.float64)


def homogeneous(n=60, vox=0.5, medium=WATER, rho=1.0, nxyz=None):
    nx, ny, nz = nxyz if nxyz else (n, n, n)
    xb = _bounds(nx, vox, -0.5 * nx * vox)
    yb = _bounds(ny, vox, -0.5 * ny * vox)
    zb = _bounds(nz, vox, 0.0)
    med = np.ones((nz, ny, nx), np.uint8)
    dens = np.full((nz, ny, nx), rho, np.float64)
    return Phantom([medium], xb, yb, zb, med, dens)


def slab(n=150, vox=0.2, layers=((0.0, 5.0, WATER, 1.0), (5.0, 15.0, LUNG, 0.26),
                                 (15.0, 18.0, BONE, 1.85), (18.0, 30.0, WATER, 1.0)), nxyz=None):
    """z-slabs; each layer is (z_lo, z_hi, medium, density) in cm."""
    nx, ny, nz = nxyz if nxyz else (n, n, n)
    xb = _bounds(nx, vox, -0.5 * nx * vox)
    yb = _bounds(ny, vox, -0.5 * ny * vox)
    zb = _bounds(nz, vox, 0.0)
    media = []
    for _, _, m, _ in layers:
        if m not in media:
            media.append(m)
    zc = 0.5 * (zb[:-1] + zb[1:])
    med = np.zeros((nz, ny, nx), np.uint8)
    dens = np.zeros((nz, ny, nx), np.float64)
    for lo, hi, m, rho in layers:
        sel = (zc >= lo) & (zc < hi)
        med[sel] = media.index(m) + 1
        dens[sel] = rho
    return Phantom(media, xb, yb, zb, med, dens)


def ct_like(nx=256, ny=256, nz=128, vox=0.2, nblobs=40, seed=2024):
    """Seeded blob phantom: rho = 1 + sum A exp(-r^2/2 s^2), A~U[-0.9,0.8],
    s~U[5,30] mm, centres uniform; clipped to [0.001, 2]; media by
    thresholds air < 0.2 <= lung < 0.85 <= water < 1.15 <= bone."""
    rng = np.random.default_rng(seed)
    xb = _bounds(nx, vox, -0.5 * nx * vox)
    yb = _bounds(ny, vox, -0.5 * ny * vox)
    zb = _bounds(nz, vox, 0.0)
    xc = 0.5 * (xb[:-1] + xb[1:])
    yc = 0.5 * (yb[:-1] + yb[1:])
    zc = 0.5 * (zb[:-1] + zb[1:])
    amp = rng.uniform(-0.9, 0.8, nblobs)
    sig = rng.uniform(0.5, 3.0, nblobs)  # cm
    cx = rng.uniform(xb[0], xb[-1], nblobs)
    cy = rng.uniform(yb[0], yb[-1], nblobs)
    cz = rng.uniform(zb[0], zb[-1], nblobs)
    rho = np.ones((nz, ny, nx), np.float64)
    for a, s, x0, y0, z0 in zip(amp, sig, cx, cy, cz):
        gx = np.exp(-((xc - x0) ** 2) / (2 * s * s))
        gy = np.exp(-((yc - y0) ** 2) / (2 * s * s))
        gz = np.exp(-((zc - z0) ** 2) / (2 * s * s))
        rho += a * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    rho = np.clip(rho, 0.001, 2.0)
    media = [AIR, LUNG, WATER, BONE]
    med = np.where(rho < 0.2, 1, np.where(rho < 0.85, 2, np.where(rho < 1.15, 3, 4))).astype(np.uint8)
    return Phantom(media, xb, yb, zb, med, rho)


@dataclass
class Beamlets:
    """matRad-style pencil beamlets (the mcSrc fields of omc_matrad):
    bixel k is corner[k] + a*side1[k] + b*side2[k], a, b in [0, 1), at the
    isocentre plane, irradiated from source[ibeam[k]]."""

    ibeam: np.ndarray   # int32 [n], 0-based beam index
    source: np.ndarray  # [nbeams, 3]
    corner: np.ndarray  # [n, 3]
    side1: np.ndarray   # [n, 3]
    side2: np.ndarray   # [n, 3]

    @property
    def n(self):
        return int(len(self.ibeam))


def beamlets(gantry_deg=(0.0,), iso=(0.0, 0.0, 15.0), sad=100.0, bixel=0.5, field=10.0, radius=None):
    """Bixel grids for beams at the given gantry angles.  Gantry angle g
    rotates the beam about the y axis through the isocentre: the source is
    at iso - sad*(sin g, 0, cos g), so g = 0 irradiates along +z.  Each
    beam carries a field x field cm grid of bixel x bixel cm bixels at the
    isocentre plane, restricted to bixels whose centre lies within
    `radius` of the axis when given."""
    iso = np.asarray(iso, dtype=np.float64)
    n1 = int(round(field / bixel))
    ib, src, cor, s1, s2 = [], [], [], [], []
    for b, g in enumerate(gantry_deg):
        t = np.deg2rad(g)
        axis = np.array([np.sin(t), 0.0, np.cos(t)])
        e1 = np.array([np.cos(t), 0.0, -np.sin(t)])
        e2 = np.array([0.0, 1.0, 0.0])
        src.append(iso - sad * axis)
        for i in range(n1):
            for j in range(n1):
                a = -0.5 * field + i * bixel
                c = -0.5 * field + j * bixel
                if radius is not None and np.hypot(a + 0.5 * bixel, c + 0.5 * bixel) > radius:
                    continue
                ib.append(b)
                cor.append(iso + a * e1 + c * e2)
                s1.append(bixel * e1)
                s2.append(bixel * e2)
    return Beamlets(np.array(ib, np.int32), np.array(src), np.array(cor), np.array(s1), np.array(s2))


def lognormal_histories(n, median=5e4, sigma=1.0, lo=1e4, hi=1e6, seed=7):
    """Histories per beamlet: lognormal with the given median and log
    standard deviation, clipped to [lo, hi], from default_rng(seed)."""
    rng = np.random.default_rng(seed)
    return np.clip(np.round(median * np.exp(sigma * rng.standard_normal(n))), lo, hi).astype(np.int64)


def write_egsphant(ph: Phantom, path: str) -> str:
    nz, ny, nx = ph.shape
    lines = [str(len(ph.media))] + list(ph.media) + ["  ".join(["0.25"] * len(ph.media)),
                                                     f"{nx} {ny} {nz}"]
    for b in (ph.xb, ph.yb, ph.zb):
        lines.append(" ".join(repr(float(v)) for v in b))
    digits = (ph.med + ord("0")).astype(np.uint8)
    parts = ["\n".join(lines), "\n"]
    for k in range(nz):
        rows = [bytes(digits[k, j]).decode("ascii") for j in range(ny)]
        parts.append("\n".join(rows) + "\n\n")
    for k in range(nz):
        sl = ph.rho[k]
        parts.append("\n".join(" ".join(repr(float(v)) for v in row) for row in sl) + "\n\n")
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        f.write("".join(parts))
    os.replace(tmp, path)
    return path


def spectrum_6mv():
    """24 bins with upper edges 0.25..6.0 MeV, counts/bin, weights
    (E/6)^-0.5 (1-E/6)^2 at the upper edge, normalised (last bin 0)."""
    e = 0.25 * np.arange(1, 25)
    w = (e / 6.0) ** -0.5 * (1.0 - e / 6.0) ** 2
    return 0.0, e, w / w.sum()


def spectrum_250kvp():
    """50 bins over 10-250 keV, counts/bin, weights (250-E) E^0.5 at the
    upper edge in keV, normalised (last bin 0)."""
    e = np.linspace(0.010, 0.250, 51)[1:]
    ek = e * 1000.0
    w = (250.0 - ek) * np.sqrt(ek)
    return 0.010, e, w / w.sum()


def write_spectrum(path, title, enmin, edges, weights, imode=0):
    with open(path, "w") as f:
        f.write(title.rstrip() + "\n")
        f.write(f"   {len(edges)} {enmin!r} {imode}\n")
        for e, w in zip(edges, weights):
            f.write(f"   {float(e)!r} {float(w)!r}\n")
    return path


@dataclass
class Job:
    """Everything the reference's omc_dosxyz .inp file holds."""

    phantom_file: str
    pegs_file: str
    pgs4form_file: str
    data_folder: str
    output_folder: str
    ncase: int = 100000
    nbatch: int = 10
    seeds: tuple = (97, 33)
    mono_energy: float = 1.25
    spectrum_file: str | None = None
    charge: int = 0
    collimator: tuple = (-5.0, 5.0, -5.0, 5.0)
    ssd: float = 100.0
    ecut: float = 0.700
    pcut: float = 0.010
    nsplit: int = 1
    extra: dict = field(default_factory=dict)

    def text(self) -> str:
        rows = ["# start source definition"]
        rows.append(f"mono energy = {self.mono_energy!r}")
        if self.spectrum_file:
            rows.append(f"spectrum file = {self.spectrum_file}")
        rows += [f"charge = {self.charge}",
                 "collimator bounds = " + " ".join(repr(float(c)) for c in self.collimator),
                 f"ssd = {self.ssd!r}",
                 "# MC control",
                 f"ncase = {self.ncase}", f"nbatch = {self.nbatch}",
                 f"rng seeds = {self.seeds[0]} {self.seeds[1]}",
                 "# geometry",
                 f"phantom file = {self.phantom_file}",
                 "# transport",
                 f"global ecut = {self.ecut!r}", f"global pcut = {self.pcut!r}",
                 f"pegs file = {self.pegs_file}", f"pgs4form file = {self.pgs4form_file}",
                 "# VRT", f"nsplit = {self.nsplit}",
                 "# environment",
                 f"data folder = {self.data_folder}", f"output folder = {self.output_folder}"]
        for k, v in self.extra.items():
            rows.append(f"{k} = {v}")
        return "\n".join(rows) + "\n"

    def write(self, path_without_ext: str) -> str:
        with open(path_without_ext + ".inp", "w") as f:
            f.write(self.text())
        return path_without_ext
