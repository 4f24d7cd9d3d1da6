"""Synthetic, spin-neutral ``spinms.data`` in the binary layout ompMC reads.

The reference reads EGSnrc's binary spin-correction table in
``initSpinData`` (ompMC ``src/ompmc.c:2376-2947``).  That file is not shipped
with the reference, so both the reference (when it is used as a checker) and
this engine read a synthetic file written here.  Its contents make every spin
correction neutral:

* the rejection function ``spin_rej`` is identically 1 (``i2 = 0xFFFF`` and
  ``fmax = 1``; ``ompmc.c:2591-2603`` and the rescale at ``:2611-2646``);
* the first-moment correction ``q1c`` is 1 (``dum1 = dum3 = 1``,
  ``ompmc.c:2587-2588, 2664-2666``);
* the second-moment correction ``q2c`` is 1 (``dum2`` is the gamma factor of
  the same screening parameter the reference recomputes, ``ompmc.c:2589,
  2658-2663``);
* the screening correction ``etap`` is close to 1 (``z^(2/3) * aux_o`` equals
  the constant ``K`` for every element, ``ompmc.c:2580, 2654-2657``).

Layout (``ompmc.c:2411-2607``): fixed 1104-byte records of 276 float32.
Record 1 is the header (32-byte version, 4-byte endianness tag, then float32
``espin_min, espin_max`` in keV and ``b2spin_min, b2spin_max``).  Element
``Z``, charge ``iq`` (0 electrons, 1 positrons) and energy ``i`` (0..31) sit at
record ``1 + (Z-1)*64 + iq*32 + i + 1`` (1-based) and hold four float32
``dum1 dum2 dum3 aux_o``, sixteen float32 ``fmax[q]`` and 512 int16
``i2[q][u]``.
"""

from __future__ import annotations

import math
import os

import numpy as np

RM = 0.5109989461  # MeV, electron rest energy (ompMC ompmc.h:46)
NREC_FLOATS = 276
NENER = 15  # MXE_SPIN (ompmc.h:257)
NZ = 100

# Header values of the synthetic table, chosen here.  The energy grid
# (1 keV-1 MeV) only sets where the reader interpolates: the rejection
# function is 1 at every grid point, so it is 1 at every energy.  The
# screening constant K = 4.25 (z^(2/3) * aux_o, the same for every element)
# gives etap ~ 1 for H2O700ICRU.
ESPIN_MIN_KEV = 1.0
ESPIN_MAX_KEV = 1000.0
B2SPIN_MAX = 0.99999
SCREEN_K = 4.25  # z^(2/3) * aux_o for every element
VERSION = b"ompmc-gb300 spin-neutral v1"


def _beta2_of_kev(e_kev: float) -> float:
    tau = e_kev / (1000.0 * RM)
    return tau * (tau + 2.0) / ((tau + 1.0) ** 2)


def _energy_grid(espin_min, espin_max, b2min, b2max):
    """Energy grid (keV) the reader builds from the header, ompmc.c:2445-2470."""
    earray = [0.0] * (2 * NENER + 2)
    dloge = math.log(espin_max / espin_min) / NENER
    eloge = math.log(espin_min)
    earray[0] = espin_min
    for i in range(1, NENER + 1):
        eloge += dloge
        earray[i] = math.exp(eloge)
    dbeta2 = (b2max - b2min) / NENER
    beta2 = b2min
    earray[NENER + 1] = espin_max
    for i in range(NENER + 2, 2 * NENER + 2):
        beta2 += dbeta2
        earray[i] = RM * 1000.0 * (1.0 / math.sqrt(1.0 - beta2) - 1) if beta2 < 0.999 else 50585.1
    return earray


def _gamma_of_eta(eta: float) -> float:
    lg = math.log(1.0 + 1.0 / eta)
    return 3.0 * (1.0 + eta) * (lg * (1.0 + 2.0 * eta) - 2.0) / (lg * (1.0 + eta) - 1.0)


def write_spin_neutral(path: str) -> str:
    """Write the synthetic table to ``path`` (little-endian) and return it."""
    f32 = np.float32
    espin_min = float(f32(ESPIN_MIN_KEV))
    espin_max = float(f32(ESPIN_MAX_KEV))
    b2min = float(f32(_beta2_of_kev(ESPIN_MAX_KEV)))
    b2max = float(f32(B2SPIN_MAX))
    earray = _energy_grid(espin_min, espin_max, b2min, b2max)

    nrec = 1 + NZ * 4 * (NENER + 1)
    buf = np.zeros((nrec, NREC_FLOATS), dtype="<f4")
    header = bytearray(NREC_FLOATS * 4)
    header[0:32] = VERSION.ljust(32, b" ")
    header[32:36] = b"1234"
    header[36:52] = np.array([espin_min, espin_max, b2min, b2max], dtype="<f4").tobytes()
    buf[0] = np.frombuffer(bytes(header), dtype="<f4")

    fsc_tf2 = (137.03604 * 0.88534138) ** 2
    dum2 = np.empty(2 * NENER + 2)
    for i, e in enumerate(earray):
        tau = e / (1000.0 * RM)
        eta = SCREEN_K / fsc_tf2 / 4.0 / tau / (tau + 2.0)
        dum2[i] = _gamma_of_eta(eta)

    i2_words = np.full(512, -1, dtype="<i2").view("<f4")  # 0xFFFF -> 65535
    for z in range(1, NZ + 1):
        aux_o = SCREEN_K / z ** (2.0 / 3.0)
        for iq in range(2):
            for i in range(2 * NENER + 2):
                rec = 1 + (z - 1) * 4 * (NENER + 1) + 2 * iq * (NENER + 1) + i  # 0-based
                row = buf[rec]
                row[0] = 1.0
                row[1] = dum2[i]
                row[2] = 1.0
                row[3] = aux_o
                row[4:20] = 1.0
                row[20:] = i2_words
    tmp = path + ".tmp"
    with open(tmp, "wb") as fh:
        fh.write(buf.tobytes())
    os.replace(tmp, path)
    return path


if __name__ == "__main__":  # pragma: no cover
    import sys

    print(write_spin_neutral(sys.argv[1] if len(sys.argv) > 1 else "spinms.data"))
