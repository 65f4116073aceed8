"""A synthetic CLOUDY-style nebular grid (the continuum and line tables of OpenSPS's ``nebular/<isoc>_<dust|nodust>``
libraries, doc/DATA_FORMAT.md of the reference), for the nebular continuum of the batched CSP.

OpenSPS reads Cloudy photoionization tables (Byler et al. 2017) from its data release, which is not available here
(the reference's coarse test subset stores them as float32, where every value, about 1e-61 L_sun/Hz per ionizing
photon per second, underflows to zero). This grid stands in for them with the same axes and units:

* ``logZ``: 11 gas metallicities log10(Z/Z_sun) (-1.98 .. 0.2), ``age``: 10 ages 0.5 .. 10 Myr (yr), ``logU``:
  7 ionization parameters (-4 .. -1);
* ``continuum`` [logZ, age, logU, wavelength]: L_sun/Hz per unit ionizing photon rate (s^-1) on a native grid of
  600 log-spaced wavelengths 91 A .. 1e8 A: hydrogen free-free and free-bound emission at an electron temperature
  T_e = 1e4 K (1 + 0.12 (-log Z)) (1 + 0.03 (7 - log age)) (1 - 0.02 (logU + 2)) -- exp(-h nu / k T_e) with the
  Balmer, Paschen and Brackett recombination edges (jumps of 1.2, 0.6 and 0.3 times the free-free level, decaying
  blueward as exp(-h (nu - nu_edge) / k T_e)) and a two-photon bump near 1500 A (0.8 of the 5000 A free-free level,
  0.12 dex wide), normalised to 10^-60.4 at 5000 A
  for solar gas at logU = -2 and 1 Myr; nothing below 912 A (1e-95, the reference's floor);
* ``lines`` [logZ, age, logU, line_wavelength]: L_sun per unit ionizing photon rate for 166 lines at log-spaced
  wavelengths 1200 .. 20000 A (written for the format's completeness; this path's lines come from the SSP library's
  line table).

The last CLOUDY age, 10 Myr, is the synthetic line list's last age, so the nebular ages of the grid are those of the
lines (log age <= 7).

``steep`` (a test grid): the continuum falls by ``STEEP_DEX`` decades per dex of age past 1 Myr (floored as above),
so that between some CLOUDY ages it drops by more than 2^64, the case the continuum kernel takes age by age.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

LOGZ = np.array([-1.98, -1.5, -0.98, -0.58, -0.39, -0.3, -0.2, -0.1, 0.0, 0.1, 0.2])
AGE = np.array([0.5, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 10.0]) * 1.0e6
LOGU = np.array([-4.0, -3.5, -3.0, -2.5, -2.0, -1.5, -1.0])
NLAM = 600
NEMLINE = 166
HC_OVER_K = 1.4387769e8          # h c / k [A K]
EDGES = ((3646.0, 1.2), (8204.0, 0.6), (14584.0, 0.3))
FLOOR = 1.0e-95
STEEP_DEX = 80.0


def wavelengths() -> np.ndarray:
    return np.geomspace(91.0, 1.0e8, NLAM)


def _continuum(lam: np.ndarray, logz: float, age: float, logu: float) -> np.ndarray:
    te = 1.0e4 * (1.0 + 0.12 * (-logz)) * (1.0 + 0.03 * (7.0 - np.log10(age))) * (1.0 - 0.02 * (logu + 2.0))
    x = HC_OVER_K / (lam * te)                   # h nu / k T_e
    c = np.exp(-x)
    for le, s in EDGES:
        xe = HC_OVER_K / (le * te)
        c = c + np.where(lam < le, s * np.exp(-xe) * np.exp(-(x - xe)), 0.0)
    x5 = HC_OVER_K / (5000.0 * te)
    c = c + 0.8 * np.exp(-x5) * np.exp(-0.5 * (np.log10(lam / 1500.0) / 0.12) ** 2)
    return np.where(lam >= 912.0, c, 0.0)


def continuum_grid(steep: bool = False) -> tuple[np.ndarray, np.ndarray]:
    """(wavelength, continuum[logZ, age, logU, wavelength]) in L_sun/Hz per ionizing photon per second."""
    lam = wavelengths()
    ref = _continuum(np.array([5000.0]), 0.0, 1.0e6, -2.0)[0]
    scale = 10.0 ** -60.4 / ref
    out = np.empty((LOGZ.size, AGE.size, LOGU.size, lam.size))
    for i, z in enumerate(LOGZ):
        for j, a in enumerate(AGE):
            for k, u in enumerate(LOGU):
                out[i, j, k] = scale * _continuum(lam, z, a, u)
                if steep:
                    out[i, j, k] *= 10.0 ** (-STEEP_DEX * max(0.0, np.log10(a) - 6.0))
    return lam, np.maximum(out, FLOOR)


def lines_grid() -> tuple[np.ndarray, np.ndarray]:
    """(line wavelength, lines[logZ, age, logU, line]) in L_sun per ionizing photon per second."""
    rng = np.random.default_rng(21)
    lw = np.geomspace(1200.0, 20000.0, NEMLINE)
    base = 10.0 ** rng.uniform(-48.0, -45.5, NEMLINE)
    out = np.empty((LOGZ.size, AGE.size, LOGU.size, NEMLINE))
    for i, z in enumerate(LOGZ):
        for j, a in enumerate(AGE):
            for k, u in enumerate(LOGU):
                out[i, j, k] = base * 10.0 ** (0.1 * z - 0.05 * (np.log10(a) - 6.0) + 0.03 * (u + 2.0))
    return lw, out


def write(root: Path, name: str = "synthetic_nodust", steep: bool = False) -> Path:
    """The grid as the standard-format library ``nebular/<name>`` under ``root``."""
    from .stdformat import write_library
    lam, cont = continuum_grid(steep)
    lw, lines = lines_grid()
    return write_library(
        root, "nebular", name,
        axes={"logZ": {"units": "log10(Z/Z_sun)", "values": LOGZ},
              "age": {"units": "yr", "values": AGE},
              "logU": {"units": "log10(ionization parameter)", "values": LOGU},
              "wavelength": {"units": "angstrom", "medium": "vacuum", "data": lam},
              "line_wavelength": {"units": "angstrom", "medium": "vacuum", "data": lw}},
        arrays={"continuum": (cont, "<f8", ["logZ", "age", "logU", "wavelength"],
                              "L_sun Hz^-1 per unit ionizing photon rate (s^-1)"),
                "lines": (lines, "<f8", ["logZ", "age", "logU", "line_wavelength"],
                          "L_sun per unit ionizing photon rate (s^-1)")},
        title="Synthetic nebular continuum and lines (the CLOUDY grid's axes and units; not for science)")
