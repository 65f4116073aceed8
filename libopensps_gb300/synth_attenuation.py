"""Synthetic stand-ins for the attenuation libraries that dust types 3 and 5 read, in the standard data format under
the data root's ``libraries/attenuation``: ``smc_bar`` (A(lambda) / A(V) over a wavelength axis) and ``dirty`` (the
optical depth of dusty environments over [structure (2), tau_v (18), model (6), wavelength (25)]). The curves are
smooth made-up functions with the libraries' shapes and ranges; the published tables are not reproduced."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import stdformat

SYNTHETIC = "synthetic stand-in (made-up smooth curves with the library's shape; not the published table)"


def generate(root: Path) -> None:
    """Write attenuation/smc_bar and attenuation/dirty under root (once)."""
    root = Path(root)
    base = root / "libraries" / "attenuation"
    if not (base / "smc_bar" / "manifest.json").exists():
        lam = np.geomspace(1160.0, 30000.0, 30)
        x = np.log(5500.0 / lam)
        ext = np.exp(1.25 * x + 0.06 * x * x)                # steep, no bump, 1 at 5500 A
        stdformat.write_library(
            root, "attenuation", "smc_bar",
            axes={"wavelength": {"units": "angstrom", "values": lam}},
            arrays={"extinction": (ext, "<f4", ["wavelength"], "A(lambda)/A(V)")},
            title="SMC-bar-like extinction curve: " + SYNTHETIC)
    if not (base / "dirty" / "manifest.json").exists():
        lam = np.geomspace(1000.0, 30000.0, 25)
        tau_v = np.geomspace(0.25, 10.0, 18)
        x = np.log(5500.0 / lam)
        att = np.empty((2, 18, 6, 25))
        for s in range(2):                                  # homogeneous, clumpy (less attenuating, greyer)
            for t in range(18):
                for m in range(6):                          # six environments: slopes 0.6 .. 1.35, a bump in three
                    slope = (0.6 + 0.15 * m) * (1.0 - 0.25 * s)
                    bump = 0.15 * (m % 2) * np.exp(-0.5 * ((lam - 2175.0) / 250.0) ** 2)
                    att[s, t, m] = tau_v[t] * (1.0 - 0.3 * s) * (np.exp(slope * x) + bump)
        stdformat.write_library(
            root, "attenuation", "dirty",
            axes={"structure": {"units": "", "labels": ["homogeneous", "clumpy"]},
                  "tau_v": {"units": "V-band optical depth", "values": tau_v},
                  "model": {"units": "", "labels": [f"environment_{k}" for k in range(6)]},
                  "wavelength": {"units": "angstrom", "values": lam}},
            arrays={"attenuation": (att, "<f4", ["structure", "tau_v", "model", "wavelength"],
                                    "attenuation optical depth")},
            title="Attenuation optical depths of dusty environments: " + SYNTHETIC)
