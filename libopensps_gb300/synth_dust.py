"""Synthetic dust emission templates (the Draine & Li 2007 grid's shape) and AGN torus templates, in this package's
data-root format.

OpenSPS reads the DL07 templates (dust emission per unit dust mass as a function of the PAH mass fraction q_PAH and
the minimum starlight intensity U_min, each as a delta-function and a power-law distribution of U) from its data
release, which is not available here. This dataset stands in for them with the grid's shapes: 7 values of q_PAH
(0.47 .. 4.58 %) x 22 values of U_min (0.1 .. 25), two components each, on the synthetic wavelength grid.

Each template, L_nu per unit luminosity on the grid: a modified blackbody (beta = 2) at T = 18 K U^(1/6) (the
delta-function component) or the U^-2 mixture of such bodies from U_min to 10^6 (the power-law component), a
stochastically heated small-grain continuum rising into the mid-infrared with U, and Gaussian PAH features at 3.3,
6.2, 7.7, 8.6 and 11.3 um whose strength follows q_PAH. (The synthetic grid stops at 10 um: the cold bodies' peaks lie
beyond it, and within the grid the PAH features and the warm continuum carry the emission.)

Contents of ``<root>/dust_dl07/`` (little-endian):

* ``manifest.json``
* ``qpah.f64``     7 q_PAH values (%)
* ``umin.f64``     22 U_min values
* ``dustem.f32``   nspec x 7 x 44 templates, column-major (pixel fastest; column 2 u + c: U_min index u, component c,
                   0 delta-function, 1 power law), as OpenSPS's dustem2_dustem(i, iq, 2 iu - 1 + c)
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from . import synthdata

QPAH = np.array([0.47, 1.12, 1.77, 2.50, 3.19, 3.90, 4.58])
UMIN = np.array([0.10, 0.15, 0.20, 0.30, 0.40, 0.50, 0.70, 0.80, 1.00, 1.20, 1.50, 2.00, 2.50, 3.00, 4.00, 5.00,
                 7.00, 8.00, 12.0, 15.0, 20.0, 25.0])
PAH_UM = np.array([3.3, 6.2, 7.7, 8.6, 11.3])
PAH_W = np.array([0.02, 0.03, 0.06, 0.03, 0.03])           # Gaussian widths / centre
PAH_A = np.array([0.4, 1.0, 2.0, 0.6, 0.8])
VERSION = 1


def _mbb(nu: np.ndarray, t: float) -> np.ndarray:
    x = synthdata.H_OVER_K * nu / synthdata.C_LIGHT / t      # h nu / k T
    with np.errstate(over="ignore"):
        return nu ** 5 / np.expm1(np.minimum(x, 700.0))


def _template(lam: np.ndarray, q: float, u: float, powerlaw: bool) -> np.ndarray:
    nu = synthdata.C_LIGHT / lam
    lam_um = lam * 1e-4
    if powerlaw:
        us = np.geomspace(u, 1.0e6, 24)
        wu = us ** -2.0 * np.gradient(us)
        cont = sum(w * _mbb(nu, 18.0 * x ** (1.0 / 6.0)) for w, x in zip(wu, us)) / wu.sum()
        hot = 0.05 * np.log10(1.0e6 / u)
    else:
        cont = _mbb(nu, 18.0 * u ** (1.0 / 6.0))
        hot = 0.01
    # small grains: a continuum rising as lambda^2 into the mid-infrared, cut below 1.5 um
    vsg = hot * (lam_um / 10.0) ** 2 * np.exp(-(1.5 / lam_um) ** 4) * u ** 0.3
    pah = sum(a * np.exp(-0.5 * ((lam_um - c) / (w * c)) ** 2) for a, c, w in zip(PAH_A, PAH_UM, PAH_W))
    t = cont / max(cont.max(), 1e-300) * 1e-3 + vsg + 0.1 * q * pah
    return t / max(np.sum(0.5 * (t[1:] + t[:-1]) * np.abs(np.diff(nu))), 1e-300)


def generate(root: Path | None = None, force: bool = False) -> Path:
    """Write the templates under ``root/dust_dl07`` (once; ``force`` rewrites)."""
    root = Path(root) if root is not None else synthdata.default_root()
    synthdata.generate(root)
    out = root / "dust_dl07"
    man = out / "manifest.json"
    if man.exists() and not force:
        try:
            if json.loads(man.read_text()).get("version") == VERSION:
                return out
        except (OSError, ValueError):
            pass
    out.mkdir(parents=True, exist_ok=True)
    lam = synthdata.wavelength_grid()
    nq, nu = QPAH.size, UMIN.size
    tab = np.empty((2 * nu, nq, lam.size))
    for k in range(2 * nu):
        for iq in range(nq):
            tab[k, iq] = _template(lam, QPAH[iq], UMIN[k // 2], powerlaw=(k % 2 == 1))
    QPAH.astype("<f8").tofile(out / "qpah.f64")
    UMIN.astype("<f8").tofile(out / "umin.f64")
    tab.astype("<f4").tofile(out / "dustem.f32")
    man.write_text(json.dumps({"version": VERSION, "nqpah": nq, "numin": nu, "nspec": int(lam.size)}, indent=1))
    return out


# The AGN torus templates (OpenSPS's agndust_spec over agndust_tau: the Nenkova clumpy-torus grid in the torus'
# optical depth): here hot-dust bodies (1500, 1000, 600, 300 K) whose mix cools as tau grows, with the 9.7 um silicate
# feature in emission at low tau and in absorption at high tau, each normalised to unit luminosity on the grid.
AGN_TAU = np.array([5.0, 10.0, 20.0, 30.0, 40.0, 60.0, 80.0, 100.0, 150.0])
AGN_VERSION = 1


def _agn_template(lam: np.ndarray, tau: float) -> np.ndarray:
    nu = synthdata.C_LIGHT / lam
    lam_um = lam * 1e-4
    x = np.log10(tau / 5.0) / np.log10(30.0)                  # 0 .. 1 over the grid
    temps = (1500.0, 1000.0, 600.0, 300.0)
    mix = np.array([1.0 - 0.7 * x, 0.8, 0.5 + 0.5 * x, 0.2 + 0.8 * x])
    body = sum(w * _mbb(nu, t) / _mbb(nu, t).max() for w, t in zip(mix, temps))
    sil = 1.0 + (0.6 - 1.4 * x) * np.exp(-0.5 * ((lam_um - 9.7) / 0.9) ** 2)
    t = np.maximum(body * sil, 0.0)
    return t / max(np.sum(0.5 * (t[1:] + t[:-1]) * np.abs(np.diff(nu))), 1e-300)


def generate_agn(root: Path | None = None, force: bool = False) -> Path:
    """Write the AGN torus templates under ``root/agn_torus`` (``tau.f64``, ``agnspec.f32``: nspec x ntau,
    column-major; once; ``force`` rewrites)."""
    root = Path(root) if root is not None else synthdata.default_root()
    synthdata.generate(root)
    out = root / "agn_torus"
    man = out / "manifest.json"
    if man.exists() and not force:
        try:
            if json.loads(man.read_text()).get("version") == AGN_VERSION:
                return out
        except (OSError, ValueError):
            pass
    out.mkdir(parents=True, exist_ok=True)
    lam = synthdata.wavelength_grid()
    tab = np.stack([_agn_template(lam, t) for t in AGN_TAU])  # (ntau, nspec)
    AGN_TAU.astype("<f8").tofile(out / "tau.f64")
    tab.astype("<f4").tofile(out / "agnspec.f32")
    man.write_text(json.dumps({"version": AGN_VERSION, "ntau": int(AGN_TAU.size), "nspec": int(lam.size)}, indent=1))
    return out


def load_agn(root: Path | None = None) -> dict:
    d = generate_agn(root)
    man = json.loads((d / "manifest.json").read_text())
    nt, ns = man["ntau"], man["nspec"]
    return {"tau": np.fromfile(d / "tau.f64", dtype="<f8"),
            "agnspec": np.fromfile(d / "agnspec.f32", dtype="<f4").reshape(nt, ns).astype(np.float64),
            "manifest": man}


def load(root: Path | None = None) -> dict:
    d = generate(root)
    man = json.loads((d / "manifest.json").read_text())
    nq, nu, ns = man["nqpah"], man["numin"], man["nspec"]
    return {"qpah": np.fromfile(d / "qpah.f64", dtype="<f8"), "umin": np.fromfile(d / "umin.f64", dtype="<f8"),
            "dustem": np.fromfile(d / "dustem.f32", dtype="<f4").reshape(2 * nu, nq, ns).astype(np.float64),
            "manifest": man}
