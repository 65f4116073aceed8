"""Synthetic data of the SSP operator (the IMF-free SSP path), in this package's data-root format.

The reference builds its SSP operator from real isochrones and stellar libraries (MIST, MILES, ...), which are not
available here. This dataset stands in for them with the shapes of the operator workload: a stellar library of
2000 spectra on a grid of 50 effective temperatures (log-uniform 2500 .. 50000 K) x 40 surface gravities (0 .. 5),
and, for each of the 107 ages x 12 metallicities of the SSP grid, 1500 isochrone points with initial masses
log-uniform in [0.08, 100] M_sun, each mapped bilinearly (in log Teff and log g) to 4 library entries, about 7.7M
operator entries in all. The 1500 stars (masses, giant temperatures, scatter) are one seeded draw shared by every
grid point, so that the points move smoothly with age and metallicity as on real isochrones.

Contents of ``<root>/ssp_op/`` (little-endian; grid point g = age + 107 metallicity):

* ``lib.f32``        2000 x nspec library spectra (template e = 50 i_logg + i_teff), L_nu per unit L_bol [1/Hz]
* ``pt_mini.f64``    12 x 107 x 1500 initial masses [M_sun], ascending within a grid point
* ``pt_idx.i32``     12 x 107 x 1500 x 4 template indices of each point
* ``pt_coef.f64``    12 x 107 x 1500 x 4 coefficients (bilinear weight x L_bol of the star [L_sun])
* ``pt_mcur.f64``    12 x 107 x 1500 current mass of the star [M_sun]
* ``pt_lum.f64``     12 x 107 x 1500 L_bol of the star [L_sun]

Stars: below the turnoff mass m_to = 10^(-0.4 (log age - 10)) M_sun they are on the main sequence (log Teff =
3.76 + 0.55 log m - 0.03 log Z/Zsun, log g = 4.44 - 0.55 log m, L = m^3.5, current mass m); above it they are giants
(log Teff = 3.62 + 0.1 u, log g = 1.5 - log(m / m_to), L = 100 m_to^2.5, current mass 0.6 m_to^0.9), with a seeded
scatter of 0.01 dex in log Teff and 0.05 in log g. Spectra: a blackbody at the grid temperature times 12 Gaussian
absorption features whose depth falls with gravity, normalised to unit bolometric luminosity. Seed 2.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from . import synthdata

NTE, NLG = 50, 40
NTEMPL = NTE * NLG
NPT = 1500
TEFF_LO, TEFF_HI = 2500.0, 50000.0
LOGG_LO, LOGG_HI = 0.0, 5.0
M_LO, M_HI = 0.08, 100.0
VERSION = 2


def _library(rng: np.random.Generator, lam: np.ndarray) -> np.ndarray:
    nu = synthdata.C_LIGHT / lam
    teff = np.geomspace(TEFF_LO, TEFF_HI, NTE)
    logg = np.linspace(LOGG_LO, LOGG_HI, NLG)
    lnl = np.log(lam)
    fc = rng.uniform(np.log(900.0), np.log(3.0e4), size=12)
    fw = rng.uniform(1.0, 4.0, size=12) * (lnl[1] - lnl[0])
    fd = rng.uniform(0.1, 0.5, size=12)
    feat = np.stack([np.exp(-0.5 * ((lnl - fc[k]) / fw[k]) ** 2) for k in range(12)])      # (12, nspec)
    lib = np.empty((NLG, NTE, lam.size))
    for it, t in enumerate(teff):
        x = synthdata.H_OVER_K / lam / t
        with np.errstate(over="ignore"):
            bb = (x ** 3) / np.expm1(np.minimum(x, 700.0))
        for ig, g in enumerate(logg):
            depth = fd * (1.0 - 0.15 * g)                                                    # deeper at low gravity
            s = bb * np.prod(1.0 - depth[:, None] * feat, axis=0)
            norm = np.sum(0.5 * (s[1:] + s[:-1]) * np.abs(np.diff(nu)))
            lib[ig, it] = s / norm
    return lib.reshape(NTEMPL, lam.size)


def _points(rng: np.random.Generator, log_age: np.ndarray, logz: np.ndarray):
    nt, nz = log_age.size, logz.size
    lt_lo, lt_hi = np.log10(TEFF_LO), np.log10(TEFF_HI)
    # one set of stars for every grid point (the masses, the giants' temperatures and the scatter): as a real
    # isochrone set, the points then move smoothly with age and metallicity
    shape = (nz, nt, NPT)
    mini = np.broadcast_to(np.sort(10.0 ** rng.uniform(np.log10(M_LO), np.log10(M_HI), size=NPT)), shape).copy()
    lm = np.log10(mini)
    mto = 10.0 ** (-0.4 * (log_age - 10.0))[None, :, None] * np.ones_like(mini)
    ms = mini <= mto
    u = np.broadcast_to(rng.uniform(size=NPT), shape)
    logt = np.where(ms, 3.76 + 0.55 * lm - 0.03 * logz[:, None, None], 3.62 + 0.1 * u)
    logg = np.where(ms, 4.44 - 0.55 * lm, 1.5 - np.log10(mini / mto))
    logt = logt + 0.01 * np.broadcast_to(rng.standard_normal(NPT), shape)
    logg = logg + 0.05 * np.broadcast_to(rng.standard_normal(NPT), shape)
    lum = np.where(ms, mini ** 3.5, 100.0 * mto ** 2.5)
    mcur = np.where(ms, mini, 0.6 * mto ** 0.9)
    # bilinear position on the library grid (log Teff, log g), clamped to it
    x = np.clip((logt - lt_lo) / (lt_hi - lt_lo) * (NTE - 1), 0.0, NTE - 1 - 1e-9)
    y = np.clip((logg - LOGG_LO) / (LOGG_HI - LOGG_LO) * (NLG - 1), 0.0, NLG - 1 - 1e-9)
    ix, iy = np.floor(x).astype(np.int32), np.floor(y).astype(np.int32)
    fx, fy = x - ix, y - iy
    idx = np.stack([iy * NTE + ix, iy * NTE + ix + 1, (iy + 1) * NTE + ix, (iy + 1) * NTE + ix + 1], axis=-1)
    wgt = np.stack([(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy], axis=-1)
    coef = wgt * lum[..., None]
    return mini, idx.astype(np.int32), coef, mcur, lum


def generate(root: Path | None = None, force: bool = False) -> Path:
    """Write the operator dataset under ``root/ssp_op`` (once; ``force`` rewrites)."""
    root = Path(root) if root is not None else synthdata.default_root()
    synthdata.generate(root)
    out = root / "ssp_op"
    man = out / "manifest.json"
    if man.exists() and not force:
        try:
            if json.loads(man.read_text()).get("version") == VERSION:
                return out
        except (OSError, ValueError):
            pass
    out.mkdir(parents=True, exist_ok=True)
    r_lib, r_pts = (np.random.default_rng(s) for s in np.random.SeedSequence(2).spawn(2))
    lam = synthdata.wavelength_grid()
    log_age = np.linspace(synthdata.LOG_AGE_LO, synthdata.LOG_AGE_HI, synthdata.NT)
    logz = np.linspace(synthdata.LOGZ_LO, synthdata.LOGZ_HI, synthdata.NZ)
    lib = _library(r_lib, lam)
    mini, idx, coef, mcur, lum = _points(r_pts, log_age, logz)
    np.ascontiguousarray(lib, dtype="<f4").tofile(out / "lib.f32")
    np.ascontiguousarray(mini, dtype="<f8").tofile(out / "pt_mini.f64")
    np.ascontiguousarray(idx, dtype="<i4").tofile(out / "pt_idx.i32")
    np.ascontiguousarray(coef, dtype="<f8").tofile(out / "pt_coef.f64")
    np.ascontiguousarray(mcur, dtype="<f8").tofile(out / "pt_mcur.f64")
    np.ascontiguousarray(lum, dtype="<f8").tofile(out / "pt_lum.f64")
    man.write_text(json.dumps({"version": VERSION, "ntempl": NTEMPL, "nte": NTE, "nlg": NLG, "npt": NPT,
                               "nt": synthdata.NT, "nz": synthdata.NZ, "nspec": synthdata.NSPEC, "seed": 2,
                               "imf_lower_bound": M_LO}, indent=1))
    return out


def load(root: Path | None = None) -> dict:
    d = generate(root)
    man = json.loads((d / "manifest.json").read_text())
    nz, nt, npt, ne, ns = man["nz"], man["nt"], man["npt"], man["ntempl"], man["nspec"]
    return {
        "manifest": man,
        "lib": np.fromfile(d / "lib.f32", dtype="<f4").reshape(ne, ns),
        "mini": np.fromfile(d / "pt_mini.f64", dtype="<f8").reshape(nz, nt, npt),
        "idx": np.fromfile(d / "pt_idx.i32", dtype="<i4").reshape(nz, nt, npt, 4),
        "coef": np.fromfile(d / "pt_coef.f64", dtype="<f8").reshape(nz, nt, npt, 4),
        "mcur": np.fromfile(d / "pt_mcur.f64", dtype="<f8").reshape(nz, nt, npt),
        "lum": np.fromfile(d / "pt_lum.f64", dtype="<f8").reshape(nz, nt, npt),
    }
