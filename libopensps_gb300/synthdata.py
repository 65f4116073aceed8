"""Synthetic SSP / filter / line library in this package's data-root format.

The reference reads real isochrone and spectral libraries (MIST, MILES, ...) from its data release.
None of those are available here, so the libraries of the benchmark workloads are synthetic and
seeded. The layout mirrors the reference's "standard" SSP kind (`ssp/bpss`: a basis of SSP spectra
over ages x metallicities with their surviving mass and log L_bol, doc/DATA_FORMAT.md) in a minimal
form of our own: a ``manifest.json`` plus raw little-endian arrays, column-major like the
reference's (pixel fastest, then age, then metallicity).

Contents of ``<root>/synthetic/``:

* ``lambda.f64``        nspec wavelengths [A], log-uniform from 91 A to 1e5 A (5994 pixels)
* ``log_age.f64``       ntfull log10 ages [yr], evenly spaced 5.5 .. 10.15 (107)
* ``zlegend.f64``       nz metallicities (mass fractions), log Z/Zsun evenly spaced -2.0 .. +0.5 (12)
* ``ssp_spec.f64``      nspec x ntfull x nz SSP spectra [L_sun/Hz per M_sun formed]
* ``ssp_mass.f64``      ntfull x nz surviving stellar mass [M_sun per M_sun formed]
* ``ssp_lbol.f64``      ntfull x nz log10 L_bol [L_sun per M_sun formed]
* ``line_lambda.f64``   nline rest wavelengths of the nebular lines [A] (128)
* ``line_lum.f64``      nline x ntfull x nz line luminosities [L_sun per M_sun formed] (zero above the
                        nebular age limit)
* ``filters_<F>.f64``   nspec x F filter responses on the grid, normalised to int T / lambda dlambda = 1
                        (trapezoid on the grid), F = 20 and 40
* ``filters_<F>_center.f64``  the F centre wavelengths [A]

Spectra: each (age, metallicity) is a sum of 3 blackbodies with temperatures uniform in
[3000, 40000] K, log-normal pixel noise (sigma 0.05) and 20 Gaussian absorption features of depth
U[0, 0.3], scaled by a luminosity that falls with age; seed 0. Lines: 128 rest wavelengths
log-uniform in [1200, 20000] A, luminosities log-uniform over three decades (10^-1.5 .. 10^1.5 L_sun
per M_sun at 1 Myr), falling as 1/age and present for log age <= 7.0 only. Filters: Gaussians with
centres log-uniform in [0.15, 5] um and R = 5 (FWHM = centre / 5), cut at 4 sigma.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np

NSPEC = 5994
LAM_LO, LAM_HI = 91.0, 1.0e5
NT = 107
LOG_AGE_LO, LOG_AGE_HI = 5.5, 10.15
NZ = 12
LOGZ_LO, LOGZ_HI = -2.0, 0.5
ZSOL = 0.0142
NLINE = 128
NEB_MAX_LOG_AGE = 7.0
LINE_LOGLUM_LO, LINE_LOGLUM_HI = -1.5, 1.5
C_LIGHT = 2.99792458e18      # A / s
H_OVER_K = 1.4387769e8       # h c / k in A K
VERSION = 1
FILTER_SETS = (20, 40)


def default_root() -> Path:
    """The data root: $OPENSPS_DATA_HOME, else ``.opensps_data`` beside the package."""
    env = os.environ.get("OPENSPS_DATA_HOME")
    if env:
        return Path(env)
    return Path(__file__).resolve().parent.parent / ".opensps_data"


def wavelength_grid() -> np.ndarray:
    dl = np.log(LAM_HI / LAM_LO) / (NSPEC - 1)
    return LAM_LO * np.exp(np.arange(NSPEC, dtype=np.float64) * dl)


def _spectra(rng: np.random.Generator, lam: np.ndarray, log_age: np.ndarray, logz: np.ndarray) -> np.ndarray:
    nspec, nt, nz = lam.size, log_age.size, logz.size
    nu_x = H_OVER_K / lam                                   # h nu / k  [K]
    spec = np.empty((nz, nt, nspec), dtype=np.float64)
    temps = rng.uniform(3000.0, 40000.0, size=(nz, nt, 3))
    amps = rng.uniform(0.2, 1.0, size=(nz, nt, 3))
    lnl = np.log(lam)
    feat_c = rng.uniform(np.log(912.0), np.log(LAM_HI), size=(nz, nt, 20))
    feat_w = rng.uniform(0.5, 3.0, size=(nz, nt, 20)) * (lnl[1] - lnl[0])
    feat_d = rng.uniform(0.0, 0.3, size=(nz, nt, 20))
    # luminosity scale per M_sun formed: ~1e-15 L_sun/Hz at 10 Gyr, rising to the youngest ages
    scale = 1.0e-15 * (10.0 ** (log_age - 10.0)) ** (-0.8)
    x_peak = 2.821439372122079                               # h nu / k T at the peak of B_nu
    peak = x_peak ** 3 / np.expm1(x_peak)
    for iz in range(nz):
        for it in range(nt):
            s = np.zeros(nspec)
            for k in range(3):
                x = nu_x / temps[iz, it, k]
                with np.errstate(over="ignore"):
                    bb = (x ** 3) / np.expm1(np.minimum(x, 700.0))
                s += amps[iz, it, k] * bb / peak
            for f in range(20):
                s *= 1.0 - feat_d[iz, it, f] * np.exp(-0.5 * ((lnl - feat_c[iz, it, f]) / feat_w[iz, it, f]) ** 2)
            spec[iz, it] = s * scale[it] * (1.0 + 0.1 * logz[iz])
    noise = np.exp(0.05 * rng.standard_normal(size=spec.shape))
    spec *= noise
    # (nz, nt, nspec) in C order is the column-major (pixel, age, metallicity) layout
    return spec


def _filters(rng: np.random.Generator, lam: np.ndarray, nb: int):
    centres = np.sort(10.0 ** rng.uniform(np.log10(1500.0), np.log10(50000.0), size=nb))
    bands = np.zeros((nb, lam.size))
    for b, c in enumerate(centres):
        sig = (c / 5.0) / (2.0 * np.sqrt(2.0 * np.log(2.0)))
        t = np.exp(-0.5 * ((lam - c) / sig) ** 2)
        t[np.abs(lam - c) > 4.0 * sig] = 0.0
        g = t / lam
        norm = np.sum(0.5 * (g[1:] + g[:-1]) * np.diff(lam))
        bands[b] = t / norm
    return np.ascontiguousarray(bands.T), centres         # (nspec, nb) column-major = bands[j + nspec*b]


def generate(root: Path | None = None, force: bool = False) -> Path:
    """Write the synthetic library under ``root/synthetic`` (once; ``force`` rewrites)."""
    root = Path(root) if root is not None else default_root()
    out = root / "synthetic"
    man = out / "manifest.json"
    if man.exists() and not force:
        try:
            if json.loads(man.read_text()).get("version") == VERSION:
                return out
        except (OSError, ValueError):
            pass
    out.mkdir(parents=True, exist_ok=True)
    ss = np.random.SeedSequence(0)
    r_spec, r_line, r_filt = (np.random.default_rng(s) for s in ss.spawn(3))

    lam = wavelength_grid()
    log_age = np.linspace(LOG_AGE_LO, LOG_AGE_HI, NT)
    logz = np.linspace(LOGZ_LO, LOGZ_HI, NZ)
    zleg = ZSOL * 10.0 ** logz

    spec = _spectra(r_spec, lam, log_age, logz)               # (nz, nt, nspec) C order == (nspec, nt, nz) F order
    mass = np.empty((NZ, NT))
    lbol = np.empty((NZ, NT))
    nu = C_LIGHT / lam
    for iz in range(NZ):
        mass[iz] = 1.0 - 0.35 * (log_age - LOG_AGE_LO) / (LOG_AGE_HI - LOG_AGE_LO) - 0.01 * logz[iz]
        s = spec[iz]                                          # (nt, nspec)
        lbol[iz] = np.log10(np.sum(0.5 * (s[:, 1:] + s[:, :-1]) * np.abs(np.diff(nu)), axis=1))

    line_lambda = np.sort(10.0 ** r_line.uniform(np.log10(1200.0), np.log10(20000.0), size=NLINE))
    line_ll = r_line.uniform(LINE_LOGLUM_LO, LINE_LOGLUM_HI, size=NLINE)
    line_lum = np.zeros((NZ, NT, NLINE))
    young = log_age <= NEB_MAX_LOG_AGE
    for iz in range(NZ):
        for it in np.nonzero(young)[0]:
            line_lum[iz, it] = 10.0 ** line_ll * 10.0 ** (-(log_age[it] - 6.0))

    def put(name, arr):
        np.ascontiguousarray(arr, dtype="<f8").tofile(out / name)

    put("lambda.f64", lam)
    put("log_age.f64", log_age)
    put("zlegend.f64", zleg)
    put("ssp_spec.f64", spec)            # (nz, nt, nspec) row-major: pixel fastest
    put("ssp_mass.f64", mass)            # (nz, nt): age fastest
    put("ssp_lbol.f64", lbol)
    put("line_lambda.f64", line_lambda)
    put("line_lum.f64", line_lum)        # (nz, nt, nline): line fastest
    for nb in FILTER_SETS:
        bands, centres = _filters(np.random.default_rng(np.random.SeedSequence([0, nb])), lam, nb)
        put(f"filters_{nb}.f64", bands.T)      # (nb, nspec) row-major: pixel fastest
        put(f"filters_{nb}_center.f64", centres)
    manifest = {
        "version": VERSION, "kind": "synthetic", "nspec": NSPEC, "ntfull": NT, "nz": NZ, "zsol": ZSOL,
        "nline": NLINE, "neb_max_log_age": NEB_MAX_LOG_AGE, "line_loglum_range": [LINE_LOGLUM_LO, LINE_LOGLUM_HI],
        "filter_sets": list(FILTER_SETS), "seed": 0,
        "layout": "little-endian float64, column-major (pixel fastest, then age, then metallicity)",
    }
    man.write_text(json.dumps(manifest, indent=1))
    return out


def load(root: Path | None = None) -> dict:
    """Read the library back as numpy arrays (generating it first if needed)."""
    d = generate(root)
    man = json.loads((d / "manifest.json").read_text())
    ns, nt, nz, nl = man["nspec"], man["ntfull"], man["nz"], man["nline"]

    def get(name, shape):
        return np.fromfile(d / name, dtype="<f8").reshape(shape)

    out = {
        "manifest": man,
        "lambda": get("lambda.f64", (ns,)),
        "log_age": get("log_age.f64", (nt,)),
        "zlegend": get("zlegend.f64", (nz,)),
        "ssp_spec": get("ssp_spec.f64", (nz, nt, ns)),
        "ssp_mass": get("ssp_mass.f64", (nz, nt)),
        "ssp_lbol": get("ssp_lbol.f64", (nz, nt)),
        "line_lambda": get("line_lambda.f64", (nl,)),
        "line_lum": get("line_lum.f64", (nz, nt, nl)),
    }
    for nb in man["filter_sets"]:
        out[f"filters_{nb}"] = get(f"filters_{nb}.f64", (nb, ns))
        out[f"filters_{nb}_center"] = get(f"filters_{nb}_center.f64", (nb,))
    return out


if __name__ == "__main__":
    import sys
    p = generate(Path(sys.argv[1]) if len(sys.argv) > 1 else None, force=True)
    print(p)
