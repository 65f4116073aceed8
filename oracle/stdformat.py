"""Oracle (test infrastructure only): the standard data format's reading and per-kind processing restated in numpy,
the checker of the C-ABI library's loader. Nothing here is used by the library.

Follows the reference's readers:
* manifests and raw arrays: src/io/opensps_datalib.f90 (open_library :161-220, datalib_check_array :346-397,
  read_descriptor_real :552-575: FP32 promoted to FP64, file size = product(shape) x itemsize);
* ssp/<name>: read_bpass_standard src/io/opensps_io.f90:3131-3155, L_bol as ssp_gen's BPASS branch
  src/physics/opensps_ssp.f90:203-218 (log10 of the |d nu| trapezoid of the spectrum, floored at tiny);
* dust_emission: opensps_io.f90:991-1060 (linear interpolation, extrapolated, at pixels from the one holding 1 um);
* agn_torus/clumpy: load_agn_dust_models opensps_io.f90:1099-1157 (log-log interpolation over the table's range);
* attenuation/smc_bar and attenuation/dirty: load_attenuation_curves opensps_io.f90:2079-2234 (linear interpolation
  inside the table's range, its first value below, zero above);
* nebular: load_nebular_grid / read_nebular_standard opensps_io.f90:749-827,910-933 (the continuum's log10(f + 1e-95)
  interpolated linearly onto the grid);
* filters: read_filter_library opensps_io.f90:1247-1318, filters_build with point resampling
  src/spectra/opensps_filters.f90:186-230 (lenient filter_clean), :362-387 (resample_point), :395-500,
  filter_pivot :521-531, the calibration of apply_standard_filter_calibration opensps_io.f90:1465-1500;
* interpolate_linear / find_interval src/math/opensps_interpolation.f90:45-72, :138-197.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

SAFE_FLOOR = 2.2250738585072014e-308
C_LIGHT = 2.99792458e18
_DT = {"<f4": np.dtype("<f4"), "<f8": np.dtype("<f8"), "<i4": np.dtype("<i4"), "<i8": np.dtype("<i8")}


def find_interval(a: np.ndarray, v: float) -> int:
    """The reference's 1-based find_interval (bisection over 0..n+1, its end cases)."""
    n = a.size
    if n < 2:
        return 1
    asc = a[-1] >= a[0]
    lo, up = 0, n + 1
    while up - lo > 1:
        mid = (up + lo) // 2
        if asc == (v >= a[mid - 1]):
            lo = mid
        else:
            up = mid
    if v == a[0]:
        return 1
    if v == a[-1]:
        return n - 1
    return lo


def interp_linear(x: np.ndarray, y: np.ndarray, v: float) -> float:
    i = min(max(find_interval(x, v), 1), x.size - 1) - 1
    slope = (y[i + 1] - y[i]) / (x[i + 1] - x[i])
    return y[i] + slope * (v - x[i])


def interp_linear_at(x: np.ndarray, y: np.ndarray, v: np.ndarray) -> np.ndarray:
    """interp_linear at many points of an ascending table: find_interval is then the count of entries <= v (the
    bisection's result), with its end cases."""
    v = np.asarray(v, dtype=np.float64)
    idx = np.searchsorted(x, v, side="right")
    idx = np.where(v == x[0], 1, np.where(v == x[-1], x.size - 1, idx))
    i = np.clip(idx, 1, x.size - 1) - 1
    slope = (y[i + 1] - y[i]) / (x[i + 1] - x[i])
    return y[i] + slope * (v - x[i])


def trapz_abs(x: np.ndarray, y: np.ndarray) -> float:
    return 0.5 * float(np.sum(np.abs(np.diff(x)) * (y[1:] + y[:-1])))


class Lib:
    """One library's manifest and arrays (no selections: extra axes of length 1 only)."""

    def __init__(self, root: Path, kind: str, name: str):
        self.dir = Path(root) / "libraries" / kind / name
        self.man = json.loads((self.dir / "manifest.json").read_text())
        assert self.man["format"] in ("opensps-data", "fsps-data") and self.man["format_version"] == 1
        assert self.man["kind"] == kind and self.man["name"] == name

    def axis(self, name: str) -> np.ndarray:
        a = self.man["axes"][name]
        if "values" in a:
            return np.asarray(a["values"], dtype=np.float64)
        return self._read(a)

    def array(self, name: str) -> np.ndarray:
        return self._read(self.man["arrays"][name])

    def _read(self, d: dict) -> np.ndarray:
        dt = _DT[d["dtype"]]
        shape = tuple(d["shape"])
        raw = np.fromfile(self.dir / d["file"], dtype=dt)
        assert raw.size == int(np.prod(shape)), "file size differs from the declared shape"
        out = raw.reshape(shape)
        return out.astype(np.float64) if dt.kind == "f" else out.astype(np.int64)


def ssp_lbol(spec: np.ndarray, lam: np.ndarray) -> np.ndarray:
    """log10 L_bol per (Z, age) of spectra (nz, nt, nspec)."""
    nu = np.where(lam > SAFE_FLOOR, C_LIGHT / lam, 0.0)
    out = np.empty(spec.shape[:2])
    for z in range(spec.shape[0]):
        for t in range(spec.shape[1]):
            out[z, t] = np.log10(max(trapz_abs(nu, spec[z, t]), SAFE_FLOOR))
    return out


def dust_emission(root: Path, lam: np.ndarray, name: str = "DL07") -> dict:
    """The templates on the grid in the oracle's dust-emission format: dustem (2 numin, nqpah, nspec)."""
    L = Lib(root, "dust_emission", name)
    q, u, wl = L.axis("qpah"), L.axis("umin"), L.axis("wavelength")
    raw = L.array("spectra")                                   # (nq, nu, 2, nw)
    start = max(find_interval(lam, 1.0e4), 1) - 1
    tab = np.zeros((2 * u.size, q.size, lam.size))
    for iq in range(q.size):
        for col in range(2 * u.size):
            tab[col, iq, start:] = interp_linear_at(wl, raw[iq, col // 2, col % 2], lam[start:])
    return {"qpah": q, "umin": u, "dustem": tab}


def nebular(root: Path, lam: np.ndarray, name: str) -> dict:
    """nebular/<name> (load_nebular_grid / read_nebular_standard, opensps_io.f90:749-827,910-933) in the oracle's
    format: cont = log10(continuum + 1e-95) interpolated linearly onto the grid, (logU, age, logZ, nspec) C order
    (nebem_cont(j, z, a, u) column-major); logz, lage (log10 of the ages), logu."""
    L = Lib(root, "nebular", name)
    lz, age, lu, wl = L.axis("logZ"), L.axis("age"), L.axis("logU"), L.axis("wavelength")
    raw = L.array("continuum")                                 # (11, 10, 7, nw)
    cont = np.empty((lu.size, age.size, lz.size, lam.size))
    for z in range(lz.size):
        for a in range(age.size):
            for u in range(lu.size):
                cont[u, a, z] = interp_linear_at(wl, np.log10(raw[z, a, u] + 1.0e-95), lam)
    return {"cont": cont, "logz": lz, "lage": np.log10(age), "logu": lu}


def agn(root: Path, lam: np.ndarray) -> dict:
    """The torus templates on the grid in the oracle's AGN format: agnspec (9, nspec)."""
    L = Lib(root, "agn_torus", "clumpy")
    tau, wl = L.axis("tau"), L.axis("wavelength")
    raw = L.array("spectra")                                   # (9, nw)
    i1 = max(find_interval(lam, wl[0]), 1) - 1
    i2 = max(find_interval(lam, wl[-1]), 1) - 1
    lw = np.log10(wl)
    tab = np.zeros((tau.size, lam.size))
    for t in range(tau.size):
        ly = np.log10(raw[t] + SAFE_FLOOR)
        hi = min(i2, lam.size - 1) + 1
        if hi > i1:
            tab[t, i1:hi] = 10.0 ** interp_linear_at(lw, ly, np.log10(lam[i1:hi])) - SAFE_FLOOR
    return {"tau": tau, "agnspec": tab}


def attenuation(root: Path, name: str, lam: np.ndarray) -> np.ndarray:
    """attenuation/smc_bar (1, nspec) or attenuation/dirty (2 x 18 x 6, nspec): each curve interpolated linearly at
    the pixels inside its wavelength range, its first value below and zero above (load_attenuation_curves,
    opensps_io.f90:2079-2234)."""
    L = Lib(root, "attenuation", name)
    wl = L.axis("wavelength")
    raw = L.array("extinction" if name == "smc_bar" else "attenuation").reshape(-1, wl.size)
    out = np.empty((raw.shape[0], lam.size))
    for k in range(raw.shape[0]):
        v = interp_linear_at(wl, raw[k], lam)
        out[k] = np.where(lam > wl[-1], 0.0, np.where(lam < wl[0], raw[k, 0], v))
    return out


def filters(root: Path, name: str, lam: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(bands (nb, nspec), pivot wavelengths)."""
    L = Lib(root, "filters", name)
    npts = L.array("npoints")
    wl, tr = L.array("wavelength"), L.array("transmission")
    meta = L.man.get("metadata", {}).get("filters", [{}] * npts.size)
    ng = lam.size
    bands = np.zeros((npts.size, ng))
    pivot = np.zeros(npts.size)
    first = 0
    for i, n in enumerate(npts):
        lc, rc = [], []
        for k in range(first, first + int(n)):
            if lc and abs(wl[k] - lc[-1]) < SAFE_FLOOR:
                continue
            lc.append(wl[k])
            rc.append(max(tr[k], 0.0))
        first += int(n)
        lc, rc = np.asarray(lc), np.asarray(rc)
        if lc.size < 2:
            continue
        b = bands[i]
        si = 1 if lc[0] <= lam[0] else max(find_interval(lam, lc[0]), 1)
        ei = ng if lc[-1] >= lam[-1] else min(find_interval(lam, lc[-1]), ng)
        if ei > si:
            b[si - 1:ei] = interp_linear_at(lc, rc, lam[si - 1:ei])
        if meta[i].get("detector") == "energy":
            b /= lam
        np.maximum(b, 0.0, out=b)
        norm = trapz_abs(lam, b / (lam + SAFE_FLOOR))
        if norm > SAFE_FLOOR:
            b /= norm
        else:
            b[:] = 0.0
        a, d = trapz_abs(lam, lam * b), trapz_abs(lam, b / lam)
        pivot[i] = 0.0 if (a != a or d != d or d <= SAFE_FLOOR) else np.sqrt(a / d)
        cal = meta[i].get("calibration")
        if cal is not None:
            # filter_calibrate_band (opensps_filters.f90:505-518)
            dc = trapz_abs(lam, (lam / cal["lambda_ref"]) ** cal["exponent"] * b / (lam + SAFE_FLOOR))
            if dc > SAFE_FLOOR:
                b /= dc
    return bands, pivot


def load_data(root: Path, isoc: str = "synthetic", filter_sets: tuple[str, ...] = ("gauss20", "gauss40")) -> dict:
    """The oracle's data dictionary (as synthdata.load gives it) from a standard-format root: the SSP basis, its L_bol
    from the spectra, its lines when present, and the filter sets resampled onto the grid."""
    L = Lib(root, "ssp", isoc)
    lam = L.axis("wavelength")
    spec = L.array("spectra")
    out = {"lambda": lam, "log_age": L.axis("log_age"), "zlegend": L.axis("Z"), "ssp_spec": spec,
           "ssp_mass": L.array("stellar_mass"), "ssp_lbol": ssp_lbol(spec, lam),
           "manifest": {"zsol": L.man["metadata"]["solar_metallicity"]}}
    if "line_luminosity" in L.man["arrays"]:
        out["line_lambda"] = L.axis("line_wavelength")
        out["line_lum"] = L.array("line_luminosity")
    else:
        out["line_lambda"] = np.zeros(0)
        out["line_lum"] = np.zeros(spec.shape[:2] + (0,))
    for fs in filter_sets:
        b, piv = filters(root, fs, lam)
        out[f"filters_{b.shape[0]}"] = b
        out[f"filters_{b.shape[0]}_center"] = piv
    return out
