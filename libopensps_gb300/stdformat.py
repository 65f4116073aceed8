"""Writing data roots in OpenSPS's standard format (version 1; doc/DATA_FORMAT.md sections 2-3 of the reference).

A standard data root holds ``opensps-data.json`` and, per library, ``libraries/<kind>/<name>/manifest.json`` with one
raw little-endian array per file (C order, slowest axis first). The context reads such a root when it is its data
root (``OPENSPS_DATA_HOME``): the SSP basis of ``ssp/<isoc>`` at setup, ``filters/<name>`` for a filter library,
``dust_emission/DL07`` and ``agn_torus/clumpy`` for the dust emission and AGN terms.

``convert_synthetic`` writes the package's synthetic libraries in that format: the SSP basis (with its nebular lines
as an extra array, ``line_luminosity`` [Z, log_age, line_wavelength]), the Gaussian filter sets as tabulated curves
(81 points over +-4 sigma; with ``energy_every`` some marked as energy-counting detectors), and the dust emission and
AGN templates on native wavelength grids of their own (so that the reader's interpolation onto the model grid is
exercised).
"""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

from . import synth_dust, synthdata

FORMAT = "opensps-data"
VERSION = 1
DTYPES = ("<f4", "<f8", "<i4", "<i8")


def _sha(path: Path) -> str:
    return hashlib.sha256(path.read_bytes()).hexdigest()


def write_library(root: Path, kind: str, name: str, axes: dict, arrays: dict, metadata: dict | None = None,
                  title: str = "") -> Path:
    """One library. ``axes``: axis name -> dict with ``units`` and ``values`` (a list), ``labels`` (strings) or
    ``data`` (an ndarray written to ``axis_<name>.bin`` as <f8). ``arrays``: name -> (ndarray, dtype, axis names or
    None, units); the ndarray's shape (C order) is the array's shape."""
    d = Path(root) / "libraries" / kind / name
    d.mkdir(parents=True, exist_ok=True)
    man_axes = {}
    for an, spec in axes.items():
        e = {"units": spec.get("units", "")}
        for k in ("medium", "description", "default"):
            if k in spec:
                e[k] = spec[k]
        if "labels" in spec:
            e["labels"] = list(spec["labels"])
        elif "values" in spec:
            e["values"] = [float(v) for v in spec["values"]]
        else:
            a = np.ascontiguousarray(spec["data"], dtype="<f8")
            fn = f"axis_{an}.bin"
            a.tofile(d / fn)
            e.update({"file": fn, "dtype": "<f8", "shape": [int(a.size)], "sha256": _sha(d / fn)})
        man_axes[an] = e
    man_arrays = {}
    for an, (a, dtype, ax, units) in arrays.items():
        assert dtype in DTYPES
        a = np.ascontiguousarray(a).astype(dtype)
        fn = f"{an}.bin"
        a.tofile(d / fn)
        e = {"file": fn, "dtype": dtype, "shape": [int(x) for x in a.shape]}
        if ax is not None:
            e["axes"] = list(ax)
        e.update({"units": units, "sha256": _sha(d / fn)})
        man_arrays[an] = e
    man = {"format": FORMAT, "format_version": VERSION, "kind": kind, "name": name, "version": 1, "title": title,
           "metadata": metadata or {}, "axes": man_axes, "arrays": man_arrays}
    (d / "manifest.json").write_text(json.dumps(man, indent=1))
    return d


def write_root_index(root: Path, release: str = "synthetic") -> Path:
    """``opensps-data.json`` listing every library under ``root/libraries``."""
    root = Path(root)
    libs = []
    for m in sorted((root / "libraries").glob("*/*/manifest.json")):
        kind, name = m.parent.parent.name, m.parent.name
        libs.append({"kind": kind, "name": name, "path": f"libraries/{kind}/{name}"})
    idx = {"format": FORMAT, "format_version": VERSION, "release": release,
           "title": "Synthetic libraries in the standard format", "libraries": libs}
    p = root / "opensps-data.json"
    p.write_text(json.dumps(idx, indent=1))
    return p


def gaussian_curves(centres: np.ndarray, npts: int = 81) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Tabulated Gaussian filter curves (R = 5: FWHM = centre / 5) over +-4 sigma: (npoints, wavelength,
    transmission), the curves concatenated."""
    sig = centres / 5.0 / (2.0 * np.sqrt(2.0 * np.log(2.0)))
    lam = np.concatenate([np.linspace(c - 4 * s, c + 4 * s, npts) for c, s in zip(centres, sig)])
    tr = np.concatenate([np.exp(-0.5 * ((np.linspace(c - 4 * s, c + 4 * s, npts) - c) / s) ** 2)
                         for c, s in zip(centres, sig)])
    return np.full(centres.size, npts, dtype=np.int32), lam, tr


def convert_synthetic(out_root: Path, src_root: Path | None = None, energy_every: int = 0, dust: bool = True,
                      agn: bool = True, ssp_dtype: str = "<f8", nebular: bool = False) -> Path:
    """The synthetic libraries of ``src_root`` (written first if missing) as a standard-format root ``out_root``.
    Libraries: ssp/synthetic, filters/gauss20, filters/gauss40, dust_emission/DL07, agn_torus/clumpy, and with
    ``nebular`` the CLOUDY-style grid nebular/synthetic_nodust (the nebular continuum of the setup's isochrones)."""
    out_root = Path(out_root)
    data = synthdata.load(src_root)
    man = data["manifest"]
    write_library(
        out_root, "ssp", "synthetic",
        axes={"Z": {"units": "mass fraction", "values": data["zlegend"]},
              "log_age": {"units": "log10(yr)", "values": data["log_age"]},
              "wavelength": {"units": "angstrom", "medium": "vacuum", "data": data["lambda"]},
              "line_wavelength": {"units": "angstrom", "values": data["line_lambda"]}},
        arrays={"spectra": (data["ssp_spec"], ssp_dtype, ["Z", "log_age", "wavelength"], "L_sun/Hz per M_sun formed"),
                "stellar_mass": (data["ssp_mass"], "<f8", ["Z", "log_age"], "M_sun per M_sun formed"),
                "line_luminosity": (data["line_lum"], "<f8", ["Z", "log_age", "line_wavelength"],
                                    "L_sun per M_sun formed")},
        metadata={"solar_metallicity": float(man["zsol"])},
        title="Synthetic SSP basis (seeded; not for science)")
    for nb in man["filter_sets"]:
        npts, lam, tr = gaussian_curves(np.asarray(data[f"filters_{nb}_center"]))
        flt = []
        for i in range(nb):
            e = {"name": f"G{nb}_{i:02d}", "description": "Gaussian, R = 5"}
            if energy_every and i % energy_every == 0:
                e["detector"] = "energy"
            flt.append(e)
        write_library(out_root, "filters", f"gauss{nb}",
                      axes={"filter": {"units": "", "labels": [f["name"] for f in flt]}},
                      arrays={"npoints": (npts, "<i4", ["filter"], "count"),
                              "wavelength": (lam, "<f8", None, "angstrom"),
                              "transmission": (tr, "<f8", None, "relative throughput")},
                      metadata={"filters": flt}, title=f"{nb} Gaussian filters (synthetic)")
    if dust:
        wl = np.geomspace(5.0e3, 1.0e7, 240)
        nq, nu = synth_dust.QPAH.size, synth_dust.UMIN.size
        tab = np.empty((nq, nu, 2, wl.size))
        for iq in range(nq):
            for iu in range(nu):
                for c in range(2):
                    tab[iq, iu, c] = synth_dust._template(wl, synth_dust.QPAH[iq], synth_dust.UMIN[iu], c == 1)
        write_library(out_root, "dust_emission", "DL07",
                      axes={"qpah": {"units": "percent", "values": synth_dust.QPAH},
                            "umin": {"units": "U_min", "values": synth_dust.UMIN},
                            "component": {"units": "", "labels": ["umin", "umin_to_umax"]},
                            "wavelength": {"units": "angstrom", "data": wl}},
                      arrays={"spectra": (tab, "<f4", ["qpah", "umin", "component", "wavelength"], "L_nu")},
                      title="Synthetic dust emission templates (the DL07 grid's shape)")
    if agn:
        wl = np.geomspace(150.0, 3.0e6, 125)
        tab = np.stack([synth_dust._agn_template(wl, t) for t in synth_dust.AGN_TAU])
        write_library(out_root, "agn_torus", "clumpy",
                      axes={"tau": {"units": "optical depth", "values": synth_dust.AGN_TAU},
                            "wavelength": {"units": "angstrom", "values": wl}},
                      arrays={"spectra": (tab, "<f4", ["tau", "wavelength"], "f_nu, normalized to unity")},
                      title="Synthetic AGN torus templates")
    if nebular:
        from . import synth_nebular
        synth_nebular.write(out_root, "synthetic_nodust")
    write_root_index(out_root)
    return out_root
