"""The standard data format (doc/DATA_FORMAT.md sections 2-3 of the reference; its reader src/io/opensps_datalib.f90):
the C-ABI library's loader (opensps_gb300_data_table, no device) against the numpy restatement in oracle/stdformat.py
on libraries written by libopensps_gb300/stdformat.py and, when OPENSPS_SOURCE_DIR names an OpenSPS source tree, on its own
test library (real DL07, THEMIS, clumpy-torus and filter manifests and arrays); and the reader's refusals (truncated
files, format versions, names, extra axes without a selection), selections and axis defaults.

Tolerances: relative 1e-13 (interpolations agree to rounding; the trapezoid sums differ only in summation order);
values of the log-interpolated AGN templates below 1e-12 of their peak absolutely.
"""
import json
import os
import shutil
from pathlib import Path

import numpy as np
import pytest

from libopensps_gb300 import stdformat, synthdata
from libopensps_gb300.capi import OpenSPSError, data_table
from oracle import stdformat as ora

# The OpenSPS source tree, when one is at hand (OPENSPS_SOURCE_DIR); its test library's cases skip otherwise.
REF_TEST_LIBRARY = Path(os.environ.get("OPENSPS_SOURCE_DIR", "/nonexistent")) / "tests" / "data" / "opensps-test-data"


@pytest.fixture(scope="module")
def lam():
    return synthdata.wavelength_grid()


@pytest.fixture(scope="module")
def std_root(tmp_path_factory):
    root = tmp_path_factory.mktemp("stdroot")
    stdformat.convert_synthetic(root, energy_every=3, nebular=True)
    return root


def test_root_index(std_root):
    idx = json.loads((std_root / "opensps-data.json").read_text())
    assert idx["format"] == "opensps-data" and idx["format_version"] == 1
    kinds = {(e["kind"], e["name"]) for e in idx["libraries"]}
    assert {("ssp", "synthetic"), ("filters", "gauss20"), ("dust_emission", "DL07"), ("agn_torus", "clumpy")} <= kinds


def test_ssp_lbol(std_root):
    got = data_table(std_root, "ssp", "synthetic")
    L = ora.Lib(std_root, "ssp", "synthetic")
    want = ora.ssp_lbol(L.array("spectra"), L.axis("wavelength")).ravel()
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13)


def test_dust_emission(std_root, lam):
    got = data_table(std_root, "dust_emission", "DL07", lam)
    want = ora.dust_emission(std_root, lam)["dustem"].reshape(-1, lam.size)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=0)
    # zero below the pixel holding 1 um, extrapolated (the native table starts at 0.5 um) above it
    start = ora.find_interval(lam, 1.0e4) - 1
    assert np.all(got[:, :start] == 0.0) and np.all(got[:, start:] != 0.0)


def test_agn(std_root, lam):
    got = data_table(std_root, "agn_torus", "clumpy", lam)
    want = ora.agn(std_root, lam)["agnspec"]
    # (interpolated in log10: an exponent near -300 carries its rounding into the value; below 1e-12 of the peak)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-12 * np.abs(want).max())


def test_nebular_continuum_table(std_root, lam):
    got = data_table(std_root, "nebular", "synthetic_nodust", lam)
    want = ora.nebular(std_root, lam, "synthetic_nodust")["cont"].reshape(-1, lam.size)
    assert got.shape == (11 * 10 * 7, lam.size)
    np.testing.assert_allclose(got, want, rtol=1e-13)


def test_filters_with_energy_detectors(std_root, lam):
    got = data_table(std_root, "filters", "gauss20", lam)
    want, _ = ora.filters(std_root, "gauss20", lam)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-300)
    # normalised: int T / lambda = 1 on the grid
    norm = 0.5 * np.sum(np.diff(lam) * (got[:, 1:] / lam[1:] + got[:, :-1] / lam[:-1]), axis=1)
    np.testing.assert_allclose(norm, 1.0, rtol=1e-12)


@pytest.mark.skipif(not REF_TEST_LIBRARY.exists(), reason="the reference's test library is not in this container")
@pytest.mark.parametrize("kind,name", [("dust_emission", "DL07"), ("dust_emission", "THEMIS"), ("agn_torus", "clumpy"),
                                       ("filters", "allfilters"), ("nebular", "mist_nodust"),
                                       ("attenuation", "smc_bar"), ("attenuation", "dirty")])
def test_reference_test_library(lam, kind, name):
    """The reader on the reference's own standard-format files (FP32 arrays, file-held axes, labels, filter
    calibrations) against the numpy restatement."""
    got = data_table(REF_TEST_LIBRARY, kind, name, lam)
    if kind == "dust_emission":
        want = ora.dust_emission(REF_TEST_LIBRARY, lam, name)["dustem"].reshape(-1, lam.size)
    elif kind == "agn_torus":
        want = ora.agn(REF_TEST_LIBRARY, lam)["agnspec"]
    elif kind == "attenuation":
        want = ora.attenuation(REF_TEST_LIBRARY, name, lam)
    elif kind == "nebular":
        # (the test subset's FP32 continuum underflows to zero: the table is the floor, log10(1e-95), everywhere)
        want = ora.nebular(REF_TEST_LIBRARY, lam, name)["cont"].reshape(-1, lam.size)
    else:
        want, _ = ora.filters(REF_TEST_LIBRARY, name, lam)
        meta = json.loads((REF_TEST_LIBRARY / "libraries/filters/allfilters/manifest.json").read_text())["metadata"]
        assert sum("calibration" in e for e in meta["filters"]) > 0
    assert got.shape == want.shape and np.any(got != 0.0)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


# ---- refusals, selections, defaults
def _copy_lib(src_root: Path, dst_root: Path, kind: str, name: str) -> Path:
    d = dst_root / "libraries" / kind / name
    shutil.copytree(src_root / "libraries" / kind / name, d)
    (dst_root / "opensps-data.json").write_text(json.dumps({"format": "opensps-data", "format_version": 1,
                                                            "libraries": []}))
    return d


def _status(fn):
    with pytest.raises(OpenSPSError) as e:
        fn()
    return e.value


def test_truncated_file(std_root, lam, tmp_path):
    d = _copy_lib(std_root, tmp_path, "dust_emission", "DL07")
    raw = (d / "spectra.bin").read_bytes()
    (d / "spectra.bin").write_bytes(raw[:-4])
    e = _status(lambda: data_table(tmp_path, "dust_emission", "DL07", lam))
    assert e.status == 4 and "bytes, expected" in e.message


def test_manifest_checks(std_root, lam, tmp_path):
    d = _copy_lib(std_root, tmp_path, "agn_torus", "clumpy")
    man = json.loads((d / "manifest.json").read_text())
    for field, value, msg in (("format_version", 2, "format_version"), ("kind", "agn", "manifest kind"),
                              ("name", "other", "directory name"), ("format", "x", "not an opensps-data manifest")):
        bad = dict(man, **{field: value})
        (d / "manifest.json").write_text(json.dumps(bad))
        e = _status(lambda: data_table(tmp_path, "agn_torus", "clumpy", lam))
        assert e.status == 4 and msg in e.message, e.message
    (d / "manifest.json").write_text(json.dumps(man)[:-2] + ",}")        # malformed JSON
    e = _status(lambda: data_table(tmp_path, "agn_torus", "clumpy", lam))
    assert e.status == 4 and "manifest.json" in e.message
    # a manifest with escapes and non-ASCII text parses
    (d / "manifest.json").write_text(json.dumps(dict(man, title="café \U0001F600 \"q\" \\ / \t")))
    want = ora.agn(std_root, lam)["agnspec"]
    np.testing.assert_allclose(data_table(tmp_path, "agn_torus", "clumpy", lam), want, rtol=1e-13,
                               atol=1e-12 * np.abs(want).max())


def test_missing_library(tmp_path, lam):
    e = _status(lambda: data_table(tmp_path, "filters", "nothing", lam))
    assert e.status == 4 and "not a standard-format data root" in e.message


def test_extra_axis_selection_and_default(std_root, lam, tmp_path):
    """An extra leading axis (here "grain", two values) must be selected ("DL07:grain=2.5") or carry a default; the
    selected block is read."""
    d = _copy_lib(std_root, tmp_path, "dust_emission", "DL07")
    man = json.loads((d / "manifest.json").read_text())
    a = man["arrays"]["spectra"]
    base = np.fromfile(d / a["file"], dtype="<f4").reshape(a["shape"])
    stacked = np.stack([base, 2.0 * base])                     # grain 1.0: the library, grain 2.5: twice it
    stacked.astype("<f4").tofile(d / a["file"])
    a["shape"] = [2] + a["shape"]
    a["axes"] = ["grain"] + a["axes"]
    man["axes"]["grain"] = {"units": "", "values": [1.0, 2.5]}
    (d / "manifest.json").write_text(json.dumps(man))
    e = _status(lambda: data_table(tmp_path, "dust_emission", "DL07", lam))
    assert e.status == 4 and "DL07:grain=<value>" in e.message
    want = data_table(std_root, "dust_emission", "DL07", lam)
    np.testing.assert_allclose(data_table(tmp_path, "dust_emission", "DL07:grain=2.5", lam), 2.0 * want, rtol=1e-6)
    np.testing.assert_allclose(data_table(tmp_path, "dust_emission", "DL07:grain=1", lam), want, rtol=0)
    e = _status(lambda: data_table(tmp_path, "dust_emission", "DL07:grain=3", lam))
    assert "has no value 3" in e.message
    e = _status(lambda: data_table(tmp_path, "dust_emission", "DL07:size=3", lam))
    assert "unknown axis" in e.message
    man["axes"]["grain"]["default"] = 2.5
    (d / "manifest.json").write_text(json.dumps(man))
    np.testing.assert_allclose(data_table(tmp_path, "dust_emission", "DL07", lam), 2.0 * want, rtol=1e-6)
