"""A context whose data root is in OpenSPS's standard format: the SSP basis from ssp/synthetic (L_bol from the
spectra), a filter library with energy-counting detectors, and the dust emission and AGN templates interpolated onto
the grid at load, through the whole mixed batch (nebular lines, IGM, dust emission, AGN), against the FP64 oracle
fed the numpy restatement of the same loaders (oracle/stdformat.py).

Tolerances as the batch's other tests: spectra <= 1e-4 relative (pixels above 1e-6 of the peak), magnitudes
<= 1e-3 mag, mass 1e-12 relative; L_bol (from the spectra's trapezoid) 1e-10 dex.
"""
import os

import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def std_root(tmp_path_factory, data):
    from libopensps_gb300 import stdformat, synthdata
    root = tmp_path_factory.mktemp("stdroot")
    stdformat.convert_synthetic(root, src_root=synthdata.default_root(), energy_every=4)
    return root


@pytest.fixture
def restore_root():
    old = os.environ.get("OPENSPS_DATA_HOME")
    yield
    if old is not None:
        os.environ["OPENSPS_DATA_HOME"] = old


def test_standard_root_batch(std_root, built_lib, restore_root):
    from libopensps_gb300.capi import Context
    from oracle import stdformat as ora
    from oracle.oracle import Oracle
    n = 24
    wz, params = config3_inputs(n, seed=931)
    rng = np.random.default_rng(932)
    params = dict(params, dust1=rng.uniform(0.1, 1.0, n), dust3=rng.uniform(0.0, 0.3, n),
                  duste_qpah=rng.uniform(0.5, 4.5, n), duste_umin=rng.uniform(0.1, 20.0, n),
                  duste_gamma=rng.uniform(0.0, 0.5, n), fagn=rng.uniform(0.0, 1.0, n), agn_tau=rng.uniform(5.0, 150.0, n))
    c = Context(data_root=std_root)
    c.set_filters_library("gauss20")
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_dust_emission", 1)
    c.set_int("add_agn_dust", 1)
    got = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    d = ora.load_data(std_root, filter_sets=("gauss20",))
    lam = d["lambda"]
    o = Oracle(d, nbands=20, dust_emission=ora.dust_emission(std_root, lam), agn=ora.agn(std_root, lam))
    want = o.csp_batch(params, wz)
    assert rel_err_spec(got["spec"], want["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - want["mags"]))) <= 1e-3
    np.testing.assert_allclose(got["mass"], want["mass"], rtol=1e-12)
    np.testing.assert_allclose(got["lbol"], want["lbol"], rtol=0, atol=1e-10)


def test_standard_root_refusals(std_root, built_lib, restore_root, tmp_path):
    """A standard root without the requested SSP library, and OPENSPS_DATA_FORMAT=standard with a library missing
    from it: status 4 with the library named."""
    from libopensps_gb300.capi import Context, OpenSPSError
    c = Context(data_root=std_root, setup=False)
    with pytest.raises(OpenSPSError) as e:
        c.setup(isoc="mist", spec="miles")
    assert e.value.status == 4 and "ssp/mist" in e.value.message
    c.setup()
    os.environ["OPENSPS_DATA_FORMAT"] = "standard"
    try:
        with pytest.raises(OpenSPSError) as e:
            c.set_filters_library("gauss99")
        assert "filters/gauss99" in e.value.message
    finally:
        del os.environ["OPENSPS_DATA_FORMAT"]
    c.close()
