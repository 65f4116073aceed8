"""The plain FP64 path on the GPU ("gb300_fp64": DGEMM age sums, every later stage in FP64) against the FP64 oracle:
two independent FP64 implementations of the batch agree to rounding (spectra <= 1e-9 relative over the pixels
above 1e-6 of the peak, magnitudes <= 1e-9 mag, mass and L_bol <= 1e-12 relative)."""
import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu


def test_fp64_path_matches_oracle(data, built_lib):
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_int("gb300_fp64", 1)
    n = 40
    wz, params = config3_inputs(n, seed=401)
    rng = np.random.default_rng(402)
    params = dict(params, dust1=rng.uniform(0.0, 1.0, n), dust3=rng.uniform(0.0, 0.3, n),
                  dust_index=rng.uniform(-1.0, -0.4, n))
    got = c.csp_batch(params, ssp_weights_z=wz)
    ora = Oracle(data, nbands=40).csp_batch(params, wz)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-9
    assert np.array_equal(np.isnan(got["mags"]), np.isnan(ora["mags"]))
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-9
    np.testing.assert_allclose(got["mass"], ora["mass"], rtol=1e-12)
    np.testing.assert_allclose(got["lbol"], ora["lbol"], rtol=1e-12)
    c.close()
