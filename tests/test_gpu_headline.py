"""The headline workload at its own size: the mixed-precision batched CSP at B = 65536 on the benchmark's own inputs
(libopensps_gb300.workloads.mixed_csp(65536, seed=1000): 107 ages x 12 metallicities per model, nebular lines, dust
tau_V 0-3, z 0-6 with the IGM, smoothing 50-300 km/s, 40 filters), through the OpenSPS C API
(opensps_context_compute_csp_batch_grad with no cotangents; the batch goes up in 16384-model chunks).

A strided sample of 512 models, one in every 128-model tile with the tile position stepping through all 128 (so every
row of the contraction's model tiles and every chunk is covered), is compared with the FP64 oracle: spectra <= 1e-4
relative over the pixels above 1e-6 of each model's peak, magnitudes <= 1e-3 mag, mass and L_bol <= 1e-12
relative. Size-independent checks on all 65536 models: every spectrum and magnitude finite, mass and L_bol equal to
the weights' FP64 sums, and a repeat call bit-identical (a checksum of the spectra).
"""
import numpy as np
import pytest

from conftest import rel_err_spec

pytestmark = pytest.mark.gpu

N = 65536


@pytest.fixture(scope="module")
def headline(data, built_lib):
    from libopensps_gb300 import workloads
    from libopensps_gb300.capi import Context
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    wz, params = workloads.mixed_csp(N, seed=1000)
    out = c.csp_batch(params, ssp_weights_z=wz)
    yield c, wz, params, out
    c.close()


def test_headline_sample_matches_oracle(headline, data):
    from oracle.oracle import Oracle
    c, wz, params, got = headline
    k = np.arange(512)
    idx = k * 128 + (k % 128)
    assert idx.max() < N and np.unique(idx % 128).size == 128 and np.unique(idx // 16384).size == 4
    ora = Oracle(data, nbands=c.nbands).csp_batch({key: v[idx] for key, v in params.items()}, wz[idx])
    e_spec = rel_err_spec(got["spec"][idx], ora["spec"])
    e_mag = float(np.nanmax(np.abs(got["mags"][idx] - ora["mags"])))
    assert np.array_equal(np.isnan(got["mags"][idx]), np.isnan(ora["mags"]))
    assert e_spec <= 1e-4, e_spec
    assert e_mag <= 1e-3, e_mag
    np.testing.assert_allclose(got["mass"][idx], ora["mass"], rtol=1e-12)
    np.testing.assert_allclose(got["lbol"][idx], ora["lbol"], rtol=1e-12)


def test_headline_whole_batch_properties(headline, data):
    c, wz, params, got = headline
    assert np.all(np.isfinite(got["spec"]))
    assert np.all(np.isfinite(got["mags"]))
    # the FP64 mass of every model: the weights' sum against the SSP masses
    mass = np.einsum("mzt,zt->m", wz, data["ssp_mass"].reshape(wz.shape[1], wz.shape[2]))
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-12)
    again = c.csp_batch(params, ssp_weights_z=wz)
    assert np.array_equal(again["mags"], got["mags"])
    assert float(np.sum(again["spec"])) == float(np.sum(got["spec"]))
