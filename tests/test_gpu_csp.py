"""Parity of the GPU batched CSP (through the C ABI) with the FP64 oracle on the same seeded inputs.

Tolerances: spectra <= 1e-4 max relative error over the pixels above 1e-6 of each model's peak; magnitudes
<= 1e-3 mag; mass and L_bol (FP64 sums) <= 1e-12 relative.
"""
import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(data, built_lib):
    from libopensps_gb300.capi import Context
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    yield c
    c.close()


@pytest.fixture(scope="module")
def oracle40(data):
    from oracle.oracle import Oracle
    return Oracle(data, nbands=40)


def _compare(got, ora, spec_tol=1e-4, mag_tol=1e-3):
    e_spec = rel_err_spec(got["spec"], ora["spec"])
    e_mag = float(np.nanmax(np.abs(got["mags"] - ora["mags"])))
    assert np.array_equal(np.isnan(got["mags"]), np.isnan(ora["mags"]))
    assert e_spec <= spec_tol, e_spec
    assert e_mag <= mag_tol, e_mag
    np.testing.assert_allclose(got["mass"], ora["mass"], rtol=1e-12)
    np.testing.assert_allclose(got["lbol"], ora["lbol"], rtol=1e-12)
    return e_spec, e_mag


@pytest.mark.parametrize("n", [1, 37, 300])
def test_mixed_csp_matches_oracle(ctx, oracle40, n):
    wz, params = config3_inputs(n, seed=100 + n)
    _compare(ctx.csp_batch(params, ssp_weights_z=wz), oracle40.csp_batch(params, wz))


def test_birth_cloud_and_old_screen(ctx, oracle40):
    """dust1 and dust3 need the young and old sums apart (two accumulators)."""
    n = 150
    wz, params = config3_inputs(n, seed=7)
    rng = np.random.default_rng(8)
    params = dict(params, dust1=rng.uniform(0.0, 2.0, n), dust3=rng.uniform(0.0, 0.5, n),
                  frac_obrun=rng.uniform(0.0, 0.3, n), frac_nodust=rng.uniform(0.0, 0.2, n),
                  dust_index=rng.uniform(-1.2, -0.3, n), dust1_index=rng.uniform(-1.5, -0.5, n))
    _compare(ctx.csp_batch(params, ssp_weights_z=wz), oracle40.csp_batch(params, wz))


def test_rest_frame_no_smoothing(ctx, oracle40):
    n = 40
    wz, params = config3_inputs(n, seed=9)
    params = {"dust2": params["dust2"], "zred": np.zeros(n), "sigma_smooth": np.zeros(n)}
    _compare(ctx.csp_batch(params, ssp_weights_z=wz), oracle40.csp_batch(params, wz))


def test_no_dust_is_sum_of_ssps(ctx, data):
    """With no dust, IGM, lines or smoothing the spectrum is sum_k w_k SSP_k (test_csp_batch.f90's identity)."""
    from libopensps_gb300.capi import Context
    c = Context()
    n = 20
    wz, _ = config3_inputs(n, seed=13)
    got = c.csp_batch({}, ssp_weights_z=wz)
    ref = np.einsum("mzt,zts->ms", wz, data["ssp_spec"])
    assert rel_err_spec(got["spec"], ref) <= 1e-4
    c.close()


def test_twenty_filters(data, built_lib):
    """The band GEMM with another band count (20 filters: 32 padded rows)."""
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_filters_library("gauss20")
    assert c.nbands == 20
    n = 70
    wz, params = config3_inputs(n, seed=21)
    _compare(c.csp_batch(params, ssp_weights_z=wz), Oracle(data, nbands=20).csp_batch(params, wz))
    c.close()


def test_weights_over_ages_blended_at_logzsol(ctx, oracle40, data):
    """ssp_weights (one weight per age) with logzsol per model: the two bracketing metallicities, linear in the
    spectra and the mass, log-linear in L_bol (compute_interpolated_ssp)."""
    n = 33
    rng = np.random.default_rng(17)
    w = rng.dirichlet(np.ones(107), size=n)
    logzsol = rng.uniform(-1.9, 0.4, n)
    _, params = config3_inputs(n, seed=18)
    params = dict(params, logzsol=logzsol)
    got = ctx.csp_batch(params, ssp_weights=w)
    lz = np.log10(data["zlegend"] / 0.0142)
    wz = np.zeros((n, 12, 107))
    lbol = np.empty(n)
    for m in range(n):
        zlo = min(max(np.searchsorted(lz, logzsol[m], side="right") - 1, 0), 10)
        dz = (logzsol[m] - lz[zlo]) / (lz[zlo + 1] - lz[zlo])
        wz[m, zlo] = (1 - dz) * w[m]
        wz[m, zlo + 1] = dz * w[m]
        lbol[m] = np.log10(np.sum(w[m] * 10.0 ** ((1 - dz) * data["ssp_lbol"][zlo] + dz * data["ssp_lbol"][zlo + 1])))
    ora = oracle40.csp_batch({k: v for k, v in params.items() if k != "logzsol"}, wz)
    ora["lbol"] = lbol
    _compare(got, ora)


def test_parts_and_emission_lines(ctx, oracle40, data):
    """compute_csp_batch_parts: the young and old age sums (nebular lines in the young), their masses and L_bol, and
    the emission-line luminosities."""
    n = 45
    rng = np.random.default_rng(31)
    w = rng.dirichlet(np.ones(107), size=n)
    logzsol = rng.uniform(-1.9, 0.4, n)
    _, params = config3_inputs(n, seed=32)
    params = dict(params, logzsol=logzsol, dust1=rng.uniform(0.0, 1.0, n))
    got = ctx.csp_batch_parts(params, w)
    lz = np.log10(data["zlegend"] / 0.0142)
    wz = np.zeros((n, 12, 107))
    for m in range(n):
        zlo = min(max(np.searchsorted(lz, logzsol[m], side="right") - 1, 0), 10)
        dz = (logzsol[m] - lz[zlo]) / (lz[zlo + 1] - lz[zlo])
        wz[m, zlo] = (1 - dz) * w[m]
        wz[m, zlo + 1] = dz * w[m]
    ora = oracle40.csp_batch({k: v for k, v in params.items() if k != "logzsol"}, wz, young=True, emlines=True)
    assert rel_err_spec(got["young"], ora["young"]) <= 1e-4
    assert rel_err_spec(got["old"], ora["old"]) <= 1e-4
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    young_ages = data["log_age"] <= 7.0
    np.testing.assert_allclose(got["mass_young"], np.einsum("mzt,zt->m", wz[:, :, young_ages],
                                                            data["ssp_mass"][:, young_ages]), rtol=1e-12)
    np.testing.assert_allclose(got["mass_young"] + got["mass_old"], got["mass"], rtol=1e-12)
    np.testing.assert_allclose(got["emlines"], ora["emlines"], rtol=1e-5)


def test_chunked_batch_pageable_and_page_locked_weights(ctx, oracle40):
    """A batch large enough to go up in chunks (40,000 models): from pageable weights (read in place where the device
    reads pageable memory) and from page-locked weights (copied) the outputs are identical, and a sample of models
    matches the oracle."""
    import torch
    n = 40000
    wz, params = config3_inputs(n, seed=77)
    a = ctx.csp_batch(params, ssp_weights_z=wz, spec=False)
    in_place = ctx.last_input_in_place()
    pinned = torch.from_numpy(wz).pin_memory()
    b = ctx.csp_batch(params, ssp_weights_z=pinned.numpy(), spec=False)
    assert not ctx.last_input_in_place()
    for k in ("mags", "mass", "lbol"):
        np.testing.assert_array_equal(a[k], b[k])
    idx = np.arange(0, n, 4999)
    ref = oracle40.csp_batch({k: v[idx] for k, v in params.items()}, wz[idx])
    assert float(np.nanmax(np.abs(a["mags"][idx] - ref["mags"]))) <= 1e-3
    np.testing.assert_allclose(a["mass"][idx], ref["mass"], rtol=1e-12)
    assert in_place in (True, False)
