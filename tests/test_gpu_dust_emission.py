"""Dust emission (add_dust_emission = 1: the energy balance of dust_emission_reductions / add_dust_emission with the
Draine & Li template grid, src/physics/opensps_csp_batch.f90:3963-4122) and the AGN torus (add_agn_dust = 1:
add_agn_batch :4342-4433) against the FP64 oracle, and the balances themselves: with IGM and smoothing off, the
spectrum's luminosity (trapezoids in frequency over the grid) equals that of the unattenuated young and old sums, and
the AGN adds fagn L_bol.

Tolerances: spectra <= 1e-4 relative (pixels above 1e-6 of the peak), magnitudes <= 1e-3 mag, the luminosity
balance <= 2e-5 relative (FP32 sums over 5994 pixels).
"""
import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu

C_LIGHT = 2.99792458e18


@pytest.fixture(scope="module")
def dust():
    from libopensps_gb300 import synth_dust
    return synth_dust.load()


def _dust_params(n, rng):
    return {"dust1": rng.uniform(0.1, 1.0, n), "dust2": rng.uniform(0.1, 2.0, n), "dust3": rng.uniform(0.0, 0.4, n),
            "frac_obrun": rng.uniform(0.0, 0.3, n), "frac_nodust": rng.uniform(0.0, 0.2, n),
            "duste_qpah": rng.uniform(0.2, 5.0, n), "duste_umin": rng.uniform(0.05, 30.0, n),
            "duste_gamma": rng.uniform(0.0, 0.6, n)}


def test_dust_emission_matches_oracle(data, built_lib, dust):
    """The mixed batch (nebular lines, IGM at z 0-6, smoothing) with dust emission, slopes of q_PAH and U_min
    reaching beyond the grid on both sides (clamped cells), and some models without dust (no emission)."""
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    n = 40
    wz, params = config3_inputs(n, seed=901)
    rng = np.random.default_rng(902)
    params = dict(params, **_dust_params(n, rng))
    params["dust1"][:4] = 0.0
    params["dust2"][:4] = 0.0
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_dust_emission", 1)
    got = c.csp_batch(params, ssp_weights_z=wz)
    ora = Oracle(data, nbands=40, dust_emission=dust).csp_batch(params, wz)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert np.array_equal(np.isnan(got["mags"]), np.isnan(ora["mags"]))
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3
    np.testing.assert_allclose(got["mass"], ora["mass"], rtol=1e-12)
    # the emission is there: the same batch without it differs, except for the dust-free models
    c.set_int("add_dust_emission", 0)
    plain = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    assert np.array_equal(got["spec"][:4], plain["spec"][:4])
    assert float(np.nanmax(np.abs(got["mags"][4:] - plain["mags"][4:]))) > 0.1


def test_energy_balance(data, built_lib):
    """IGM and smoothing off: the trapezoid luminosity of the spectrum equals that of the intrinsic young + old sums
    (what the screens absorb comes back as dust emission)."""
    from libopensps_gb300.capi import Context
    n = 24
    rng = np.random.default_rng(903)
    w = rng.dirichlet(np.ones(107), size=n)
    params = dict(_dust_params(n, rng), logzsol=rng.uniform(-1.5, 0.3, n))
    c = Context()
    c.set_int("add_dust_emission", 1)
    got = c.csp_batch_parts(params, w, emlines=False)
    c.close()
    nu = C_LIGHT / data["lambda"]
    tr = lambda s: np.sum(0.5 * np.abs(np.diff(nu)) * (s[:, 1:] + s[:, :-1]), axis=1)
    np.testing.assert_allclose(tr(got["spec"]), tr(got["young"] + got["old"]), rtol=2e-5)


def test_dust_emission_through_the_operator(data, built_lib, dust):
    """The SSP operator's batch (an IMF per model) with dust emission: the same epilogue after the operator's young
    and old sums."""
    from libopensps_gb300 import synth_ops
    from libopensps_gb300.capi import Context
    from oracle.oracle import OpsOracle, Oracle
    ops = synth_ops.load()
    n = 16
    wz, params = config3_inputs(n, seed=904)
    rng = np.random.default_rng(905)
    alpha = np.stack([rng.uniform(0.3, 1.8, n), rng.uniform(1.3, 2.8, n), rng.uniform(1.8, 3.3, n)], axis=1)
    params = dict(params, imf1=alpha[:, 0], imf2=alpha[:, 1], imf3=alpha[:, 2], **_dust_params(n, rng))
    c = Context()
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_dust_emission", 1)
    c.build_ssp_ops()
    got = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    itesc = int(np.clip(np.searchsorted(data["log_age"], 7.0, side="right"), 1, data["log_age"].size))
    y, o, _, _ = OpsOracle(ops).parts(alpha, wz, itesc)
    ora = Oracle(data, nbands=40, add_neb=False, dust_emission=dust).csp_from_parts(
        {k: v for k, v in params.items() if not k.startswith("imf")}, y, o)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3


def test_dust_emission_refusals(data, built_lib):
    from libopensps_gb300.capi import Context, OpenSPSError
    n = 4
    wz, params = config3_inputs(n, seed=906)
    params = dict(params, dust1=np.full(n, 0.3))
    c = Context()
    c.set_int("add_dust_emission", 1)
    c.set_int("gb300_fp64", 1)
    with pytest.raises(OpenSPSError) as e:
        c.csp_batch(params, ssp_weights_z=wz)
    assert e.value.status == 2
    c.close()


@pytest.fixture(scope="module")
def agn():
    from libopensps_gb300 import synth_dust
    return synth_dust.load_agn()


def test_agn_and_dust_emission_match_oracle(data, built_lib, dust, agn):
    """The AGN torus (add_agn_dust: fagn L_bol times the template at agn_tau through the diffuse dust, after the IGM)
    with dust emission on the mixed batch, agn_tau beyond the grid on both sides, some models without AGN."""
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    n = 32
    wz, params = config3_inputs(n, seed=911)
    rng = np.random.default_rng(912)
    params = dict(params, **_dust_params(n, rng), fagn=rng.uniform(0.01, 3.0, n), agn_tau=rng.uniform(2.0, 200.0, n))
    params["fagn"][:5] = 0.0
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_dust_emission", 1)
    c.set_int("add_agn_dust", 1)
    got = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    ora = Oracle(data, nbands=40, dust_emission=dust, agn=agn).csp_batch(params, wz)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3


@pytest.mark.parametrize("weights", ["over_z", "sfh"])
def test_agn_luminosity(data, built_lib, weights):
    """Without dust, IGM and smoothing the AGN adds fagn L_bol (the model's L_bol output: the linear sum, or
    log-blended for weights formed on the device) to the spectrum's trapezoid luminosity (within 2e-5 of the whole,
    the two runs taking different kernel paths)."""
    from libopensps_gb300.capi import Context
    n = 16
    wz, params = config3_inputs(n, seed=913)
    rng = np.random.default_rng(914)
    params = {"fagn": rng.uniform(0.05, 2.0, n), "agn_tau": rng.uniform(5.0, 150.0, n)}
    c = Context()
    if weights == "sfh":
        c.set_int("sfh", 4)
        params.update(tage=rng.uniform(2.0, 12.0, n), tau=rng.uniform(0.3, 5.0, n), logzsol=rng.uniform(-1.5, 0.3, n))
        run = lambda: c.csp_batch(params)
    else:
        run = lambda: c.csp_batch(params, ssp_weights_z=wz)
    plain = run()
    c.set_int("add_agn_dust", 1)
    got = run()
    c.close()
    nu = C_LIGHT / data["lambda"]
    tr = lambda s: np.sum(0.5 * np.abs(np.diff(nu)) * (s[:, 1:] + s[:, :-1]), axis=1)
    np.testing.assert_allclose(got["lbol"], plain["lbol"], rtol=1e-12)
    want = params["fagn"] * 10.0 ** got["lbol"]
    assert np.all(np.abs(tr(got["spec"]) - tr(plain["spec"]) - want) <= 2e-5 * tr(got["spec"]))


def test_agn_through_the_operator(data, built_lib, agn):
    """The operator's batch with AGN: L_bol is the operator's linear row."""
    from libopensps_gb300 import synth_ops
    from libopensps_gb300.capi import Context
    from oracle.oracle import OpsOracle, Oracle
    ops = synth_ops.load()
    n = 12
    wz, params = config3_inputs(n, seed=915)
    rng = np.random.default_rng(916)
    alpha = np.stack([rng.uniform(0.3, 1.8, n), rng.uniform(1.3, 2.8, n), rng.uniform(1.8, 3.3, n)], axis=1)
    params = dict(params, imf1=alpha[:, 0], imf2=alpha[:, 1], imf3=alpha[:, 2], fagn=rng.uniform(0.05, 1.0, n),
                  agn_tau=rng.uniform(5.0, 150.0, n))
    c = Context()
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_agn_dust", 1)
    c.build_ssp_ops()
    got = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    itesc = int(np.clip(np.searchsorted(data["log_age"], 7.0, side="right"), 1, data["log_age"].size))
    y, o, _, ls = OpsOracle(ops).parts(alpha, wz, itesc)
    ora = Oracle(data, nbands=40, add_neb=False, agn=agn).csp_from_parts(
        {k: v for k, v in params.items() if not k.startswith("imf")}, y, o, lsum=ls)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3
