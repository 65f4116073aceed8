"""The SSP operator with a Kroupa IMF per model (opensps_context_build_ssp_ops / evaluate_ssp_op, and the batch with
operators) against the FP64 oracle (ops_oracle.c) over the synthetic operator dataset.

Tolerances: spectra <= 1e-4 relative over the pixels above 1e-6 of each spectrum's peak (FP32 IMF bin weights, the
split-BF16 template GEMM); magnitudes <= 1e-3 mag; mass and L_bol <= 1e-5 relative (FP32 bin weights, FP64 sums).
"""
import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops_data():
    from libopensps_gb300 import synth_ops
    return synth_ops.load()


@pytest.fixture(scope="module")
def octx(data, built_lib, ops_data):
    from libopensps_gb300.capi import Context
    c = Context()
    c.set_int("add_igm_absorption", 1)
    c.build_ssp_ops()
    assert c.has_ssp_ops
    yield c
    c.close()


@pytest.mark.parametrize("imf,zmet", [((1.3, 2.3, 2.3), 1), ((0.5, 1.5, 3.0), 5), ((1.8, 2.8, 1.9), 12)])
def test_evaluate_ssp_op_matches_oracle(octx, ops_data, imf, zmet):
    from oracle.oracle import OpsOracle
    octx.set_int("zmet", zmet)
    got = octx.evaluate_ssp_op([imf[0], imf[1], imf[2], 0.08, 0.5])
    nt, nz = octx.ntfull, octx.nz
    wz = np.zeros((nt, nz, nt))
    for t in range(nt):
        wz[t, zmet - 1, t] = 1.0
    y, o, mass, ls = OpsOracle(ops_data).parts(np.tile(imf, (nt, 1)), wz, nt)
    assert np.all(o == 0.0)
    assert rel_err_spec(got["spec"], y) <= 1e-4
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)
    np.testing.assert_allclose(got["lbol"], np.log10(ls), rtol=1e-5)
    octx.set_int("zmet", 1)


def test_batch_with_imf_per_model_matches_oracle(octx, data, ops_data):
    """The IMF-free batch: slopes uniform in [0.3, 1.8], [1.3, 2.8], [1.8, 3.3] per model, weights over ages and
    metallicities, dust, redshift with IGM, velocity smoothing."""
    from oracle.oracle import Oracle, OpsOracle
    n = 48
    wz, params = config3_inputs(n, seed=301)
    rng = np.random.default_rng(302)
    alpha = np.stack([rng.uniform(0.3, 1.8, n), rng.uniform(1.3, 2.8, n), rng.uniform(1.8, 3.3, n)], axis=1)
    params = dict(params, imf1=alpha[:, 0], imf2=alpha[:, 1], imf3=alpha[:, 2], dust1=rng.uniform(0.0, 1.0, n))
    got = octx.csp_batch(params, ssp_weights_z=wz)
    assert octx.ops_last_interpolated()          # every slope inside the interpolated fold's range
    itesc = int(np.clip(np.searchsorted(data["log_age"], 7.0, side="right"), 1, data["log_age"].size))
    y, o, mass, ls = OpsOracle(ops_data).parts(alpha, wz, itesc)
    ora = Oracle(data, nbands=40, add_neb=False).csp_from_parts(
        {k: v for k, v in params.items() if not k.startswith("imf")}, y, o)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert np.array_equal(np.isnan(got["mags"]), np.isnan(ora["mags"]))
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)
    np.testing.assert_allclose(got["lbol"], np.log10(ls), rtol=1e-5)


def test_interpolated_and_exact_folds_agree(octx, data, ops_data):
    """The interpolated fold (the GEMM against the Lagrange basis in ln m) against the exact fold on the same batch:
    spectra within 2e-5 relative (above 1e-6 of the peak), mass and L_bol within 1e-6; a batch with one slope
    outside the interpolated range (imf1 = 2.8) takes the exact fold and matches the oracle."""
    from oracle.oracle import Oracle, OpsOracle
    n = 40
    wz, params = config3_inputs(n, seed=311)
    rng = np.random.default_rng(312)
    alpha = np.stack([rng.uniform(-0.5, 2.6, n), rng.uniform(0.5, 3.0, n), rng.uniform(1.0, 3.5, n)], axis=1)
    params = dict(params, imf1=alpha[:, 0], imf2=alpha[:, 1], imf3=alpha[:, 2])
    a = octx.csp_batch(params, ssp_weights_z=wz)
    assert octx.ops_last_interpolated()
    octx.set_int("gb300_ops_exact", 1)
    try:
        b = octx.csp_batch(params, ssp_weights_z=wz)
        assert not octx.ops_last_interpolated()
    finally:
        octx.set_int("gb300_ops_exact", 0)
    assert rel_err_spec(a["spec"], b["spec"]) <= 2e-5
    np.testing.assert_allclose(a["mass"], b["mass"], rtol=1e-6)
    np.testing.assert_allclose(a["lbol"], b["lbol"], rtol=1e-6)
    # outside the range: the exact fold, against the oracle
    alpha[3, 0] = 2.8
    params["imf1"] = alpha[:, 0]
    got = octx.csp_batch(params, ssp_weights_z=wz)
    assert not octx.ops_last_interpolated()
    itesc = int(np.clip(np.searchsorted(data["log_age"], 7.0, side="right"), 1, data["log_age"].size))
    y, o, mass, ls = OpsOracle(ops_data).parts(alpha, wz, itesc)
    ora = Oracle(data, nbands=40, add_neb=False).csp_from_parts(
        {k: v for k, v in params.items() if not k.startswith("imf")}, y, o)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)


def test_operator_refusals(data, built_lib, ops_data):
    from libopensps_gb300.capi import Context, OpenSPSError
    c = Context()
    wz, params = config3_inputs(4, seed=5)
    # an IMF per model without operators
    with pytest.raises(OpenSPSError) as e:
        c.csp_batch(dict(params, imf1=np.array([1.0, 1.3, 1.3, 1.3])), ssp_weights_z=wz)
    assert e.value.status == 2
    c.build_ssp_ops()
    # nebular emission with the operators
    c.set_int("add_neb_emission", 1)
    with pytest.raises(OpenSPSError) as e:
        c.csp_batch(params, ssp_weights_z=wz)
    assert e.value.status == 2
    c.set_int("add_neb_emission", 0)
    # an IMF type beyond the reference's 0 - 5
    with pytest.raises(OpenSPSError) as e:
        c.evaluate_ssp_op([1.3, 2.3, 2.3, 0.08, 0.5], imf_type=6)
    assert e.value.status == 2
    c.free_ssp_ops()
    assert not c.has_ssp_ops
    with pytest.raises(OpenSPSError) as e:
        c.evaluate_ssp_op()
    assert e.value.status == 303
    c.close()
