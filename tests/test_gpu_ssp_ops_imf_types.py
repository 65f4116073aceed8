"""The SSP operator with the Salpeter (imf_type 0, slope 2.35: the Kroupa form with equal slopes) and Chabrier 2003
(imf_type 1: the lognormal below 1 M_sun, the power law above; the interpolated fold's node values from its density)
IMFs, against the FP64 oracle's bin integrals of the same IMFs (ops_oracle.c, imf_integral cases 0 and 1 of
src/physics/opensps_imf.f90:206-315): evaluate_ssp_op at every age, the batch through the operator, the reverse
pass's weights' cotangent along a random direction against central differences, the slopes' rows zero (no
parameters), and the refusals (imf_type 3-5; Chabrier with the exact fold forced).

Tolerances as the Kroupa tests: spectra <= 1e-4 relative (pixels above 1e-6 of the peak), magnitudes <= 1e-3 mag,
mass and L_bol <= 1e-5 relative; gradients 2e-3.
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
    yield c
    c.set_int("imf_type", 2)
    c.close()


def _itesc(data):
    return int(np.clip(np.searchsorted(data["log_age"], 7.0, side="right"), 1, data["log_age"].size))


@pytest.mark.parametrize("imf_type", [0, 1])
def test_evaluate_ssp_op(octx, ops_data, imf_type):
    from oracle.oracle import OpsOracle
    octx.set_int("zmet", 4)
    got = octx.evaluate_ssp_op([1.3, 2.3, 2.3, 0.08, 0.5], imf_type=imf_type)
    octx.set_int("zmet", 1)
    nt, nz = octx.ntfull, octx.nz
    wz = np.zeros((nt, nz, nt))
    for t in range(nt):
        wz[t, 3, t] = 1.0
    y, o, mass, ls = OpsOracle(ops_data, imf_type=imf_type).parts(np.tile([1.3, 2.3, 2.3], (nt, 1)), wz, nt)
    assert rel_err_spec(got["spec"], y) <= 1e-4
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)
    np.testing.assert_allclose(got["lbol"], np.log10(ls), rtol=1e-5)


@pytest.mark.parametrize("imf_type", [0, 1])
def test_batch_matches_oracle(octx, data, ops_data, imf_type):
    from oracle.oracle import Oracle, OpsOracle
    n = 40
    wz, params = config3_inputs(n, seed=330 + imf_type)
    rng = np.random.default_rng(332)
    params = dict(params, dust1=rng.uniform(0.0, 1.0, n))
    octx.set_int("imf_type", imf_type)
    try:
        got = octx.csp_batch(params, ssp_weights_z=wz)
        assert octx.ops_last_interpolated()
        if imf_type == 0:
            # the exact fold (Kroupa segments with equal slopes) gives the same
            octx.set_int("gb300_ops_exact", 1)
            exact = octx.csp_batch(params, ssp_weights_z=wz)
            octx.set_int("gb300_ops_exact", 0)
            assert rel_err_spec(exact["spec"], got["spec"]) <= 5e-5
    finally:
        octx.set_int("imf_type", 2)
    y, o, mass, ls = OpsOracle(ops_data, imf_type=imf_type).parts(np.tile([2.35] * 3, (n, 1)), wz, _itesc(data))
    ora = Oracle(data, nbands=40, add_neb=False).csp_from_parts(params, y, o)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)
    np.testing.assert_allclose(got["lbol"], np.log10(ls), rtol=1e-5)
    # Salpeter and Chabrier differ (the IMF is in effect)
    if imf_type == 1:
        y0, _, m0, _ = OpsOracle(ops_data, imf_type=0).parts(np.tile([2.35] * 3, (n, 1)), wz, _itesc(data))
        assert float(np.max(np.abs(mass / m0 - 1.0))) > 1e-3


@pytest.mark.parametrize("imf_type", [0, 1])
def test_reverse_pass(octx, data, ops_data, imf_type):
    """The weights' cotangent along a random relative direction against central differences of the oracle; the
    slopes' rows (26-28) zero."""
    from libopensps_gb300.workloads import adjoint_cotangents
    from oracle.oracle import Oracle, OpsOracle
    n = 5
    wz, params = config3_inputs(n, seed=340 + imf_type)
    mb, sb = adjoint_cotangents(n, data["lambda"].size, 40, seed=341)
    octx.set_int("imf_type", imf_type)
    try:
        got = octx.csp_batch_grad(dict(params, imf1=np.full(n, 1.1)), wz, mags_bar=mb, spec_bar=sb)
    finally:
        octx.set_int("imf_type", 2)
    assert np.all(got["params_bar"][:, 26:29] == 0.0)
    ops = OpsOracle(ops_data, imf_type=imf_type)
    csp = Oracle(data, nbands=40, add_neb=False)
    alpha = np.tile([2.35] * 3, (n, 1))

    def loss(w):
        y, o, mass, ls = ops.parts(alpha, w, _itesc(data))
        out = csp.csp_from_parts(params, y, o)
        return np.nansum(mb * out["mags"], axis=1) + np.sum(sb * out["spec"], axis=1)

    rng = np.random.default_rng(342)
    dw = wz * rng.standard_normal(wz.shape)
    fd = (loss(wz + 1e-4 * dw) - loss(wz - 1e-4 * dw)) / 2e-4
    g = np.sum(got["weights_z_bar"] * dw, axis=(1, 2))
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert float(err.max()) <= 2e-3, (g, fd)


def test_refusals(octx, data):
    from libopensps_gb300.capi import OpenSPSError
    n = 4
    wz, params = config3_inputs(n, seed=350)
    for t in (3, 4, 5):
        octx.set_int("imf_type", t)
        with pytest.raises(OpenSPSError) as e:
            octx.csp_batch(params, ssp_weights_z=wz)
        assert e.value.status == 2
    octx.set_int("imf_type", 1)
    octx.set_int("gb300_ops_exact", 1)
    try:
        with pytest.raises(OpenSPSError) as e:
            octx.csp_batch(params, ssp_weights_z=wz)
        assert e.value.status == 2 and "Chabrier" in e.value.message
    finally:
        octx.set_int("gb300_ops_exact", 0)
        octx.set_int("imf_type", 2)
