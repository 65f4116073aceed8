"""The SSP operator with the Salpeter (imf_type 0, slope 2.35: the Kroupa form with equal slopes), Chabrier 2003
(imf_type 1: the lognormal below 1 M_sun, the power law above; the interpolated fold's node values from its density),
van Dokkum 2008 (imf_type 3: vdmc per model, a lognormal up to 25 vdmc) and Dave 2008 (imf_type 4: imf1, imf2 and
mdave per model) IMFs, the last two through the exact fold (their breaks move with the model), against the FP64
oracle's bin integrals of the same IMFs (ops_oracle.c, imf_integral cases 0, 1, 3, 4 of
src/physics/opensps_imf.f90:206-315): evaluate_ssp_op at every age, the batch through the operator, the reverse
pass's weights' cotangent along a random direction against central differences, the IMF's rows (zero for
Salpeter, Chabrier and van Dokkum, which have no parameters there; Dave's imf1, imf2 and mdave against central
differences, imf_integral_dp :833-900), Chabrier's exact fold against its interpolated one, and the refusal of
an IMF type beyond 5 (the user IMF, type 5, and other mass limits: test_gpu_ssp_ops_user_imf.py).

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


def _packed(imf_type, imf1, imf2, imf3, vdmc, mdave):
    """The oracle's three IMF parameters per model (as the operator kernels take them)."""
    if imf_type == 3:
        return np.stack([vdmc, np.zeros_like(vdmc), np.zeros_like(vdmc)], axis=1)
    if imf_type == 4:
        return np.stack([imf1, imf2, mdave], axis=1)
    if imf_type == 2:
        return np.stack([imf1, imf2, imf3], axis=1)
    return np.full((np.size(imf1), 3), 2.35)


@pytest.mark.parametrize("imf_type", [0, 1, 3, 4])
def test_evaluate_ssp_op(octx, ops_data, imf_type):
    from oracle.oracle import OpsOracle
    octx.set_int("zmet", 4)
    pv = [1.1, 2.1, 2.6, 0.3, 0.9]
    got = octx.evaluate_ssp_op(pv, imf_type=imf_type)
    octx.set_int("zmet", 1)
    nt, nz = octx.ntfull, octx.nz
    wz = np.zeros((nt, nz, nt))
    for t in range(nt):
        wz[t, 3, t] = 1.0
    one = np.ones(nt)
    al = _packed(imf_type, *(v * one for v in pv))
    y, o, mass, ls = OpsOracle(ops_data, imf_type=imf_type).parts(al, wz, nt)
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


def _imf_params(n, seed):
    rng = np.random.default_rng(seed)
    return {"imf1": rng.uniform(0.6, 1.8, n), "imf2": rng.uniform(1.8, 2.8, n), "imf3": np.full(n, 2.3),
            "vdmc": 10.0 ** rng.uniform(-1.2, 0.0, n), "mdave": 10.0 ** rng.uniform(-0.6, 0.4, n)}


@pytest.mark.parametrize("imf_type", [3, 4])
def test_breaks_per_model_batch(octx, data, ops_data, imf_type):
    """van Dokkum with vdmc and Dave with imf1, imf2 and mdave per model, through the exact fold."""
    from oracle.oracle import Oracle, OpsOracle
    n = 40
    wz, params = config3_inputs(n, seed=360 + imf_type)
    ip = _imf_params(n, 362 + imf_type)
    octx.set_int("imf_type", imf_type)
    try:
        got = octx.csp_batch(dict(params, **ip), ssp_weights_z=wz)
        assert not octx.ops_last_interpolated()
    finally:
        octx.set_int("imf_type", 2)
    al = _packed(imf_type, ip["imf1"], ip["imf2"], ip["imf3"], ip["vdmc"], ip["mdave"])
    y, o, mass, ls = OpsOracle(ops_data, imf_type=imf_type).parts(al, wz, _itesc(data))
    ora = Oracle(data, nbands=40, add_neb=False).csp_from_parts(params, y, o)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)
    np.testing.assert_allclose(got["lbol"], np.log10(ls), rtol=1e-5)


@pytest.mark.parametrize("imf_type", [3, 4])
def test_breaks_per_model_reverse(octx, data, ops_data, imf_type):
    """The weights' cotangent along a random direction; Dave's imf1, imf2 and mdave rows (26, 27, 30) against central
    differences (h = 1e-4 relative), the other IMF rows zero; van Dokkum's rows zero (vdmc has no row in the
    reference's reverse pass)."""
    from libopensps_gb300.workloads import adjoint_cotangents
    from oracle.oracle import Oracle, OpsOracle
    n = 5
    wz, params = config3_inputs(n, seed=370 + imf_type)
    ip = _imf_params(n, 372 + imf_type)
    mb, sb = adjoint_cotangents(n, data["lambda"].size, 40, seed=371)
    octx.set_int("imf_type", imf_type)
    try:
        got = octx.csp_batch_grad(dict(params, **ip), wz, mags_bar=mb, spec_bar=sb)
    finally:
        octx.set_int("imf_type", 2)
    pb = got["params_bar"]
    ops = OpsOracle(ops_data, imf_type=imf_type)
    csp = Oracle(data, nbands=40, add_neb=False)

    def loss(w, q):
        al = _packed(imf_type, q["imf1"], q["imf2"], q["imf3"], q["vdmc"], q["mdave"])
        y, o, mass, ls = ops.parts(al, w, _itesc(data))
        out = csp.csp_from_parts(params, y, o)
        return np.nansum(mb * out["mags"], axis=1) + np.sum(sb * out["spec"], axis=1)

    rng = np.random.default_rng(373)
    dw = wz * rng.standard_normal(wz.shape)
    fd = (loss(wz + 1e-4 * dw, ip) - loss(wz - 1e-4 * dw, ip)) / 2e-4
    g = np.sum(got["weights_z_bar"] * dw, axis=(1, 2))
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert float(err.max()) <= 2e-3, (g, fd)
    if imf_type == 3:
        assert np.all(pb[:, 26:31] == 0.0)
        return
    assert np.all(pb[:, 28] == 0.0) and np.all(pb[:, 29] == 0.0)
    for k, row in (("imf1", 26), ("imf2", 27), ("mdave", 30)):
        h = 1e-4 * np.abs(ip[k])
        up = loss(wz, dict(ip, **{k: ip[k] + h}))
        dn = loss(wz, dict(ip, **{k: ip[k] - h}))
        fdk = (up - dn) / (2.0 * h)
        e = np.abs(pb[:, row] - fdk) / np.maximum(np.abs(fdk), 1e-3 * np.max(np.abs(fdk)))
        assert float(e.max()) <= 2e-3, (k, pb[:, row], fdk)


def test_chabrier_exact_fold_and_refusal(octx, data):
    """Chabrier through the exact fold (its lognormal's bin integrals as van Dokkum's, the power law above 1 M_sun)
    against the interpolated fold; an IMF type beyond 5 refused."""
    from libopensps_gb300.capi import OpenSPSError
    n = 24
    wz, params = config3_inputs(n, seed=350)
    octx.set_int("imf_type", 1)
    try:
        a = octx.csp_batch(params, ssp_weights_z=wz)
        assert octx.ops_last_interpolated()
        octx.set_int("gb300_ops_exact", 1)
        b = octx.csp_batch(params, ssp_weights_z=wz)
        assert not octx.ops_last_interpolated()
    finally:
        octx.set_int("gb300_ops_exact", 0)
        octx.set_int("imf_type", 2)
    assert rel_err_spec(a["spec"], b["spec"]) <= 5e-5
    np.testing.assert_allclose(a["mass"], b["mass"], rtol=2e-6)
    np.testing.assert_allclose(a["lbol"], b["lbol"], rtol=2e-6)
    octx.set_int("imf_type", 6)
    try:
        with pytest.raises(OpenSPSError) as e:
            octx.csp_batch(params, ssp_weights_z=wz)
        assert e.value.status == 2
    finally:
        octx.set_int("imf_type", 2)
