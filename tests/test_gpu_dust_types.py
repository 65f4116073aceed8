"""The diffuse dust curves other than the power law (dust_type 1 CCM89 with mwr and uvb, 2 Calzetti, 4 Kriek &
Conroy with dust_index, 6 Reddy: the reference's tabulated curves, attenuation_tables_cached / pixel_transmissions,
src/physics/opensps_csp_batch.f90:3494-3560,3765-3818; 3 the dusty environments' optical depth chosen by wgp1-3, dust2
not applied, and 5 the SMC bar: table lookups of the data root's attenuation libraries, here the synthetic stand-ins)
through the C API against the FP64 oracle, which evaluates the curve functions themselves
(compute_attenuation_curve_point; for 3 and 5 the library's curve interpolated onto the grid by the numpy
restatement of load_attenuation_curves): the mixed batch (nebular lines, birth-cloud,
diffuse and old-star screens, IGM, smoothing, 40 filters) with the curve's parameters shared by the batch (the
pixel table's FP64 curve) and per model (each model's curve from the FP32 tables), with dust emission too; the
reverse pass's dust rows (dust2, dust3, dust_index with type 4, mwr and uvb with type 1) against FP64 central
differences, shared and per model; the refusals.

Tolerances as the other tests: spectra <= 1e-4 relative (pixels above 1e-6 of the peak), magnitudes <= 1e-3 mag;
gradients |g - g_fd| <= 2e-3 max(|g_fd|, 1e-3 max_rows |g_fd|).
"""
import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu

CURVE = {1: dict(mwr=3.4, uvb=0.7), 2: {}, 3: {}, 4: dict(dust_index=-0.35), 5: {}, 6: {}}
WGP = (7, 4, 2)     # dust_type 3: tau_v 7, model 4, clumpy


def _att_curve(data, dust_type):
    """The table lookup's curve on the grid (types 3, 5) from the data root's attenuation libraries."""
    import os
    from pathlib import Path
    from libopensps_gb300 import synth_attenuation
    from oracle import stdformat as ora
    root = Path(os.environ["OPENSPS_DATA_HOME"])
    synth_attenuation.generate(root)
    if dust_type == 5:
        return ora.attenuation(root, "smc_bar", data["lambda"])[0]
    t, m, s = WGP
    return ora.attenuation(root, "dirty", data["lambda"])[((s - 1) * 18 + (t - 1)) * 6 + (m - 1)]


def _oracle(data, dust_type, **kw):
    from oracle.oracle import Oracle
    att = _att_curve(data, dust_type) if dust_type in (3, 5) else None
    return Oracle(data, nbands=40, dust_type=dust_type, att_curve=att, **kw)


def _inputs(n, seed, dust_type, per_model=False):
    wz, params = config3_inputs(n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    params = dict(params, dust1=rng.uniform(0.1, 1.0, n), dust3=rng.uniform(0.0, 0.4, n),
                  frac_nodust=rng.uniform(0.0, 0.2, n), frac_obrun=rng.uniform(0.0, 0.3, n),
                  dust_index=rng.uniform(-1.0, -0.3, n))
    if per_model:
        params.update(mwr=rng.uniform(2.2, 5.0, n), uvb=rng.uniform(0.0, 1.5, n))
    else:
        for k, v in CURVE[dust_type].items():
            params[k] = np.full(n, v)
    return wz, params


def _ctx(dust_type, **flags):
    from libopensps_gb300.capi import Context
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_int("dust_type", dust_type)
    if dust_type == 3:
        for k, v in zip(("wgp1", "wgp2", "wgp3"), WGP):
            c.set_int(k, v)
    for k, v in flags.items():
        c.set_int(k, v)
    return c


@pytest.mark.parametrize("dust_type,per_model", [(1, False), (2, False), (3, False), (4, False), (5, False),
                                                 (6, False), (1, True), (4, True)])
def test_dust_type_matches_oracle(data, built_lib, dust_type, per_model):
    from oracle.oracle import Oracle
    n = 60
    wz, params = _inputs(n, 1400 + dust_type + (10 if per_model else 0), dust_type, per_model)
    c = _ctx(dust_type)
    got = c.csp_batch(params, ssp_weights_z=wz)
    plain = None
    if dust_type in (2, 3, 5):
        c.set_int("dust_type", 0)
        plain = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    want = _oracle(data, dust_type).csp_batch(params, wz)
    assert rel_err_spec(got["spec"], want["spec"]) <= 1e-4
    assert np.array_equal(np.isnan(got["mags"]), np.isnan(want["mags"]))
    assert float(np.nanmax(np.abs(got["mags"] - want["mags"]))) <= 1e-3
    if plain is not None:
        # the curve is in effect: Calzetti and the power law differ
        assert float(np.nanmax(np.abs(got["mags"] - plain["mags"]))) > 0.05


def test_dust_type_with_dust_emission(data, built_lib):
    """The absorbed light of the energy balance goes through the same curve (Calzetti)."""
    from libopensps_gb300 import synth_dust
    from oracle.oracle import Oracle
    n = 24
    wz, params = _inputs(n, 1450, 2)
    rng = np.random.default_rng(1451)
    params = dict(params, duste_qpah=rng.uniform(0.5, 4.5, n), duste_umin=rng.uniform(0.1, 20.0, n),
                  duste_gamma=rng.uniform(0.0, 0.5, n))
    c = _ctx(2, add_dust_emission=1)
    got = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    want = Oracle(data, nbands=40, dust_type=2, dust_emission=synth_dust.load()).csp_batch(params, wz)
    assert rel_err_spec(got["spec"], want["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - want["mags"]))) <= 1e-3


def _loss(out, mb, sb):
    return np.nansum(mb * out["mags"], axis=1) + np.sum(sb * out["spec"], axis=1)


@pytest.mark.parametrize("dust_type,rows,per_model", [(1, {"dust2": 2, "dust3": 3, "mwr": 8, "uvb": 9}, False),
                                                      (2, {"dust2": 2, "dust3": 3}, False),
                                                      (3, {"dust1": 1, "dust3": 3, "frac_nodust": 7}, False),
                                                      (5, {"dust2": 2, "dust3": 3}, False),
                                                      (4, {"dust2": 2, "dust3": 3, "dust_index": 4}, False),
                                                      (1, {"dust2": 2, "mwr": 8, "uvb": 9}, True),
                                                      (4, {"dust2": 2, "dust_index": 4}, True)])
def test_dust_type_gradients(data, built_lib, dust_type, rows, per_model):
    """Rows against FP64 central differences of the oracle (h = 1e-4 relative), each model's own parameter moved.
    Without IGM and smoothing, at z = 0: the curve's rows alone."""
    from libopensps_gb300.workloads import adjoint_cotangents
    from oracle.oracle import Oracle
    n = 6
    wz, params = _inputs(n, 1460 + dust_type + (10 if per_model else 0), dust_type, per_model)
    params = dict(params, zred=np.zeros(n), sigma_smooth=np.zeros(n))
    mb, sb = adjoint_cotangents(n, data["lambda"].size, 40, seed=1470 + dust_type)
    c = _ctx(dust_type)
    got = c.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb)
    c.close()
    o = _oracle(data, dust_type)
    names = list(rows)
    g = np.stack([got["params_bar"][:, rows[k]] for k in names], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(names):
        h = 1e-4 * np.abs(params[k])
        up = o.csp_batch(dict(params, **{k: params[k] + h}), wz)
        dn = o.csp_batch(dict(params, **{k: params[k] - h}), wz)
        fd[:, i] = (_loss(up, mb, sb) - _loss(dn, mb, sb)) / (2.0 * h)
    scale = np.max(np.abs(fd), axis=1, keepdims=True)
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * scale)
    assert float(err.max()) <= 2e-3, {names[i]: float(err[:, i].max()) for i in range(len(names))}
    if dust_type != 4:
        assert np.all(got["params_bar"][:, 4] == 0.0)     # dust_index does not act
    if dust_type != 1:
        assert np.all(got["params_bar"][:, 8:10] == 0.0)  # nor mwr and uvb
    if dust_type == 3:
        assert np.all(got["params_bar"][:, 2] == 0.0)     # nor dust2 (the optical depth is the curve itself)


def test_dust_type_refusals(data, built_lib):
    from libopensps_gb300.capi import OpenSPSError
    n = 8
    wz, params = _inputs(n, 1480, 1)
    c = _ctx(1)
    c.set_int("dust_type", 7)
    with pytest.raises(OpenSPSError) as e:
        c.csp_batch(params, ssp_weights_z=wz)
    assert e.value.status == 2
    c.set_int("dust_type", 3)
    c.set_int("wgp1", 19)
    with pytest.raises(OpenSPSError) as e:
        c.csp_batch(params, ssp_weights_z=wz)
    assert e.value.status == 3
    c.set_int("wgp1", 1)
    c.set_int("dust_type", 2)
    c.set_int("gb300_fp64", 1)
    with pytest.raises(OpenSPSError) as e:
        c.csp_batch(params, ssp_weights_z=wz)
    assert e.value.status == 2
    c.close()
