"""The CLOUDY-grid nebular continuum (nebular_kernels step 3 of OpenSPS, src/physics/opensps_csp_batch.f90:2760-2910):
a standard-format data root with the grid of the setup's isochrones (nebular/synthetic_nodust, written by
libopensps_gb300.synth_nebular), add_neb_emission and add_neb_continuum on, gas_logz, gas_logu and frac_obrun per
model, through the whole mixed batch (lines, the escaping ionizing light, birth-cloud and diffuse dust, IGM,
smoothing, 40 filters) against the FP64 oracle fed the numpy restatement of the grid's loader; with dust emission on
as well; the continuum's share of the spectrum; its reverse pass (the gas_logz, gas_logu and frac_obrun rows and the
weights' cotangent against central differences of the oracle, backward_nebular :5334-5606); and the refusal of the
missing _dust table.

Tolerances as the batch's other tests: spectra <= 1e-4 relative (pixels above 1e-6 of the peak), magnitudes
<= 1e-3 mag, mass 1e-12 relative.
"""
import os

import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def neb_root(tmp_path_factory, data):
    from libopensps_gb300 import stdformat, synthdata
    root = tmp_path_factory.mktemp("nebroot")
    stdformat.convert_synthetic(root, src_root=synthdata.default_root(), nebular=True)
    return root


@pytest.fixture
def restore_root():
    old = os.environ.get("OPENSPS_DATA_HOME")
    yield
    if old is not None:
        os.environ["OPENSPS_DATA_HOME"] = old


def _inputs(n, seed):
    wz, params = config3_inputs(n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    return wz, dict(params, gas_logz=rng.uniform(-2.2, 0.4, n), gas_logu=rng.uniform(-4.2, -0.8, n),
                    frac_obrun=rng.uniform(0.0, 0.4, n), dust1=rng.uniform(0.0, 1.0, n))


def _oracle(root, **kw):
    from oracle import stdformat as ora
    from oracle.oracle import Oracle
    d = ora.load_data(root, filter_sets=("gauss40",))
    lam = d["lambda"]
    return Oracle(d, nbands=40, nebular=ora.nebular(root, lam, "synthetic_nodust"), **kw), d


@pytest.mark.parametrize("n", [37, 300])
def test_continuum_matches_oracle(neb_root, built_lib, restore_root, n):
    """gas_logz and gas_logu drawn past both ends of the grid (the cell and its weights clamp), frac_obrun 0-0.4."""
    from libopensps_gb300.capi import Context
    wz, params = _inputs(n, seed=1200 + n)
    c = Context(data_root=neb_root)
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    got = c.csp_batch(params, ssp_weights_z=wz)
    plain = None
    if n == 37:
        c.set_int("add_neb_continuum", 0)
        plain = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    o, _ = _oracle(neb_root)
    want = o.csp_batch(params, wz)
    assert rel_err_spec(got["spec"], want["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - want["mags"]))) <= 1e-3
    np.testing.assert_allclose(got["mass"], want["mass"], rtol=1e-12)
    if plain is not None:
        # the continuum is a visible part of the optical spectrum of these young-weighted models
        sel = (o.lam > 3000.0) & (o.lam < 9000.0)
        assert np.median(got["spec"][:, sel] / plain["spec"][:, sel] - 1.0) > 1e-3


def test_continuum_with_dust_emission(neb_root, built_lib, restore_root):
    """The continuum joins the young and old sums before the attenuation, so the dust emission's energy balance
    counts its absorbed light."""
    from libopensps_gb300 import synth_dust
    from libopensps_gb300.capi import Context
    from oracle import stdformat as ora
    n = 24
    wz, params = _inputs(n, seed=1250)
    rng = np.random.default_rng(1251)
    params = dict(params, duste_qpah=rng.uniform(0.5, 4.5, n), duste_umin=rng.uniform(0.1, 20.0, n),
                  duste_gamma=rng.uniform(0.0, 0.5, n))
    c = Context(data_root=neb_root)
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_dust_emission", 1)
    got = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    lam = ora.load_data(neb_root, filter_sets=("gauss40",))["lambda"]
    o, _ = _oracle(neb_root, dust_emission=ora.dust_emission(neb_root, lam))
    want = o.csp_batch(params, wz)
    assert rel_err_spec(got["spec"], want["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - want["mags"]))) <= 1e-3


def test_continuum_steep_grid(tmp_path, data, built_lib, restore_root):
    """synth_nebular's steep test grid (the continuum falls by 80 decades per dex of age past 1 Myr, floored at
    1e-95): between the CLOUDY ages 1 and 2 Myr it drops by 2^80, past the 2^64 the kernel's polynomial takes, so
    those runs go age by age; the next intervals fall by 2^35 and 2^26 (the polynomial with its ratio above 1). The
    weights sit on the ages 1-4 Myr (the others at 1e-6 of theirs): the continuum's part of the spectrum (the batch
    less the same batch without it) against the oracle's within 1e-2 wherever it is at least 1e-3 of the spectrum
    (FP32 spectra differenced), and the whole batch as the other tests."""
    from libopensps_gb300 import stdformat, synth_nebular, synthdata
    from libopensps_gb300.capi import Context
    from oracle import stdformat as ora
    from oracle.oracle import Oracle
    root = tmp_path / "steep"
    stdformat.convert_synthetic(root, src_root=synthdata.default_root(), dust=False, agn=False)
    synth_nebular.write(root, "synthetic_nodust", steep=True)
    n = 40
    wz, params = _inputs(n, seed=1270)
    la = data["log_age"]
    wz[:, :, ~((la >= 6.0) & (la < 6.6))] *= 1e-6
    c = Context(data_root=root)
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    got = c.csp_batch(params, ssp_weights_z=wz)
    c.set_int("add_neb_continuum", 0)
    plain = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    d = ora.load_data(root, filter_sets=("gauss40",))
    want = Oracle(d, nbands=40, nebular=ora.nebular(root, d["lambda"], "synthetic_nodust")).csp_batch(params, wz)
    want_plain = Oracle(d, nbands=40).csp_batch(params, wz)
    assert rel_err_spec(got["spec"], want["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - want["mags"]))) <= 1e-3
    cont, cont_want = got["spec"] - plain["spec"], want["spec"] - want_plain["spec"]
    sel = cont_want >= 1e-3 * want["spec"]
    assert sel.sum() > 1000
    assert np.max(np.abs(cont[sel] - cont_want[sel]) / cont_want[sel]) <= 1e-2


def test_continuum_refusals(neb_root, built_lib, restore_root):
    from libopensps_gb300.capi import Context, OpenSPSError
    n = 8
    wz, params = _inputs(n, seed=1260)
    c = Context(data_root=neb_root)
    c.set_int("add_neb_emission", 1)
    c.set_int("cloudy_dust", 1)
    with pytest.raises(OpenSPSError) as e:
        c.csp_batch(params, ssp_weights_z=wz)
    assert e.value.status == 4 and "synthetic_dust" in e.value.message
    c.close()


def test_continuum_reverse_pass(neb_root, built_lib, restore_root):
    """gas_logz and gas_logu inside a cell of the grid (0.2 .. 0.8 of it), frac_obrun 0.05-0.4: the gas_logz (13),
    gas_logu (14), frac_obrun (6) and dust2 (2) rows and the weights' cotangent along a random direction against
    central differences (h = 1e-4 relative) of the oracle. Tolerance |g - g_fd| <= 2e-3 max(|g_fd|, 1e-3 max_rows)."""
    from libopensps_gb300.capi import Context
    from libopensps_gb300.workloads import adjoint_cotangents
    from oracle import stdformat as ora
    n = 5
    wz, params = _inputs(n, seed=1280)
    o, d = _oracle(neb_root)
    grid = ora.nebular(neb_root, d["lambda"], "synthetic_nodust")
    rng = np.random.default_rng(1281)

    def mid(g):
        i = rng.integers(0, g.size - 1, n)
        return g[i] + rng.uniform(0.2, 0.8, n) * (g[i + 1] - g[i])

    params = dict(params, gas_logz=mid(grid["logz"]), gas_logu=mid(grid["logu"]),
                  frac_obrun=rng.uniform(0.05, 0.4, n), dust2=rng.uniform(0.1, 1.0, n))
    c = Context(data_root=neb_root)
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    mb, sb = adjoint_cotangents(n, c.nspec, c.nbands, seed=1282)
    got = c.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb)
    c.close()

    def loss(out):
        return np.nansum(mb * out["mags"], axis=1) + np.sum(sb * out["spec"], axis=1)

    rows = {"gas_logz": 13, "gas_logu": 14, "frac_obrun": 6, "dust2": 2}
    g = np.stack([got["params_bar"][:, r] for r in rows.values()], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(rows):
        h = 1e-4 * np.abs(params[k])
        fd[:, i] = (loss(o.csp_batch(dict(params, **{k: params[k] + h}), wz))
                    - loss(o.csp_batch(dict(params, **{k: params[k] - h}), wz))) / (2.0 * h)
    scale = np.max(np.abs(fd), axis=1, keepdims=True)
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * scale)
    assert float(err.max()) <= 2e-3, {k: float(err[:, i].max()) for i, k in enumerate(rows)}
    dw = wz * rng.standard_normal(wz.shape)
    fdw = (loss(o.csp_batch(params, wz + 1e-4 * dw)) - loss(o.csp_batch(params, wz - 1e-4 * dw))) / 2e-4
    gw = np.sum(got["weights_z_bar"] * dw, axis=(1, 2))
    e = np.abs(gw - fdw) / np.maximum(np.abs(fdw), 1e-3 * np.max(np.abs(fdw)))
    assert float(e.max()) <= 2e-3, (gw, fdw)
