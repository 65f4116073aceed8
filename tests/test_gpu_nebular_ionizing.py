"""Nebular emission's gas absorption (nebular_kernels step 2, src/physics/opensps_csp_batch.f90:2726-2750): with
add_neb_emission the ionizing pixels (below 912 A) of the nebular ages keep only the escaping fraction
fesc = clamp(frac_obrun, 0, 1) of their light. The batch against the FP64 oracle with frac_obrun per model (0 and
above), the identity fesc = 1 <-> no absorption, and the gradients' frac_obrun row and weights' cotangent through the
escaping light against central differences of the batch.

Tolerances: spectra <= 1e-4 relative (pixels above 1e-6 of the peak), magnitudes <= 1e-3 mag; the identity 1e-5
relative (FP32 sums of the escaping light against the split-BF16 contraction); gradients as the other gradient tests.
"""
import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("igm,n,birth,tesc", [(0, 32, True, 7.0), (1, 32, True, 7.0), (0, 300, False, 7.0),
                                               (0, 300, True, 6.5), (1, 300, True, 6.5)])
def test_ionizing_absorption_matches_oracle(data, built_lib, igm, n, birth, tesc):
    """With the IGM off the ionizing pixels themselves are compared (with it on they fall below the comparison's
    floor at most redshifts). 300 models: several model tiles of the contraction and a ragged last one; without a
    birth cloud one accumulator (the escaping light in the same sums), with it young and old ones; dust_tesc 7.0 puts
    every nebular age among the young ones, 6.5 splits them (escaping-light blocks for both)."""
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    wz, params = config3_inputs(n, seed=941 + n)
    rng = np.random.default_rng(942)
    fo = rng.uniform(0.0, 0.6, n)
    fo[:8] = 0.0
    params = dict(params, frac_obrun=fo, dust_tesc=np.full(n, tesc))
    if birth:
        params["dust1"] = rng.uniform(0.0, 0.8, n)
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", igm)
    got = c.csp_batch(params, ssp_weights_z=wz)
    c.close()
    want = Oracle(data, nbands=40, add_igm=bool(igm)).csp_batch(params, wz)
    assert rel_err_spec(got["spec"], want["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - want["mags"]))) <= 1e-3


def test_escaping_light_in_chunks_and_from_device_inputs(data, built_lib):
    """A batch large enough to go up in chunks (40,000 models) with frac_obrun above 0, against the oracle on a sample
    of models; and the same inputs from device memory (opensps_gb300_batch_device) give the same magnitudes to FP32
    rounding (1e-4 mag)."""
    import torch
    from libopensps_gb300 import workloads
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    n = 40000
    wz, params = config3_inputs(n, seed=946)
    rng = np.random.default_rng(947)
    params = dict(params, frac_obrun=rng.uniform(0.0, 0.5, n))
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    got = c.csp_batch(params, ssp_weights_z=wz, spec=False)
    idx = np.arange(0, n, 997)
    want = Oracle(data, nbands=40).csp_batch({k: v[idx] for k, v in params.items()}, wz[idx])
    assert float(np.nanmax(np.abs(got["mags"][idx] - want["mags"]))) <= 1e-3
    d_wz = torch.from_numpy(wz).cuda()
    d_par = torch.from_numpy(workloads.device_param_table(params, n)).cuda()
    d_mags = torch.empty((n, c.nbands), dtype=torch.float64, device="cuda")
    c.batch_device(n, d_par.data_ptr(), d_wz.data_ptr(), d_mags.data_ptr(), sync=True)
    # (the band GEMM splits the pixels over CTAs by the batch's size: 16384-model chunks and one 40,000-model batch
    # sum the band fluxes in different FP32 orders)
    np.testing.assert_allclose(d_mags.cpu().numpy(), got["mags"], rtol=0, atol=1e-4)
    c.close()


def test_escaping_fraction_one_is_no_absorption(data, built_lib):
    """frac_obrun = 1: the ionizing pixels of the young and old sums with nebular emission equal those without it
    (the lines lie above 912 A)."""
    from libopensps_gb300.capi import Context
    n = 12
    rng = np.random.default_rng(943)
    w = rng.dirichlet(np.ones(107), size=n)
    params = {"frac_obrun": np.ones(n), "logzsol": rng.uniform(-1.5, 0.3, n)}
    c = Context()
    plain = c.csp_batch_parts(params, w, emlines=False)
    c.set_int("add_neb_emission", 1)
    neb = c.csp_batch_parts(params, w, emlines=False)
    half = dict(params, frac_obrun=np.full(n, 0.5))
    neb_half = c.csp_batch_parts(half, w, emlines=False)
    c.close()
    whl = int(np.searchsorted(data["lambda"], 912.0, side="right"))
    for part in ("young", "old"):
        np.testing.assert_allclose(neb[part][:, :whl], plain[part][:, :whl], rtol=1e-5, atol=1e-30)
    # absorbed: the young ages' ionizing light halves at fesc = 1/2 where the nebular ages dominate
    assert np.all(neb_half["young"][:, :whl].sum(axis=1) < 0.75 * neb["young"][:, :whl].sum(axis=1))


def test_gradient_through_escaping_light(data, built_lib):
    """The frac_obrun row and the weights' cotangent with the escaping light on, against central differences of the
    FP64 oracle's loss (spectra and magnitudes weighted by fixed cotangents; differences of the FP32 batch itself are
    too noisy at these steps)."""
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    n = 6
    wz, params = config3_inputs(n, seed=944)
    rng = np.random.default_rng(945)
    params = dict(params, frac_obrun=rng.uniform(0.1, 0.5, n), zred=rng.uniform(0.8, 3.0, n))
    c = Context()
    c.set_int("add_neb_emission", 1)
    ns, nb = c.nspec, c.nbands
    mags_bar = rng.standard_normal((n, nb))
    spec_bar = rng.standard_normal((n, ns)) * 1e-3
    out = c.csp_batch_grad(params, wz, mags_bar=mags_bar, spec_bar=spec_bar, weights_z_bar=True)
    c.close()
    pb, wzb = out["params_bar"], out["weights_z_bar"]
    o = Oracle(data, nbands=40, add_igm=False)      # (the context's IGM is off)

    def loss(p, w):
        r = o.csp_batch(p, w)
        return np.nansum(mags_bar * r["mags"], axis=1) + np.sum(spec_bar * r["spec"], axis=1)

    h = 1e-4
    fd = (loss(dict(params, frac_obrun=params["frac_obrun"] + h), wz)
          - loss(dict(params, frac_obrun=params["frac_obrun"] - h), wz)) / (2 * h)
    row = 6                                   # frac_obrun's params_bar row (opensps.h)
    np.testing.assert_allclose(pb[:, row], fd, rtol=2e-2, atol=2e-3 * np.max(np.abs(fd)))
    # the weights' cotangent at the largest young nebular (age, metallicity) weight of each model
    for m in range(n):
        z, t = np.unravel_index(np.argmax(wz[m, :, :10]), (wz.shape[1], 10))
        dw = np.zeros_like(wz)
        dw[:, z, t] = 1e-4 * wz[m, z, t]
        fdw = (loss(params, wz + dw)[m] - loss(params, wz - dw)[m]) / (2 * dw[m, z, t])
        np.testing.assert_allclose(wzb[m, z, t], fdw, rtol=2e-2)
