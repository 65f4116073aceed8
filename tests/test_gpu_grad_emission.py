"""The reverse pass with dust emission and the AGN torus (backward_emission_sums and backward_agn,
src/physics/opensps_csp_batch.f90:6667-6845, and the absorbed light's share of the attenuation adjoint) through the C
ABI, against central finite differences of the FP64 oracle: the dust rows, the dust emission's q_PAH, U_min and gamma
rows, the AGN's fagn and agn_tau rows, redshift, smoothing and IGM, and the weights' cotangent along a random
direction (the AGN's L_bol scale included).

Loss and steps as tests/test_gpu_grad.py (central differences of relative step 1e-4; redshifts mid-pixel, the
smoothing window's edge away from a pixel boundary); q_PAH, U_min and agn_tau are drawn inside a cell of their grids
(0.2 .. 0.8 of the cell) so that the step stays on one smooth piece. Tolerance: |g - g_fd| <= 2e-3 max(|g_fd|,
1e-3 max_rows |g_fd|) per model and row.
"""
import numpy as np
import pytest

from test_gpu_grad import _check_rows, _cotangents, _inputs, _loss

pytestmark = pytest.mark.gpu

RTOL = 2e-3
H_REL = 1e-4
ROWS = {"fagn": 0, "dust1": 1, "dust2": 2, "dust3": 3, "dust_index": 4, "dust1_index": 5, "frac_obrun": 6,
        "frac_nodust": 7, "duste_qpah": 10, "duste_umin": 11, "duste_gamma": 12, "zred": 22, "sigma_smooth": 23,
        "agn_tau": 31, "igm_factor": 32}


def _mid_cell(grid, rng, n):
    i = rng.integers(0, grid.size - 1, n)
    return grid[i] + rng.uniform(0.2, 0.8, n) * (grid[i + 1] - grid[i])


def _emission_inputs(data, n, seed):
    from libopensps_gb300 import synth_dust
    wz, params = _inputs(data, n, seed)
    rng = np.random.default_rng(seed + 11)
    params = dict(params, duste_qpah=_mid_cell(synth_dust.QPAH, rng, n),
                  duste_umin=_mid_cell(synth_dust.UMIN, rng, n), duste_gamma=rng.uniform(0.05, 0.6, n),
                  fagn=rng.uniform(0.05, 1.0, n), agn_tau=_mid_cell(synth_dust.AGN_TAU, rng, n))
    return wz, params


@pytest.fixture(scope="module")
def ectx(data, built_lib):
    from libopensps_gb300.capi import Context
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_dust_emission", 1)
    c.set_int("add_agn_dust", 1)
    yield c
    c.close()


@pytest.fixture(scope="module")
def eoracle(data):
    from libopensps_gb300 import synth_dust
    from oracle.oracle import Oracle
    return Oracle(data, nbands=40, dust_emission=synth_dust.load(), agn=synth_dust.load_agn())


@pytest.mark.parametrize("n,seed", [(5, 140), (8, 141)])
def test_emission_and_agn_rows_match_central_differences(ectx, eoracle, data, n, seed):
    wz, params = _emission_inputs(data, n, seed)
    mb, sb, massb, lbolb = _cotangents(n, ectx.nspec, ectx.nbands, seed)
    got = ectx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
    pb = got["params_bar"]
    names = list(ROWS)
    g = np.stack([pb[:, ROWS[k]] for k in names], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(names):
        h = H_REL * np.abs(params[k])
        up = eoracle.csp_batch(dict(params, **{k: params[k] + h}), wz)
        dn = eoracle.csp_batch(dict(params, **{k: params[k] - h}), wz)
        fd[:, i] = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * h)
    worst, err = _check_rows(g, fd)
    assert worst <= RTOL, {names[i]: float(err[:, i].max()) for i in range(len(names))}


def test_weights_cotangent_with_emission_and_agn(ectx, eoracle, data):
    n, seed = 6, 152
    wz, params = _emission_inputs(data, n, seed)
    mb, sb, massb, lbolb = _cotangents(n, ectx.nspec, ectx.nbands, seed)
    got = ectx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
    wzb = got["weights_z_bar"]
    rng = np.random.default_rng(seed + 3)
    dw = wz * rng.standard_normal(wz.shape)
    up = eoracle.csp_batch(params, wz + H_REL * dw)
    dn = eoracle.csp_batch(params, wz - H_REL * dw)
    fd = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * H_REL)
    g = np.sum(wzb * dw, axis=(1, 2))
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert float(err.max()) <= RTOL, (g, fd)


def test_agn_gradients_refused_with_weights_formed_on_the_device(data, built_lib):
    """The AGN scales with the batch's L_bol output; with weights over ages blended at logzsol on the device that is
    the log-blended L_bol, whose cotangent this path does not carry: status 2."""
    from libopensps_gb300.capi import Context, OpenSPSError
    n = 3
    rng = np.random.default_rng(7)
    w = rng.dirichlet(np.ones(107), size=n)
    c = Context()
    c.set_int("add_agn_dust", 1)
    with pytest.raises(OpenSPSError) as e:
        c.csp_batch_grad({"fagn": np.full(n, 0.3), "logzsol": np.zeros(n)}, ssp_weights=w, mags_bar=np.ones((n, c.nbands)))
    assert e.value.status == 2
    c.close()
