"""The reverse pass (compute_csp_batch_grad_rows through the C ABI) against central finite differences of the FP64
oracle, as the reference's tests/test_csp_batch_grad.f90 checks its adjoints (central differences, relative step).

The loss is L_m = sum_b mags_bar mags + sum_i spec_bar spec + mass_bar mass + lbol_bar lbol per model, with the
cotangents N(0, 1) (magnitudes, 512 binned spectral pixels, mass, L_bol). Redshifts sit mid-pixel and sigma_smooth
away from a change of the smoothing window, so that a step of 1e-4 (relative) stays on one smooth piece.

Tolerance: |g - g_fd| <= 2e-3 max(|g_fd|, 1e-3 max_rows |g_fd|) per model and parameter row; the weights'
cotangent along a random relative direction of the weights within 2e-3 of its difference quotient.
"""
import numpy as np
import pytest

from conftest import config3_inputs

pytestmark = pytest.mark.gpu

RTOL = 2e-3
H_REL = 1e-4
ROWS = {"dust1": 1, "dust2": 2, "dust3": 3, "dust_index": 4, "dust1_index": 5, "frac_obrun": 6, "frac_nodust": 7,
        "zred": 22, "sigma_smooth": 23, "igm_factor": 32}
C_KMS = 2.99792458e5


def _inputs(data, n, seed):
    wz, params = config3_inputs(n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    lam = data["lambda"]
    dlnl = np.log(lam[-1] / lam[0]) / (lam.size - 1)
    # redshift mid-pixel: s = ln(1 + z) / dlnl with a fractional part in [0.25, 0.75]
    s = np.floor(np.log1p(rng.uniform(0.3, 6.0, n)) / dlnl) + rng.uniform(0.25, 0.75, n)
    zred = np.expm1(s * dlnl)
    # sigma_smooth with the window edge (4 sigma / c in pixels) away from a pixel boundary
    e = np.floor(4.0 * rng.uniform(60.0, 300.0, n) / C_KMS / dlnl) + rng.uniform(0.2, 0.8, n)
    sigma = e * dlnl * C_KMS / 4.0
    params = dict(dust2=rng.uniform(0.2, 2.0, n), zred=zred, sigma_smooth=sigma,
                  dust1=rng.uniform(0.2, 1.5, n), dust3=rng.uniform(0.1, 0.5, n),
                  frac_obrun=rng.uniform(0.05, 0.3, n), frac_nodust=rng.uniform(0.05, 0.2, n),
                  dust_index=rng.uniform(-1.2, -0.3, n), dust1_index=rng.uniform(-1.5, -0.5, n),
                  igm_factor=rng.uniform(0.5, 1.5, n))
    return wz, params


def _cotangents(n, ns, nb, seed):
    from libopensps_gb300.workloads import adjoint_cotangents
    mags_bar, spec_bar = adjoint_cotangents(n, ns, nb, seed=seed)
    rng = np.random.default_rng(seed + 7)
    return mags_bar, spec_bar, rng.standard_normal(n), rng.standard_normal(n)


def _loss(out, mags_bar, spec_bar, mass_bar, lbol_bar):
    return (np.nansum(mags_bar * out["mags"], axis=1) + np.sum(spec_bar * out["spec"], axis=1)
            + mass_bar * out["mass"] + lbol_bar * out["lbol"])


@pytest.fixture(scope="module")
def gctx(data, built_lib):
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


def _check_rows(got, fd):
    scale = np.max(np.abs(fd), axis=1, keepdims=True)
    den = np.maximum(np.abs(fd), 1e-3 * scale)
    err = np.abs(got - fd) / den
    return float(np.max(err)), err


@pytest.mark.parametrize("n,seed", [(5, 40), (9, 41)])
def test_parameter_gradients_match_central_differences(gctx, oracle40, data, n, seed):
    wz, params = _inputs(data, n, seed)
    mb, sb, massb, lbolb = _cotangents(n, gctx.nspec, gctx.nbands, seed)
    got = gctx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
    pb = got["params_bar"]
    assert pb.shape == (n, 44)
    names = list(ROWS)
    g = np.stack([pb[:, ROWS[k]] for k in names], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(names):
        h = H_REL * np.abs(params[k])
        up = oracle40.csp_batch(dict(params, **{k: params[k] + h}), wz)
        dn = oracle40.csp_batch(dict(params, **{k: params[k] - h}), wz)
        fd[:, i] = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * h)
    worst, err = _check_rows(g, fd)
    assert worst <= RTOL, {names[i]: float(err[:, i].max()) for i in range(len(names))}
    # the rows this path does not vary are written as zero
    others = [r for r in range(44) if r not in ROWS.values()]
    assert np.all(pb[:, others] == 0.0)


def test_weights_cotangent_matches_directional_difference(gctx, oracle40, data):
    n, seed = 7, 52
    wz, params = _inputs(data, n, seed)
    mb, sb, massb, lbolb = _cotangents(n, gctx.nspec, gctx.nbands, seed)
    got = gctx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
    wzb = got["weights_z_bar"]
    rng = np.random.default_rng(seed + 3)
    dw = wz * rng.standard_normal(wz.shape)          # relative perturbations of the weights
    h = H_REL
    up = oracle40.csp_batch(params, wz + h * dw)
    dn = oracle40.csp_batch(params, wz - h * dw)
    fd = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * h)
    g = np.sum(wzb * dw, axis=(1, 2))
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert float(err.max()) <= RTOL, (g, fd)


def test_mass_and_lbol_cotangents_alone(gctx, data):
    """With only mass_bar and lbol_bar the weights' cotangent is mass_bar M(t, z) + lbol_bar L(t, z) / (ln 10 L_bol)."""
    n = 4
    wz, params = _inputs(data, n, 60)
    rng = np.random.default_rng(61)
    massb, lbolb = rng.standard_normal(n), rng.standard_normal(n)
    got = gctx.csp_batch_grad(params, wz, mass_bar=massb, lbol_bar=lbolb)
    llin = 10.0 ** data["ssp_lbol"]                   # (nz, nt)
    lsum = np.einsum("mzt,zt->m", wz, llin)
    want = massb[:, None, None] * data["ssp_mass"][None] + (lbolb / (np.log(10.0) * lsum))[:, None, None] * llin[None]
    np.testing.assert_allclose(got["weights_z_bar"], want, rtol=1e-6, atol=1e-12 * np.max(np.abs(want)))
    np.testing.assert_allclose(got["params_bar"], 0.0)


def test_sigma_smooth_gradient_from_spectrum_cotangents(gctx, oracle40, data):
    """sigma_smooth alone: spectrum cotangents only inside the smoothing range, where the gradient is a second
    difference of the spectrum. Within 2e-3 of the central difference (floor 1e-3 of the batch's largest)."""
    n, seed = 8, 90
    wz, params = _inputs(data, n, seed)
    lam = data["lambda"]
    rng = np.random.default_rng(seed)
    sel = (lam >= 1e3) & (lam <= 1e4)
    sb = np.zeros((n, lam.size))
    sb[:, sel] = rng.standard_normal((n, int(sel.sum())))
    got = gctx.csp_batch_grad(params, wz, spec_bar=sb)
    k = "sigma_smooth"
    h = H_REL * np.abs(params[k])
    up = oracle40.csp_batch(dict(params, **{k: params[k] + h}), wz)
    dn = oracle40.csp_batch(dict(params, **{k: params[k] - h}), wz)
    fd = (np.sum(sb * up["spec"], axis=1) - np.sum(sb * dn["spec"], axis=1)) / (2.0 * h)
    g = got["params_bar"][:, ROWS[k]]
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert float(err.max()) <= RTOL, (g, fd)
