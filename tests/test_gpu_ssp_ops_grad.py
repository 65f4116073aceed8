"""The reverse pass with the SSP operators (compute_csp_batch_grad_rows with a Kroupa IMF per model): the three IMF
slopes' rows (imf1..imf3, params_bar rows 26..28), a dust row, the weights' cotangent over ages and metallicities
and, with weights formed on the device (sfh = 4), the SFH and logzsol rows, against central differences
(h = 1e-4 relative) of the FP64 oracle (ops_oracle.c for the operator, the CSP oracle for the stages after it), as
the reference's tests/test_csp_batch_grad.f90 checks its adjoints.

Tolerance as the other gradient tests: |g - g_fd| <= 2e-3 max(|g_fd|, 1e-3 max_rows |g_fd|).
"""
import numpy as np
import pytest

from conftest import blend_at_logzsol, config3_inputs

pytestmark = pytest.mark.gpu

RTOL = 2e-3
H_REL = 1e-4
IMF_ROWS = {"imf1": 26, "imf2": 27, "imf3": 28}


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
    c.close()


@pytest.fixture(scope="module")
def oracles(data, ops_data):
    from oracle.oracle import OpsOracle, Oracle
    return OpsOracle(ops_data), Oracle(data, nbands=40, add_neb=False)


def _itesc(data):
    return int(np.clip(np.searchsorted(data["log_age"], 7.0, side="right"), 1, data["log_age"].size))


def _cot(c, n, seed):
    from libopensps_gb300.workloads import adjoint_cotangents
    mb, sb = adjoint_cotangents(n, c.nspec, c.nbands, seed=seed)
    rng = np.random.default_rng(seed + 1)
    return mb, sb, rng.standard_normal(n), rng.standard_normal(n)


def _loss(out, mb, sb, massb, lbolb):
    return (np.nansum(mb * out["mags"], axis=1) + np.sum(sb * out["spec"], axis=1) + massb * out["mass"]
            + lbolb * out["lbol"])


def _oracle_run(oracles, data, params, wz):
    """The operator's young and old sums for the slopes in params, then the CSP's stages after the age sums; mass
    and L_bol from the operator's rows."""
    ops, csp = oracles
    alpha = np.stack([params["imf1"], params["imf2"], params["imf3"]], axis=1)
    y, o, mass, ls = ops.parts(alpha, wz, _itesc(data))
    out = csp.csp_from_parts({k: v for k, v in params.items() if not k.startswith("imf")}, y, o)
    out["mass"] = mass
    out["lbol"] = np.log10(ls)
    return out


def _slopes(n, rng):
    return {"imf1": rng.uniform(0.3, 1.8, n), "imf2": rng.uniform(1.3, 2.8, n), "imf3": rng.uniform(1.8, 3.3, n)}


def _check(g, fd, names):
    scale = np.max(np.abs(fd), axis=1, keepdims=True)
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * scale)
    assert float(err.max()) <= RTOL, {names[i]: float(err[:, i].max()) for i in range(len(names))}


@pytest.mark.parametrize("fold", ["interpolated", "exact"])
@pytest.mark.parametrize("n,seed", [(5, 510), (6, 511)])
def test_slope_rows_and_weights_cotangent(octx, oracles, data, n, seed, fold):
    """Both folds' reverses: the interpolated one (GEMMs against the transposed operator basis) and the exact one
    (gb300_ops_exact = 1)."""
    wz, params = config3_inputs(n, seed=seed)
    rng = np.random.default_rng(seed + 5)
    params = dict(params, **_slopes(n, rng))
    mb, sb, massb, lbolb = _cot(octx, n, seed)
    octx.set_int("gb300_ops_exact", 1 if fold == "exact" else 0)
    try:
        got = octx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
        assert octx.ops_last_interpolated() == (fold == "interpolated")
    finally:
        octx.set_int("gb300_ops_exact", 0)
    rows = dict(IMF_ROWS, dust2=2)
    names = list(rows)
    g = np.stack([got["params_bar"][:, rows[k]] for k in names], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(names):
        h = H_REL * np.abs(params[k])
        up = _oracle_run(oracles, data, dict(params, **{k: params[k] + h}), wz)
        dn = _oracle_run(oracles, data, dict(params, **{k: params[k] - h}), wz)
        fd[:, i] = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * h)
    _check(g, fd, names)
    # the weights' cotangent along a random relative direction
    dw = wz * rng.standard_normal(wz.shape)
    up = _oracle_run(oracles, data, params, wz + H_REL * dw)
    dn = _oracle_run(oracles, data, params, wz - H_REL * dw)
    fd_w = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * H_REL)
    g_w = np.sum(got["weights_z_bar"] * dw, axis=(1, 2))
    err = np.abs(g_w - fd_w) / np.maximum(np.abs(fd_w), 1e-3 * np.max(np.abs(fd_w)))
    assert float(err.max()) <= RTOL, (g_w, fd_w)


def test_interpolated_reverse_matches_exact(octx, data):
    """The interpolated reverse fold against the exact one on 300 models of the operator leg's batch (slopes per
    model, every grid point weighted): the slope rows and the weights' cotangent within 1e-4 of each row's largest
    value (the interpolation and the split-BF16 GEMMs against FP32 sums)."""
    from libopensps_gb300 import workloads
    n = 300
    wz, params = workloads.mixed_csp(n, seed=530)
    rng = np.random.default_rng(531)
    params = dict(params, **_slopes(n, rng))
    mb, sb, massb, lbolb = _cot(octx, n, 532)
    out = {}
    for fold in ("interpolated", "exact"):
        octx.set_int("gb300_ops_exact", 1 if fold == "exact" else 0)
        try:
            out[fold] = octx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
        finally:
            octx.set_int("gb300_ops_exact", 0)
    gi, ge = out["interpolated"]["params_bar"][:, 26:29], out["exact"]["params_bar"][:, 26:29]
    assert np.all(np.abs(gi - ge) <= 1e-4 * np.max(np.abs(ge), axis=0))
    wi, we = out["interpolated"]["weights_z_bar"], out["exact"]["weights_z_bar"]
    scale = np.max(np.abs(we), axis=(1, 2), keepdims=True)
    assert float(np.max(np.abs(wi - we) / scale)) <= 1e-4


def test_slope_rows_without_weights_cotangent(octx, data):
    """params_bar alone (no weights' cotangent asked): the reverse fold visits only the grid points with weight and
    gives the same slope rows."""
    n, seed = 7, 520
    wz, params = config3_inputs(n, seed=seed)
    wz[:, :, 40:] = 0.0                            # weight only at the youngest 40 ages
    params = dict(params, **_slopes(n, np.random.default_rng(seed + 1)))
    mb, sb, massb, lbolb = _cot(octx, n, seed)
    full = octx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
    rows = octx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb,
                               weights_z_bar=False)
    # (two forward runs: the fold's shared-memory float atomics make them differ at FP32 rounding)
    pb, ref = rows["params_bar"], full["params_bar"]
    np.testing.assert_allclose(pb, ref, rtol=1e-4, atol=1e-6 * np.max(np.abs(ref)))
    assert np.any(pb[:, 26:29] != 0.0)


def test_mass_and_lbol_cotangents_alone(octx, oracles, data):
    """mass_bar and lbol_bar only: the weights' cotangent is mass_bar M_g + lbol_bar L_g / (ln 10 L_bol), M_g and
    L_g the operator's mass and L_bol rows of grid point g for the model's IMF, and the slopes' rows their
    derivatives."""
    n, seed = 4, 530
    wz, params = config3_inputs(n, seed=seed)
    params = dict(params, **_slopes(n, np.random.default_rng(seed + 1)))
    rng = np.random.default_rng(seed + 2)
    massb, lbolb = rng.standard_normal(n), rng.standard_normal(n)
    got = octx.csp_batch_grad(params, wz, mass_bar=massb, lbol_bar=lbolb)
    ops, _ = oracles
    alpha = np.stack([params[k] for k in IMF_ROWS], axis=1)
    nz, nt = wz.shape[1:]
    _, _, _, lsum = ops.parts(alpha, wz, _itesc(data))
    # the rows at a sample of grid points: one model per (model, grid point) with a unit weight there
    picks = [(z, t) for z, t in zip(rng.integers(0, nz, 12), rng.integers(0, nt, 12))]
    e = np.zeros((n * len(picks), nz, nt))
    for i, (z, t) in enumerate(picks):
        e[i * n:(i + 1) * n, z, t] = 1.0
    _, _, M, L = ops.parts(np.tile(alpha, (len(picks), 1)), e, nt)
    for i, (z, t) in enumerate(picks):
        want = massb * M[i * n:(i + 1) * n] + lbolb / (np.log(10.0) * lsum) * L[i * n:(i + 1) * n]
        np.testing.assert_allclose(got["weights_z_bar"][:, z, t], want, rtol=2e-5,
                                   atol=2e-5 * np.max(np.abs(want)))
    # the slopes' rows: central differences of mass_bar mass + lbol_bar lbol
    g = got["params_bar"][:, 26:29]
    fd = np.empty_like(g)
    for j in range(3):
        h = H_REL * np.abs(alpha[:, j])
        au, ad = alpha.copy(), alpha.copy()
        au[:, j] += h
        ad[:, j] -= h
        _, _, mu, lu = ops.parts(au, wz, _itesc(data))
        _, _, md, ld = ops.parts(ad, wz, _itesc(data))
        fd[:, j] = (massb * (mu - md) + lbolb * (np.log10(lu) - np.log10(ld))) / (2.0 * h)
    _check(g, fd, list(IMF_ROWS))


def test_sfh_and_slope_rows_with_weights_on_the_device(octx, oracles, data):
    """sfh = 4 with the operators: tage, tau, logzsol and the slopes' rows, the weights formed and blended on the
    device; L_bol is the operator's linear row."""
    from oracle.oracle import sfh_weights
    n, seed = 5, 540
    rng = np.random.default_rng(seed)
    la = data["log_age"]
    tage = rng.uniform(3.0, 12.0, n)
    for i in range(n):                             # away from the grid ages (the weights' kinks)
        while np.min(np.abs(np.log10(tage[i] * 1e9) - la)) < 5e-3:
            tage[i] *= 1.015
    params = dict(tage=tage, tau=10.0 ** rng.uniform(-0.3, 0.8, n), logzsol=rng.uniform(-1.5, 0.3, n),
                  dust2=rng.uniform(0.1, 1.0, n), zred=rng.uniform(0.2, 2.0, n),
                  sigma_smooth=rng.uniform(60.0, 250.0, n), **_slopes(n, rng))
    octx.set_int("sfh", 4)
    try:
        mb, sb, massb, lbolb = _cot(octx, n, seed)
        got = octx.csp_batch_grad(params, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb, n=n)
    finally:
        octx.set_int("sfh", 0)

    def run(p):
        w, _ = sfh_weights(la, 4, p, n)
        wz, _ = blend_at_logzsol(data, w, p["logzsol"])
        return _loss(_oracle_run(oracles, data, {k: v for k, v in p.items() if k not in ("tage", "tau", "logzsol")},
                                 wz), mb, sb, massb, lbolb)

    rows = dict(IMF_ROWS, logzsol=15, tage=16, tau=17)
    names = list(rows)
    g = np.stack([got["params_bar"][:, rows[k]] for k in names], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(names):
        h = H_REL * np.maximum(np.abs(params[k]), 1e-2)
        fd[:, i] = (run(dict(params, **{k: params[k] + h})) - run(dict(params, **{k: params[k] - h}))) / (2.0 * h)
    _check(g, fd, names)
