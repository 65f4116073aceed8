"""The reverse pass with weights formed on the device: the SFH parameters' rows (tage, tau, const, fburst, tburst,
sf_start, sf_trunc, and sf_slope for sfh 5: forward-mode tangents of the weights), logzsol's row and weights_bar (the
cotangent of the weights over ages), against central differences (h = 1e-4 relative) of the FP64 oracle. Tolerance as the other
gradient tests: |g - g_fd| <= 2e-3 max(|g_fd|, 1e-3 max_rows |g_fd|)."""
import numpy as np
import pytest

from conftest import blend_at_logzsol, oracle_sfh_csp

pytestmark = pytest.mark.gpu

RTOL = 2e-3
H_REL = 1e-4
ROWS = {"logzsol": 15, "tage": 16, "tau": 17, "const": 18, "fburst": 19, "tburst": 20, "sf_start": 21,
        "sf_trunc": 24}
ROWS_SIMHA = {"logzsol": 15, "tage": 16, "tau": 17, "sf_start": 21, "sf_trunc": 24, "sf_slope": 25}


def _loss(out, mb, sb, massb, lbolb):
    return (np.nansum(mb * out["mags"], axis=1) + np.sum(sb * out["spec"], axis=1) + massb * out["mass"]
            + lbolb * out["lbol"])


def _cot(c, n, seed):
    from libopensps_gb300.workloads import adjoint_cotangents
    mb, sb = adjoint_cotangents(n, c.nspec, c.nbands, seed=seed)
    rng = np.random.default_rng(seed + 1)
    return mb, sb, rng.standard_normal(n), rng.standard_normal(n)


def _away_from_nodes(log_age, x_gyr, rng, margin=2e-3):
    """Values (Gyr) whose log10(years) lies at least margin dex from any grid age (the weights' kinks)."""
    x = np.array(x_gyr, dtype=np.float64)
    for i in range(x.size):
        while np.min(np.abs(np.log10(x[i] * 1e9) - log_age)) < margin:
            x[i] *= 1.0 + 3 * margin
    return x


def test_sfh_rows_match_central_differences(data, built_lib):
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    n = 6
    rng = np.random.default_rng(81)
    la = data["log_age"]
    # the kinks of the weights lie where the star-forming age tage - sf_start, the burst's lookback time
    # tage - tburst or the truncation's tage - sf_trunc crosses a grid age: each is drawn away from them
    start = rng.uniform(0.05, 0.3, n)
    age = _away_from_nodes(la, rng.uniform(3.0, 12.0, n), rng, 5e-3)
    tb = _away_from_nodes(la, rng.uniform(0.8, 2.5, n), rng, 5e-3)
    tq = _away_from_nodes(la, rng.uniform(0.3, 1.0, n), rng, 5e-3)
    params = {"tau": 10.0 ** rng.uniform(-0.3, 0.8, n), "tage": age + start, "sf_start": start,
              "tburst": age + start - tb, "sf_trunc": age + start - tq,
              "logzsol": rng.uniform(-1.5, 0.3, n), "dust2": rng.uniform(0.1, 1.0, n),
              "const": rng.uniform(0.05, 0.3, n), "fburst": rng.uniform(0.05, 0.2, n),
              "zred": rng.uniform(0.2, 2.0, n), "sigma_smooth": rng.uniform(60.0, 250.0, n)}
    c = Context()
    c.set_int("sfh", 4)
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    mb, sb, massb, lbolb = _cot(c, n, 82)
    got = c.csp_batch_grad(params, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb, n=n)
    o = Oracle(data, nbands=40)
    names = list(ROWS)
    g = np.stack([got["params_bar"][:, ROWS[k]] for k in names], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(names):
        h = H_REL * np.maximum(np.abs(params[k]), 1e-2)
        up = oracle_sfh_csp(o, data, 4, dict(params, **{k: params[k] + h}))
        dn = oracle_sfh_csp(o, data, 4, dict(params, **{k: params[k] - h}))
        fd[:, i] = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * h)
    scale = np.max(np.abs(fd), axis=1, keepdims=True)
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * scale)
    assert float(err.max()) <= RTOL, {names[i]: float(err[:, i].max()) for i in range(len(names))}
    c.close()


def test_simha_rows_match_central_differences(data, built_lib):
    """sfh 5: the ramp's start (the truncation's lookback time tq), its zero t0 = tq - 1 / slope (for the falling
    ramps) and the star-forming age each drawn away from the grid ages; half the ramps reach zero before tage."""
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    n = 6
    rng = np.random.default_rng(83)
    la = data["log_age"]
    start = rng.uniform(0.05, 0.3, n)
    age = _away_from_nodes(la, rng.uniform(4.0, 12.0, n), rng, 5e-3)
    tq = _away_from_nodes(la, rng.uniform(1.0, 3.0, n), rng, 5e-3)
    t0 = _away_from_nodes(la, tq * rng.uniform(0.2, 0.6, n), rng, 5e-3)
    falling_to_zero = np.arange(n) % 2 == 0
    slope = np.where(falling_to_zero, -1.0 / (tq - t0), -1.0 / (3.0 * tq))
    params = {"tau": 10.0 ** rng.uniform(-0.3, 0.8, n), "tage": age + start, "sf_start": start,
              "sf_trunc": age + start - tq, "sf_slope": slope, "logzsol": rng.uniform(-1.5, 0.3, n),
              "dust2": rng.uniform(0.1, 1.0, n), "zred": rng.uniform(0.2, 2.0, n),
              "sigma_smooth": rng.uniform(60.0, 250.0, n)}
    c = Context()
    c.set_int("sfh", 5)
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    mb, sb, massb, lbolb = _cot(c, n, 84)
    got = c.csp_batch_grad(params, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb, n=n)
    o = Oracle(data, nbands=40)
    names = list(ROWS_SIMHA)
    g = np.stack([got["params_bar"][:, ROWS_SIMHA[k]] for k in names], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(names):
        h = H_REL * np.maximum(np.abs(params[k]), 1e-2)
        up = oracle_sfh_csp(o, data, 5, dict(params, **{k: params[k] + h}))
        dn = oracle_sfh_csp(o, data, 5, dict(params, **{k: params[k] - h}))
        fd[:, i] = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * h)
    scale = np.max(np.abs(fd), axis=1, keepdims=True)
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * scale)
    assert float(err.max()) <= RTOL, {names[i]: float(err[:, i].max()) for i in range(len(names))}
    assert np.all(np.abs(fd[:, names.index("sf_slope")]) > 1e-6 * scale[:, 0])
    c.close()


def test_tabular_sfh_rows(data, built_lib):
    """sfh 3: the SFH rows are zero (the tabular SFH has no parameters in the reference's tangents); logzsol's row
    against central differences."""
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    n = 5
    rng = np.random.default_rng(85)
    t = np.linspace(0.0, 13.0, 60)
    table = (t, 1.0 + 0.5 * np.sin(t))
    params = {"tage": rng.uniform(3.0, 12.0, n), "logzsol": rng.uniform(-1.5, 0.3, n),
              "dust2": rng.uniform(0.1, 1.0, n), "zred": rng.uniform(0.2, 2.0, n),
              "sigma_smooth": rng.uniform(60.0, 250.0, n)}
    c = Context()
    c.set_int("sfh", 3)
    c.set_sfh_tab(*table)
    c.set_int("add_neb_emission", 1)
    mb, sb, massb, lbolb = _cot(c, n, 86)
    got = c.csp_batch_grad(params, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb, n=n)
    for k in ("tage", "tau", "const", "fburst", "tburst", "sf_start", "sf_trunc"):
        assert np.all(got["params_bar"][:, ROWS[k]] == 0.0)
    assert np.all(got["params_bar"][:, 25] == 0.0)
    o = Oracle(data, nbands=40, add_igm=False)
    h = H_REL * np.abs(params["logzsol"])
    up = oracle_sfh_csp(o, data, 3, dict(params, logzsol=params["logzsol"] + h), table=table)
    dn = oracle_sfh_csp(o, data, 3, dict(params, logzsol=params["logzsol"] - h), table=table)
    fd = (_loss(up, mb, sb, massb, lbolb) - _loss(dn, mb, sb, massb, lbolb)) / (2.0 * h)
    g = got["params_bar"][:, ROWS["logzsol"]]
    assert float(np.max(np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd))))) <= RTOL
    c.close()


def test_weights_bar_and_logzsol_with_given_weights(data, built_lib):
    """ssp_weights (one weight per age) blended at logzsol: weights_bar along a random relative direction, and
    logzsol's row."""
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle
    n = 7
    rng = np.random.default_rng(91)
    w = rng.dirichlet(np.ones(107), size=n)
    params = {"logzsol": rng.uniform(-1.8, 0.3, n), "dust2": rng.uniform(0.1, 1.5, n),
              "zred": rng.uniform(0.2, 3.0, n), "sigma_smooth": rng.uniform(60.0, 250.0, n)}
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    mb, sb, massb, lbolb = _cot(c, n, 92)
    got = c.csp_batch_grad(params, ssp_weights=w, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
    o = Oracle(data, nbands=40)

    def run(wv, lz):
        wz, lb = blend_at_logzsol(data, wv, lz)
        out = o.csp_batch({k: v for k, v in params.items() if k != "logzsol"}, wz)
        out["lbol"] = np.log10(lb[:, 0])
        return _loss(out, mb, sb, massb, lbolb)

    dw = w * rng.standard_normal(w.shape)
    fd_w = (run(w + H_REL * dw, params["logzsol"]) - run(w - H_REL * dw, params["logzsol"])) / (2 * H_REL)
    g_w = np.sum(got["weights_bar"] * dw, axis=1)
    assert float(np.max(np.abs(g_w - fd_w) / np.maximum(np.abs(fd_w), 1e-3 * np.max(np.abs(fd_w))))) <= RTOL
    h = H_REL * np.abs(params["logzsol"])
    fd_z = (run(w, params["logzsol"] + h) - run(w, params["logzsol"] - h)) / (2 * h)
    g_z = got["params_bar"][:, 15]
    assert float(np.max(np.abs(g_z - fd_z) / np.maximum(np.abs(fd_z), 1e-3 * np.max(np.abs(fd_z))))) <= RTOL
    c.close()
