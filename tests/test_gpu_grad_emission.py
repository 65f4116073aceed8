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


def _away_from_nodes(log_age, x_gyr, margin=5e-3):
    x = np.array(x_gyr, dtype=np.float64)
    for i in range(x.size):
        while np.min(np.abs(np.log10(x[i] * 1e9) - log_age)) < margin:
            x[i] *= 1.0 + 3 * margin
    return x


def test_agn_with_sfh_weights_matches_central_differences(data, built_lib):
    """Weights formed on the device from delayed-tau SFH parameters and blended at logzsol: the AGN scales with the
    log-blended L_bol (the model's L_bol output), whose cotangent goes through the SFH reverse pass (the tage, tau
    and logzsol rows), beside the fagn and agn_tau rows."""
    from libopensps_gb300 import synth_dust
    from libopensps_gb300.capi import Context
    from oracle.oracle import SFH_NAMES, Oracle, sfh_weights
    from conftest import blend_at_logzsol
    n = 5
    rng = np.random.default_rng(160)
    params = {"tau": 10.0 ** rng.uniform(-0.3, 0.8, n), "tage": _away_from_nodes(data["log_age"], rng.uniform(2.0, 12.0, n)),
              "logzsol": rng.uniform(-1.5, 0.3, n), "dust2": rng.uniform(0.1, 1.0, n), "zred": rng.uniform(0.2, 2.0, n),
              "sigma_smooth": rng.uniform(60.0, 250.0, n), "fagn": rng.uniform(0.05, 1.0, n),
              "agn_tau": _mid_cell(synth_dust.AGN_TAU, rng, n)}
    c = Context()
    c.set_int("sfh", 4)
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_agn_dust", 1)
    mb, sb, massb, lbolb = _cotangents(n, c.nspec, c.nbands, 161)
    got = c.csp_batch_grad(params, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb, n=n)
    c.close()
    o = Oracle(data, nbands=40, agn=synth_dust.load_agn())

    def run(q):
        w, _ = sfh_weights(data["log_age"], 4, q, n)
        wz, lb = blend_at_logzsol(data, w, q["logzsol"])
        rest = {k: v for k, v in q.items() if k not in SFH_NAMES and k != "logzsol"}
        parts = o.csp_batch(rest, wz, young=True)
        out = o.csp_from_parts(rest, parts["young"], parts["old"], lsum=lb[:, 0])
        out["mass"], out["lbol"] = parts["mass"], np.log10(lb[:, 0])
        return _loss(out, mb, sb, massb, lbolb)

    rows = {"fagn": 0, "agn_tau": 31, "logzsol": 15, "tage": 16, "tau": 17}
    g = np.stack([got["params_bar"][:, r] for r in rows.values()], axis=1)
    fd = np.empty_like(g)
    for i, k in enumerate(rows):
        h = H_REL * np.abs(params[k])
        fd[:, i] = (run(dict(params, **{k: params[k] + h})) - run(dict(params, **{k: params[k] - h}))) / (2.0 * h)
    worst, err = _check_rows(g, fd)
    assert worst <= RTOL, {k: float(err[:, i].max()) for i, k in enumerate(rows)}


def test_agn_through_the_operator_reverse(data, built_lib):
    """The AGN with the SSP operators (its scale the operator's linear L_bol row): the imf1-3 rows and the weights'
    cotangent along a random direction, beside fagn, against central differences."""
    from libopensps_gb300 import synth_dust, synth_ops
    from libopensps_gb300.capi import Context
    from oracle.oracle import Oracle, OpsOracle
    from conftest import config3_inputs
    n = 5
    wz, params = config3_inputs(n, seed=170)
    rng = np.random.default_rng(171)
    alpha = np.stack([rng.uniform(0.9, 1.6, n), rng.uniform(1.9, 2.6, n), rng.uniform(2.0, 2.9, n)], axis=1)
    params = dict(params, imf1=alpha[:, 0], imf2=alpha[:, 1], imf3=alpha[:, 2], fagn=rng.uniform(0.05, 1.0, n),
                  agn_tau=_mid_cell(synth_dust.AGN_TAU, rng, n))
    c = Context()
    c.set_int("add_igm_absorption", 1)
    c.set_int("add_agn_dust", 1)
    c.build_ssp_ops()
    mb, sb, massb, lbolb = _cotangents(n, c.nspec, c.nbands, 172)
    got = c.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb, mass_bar=massb, lbol_bar=lbolb)
    c.close()
    ops = OpsOracle(synth_ops.load())
    o = Oracle(data, nbands=40, add_neb=False, agn=synth_dust.load_agn())
    itesc = int(np.clip(np.searchsorted(data["log_age"], 7.0, side="right"), 1, data["log_age"].size))
    base = {k: v for k, v in params.items() if k not in ("imf1", "imf2", "imf3")}

    def run(al, w):
        y, old, mass, ls = ops.parts(al, w, itesc)
        out = o.csp_from_parts(base, y, old, lsum=ls)
        out["mass"], out["lbol"] = mass, np.log10(ls)
        return _loss(out, mb, sb, massb, lbolb)

    pb = got["params_bar"]
    for j in range(3):
        h = H_REL * np.abs(alpha[:, j])
        up, dn = alpha.copy(), alpha.copy()
        up[:, j] += h
        dn[:, j] -= h
        fd = (run(up, wz) - run(dn, wz)) / (2.0 * h)
        e = np.abs(pb[:, 26 + j] - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
        assert float(e.max()) <= RTOL, (j, pb[:, 26 + j], fd)
    # fagn: the AGN's own row (its scale the operator's linear L_bol)
    h = H_REL * params["fagn"]
    y, old, mass, ls = ops.parts(alpha, wz, itesc)

    def run_f(f):
        out = o.csp_from_parts(dict(base, fagn=f), y, old, lsum=ls)
        out["mass"], out["lbol"] = mass, np.log10(ls)
        return _loss(out, mb, sb, massb, lbolb)

    fd = (run_f(params["fagn"] + h) - run_f(params["fagn"] - h)) / (2.0 * h)
    e = np.abs(pb[:, 0] - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert float(e.max()) <= RTOL, (pb[:, 0], fd)
    dwz = wz * rng.standard_normal(wz.shape)
    fdw = (run(alpha, wz + H_REL * dwz) - run(alpha, wz - H_REL * dwz)) / (2.0 * H_REL)
    gw = np.sum(got["weights_z_bar"] * dwz, axis=(1, 2))
    e = np.abs(gw - fdw) / np.maximum(np.abs(fdw), 1e-3 * np.max(np.abs(fdw)))
    assert float(e.max()) <= RTOL, (gw, fdw)
