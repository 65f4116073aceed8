"""SFH weights formed on the device (sfh 0, 1, 4 with the constant and burst components; sfh 5, the delayed tau
with a linear ramp after the truncation; the tabular sfh 2 and 3), blended at logzsol,
through the batch, against the FP64 oracle: spectra <= 1e-4 relative, magnitudes <= 1e-3 mag, mass <= 1e-12
relative, log L_bol <= 1e-9 relative, the SFR per unit mass formed <= 1e-12 relative.

(L_bol is set by the youngest ages, whose weights are differences of the closed-form moments ~ e^(t/tau) over bins
short against tau: a 1-ulp difference between the host's and the device's exp / pow grows by ~tau / dt there, up
to ~1e-10 relative in those weights; the mass is set by the old ages and keeps 1e-12.)"""
import numpy as np
import pytest

from conftest import oracle_sfh_csp, rel_err_spec

pytestmark = pytest.mark.gpu


def _ctx(sfh, nbands=40, neb=False, igm=False):
    from libopensps_gb300.capi import Context
    c = Context()
    c.set_int("sfh", sfh)
    if neb:
        c.set_int("add_neb_emission", 1)
    if igm:
        c.set_int("add_igm_absorption", 1)
    if nbands == 20:
        c.set_filters_library("gauss20")
    return c


def _forward(c, params, n):
    import ctypes as C
    from libopensps_gb300 import capi
    k, names, vals, keep = capi._names_values(params, n)
    out = {"mags": np.empty((n, c.nbands)), "spec": np.empty((n, c.nspec)), "mass": np.empty(n),
           "lbol": np.empty(n), "sfr": np.empty(n)}
    st = C.c_int(0)
    c.lib.opensps_context_compute_csp_batch(c.handle, n, k, names, vals, None, capi._ptr(out["mags"]),
                                            capi._ptr(out["spec"]), capi._ptr(out["mass"]), capi._ptr(out["lbol"]),
                                            None, capi._ptr(out["sfr"]), None, None, C.byref(st))
    capi._check(st, c.lib)
    del keep
    return out


def _check(got, ora):
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert np.array_equal(np.isnan(got["mags"]), np.isnan(ora["mags"]))
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3
    np.testing.assert_allclose(got["mass"], ora["mass"], rtol=1e-12)
    np.testing.assert_allclose(got["lbol"], ora["lbol"], rtol=1e-9)
    np.testing.assert_allclose(got["sfr"], ora["sfr"], rtol=1e-12)


def test_delayed_tau_plain_config(data, built_lib):
    """The plain-CSP workload: delayed tau, tau log-uniform 0.1-10 Gyr, age 1-13.7 Gyr, logZ on the grid's range,
    power-law dust, z = 0, no nebular emission, 20 filters."""
    from oracle.oracle import Oracle
    n = 64
    rng = np.random.default_rng(0)
    params = {"tau": 10.0 ** rng.uniform(-1.0, 1.0, n), "tage": rng.uniform(1.0, 13.7, n),
              "logzsol": rng.uniform(-2.0, 0.5, n), "dust2": rng.uniform(0.0, 2.0, n)}
    c = _ctx(4, nbands=20)
    got = _forward(c, params, n)
    _check(got, oracle_sfh_csp(Oracle(data, nbands=20, add_neb=False, add_igm=False), data, 4, params))
    c.close()


@pytest.mark.parametrize("sfh", [0, 1, 4])
def test_sfh_types_with_constant_and_burst(data, built_lib, sfh):
    from oracle.oracle import Oracle
    n = 40
    rng = np.random.default_rng(10 + sfh)
    params = {"tau": 10.0 ** rng.uniform(-0.5, 1.0, n), "tage": rng.uniform(0.5, 13.0, n),
              "logzsol": rng.uniform(-1.5, 0.3, n), "dust2": rng.uniform(0.0, 1.0, n),
              "zred": rng.uniform(0.1, 3.0, n), "sigma_smooth": rng.uniform(60.0, 250.0, n)}
    if sfh != 0:
        params.update({"const": rng.uniform(0.0, 0.3, n), "fburst": rng.uniform(0.0, 0.2, n),
                       "tburst": rng.uniform(0.2, 10.0, n), "sf_trunc": np.where(rng.uniform(size=n) < 0.5, 0.0,
                                                                                  rng.uniform(0.5, 12.0, n)),
                       "sf_start": rng.uniform(0.0, 0.3, n)})
    c = _ctx(sfh, neb=True, igm=True)
    got = _forward(c, params, n)
    _check(got, oracle_sfh_csp(Oracle(data, nbands=40), data, sfh, params))
    c.close()


def test_simha_sfh(data, built_lib):
    """sfh 5: truncations inside the star-forming age (and none), ramps falling to zero before tage, falling but not
    to zero, and rising; sf_start and logzsol per model."""
    from oracle.oracle import Oracle
    n = 48
    rng = np.random.default_rng(55)
    tage = rng.uniform(1.0, 13.0, n)
    start = rng.uniform(0.0, 0.3, n)
    trunc = np.where(rng.uniform(size=n) < 0.2, 0.0, start + rng.uniform(0.2, 0.9, n) * (tage - start))
    kind = rng.integers(0, 3, n)
    ramp = np.maximum(tage - trunc, 0.05)
    slope = np.select([kind == 0, kind == 1], [-1.0 / (rng.uniform(0.3, 0.9, n) * ramp),
                                                -1.0 / (rng.uniform(1.2, 4.0, n) * ramp)], rng.uniform(0.05, 1.0, n))
    params = {"tau": 10.0 ** rng.uniform(-0.5, 1.0, n), "tage": tage, "sf_start": start, "sf_trunc": trunc,
              "sf_slope": slope, "logzsol": rng.uniform(-1.5, 0.3, n), "dust2": rng.uniform(0.0, 1.0, n),
              "zred": rng.uniform(0.1, 3.0, n), "sigma_smooth": rng.uniform(60.0, 250.0, n)}
    c = _ctx(5, neb=True, igm=True)
    got = _forward(c, params, n)
    ora = oracle_sfh_csp(Oracle(data, nbands=40), data, 5, params)
    _check(got, ora)
    assert np.any(ora["sfr"] == 0.0) and np.any(ora["sfr"] > 0.0)
    c.close()


def _table(seed=71, ntab=300):
    """A tabular SFH over 0-13.5 Gyr: a bump at 3 Gyr on a wave, one repeated age (a bin of zero width)."""
    rng = np.random.default_rng(seed)
    t = np.sort(rng.uniform(0.0, 13.5, ntab))
    t[0] = 0.0
    t[100] = t[99]
    sfr = 1.0 + 0.5 * np.sin(2.0 * t) + 2.0 * np.exp(-0.5 * ((t - 3.0) / 0.7) ** 2)
    sfr[100] = sfr[99]
    return t, sfr


def _check_tab(got, ora):
    """The tabular SFH's weights are masses formed, each bin a difference of moments ~ slope t^2 much larger than its
    mass: the host's and the device's pow differ by an ulp there, so the FP64 sums agree to 1e-10."""
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    assert float(np.nanmax(np.abs(got["mags"] - ora["mags"]))) <= 1e-3
    np.testing.assert_allclose(got["mass"], ora["mass"], rtol=1e-10)
    np.testing.assert_allclose(got["lbol"], ora["lbol"], rtol=1e-9)
    np.testing.assert_allclose(got["sfr"], ora["sfr"], rtol=1e-12)


def _tab_params(n, seed):
    rng = np.random.default_rng(seed)
    return {"tage": rng.uniform(0.5, 14.0, n), "logzsol": rng.uniform(-1.5, 0.3, n),
            "dust2": rng.uniform(0.0, 1.0, n), "zred": rng.uniform(0.1, 3.0, n),
            "sigma_smooth": rng.uniform(60.0, 250.0, n)}


def test_tabular_sfh_from_the_array(data, built_lib):
    """sfh 3: the table set by opensps_context_set_sfh_tab; models older and younger than the table's span."""
    from oracle.oracle import Oracle
    n = 40
    table = _table()
    params = _tab_params(n, 72)
    c = _ctx(3, neb=True, igm=True)
    c.set_sfh_tab(*table)
    got = _forward(c, params, n)
    _check_tab(got, oracle_sfh_csp(Oracle(data, nbands=40), data, 3, params, table=table))
    c.close()


def test_tabular_sfh_from_the_file(data, built_lib):
    """sfh 2: the table read from sfh_filename under the data root (three columns, the third not read); a missing
    file and sfh 3 without a table are status 508."""
    import os
    from pathlib import Path
    from libopensps_gb300.capi import OpenSPSError
    from oracle.oracle import Oracle
    n = 24
    t, sfr = _table(seed=73, ntab=120)
    path = Path(os.environ["OPENSPS_DATA_HOME"]) / "sfh_tab_test.dat"
    path.write_text("".join(f"{a:.17g} {b:.17g} 0.0142\n" for a, b in zip(t, sfr)))
    params = _tab_params(n, 74)
    c = _ctx(2)
    c.set_str("sfh_filename", "sfh_tab_test.dat")
    got = _forward(c, params, n)
    _check_tab(got, oracle_sfh_csp(Oracle(data, nbands=40, add_neb=False, add_igm=False), data, 2, params,
                                   table=(t, sfr)))
    c.set_str("sfh_filename", "no_such_sfh.dat")
    with pytest.raises(OpenSPSError) as e:
        _forward(c, params, n)
    assert e.value.status == 508
    c.close()
    c = _ctx(3)
    with pytest.raises(OpenSPSError) as e:
        _forward(c, params, n)
    assert e.value.status == 508
    c.close()


def test_sfh_rejects_nonpositive_age(data, built_lib):
    from libopensps_gb300.capi import OpenSPSError
    c = _ctx(4)
    with pytest.raises(OpenSPSError) as e:
        _forward(c, {"tage": np.array([1.0, 0.0]), "tau": np.array([1.0, 1.0])}, 2)
    assert e.value.status == 2
    c.close()
