"""The SSP operator with the user IMF and with IMF mass limits other than 0.08 - 120 M_sun, through the exact fold,
against the FP64 oracle (ops_oracle.c).

* imf_type 5: segments (lower mass, upper mass, slope) read from imf_filename under the data root, imf.dat when no
  name is set (src/physics/opensps_ssp.f90:1756-1808); the IMF limits become the first lower and the last upper mass;
  imf_integral case 5 (src/physics/opensps_imf.f90:287-305): each segment a power law over its own mass range,
  continuous at its lower mass, overlapping segments adding, gaps empty.
* imf_lower_limit / imf_upper_limit: points whose initial mass lies outside weigh nothing, each age's first bin
  starts at the lower limit, the normalisation is the IMF's mass between the limits (compute_imf_weights :111-172);
  Salpeter and Chabrier have no cut at 0.08 M_sun, Kroupa and Dave do.

Tolerances as the other operator tests: spectra <= 1e-4 relative (pixels above 1e-6 of the peak), magnitudes
<= 1e-3 mag over the bands less than 30 mag fainter than the model's brightest, mass and L_bol <= 1e-5 relative;
gradients 2e-3. (Without stars above 60 M_sun the far-UV bands of the models at high redshift, behind the IGM, sit
near 1e-43 in the FP32 band sums, in FP32's subnormal range, where a sum keeps three digits: their magnitudes, some
60 mag fainter than the model's brightest band, are only checked to stay that faint.)
"""
import os
from pathlib import Path

import numpy as np
import pytest

from conftest import config3_inputs, rel_err_spec

pytestmark = pytest.mark.gpu

# four segments: a gap-free chain to 60 M_sun and a fourth overlapping the third over 3 - 10 M_sun
USER = np.array([[0.1, 0.4, 1.1], [0.4, 2.0, 2.0], [2.0, 60.0, 2.6], [3.0, 10.0, 1.0]])
# three segments with an empty gap over 0.4 - 0.5 M_sun, to 80 M_sun
USER_GAP = np.array([[0.1, 0.4, 1.1], [0.5, 2.0, 2.0], [2.0, 80.0, 2.6]])
# the rows of the reference's test imf.dat: Kroupa's slopes, to 100 M_sun
KROUPA_ROWS = np.array([[0.08, 0.5, 1.3], [0.5, 1.0, 2.3], [1.0, 100.0, 2.3]])


def _write(name, rows):
    path = Path(os.environ["OPENSPS_DATA_HOME"]) / name
    path.write_text("".join(f"{a:.17g} {b:.17g} {c:.17g}\n" for a, b, c in rows))


@pytest.fixture(scope="module")
def ops_data():
    from libopensps_gb300 import synth_ops
    return synth_ops.load()


@pytest.fixture(scope="module")
def octx(data, built_lib, ops_data):
    from libopensps_gb300.capi import Context
    _write("imf_user_test.dat", USER)
    c = Context()
    c.set_int("add_igm_absorption", 1)
    c.build_ssp_ops()
    c.set_str("imf_filename", "imf_user_test.dat")
    yield c
    c.close()


class _Imf:
    """The context's imf_type and mass limits for a block, restored after."""

    def __init__(self, c, imf_type, lo=0.08, hi=120.0):
        self.c, self.t, self.lo, self.hi = c, imf_type, lo, hi

    def __enter__(self):
        self.c.set_int("imf_type", self.t)
        self.c.set_float("imf_lower_limit", self.lo)
        self.c.set_float("imf_upper_limit", self.hi)

    def __exit__(self, *exc):
        self.c.set_int("imf_type", 2)
        self.c.set_float("imf_lower_limit", 0.08)
        self.c.set_float("imf_upper_limit", 120.0)


def _check_mags(got, ora):
    ref = np.nanmin(ora, axis=1, keepdims=True)
    sel = ora < ref + 30.0
    assert np.array_equal(np.isnan(got[sel]), np.isnan(ora[sel]))
    assert float(np.nanmax(np.abs(got[sel] - ora[sel]))) <= 1e-3
    assert np.all(np.nan_to_num(got[~sel], nan=np.inf) > (ref + 25.0).repeat(ora.shape[1], axis=1)[~sel])


def _bright_only(mb, mags):
    """The magnitudes' cotangents with those of the bands more than 30 mag fainter than the model's brightest zero."""
    ref = np.nanmin(mags, axis=1, keepdims=True)
    return np.where(mags < ref + 30.0, mb, 0.0)


def _itesc(data):
    return int(np.clip(np.searchsorted(data["log_age"], 7.0, side="right"), 1, data["log_age"].size))


def _grid_weights(nt, nz, z):
    wz = np.zeros((nt, nz, nt))
    for t in range(nt):
        wz[t, z, t] = 1.0
    return wz


def _packed(imf_type, n, ip=None):
    if ip is None:
        return np.tile([1.3, 2.3, 2.3] if imf_type == 2 else [2.35] * 3, (n, 1))
    if imf_type == 3:
        return np.stack([ip["vdmc"], np.zeros(n), np.zeros(n)], axis=1)
    if imf_type == 4:
        return np.stack([ip["imf1"], ip["imf2"], ip["mdave"]], axis=1)
    if imf_type == 2:
        return np.stack([ip["imf1"], ip["imf2"], ip["imf3"]], axis=1)
    return np.tile([2.35] * 3, (n, 1))


def _imf_params(n, seed):
    rng = np.random.default_rng(seed)
    return {"imf1": rng.uniform(0.6, 1.8, n), "imf2": rng.uniform(1.8, 2.8, n), "imf3": rng.uniform(1.9, 2.7, n),
            "vdmc": 10.0 ** rng.uniform(-1.2, 0.0, n), "mdave": 10.0 ** rng.uniform(-0.6, 0.4, n)}


@pytest.mark.parametrize("table", ["overlap", "gap"])
def test_user_imf_evaluate(octx, ops_data, table):
    from oracle.oracle import OpsOracle
    rows = USER if table == "overlap" else USER_GAP
    if table == "gap":
        _write("imf_gap_test.dat", USER_GAP)
        octx.set_str("imf_filename", "imf_gap_test.dat")
    octx.set_int("zmet", 4)
    try:
        got = octx.evaluate_ssp_op(imf_type=5)
    finally:
        octx.set_int("zmet", 1)
        octx.set_str("imf_filename", "imf_user_test.dat")
    nt, nz = octx.ntfull, octx.nz
    y, o, mass, ls = OpsOracle(ops_data, imf_type=5, user=rows).parts(np.zeros((nt, 3)), _grid_weights(nt, nz, 3), nt)
    assert np.all(o == 0.0)
    assert rel_err_spec(got["spec"], y) <= 1e-4
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)
    np.testing.assert_allclose(got["lbol"], np.log10(ls), rtol=1e-5)


def test_default_file_with_kroupa_rows_is_kroupa(octx, ops_data):
    """With no name the file is imf.dat; with the reference's test rows (Kroupa to 100 M_sun) the user IMF gives what
    the Kroupa IMF gives with the upper limit 100 M_sun (two paths of the fold), both the oracle's."""
    from oracle.oracle import OpsOracle
    _write("imf.dat", KROUPA_ROWS)
    nt, nz = octx.ntfull, octx.nz
    octx.set_str("imf_filename", "")
    try:
        u = octx.evaluate_ssp_op(imf_type=5)
    finally:
        octx.set_str("imf_filename", "imf_user_test.dat")
    with _Imf(octx, 2, 0.08, 100.0):
        k = octx.evaluate_ssp_op([1.3, 2.3, 2.3, 0.08, 0.5], imf_type=2)
    assert rel_err_spec(u["spec"], k["spec"]) <= 2e-6
    np.testing.assert_allclose(u["mass"], k["mass"], rtol=1e-6)
    y, o, mass, ls = OpsOracle(ops_data, imf_type=5, user=KROUPA_ROWS).parts(np.zeros((nt, 3)),
                                                                             _grid_weights(nt, nz, 0), nt)
    assert rel_err_spec(u["spec"], y) <= 1e-4
    np.testing.assert_allclose(u["mass"], mass, rtol=1e-5)


def test_user_imf_batch(octx, data, ops_data):
    from oracle.oracle import Oracle, OpsOracle
    n = 40
    wz, params = config3_inputs(n, seed=380)
    rng = np.random.default_rng(381)
    params = dict(params, dust1=rng.uniform(0.0, 1.0, n))
    with _Imf(octx, 5):
        got = octx.csp_batch(params, ssp_weights_z=wz)
        assert not octx.ops_last_interpolated()
    y, o, mass, ls = OpsOracle(ops_data, imf_type=5, user=USER).parts(np.zeros((n, 3)), wz, _itesc(data))
    ora = Oracle(data, nbands=40, add_neb=False).csp_from_parts(params, y, o)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    _check_mags(got["mags"], ora["mags"])
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)
    np.testing.assert_allclose(got["lbol"], np.log10(ls), rtol=1e-5)


def test_user_imf_reverse(octx, data, ops_data):
    """The weights' cotangent along a random direction against central differences of the oracle; the IMF rows
    (26-30) zero (the user IMF has no parameters per model)."""
    from libopensps_gb300.workloads import adjoint_cotangents
    from oracle.oracle import Oracle, OpsOracle
    n = 5
    wz, params = config3_inputs(n, seed=390)
    mb, sb = adjoint_cotangents(n, data["lambda"].size, 40, seed=391)
    ops = OpsOracle(ops_data, imf_type=5, user=USER)
    csp = Oracle(data, nbands=40, add_neb=False)
    mb = _bright_only(mb, csp.csp_from_parts(params, *ops.parts(np.zeros((n, 3)), wz, _itesc(data))[:2])["mags"])
    with _Imf(octx, 5):
        got = octx.csp_batch_grad(params, wz, mags_bar=mb, spec_bar=sb)
    assert np.all(got["params_bar"][:, 26:31] == 0.0)

    def loss(w):
        y, o, mass, ls = ops.parts(np.zeros((n, 3)), w, _itesc(data))
        out = csp.csp_from_parts(params, y, o)
        return np.nansum(mb * out["mags"], axis=1) + np.sum(sb * out["spec"], axis=1)

    rng = np.random.default_rng(392)
    dw = wz * rng.standard_normal(wz.shape)
    fd = (loss(wz + 1e-4 * dw) - loss(wz - 1e-4 * dw)) / 2e-4
    g = np.sum(got["weights_z_bar"] * dw, axis=(1, 2))
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert float(err.max()) <= 2e-3, (g, fd)


@pytest.mark.parametrize("imf_type,lo,hi", [(2, 0.15, 60.0), (4, 0.15, 60.0), (3, 0.15, 60.0), (0, 0.05, 80.0),
                                            (1, 0.05, 80.0), (2, 0.05, 150.0)])
def test_mass_limits_batch(octx, data, ops_data, imf_type, lo, hi):
    """The reference's operator cases (Kroupa 0.15 - 60 M_sun, Salpeter to 80 M_sun) and more: the first bins open
    below 0.08 M_sun for Salpeter and Chabrier (no cut there) and stay cut for Kroupa."""
    from oracle.oracle import Oracle, OpsOracle
    n = 32
    wz, params = config3_inputs(n, seed=400 + imf_type)
    ip = _imf_params(n, 401 + imf_type)
    with _Imf(octx, imf_type, lo, hi):
        got = octx.csp_batch(dict(params, **ip) if imf_type in (2, 3, 4) else params, ssp_weights_z=wz)
        assert not octx.ops_last_interpolated()
    al = _packed(imf_type, n, ip if imf_type in (2, 3, 4) else None)
    y, o, mass, ls = OpsOracle(ops_data, imf_type=imf_type, lim_lo=lo, lim_hi=hi, lower_bound=lo).parts(
        al, wz, _itesc(data))
    ora = Oracle(data, nbands=40, add_neb=False).csp_from_parts(params, y, o)
    assert rel_err_spec(got["spec"], ora["spec"]) <= 1e-4
    _check_mags(got["mags"], ora["mags"])
    np.testing.assert_allclose(got["mass"], mass, rtol=1e-5)
    np.testing.assert_allclose(got["lbol"], np.log10(ls), rtol=1e-5)
    # the limits are in effect
    y0, _, m0, _ = OpsOracle(ops_data, imf_type=imf_type).parts(al, wz, _itesc(data))
    assert float(np.max(np.abs(mass / m0 - 1.0))) > 1e-4


def test_mass_limits_reverse(octx, data, ops_data):
    """Kroupa per model between 0.15 and 60 M_sun: the weights' cotangent and the imf1-3 rows (26-28) against
    central differences of the oracle (the normalisation's derivative over the limits)."""
    from libopensps_gb300.workloads import adjoint_cotangents
    from oracle.oracle import Oracle, OpsOracle
    n = 5
    wz, params = config3_inputs(n, seed=410)
    ip = _imf_params(n, 411)
    mb, sb = adjoint_cotangents(n, data["lambda"].size, 40, seed=412)
    ops = OpsOracle(ops_data, imf_type=2, lim_lo=0.15, lim_hi=60.0, lower_bound=0.15)
    csp = Oracle(data, nbands=40, add_neb=False)
    mb = _bright_only(mb, csp.csp_from_parts(params, *ops.parts(_packed(2, n, ip), wz, _itesc(data))[:2])["mags"])
    with _Imf(octx, 2, 0.15, 60.0):
        got = octx.csp_batch_grad(dict(params, **ip), wz, mags_bar=mb, spec_bar=sb)
    pb = got["params_bar"]

    def loss(w, q):
        y, o, mass, ls = ops.parts(_packed(2, n, q), w, _itesc(data))
        out = csp.csp_from_parts(params, y, o)
        return np.nansum(mb * out["mags"], axis=1) + np.sum(sb * out["spec"], axis=1)

    rng = np.random.default_rng(413)
    dw = wz * rng.standard_normal(wz.shape)
    fd = (loss(wz + 1e-4 * dw, ip) - loss(wz - 1e-4 * dw, ip)) / 2e-4
    g = np.sum(got["weights_z_bar"] * dw, axis=(1, 2))
    err = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert float(err.max()) <= 2e-3, (g, fd)
    for k, row in (("imf1", 26), ("imf2", 27), ("imf3", 28)):
        h = 1e-4 * np.abs(ip[k])
        fdk = (loss(wz, dict(ip, **{k: ip[k] + h})) - loss(wz, dict(ip, **{k: ip[k] - h}))) / (2.0 * h)
        e = np.abs(pb[:, row] - fdk) / np.maximum(np.abs(fdk), 1e-3 * np.max(np.abs(fdk)))
        assert float(e.max()) <= 2e-3, (k, pb[:, row], fdk)


def test_refusals(octx, data):
    """A user IMF file that is not there or holds no segments: status 504 (OPENSPS_ERR_SSP_IMF_FILE); limits out of
    order: 3; an IMF type beyond 5: 2; limits other than 0.08 - 120 M_sun without the operators: 2."""
    from libopensps_gb300.capi import Context, OpenSPSError
    n = 4
    wz, params = config3_inputs(n, seed=420)
    (Path(os.environ["OPENSPS_DATA_HOME"]) / "imf_empty_test.dat").write_text("\n")
    with _Imf(octx, 5):
        for name in ("no_such_imf.dat", "imf_empty_test.dat"):
            octx.set_str("imf_filename", name)
            with pytest.raises(OpenSPSError) as e:
                octx.csp_batch(params, ssp_weights_z=wz)
            assert e.value.status == 504
        octx.set_str("imf_filename", "imf_user_test.dat")
        octx.csp_batch(params, ssp_weights_z=wz)   # (readable again)
    with _Imf(octx, 2, 0.5, 0.4):
        with pytest.raises(OpenSPSError) as e:
            octx.csp_batch(params, ssp_weights_z=wz)
        assert e.value.status == 3
    with _Imf(octx, 6):
        with pytest.raises(OpenSPSError) as e:
            octx.csp_batch(params, ssp_weights_z=wz)
        assert e.value.status == 2
    c = Context()
    try:
        c.set_float("imf_upper_limit", 80.0)
        with pytest.raises(OpenSPSError) as e:
            c.csp_batch(params, ssp_weights_z=wz)
        assert e.value.status == 2
    finally:
        c.close()
