"""The reference's analytic unit checks of the path's building blocks, run on the FP64 oracle (CPU, no GPU): the same
inputs, the same closed forms or direct evaluations, the same tolerances as OpenSPS's own tests.

* Cosmology (tests/physics/test_opensps_cosmology.f90:142-183): the Einstein-de Sitter luminosity distance in closed
  form at z = 2 (5e-4 relative) and the low-z Hubble law at z = 1e-3 (1e-3 relative).
* SFH moment method (tests/physics/test_opensps_sfh.f90:158-278,1115-1243): the tau model's total mass against its
  integral (5e-3), the delayed tau's mass invariant under a grid refinement (1e-5), the youngest edge bin, and the
  weights against Simpson quadrature of the SFR for the analytic types 0, 1, 4 and 5 with tage on and off a node
  (mass 1e-6, mean log age 1e-8, weights non-negative).
* Simha SFH properties (tests/physics/test_opensps_sfh.f90:379-404,955-1016): the SFR is zero past the ramp's zero
  and the ramp's mass fraction positive; a truncation past the grid's oldest age leaves no ramp; before sf_start the
  mass fraction, SFR and ramp fraction are zero.
* Velocity smoothing (tests/spectra/test_opensps_smoothing.f90:384-474,586-614): the sparse operator against the
  direct convolution integral on a grid with a spacing jump (1e-12 relative) and on the synthetic log-uniform grid;
  a flat spectrum stays flat; pixels outside [minl, maxl] pass through unchanged.
* Batch photometry (tests/spectra/test_opensps_batch_photometry.f90:21-131,135-212): band integrals on the reference
  test's synthetic data (700 pixels, 12 bands with edge supports, two skipped) against a direct FP64 sum (1e-11),
  bit-identical repeats, exact scaling, a model with no flux giving exactly 0, skipped bands exactly 0; the observed
  frame against a direct evaluation on a non-uniform grid for redshifts below, at and above the grid's range.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

C_LIGHT = 2.99792458e18          # src/core/opensps_constants.f90:41 [A/s]


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


# ----------------------------------------------------------------------------------------------------- cosmology
def test_eds_luminosity_distance():
    h0, z = 70.0, 2.0
    dh = (C_LIGHT * 1.0e-13 / h0) * 1.0e6
    expected = (1.0 + z) * dh * (2.0 * (1.0 - 1.0 / math.sqrt(1.0 + z)))
    got = O.lum_distance(h0, 1.0, 0.0, z)
    assert abs(got / expected - 1.0) <= 5.0e-4


def test_low_z_hubble_law():
    h0, z = 70.0, 1.0e-3
    dh = (C_LIGHT * 1.0e-13 / h0) * 1.0e6
    got = O.lum_distance(h0, 0.3, 0.7, z)
    assert abs(got / (dh * z) - 1.0) <= 1.0e-3


# ----------------------------------------------------------------------------------------------------- SFH
def log_grid(n, a, b):
    return a + (b - a) * np.arange(n) / (n - 1)


def test_tau_model_mass_conservation():
    tf = log_grid(60, 6.0, 10.0)
    w = O.ssp_weights_raw(tf, 1, tage=1.0e9, tau=1.0e9, idx_min=1, idx_max=59, tiny_logt=4.0)
    expected = math.exp(1.0) - 1.0
    assert abs(w.sum() / expected - 1.0) <= 5.0e-3


def test_delayed_tau_mass_invariant_under_refinement():
    a = log_grid(40, 6.0, 10.0)
    b = np.concatenate([a[:20], [0.5 * (a[19] + a[20])], a[20:]])
    wa = O.ssp_weights_raw(a, 4, tage=6.0e9, tau=2.0e9, idx_min=1, idx_max=a.size - 1, tiny_logt=4.0)
    wb = O.ssp_weights_raw(b, 4, tage=6.0e9, tau=2.0e9, idx_min=1, idx_max=b.size - 1, tiny_logt=4.0)
    assert abs(wa.sum() / wb.sum() - 1.0) <= 1.0e-5


def test_youngest_edge_includes_zero_bin():
    tf = log_grid(30, 6.0, 9.5)
    w0 = O.ssp_weights_raw(tf, 0, tage=3.0e9, tau=1.0, idx_min=0, idx_max=29, tiny_logt=4.0)
    w1 = O.ssp_weights_raw(tf, 0, tage=3.0e9, tau=1.0, idx_min=1, idx_max=29, tiny_logt=4.0)
    assert w0[0] > w1[0]


def _simpson_moments(sfh_type, tau, tage, t_lo, t_hi, n_steps=200000, trunc=0.0, slope=0.0):
    """M0 = int SFR dt, M1 = int SFR log10(t) dt over lookback [t_lo, t_hi] by composite Simpson in u = log10 t (the
    reference test's sfh_moments_quadrature, log interpolation)."""
    u = np.log10(t_lo) + (np.log10(t_hi) - np.log10(t_lo)) * np.arange(n_steps + 1) / n_steps
    t = 10.0 ** u
    if sfh_type == 0:
        sfr = np.ones_like(t)
    elif sfh_type == 1:
        sfr = np.exp(t / tau) / tau
    elif sfh_type == 5:
        sfr = 1.0 - slope * max(0.0, tage - trunc) + slope * t
    else:
        sfr = (tage - t) * np.exp(t / tau) / tau
    c = np.where(np.arange(n_steps + 1) % 2 == 1, 4.0, 2.0)
    c[0] = c[-1] = 1.0
    jac = t * math.log(10.0)
    du = (u[-1] - u[0]) / n_steps
    return float(np.sum(c * sfr * jac)) * du / 3.0, float(np.sum(c * sfr * u * jac)) * du / 3.0


@pytest.mark.parametrize("sfh_type", [0, 1, 4, 5])
@pytest.mark.parametrize("on_node", [True, False])
def test_moments_match_quadrature(sfh_type, on_node):
    tf = log_grid(60, 6.0, 10.2)
    tau = 2.0e9
    tage = 10.0 ** tf[54] if on_node else 10.0 ** (0.3 * tf[54] + 0.7 * tf[55])
    trunc, slope = 2.0e9, 1.0e-10
    w = O.ssp_weights_raw(tf, sfh_type, tage=tage, tau=tau, idx_min=1, idx_max=tf.size, tiny_logt=4.0, trunc=trunc,
                          slope=slope)
    m0, m1 = _simpson_moments(sfh_type, tau, tage, 10.0 ** tf[0], tage, trunc=trunc, slope=slope)
    assert abs(w.sum() / m0 - 1.0) <= 1.0e-6
    assert abs((np.sum(w * tf) / w.sum()) / (m1 / m0) - 1.0) <= 1.0e-8
    assert np.all(w >= 0.0)


def test_simha_truncation_logic():
    mf, sfr, fl = O.sfh_properties(log_grid(30, 6.0, 10.0), 5, {"tau": 1.0, "sf_start": 0.0, "sf_trunc": 2.0,
                                                                 "sf_slope": -1.0}, 4.0)
    assert abs(sfr) <= 1.0e-12
    assert fl > 0.0


def test_simha_no_truncation_effective():
    mf, sfr, fl = O.sfh_properties(log_grid(10, 6.0, 10.0), 5, {"tau": 1.0, "sf_start": 0.0, "sf_trunc": 20.0,
                                                                 "sf_slope": -1.0}, 5.0)
    assert fl == 0.0


def test_simha_before_sf_start():
    mf, sfr, fl = O.sfh_properties(log_grid(10, 6.0, 10.0), 5, {"tau": 1.0, "sf_start": 5.0, "sf_trunc": 7.0,
                                                                 "sf_slope": -1.0}, 3.0)
    assert mf == 0.0 and sfr == 0.0 and fl == 0.0


# ----------------------------------------------------------------------------------------------------- smoothing
def test_velocity_operator_matches_direct_convolution():
    n = 600
    i = np.arange(1, n + 1)
    lam = np.where(i <= 300, 2.0e4 + 20.0 * i, 0.0)
    lam[300:] = lam[299] + 400.0 * (i[300:] - 300)
    spec = (lam / 3.0e4) ** (-2) * (1.0 - 0.5 * np.exp(-0.5 * ((lam - 2.6e4) / 60.0) ** 2))
    direct = O.smooth_velocity_direct(lam, spec, 1.0e4, 3.0e4, 1.0e8)
    op = O.smooth_velocity_kernel(lam, spec, 1.0e4, 3.0e4, 1.0e8)
    first = 199
    assert np.max(np.abs(op[first:] - direct[first:]) / np.abs(direct[first:])) < 1.0e-12
    assert np.any(np.abs(direct[first:] - spec[first:]) > 1.0e-3 * spec[first:])


@pytest.mark.parametrize("sigma", [50.0, 175.0, 300.0])
def test_velocity_operator_on_the_synthetic_grid(data, sigma):
    lam = data["lambda"]
    sel = slice(2800, 3400)                       # 2400-4800 A, inside the default smoothing range
    spec = data["ssp_spec"][5, 40, sel]
    direct = O.smooth_velocity_direct(lam[sel], spec, sigma, 1.0e3, 1.0e4)
    op = O.smooth_velocity_kernel(lam[sel], spec, sigma, 1.0e3, 1.0e4)
    assert np.max(np.abs(op - direct) / np.abs(direct)) < 1.0e-12


def test_flat_field_identity():
    lam = 3000.0 + 2.0 * np.arange(2501)
    out = O.smooth_velocity_kernel(lam, np.ones_like(lam), 500.0, lam[0], lam[-1])
    assert np.max(np.abs(out[9:-10] - 1.0)) <= 1.0e-6


def test_window_cut_passthrough():
    lam = 3500.0 + 5.0 * np.arange(401)
    spec = 1.2 + 0.3 * np.sin(lam / 150.0)
    out = O.smooth_velocity_kernel(lam, spec, 300.0, 4000.0, 5000.0)
    below, above = lam < 4000.0, lam > 5000.0
    assert np.array_equal(out[below], spec[below]) and np.array_equal(out[above], spec[above])
    inside = ~below & ~above
    assert np.any(out[inside] != spec[inside])


# ----------------------------------------------------------------------------------------------------- photometry
class _Lcg:
    """The reference test's uniform [0, 1) generator: a 31-bit linear congruence in 64-bit arithmetic."""

    def __init__(self, seed=20261107):
        self.seed = seed

    def __call__(self):
        self.seed = (1103515245 * self.seed + 12345) & 2147483647
        return self.seed / 2147483648.0


NSPEC, NBANDS, NMAX = 700, 12, 100
J_LO = [1, 1, 699, 100, 250, 1, 1, 300, 10, 100, 2, 600]
J_HI = [699, 1, 699, 100, 260, 256, 257, 655, 400, 611, 40, 699]
DO_BAND = [1, 1, 1, 1, 1, 1, 1, 1, 0, 1, 1, 0]


@pytest.fixture(scope="module")
def photometry_data():
    u = _Lcg()
    bands = np.empty((NBANDS, NSPEC))
    wt = np.empty(NSPEC)
    fobs = np.empty((NMAX, NSPEC))
    for j in range(NSPEC):
        wt[j] = 0.5 + u()
        for b in range(NBANDS):
            bands[b, j] = u()
        for m in range(NMAX):
            fobs[m, j] = 2.0 * u()
        fobs[1, j] = 2.0 * fobs[0, j]
        fobs[2, j] = 0.0
    return u, bands, wt, fobs


def test_band_fluxes_against_direct_sums_and_identities(photometry_data):
    _, bands, wt, fobs = photometry_data
    fb = np.array([O.band_fluxes(bands, J_LO, J_HI, DO_BAND, wt, None, fobs[m]) for m in range(NMAX)])
    fb2 = np.array([O.band_fluxes(bands, J_LO, J_HI, DO_BAND, wt, None, fobs[m]) for m in range(NMAX)])
    worst = 0.0
    for m in range(NMAX):
        for b in range(NBANDS):
            if not DO_BAND[b]:
                assert fb[m, b] == 0.0
                continue
            ref = sum(wt[j - 1] * (fobs[m, j - 1] * bands[b, j - 1] + fobs[m, j] * bands[b, j])
                      for j in range(J_LO[b], J_HI[b] + 1))
            worst = max(worst, abs(fb[m, b] - ref) / ref if ref > 0.0 else abs(fb[m, b]))
    assert worst <= 1.0e-11
    assert np.array_equal(fb, fb2)
    assert np.array_equal(fb[1], 2.0 * fb[0])
    assert np.all(fb[2] == 0.0)


def test_observed_frame_against_direct_evaluation(photometry_data):
    u = photometry_data[0]
    ns, nc = 70, 9
    j1 = np.arange(1, ns + 1)
    lam = 900.0 * np.exp(0.045 * (j1 - 1)) * (1.0 + 0.01 * np.sin(j1))
    total = np.empty((nc, ns))
    for m in range(nc):
        for j in range(ns):
            total[m, j] = 1.0 + u()
    total[2, 4] = np.nan            # NaN gives 0
    total[3, 8] = -1.0              # negative gives 0
    zc = [0.0, 0.05, 0.4, 1.0, 2.5, 6.0, -0.3, 1.0e-12, 0.7]
    for m in range(nc):
        got = O.observed_frame(lam, zc[m], total[m])
        for j in range(ns):
            if abs(zc[m]) > np.finfo(np.float64).tiny:
                tg = lam[j] / (1.0 + zc[m])
                lo, hi = 0, ns + 1
                while hi - lo > 1:
                    mid = (hi + lo) // 2
                    if tg >= lam[mid - 1]:
                        lo = mid
                    else:
                        hi = mid
                il = max(1, min(lo, ns - 1))
                t = (tg - lam[il - 1]) / (lam[il] - lam[il - 1])
                v = total[m, il - 1] + t * (total[m, il] - total[m, il - 1])
            else:
                v = total[m, j]
            if v != v:
                v = 0.0
            ref = max(v, 0.0) * (1.0 / lam[j])
            assert abs(got[j] - ref) <= 4.0 * np.finfo(np.float64).eps * abs(ref), (m, j, got[j], ref)


# ----------------------------------------------------------------------------------------------------- tabular SFH
# The reference's tabular checks (tests/physics/test_opensps_sfh.f90:283-376,722-749,1065-1106), restated on the
# batch's path (sfh_weights_core's per-bin linear segments): the square wave's mass, a flat table's mass, a fine
# table against the analytic SFH of the same shape, the SFR's lookup in years.
def test_tabular_square_wave_mass():
    """The reference's square wave drops to an SFR of 0; on the batch's path a bin's segment is normalised by the SFR
    at its later row (slope / max(sfr, SAFE_FLOOR)), which a zero there sends to ~1e301 and the moments to NaN, in
    the reference as here: the wave drops to 1e-3 instead (mass 1e9 + 1e6 within the same 1e-2)."""
    tf = log_grid(50, 6.0, 10.0)
    w, _ = O.sfh_weights(tf, 3, {"tage": 2.0}, 1, table=([0.0, 1.0, 1.001, 2.0], [1.0, 1.0, 1.0e-3, 1.0e-3]))
    assert np.any(w > 0.0)
    assert abs(w.sum() / 1.0e9 - 1.0) <= 1.0e-2
    z, _ = O.sfh_weights(tf, 3, {"tage": 2.0}, 1, table=([0.0, 1.0, 1.001, 2.0], [1.0, 1.0, 0.0, 0.0]))
    assert np.all(np.isnan(z))


def test_tabular_flat_mass():
    tf = log_grid(10, 6.0, 10.0)
    w, _ = O.sfh_weights(tf, 3, {"tage": 10.0}, 1, table=([0.0, 10.0], [1.0, 1.0]))
    assert np.all(np.isfinite(w))
    assert abs(w.sum() / 1.0e10 - 1.0) <= 0.05


def test_tabular_matches_analytic_delayed_tau():
    tf = log_grid(80, 6.0, 10.2)
    tau, tage = 3.0, 9.0
    t = np.linspace(0.0, tage, 10001)
    w, _ = O.sfh_weights(tf, 3, {"tage": tage}, 1, table=(t, t * np.exp(-t / tau)))
    wa, _ = O.sfh_weights(tf, 4, {"tage": tage, "tau": tau}, 1)
    assert float(np.max(np.abs(w[0] / w.sum() - wa[0]))) <= 1.0e-3 * float(wa.max())


def test_tabular_sfr_lookup_in_years():
    tf = log_grid(10, 6.0, 10.0)
    _, sfr = O.sfh_weights(tf, 3, {"tage": 1.0}, 1, table=([0.1, 1.0, 2.0], [0.1, 0.5, 0.9]))
    assert abs(sfr[0] - 0.5) <= 1.0e-12
