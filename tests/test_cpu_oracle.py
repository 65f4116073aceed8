"""The FP64 oracle pinned against the reference's known answers and identities (CPU only).

* the IMF power-law bin integrals against the reference's 60-digit known-answer table
  (tests/golden/imf_powerlaw_bins.txt, made by the reference's own generator), within 1e-14 as the reference's
  test_powerlaw_bin_worst_cases;
* the IMF integrals of every analytic type (Salpeter, Chabrier, Kroupa, van Dokkum, Dave) against Simpson quadrature
  of the IMF's density, number and mass weighted, on the reference's intervals within its 1e-8
  (tests/physics/test_opensps_imf.f90:236-255,383-408, the density of get_imf_value src/physics/opensps_imf.f90:
  903-1010), and a wide lognormal bin equal to the sum of its narrow bins within 1e-13 (:344-381);
* identities the reference's batch tests use (tests/test_csp_batch.f90): with no dust, IGM, lines or smoothing the
  spectrum is sum_k w_k SSP_k; linearity in the weights; the velocity-smoothing rows sum to one; the distance term.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def olib():
    from oracle import oracle
    L = oracle.lib()
    L.oracle_powerlaw_bin.restype = C.c_double
    L.oracle_powerlaw_bin.argtypes = [C.c_double] * 4
    return L


def test_imf_powerlaw_bins_known_answers(olib):
    lines = (GOLDEN / "imf_powerlaw_bins.txt").read_text().splitlines()
    n = int(lines[1])
    rows = [tuple(float(x) for x in l.split()) for l in lines[2:2 + n]]
    assert len(rows) == n == 444
    worst = 0.0
    for alpha, lo, hi, ref in rows:
        got = olib.oracle_powerlaw_bin(alpha, 1.0, lo, hi)
        worst = max(worst, abs(got / ref - 1.0))
    assert worst <= 1e-14, worst


def _oracle(data, **kw):
    from oracle.oracle import Oracle
    return Oracle(data, **kw)


def _imf_density(t, m, vdmc=0.3, mdave=0.7, alpha=(1.3, 2.3, 2.3)):
    """get_imf_value (number per unit mass) restated for the test: the analytic types 0-4."""
    m = np.asarray(m, dtype=np.float64)
    if t == 0:
        return m ** -2.35
    if t == 1:
        lmc, s2 = np.log10(0.08), 0.69 ** 2
        high = np.exp(-lmc ** 2 / (2 * s2)) * m ** -2.3
        return np.where(m < 1.0, np.exp(-(np.log10(m) - lmc) ** 2 / (2 * s2)) / m, high)
    if t == 2:
        c2 = 0.5 ** (-alpha[0] + alpha[1])
        return np.where(m < 0.08, 0.0, np.where(m < 0.5, m ** -alpha[0], np.where(m < 1.0, c2 * m ** -alpha[1],
                                                                                 c2 * m ** -alpha[2])))
    if t == 3:
        br = 25.0 * vdmc
        low = 0.14 * (0.5 * br) ** -1.3 * np.exp(-(np.log10(m) - np.log10(vdmc)) ** 2 / (2 * 0.69 ** 2))
        return np.where(m <= br, low, 0.0443 * m ** -1.3) / m
    return np.where(m < 0.08, 0.0, np.where(m < mdave, m ** -alpha[0], mdave ** (-alpha[0] + alpha[1]) * m ** -alpha[1]))


@pytest.mark.parametrize("imf_type", [0, 1, 2, 3, 4])
def test_imf_integrals_match_quadrature(imf_type):
    from oracle.oracle import imf_integral
    a = {3: (0.3, 0.0, 0.0), 4: (1.3, 2.3, 0.7)}.get(imf_type, (1.3, 2.3, 2.3))
    for lo, hi in ((0.08, 0.3), (0.3, 0.7), (0.4, 2.0), (0.9, 1.1), (5.0, 120.0), (0.08, 120.0)):
        n = 200000
        u = np.log(lo) + (np.log(hi) - np.log(lo)) * np.arange(n + 1) / n
        m = np.exp(u)
        m[0], m[-1] = lo, hi
        c = np.where(np.arange(n + 1) % 2 == 1, 4.0, 2.0)
        c[0] = c[-1] = 1.0
        f = _imf_density(imf_type, m) * m
        du = (u[-1] - u[0]) / n
        for mw in (False, True):
            q = float(np.sum(c * f * (m if mw else 1.0))) * du / 3.0
            got = imf_integral(imf_type, lo, hi, mw, alpha=a)
            assert abs(got / q - 1.0) <= 1.0e-8, (imf_type, lo, hi, mw, got, q)


def _user_density(user, m):
    """get_imf_value case 5 restated for the test: each segment c_s m^-alpha_s on [lo_s, hi_s), c_s continuous at
    lo_s; overlapping segments add."""
    v, cu = np.zeros_like(m), 1.0
    for s, (lo, hi, al) in enumerate(user):
        if s:
            cu *= lo ** (-user[s - 1][2] + al)
        v += np.where((m >= lo) & (m < hi), cu * m ** -al, 0.0)
    return v


def test_user_imf_integral_matches_quadrature():
    """imf_integral case 5 (src/physics/opensps_imf.f90:287-305) against Simpson's rule between the segments'
    edges: a chain with a gap (0.4 - 0.5 M_sun empty) and a segment overlapping another (3 - 10 M_sun); with the rows
    of the reference's test imf.dat (Kroupa's slopes to 100 M_sun) it is the Kroupa integral."""
    from oracle.oracle import imf_integral, user_imf_integral
    user = [(0.1, 0.4, 1.1), (0.5, 2.0, 2.0), (2.0, 60.0, 2.6), (3.0, 10.0, 1.0)]
    edges = sorted({e for r in user for e in r[:2]})
    for lo, hi in ((0.08, 0.3), (0.2, 0.7), (0.45, 2.5), (2.5, 12.0), (0.05, 100.0), (0.1, 60.0)):
        cuts = [lo] + [e for e in edges if lo < e < hi] + [hi]
        for mw in (False, True):
            q = 0.0
            for a, b in zip(cuts[:-1], cuts[1:]):
                n = 20000
                u = np.log(a) + (np.log(b) - np.log(a)) * np.arange(n + 1) / n
                m = np.exp(u)
                m[0], m[-1] = a, b * (1.0 - 1e-15)   # (the piece's own side of its upper edge)
                c = np.where(np.arange(n + 1) % 2 == 1, 4.0, 2.0)
                c[0] = c[-1] = 1.0
                f = _user_density(user, m) * m * (m if mw else 1.0)
                q += float(np.sum(c * f)) * (u[-1] - u[0]) / n / 3.0
            got = user_imf_integral(user, lo, hi, mw)
            assert abs(got / q - 1.0) <= 1.0e-8, (lo, hi, mw, got, q)
    kroupa_rows = [(0.08, 0.5, 1.3), (0.5, 1.0, 2.3), (1.0, 100.0, 2.3)]
    for lo, hi in ((0.08, 100.0), (0.3, 0.7), (0.9, 40.0)):
        for mw in (False, True):
            assert user_imf_integral(kroupa_rows, lo, hi, mw) == pytest.approx(imf_integral(2, lo, hi, mw), rel=1e-14)


@pytest.mark.parametrize("imf_type", [1, 3])
def test_lognormal_wide_bin_is_the_sum_of_narrow_bins(imf_type):
    from oracle.oracle import imf_integral
    a = (0.13, 0.0, 0.0) if imf_type == 3 else (1.3, 2.3, 2.3)
    for lo, hi in ((0.1, 0.9), (0.2, 1.0), (0.5, 0.95), (30.0, 100.0), (1.0e-4, 1.0e-3)):
        e = lo * (hi / lo) ** (np.arange(4001) / 4000)
        for mw in (False, True):
            whole = imf_integral(imf_type, e[0], e[-1], mw, alpha=a)
            parts = sum(imf_integral(imf_type, e[k - 1], e[k], mw, alpha=a) for k in range(1, e.size))
            assert abs(parts / whole - 1.0) < 1.0e-13


def test_no_dust_sum_of_ssps(data):
    o = _oracle(data, add_neb=False, add_igm=False, smooth=False)
    rng = np.random.default_rng(0)
    wz = rng.dirichlet(np.ones(12 * 107), size=5).reshape(5, 12, 107)
    r = o.csp_batch({}, wz)
    ref = np.einsum("mzt,zts->ms", wz, data["ssp_spec"])
    np.testing.assert_allclose(r["spec"], ref, rtol=1e-12, atol=0)
    np.testing.assert_allclose(r["mass"], np.einsum("mzt,zt->m", wz, data["ssp_mass"]), rtol=1e-12)


def test_linear_in_weights(data):
    o = _oracle(data)
    rng = np.random.default_rng(1)
    w1 = rng.dirichlet(np.ones(1284), size=3).reshape(3, 12, 107)
    w2 = rng.dirichlet(np.ones(1284), size=3).reshape(3, 12, 107)
    p = {"dust2": np.array([0.3, 1.0, 2.0]), "zred": np.array([0.5, 2.0, 4.0]), "sigma_smooth": [100.0, 150.0, 250.0]}
    a, b, ab = o.csp_batch(p, w1), o.csp_batch(p, w2), o.csp_batch(p, w1 + 2.0 * w2)
    np.testing.assert_allclose(ab["spec"], a["spec"] + 2.0 * b["spec"], rtol=1e-11, atol=1e-300)


def test_velocity_rows_normalised(data):
    o = _oracle(data)
    for sigma in (50.0, 150.0, 300.0):
        i = int(np.searchsorted(o.lam, 5000.0))
        lo, coef = o.velocity_row(sigma, i)
        assert coef.size in (3, 5, 7, 9)
        assert lo == i - coef.size // 2
        assert abs(coef.sum() - 1.0) < 1e-14
        # nearly symmetric on a log-uniform grid (the trapezoid widths grow by e^dlnl per pixel)
        np.testing.assert_allclose(coef, coef[::-1], rtol=3e-3)


def test_distance_term(data):
    o = _oracle(data)
    assert o.distance_term(0.0) == 0.0
    d1, d2 = o.distance_term(1.0), o.distance_term(2.0)
    assert 43.0 < d1 < 44.5 and d2 > d1


def test_igm_only_below_lyman_alpha(data):
    o = _oracle(data, add_neb=False, smooth=False)
    rng = np.random.default_rng(2)
    wz = rng.dirichlet(np.ones(1284), size=2).reshape(2, 12, 107)
    a = o.csp_batch({"zred": np.array([3.0, 3.0])}, wz)
    b = _oracle(data, add_neb=False, add_igm=False, smooth=False).csp_batch({"zred": np.array([3.0, 3.0])}, wz)
    red = o.lam >= 1215.67
    np.testing.assert_array_equal(a["spec"][:, red], b["spec"][:, red])
    assert np.all(a["spec"][:, ~red] <= b["spec"][:, ~red])


def test_oracle_escaping_ionizing_light(data):
    """The oracle's gas absorption: with nebular emission and frac_obrun = 1 (fesc = 1) the ionizing pixels of the
    young and old sums equal those without nebular emission; with frac_obrun = 0 the nebular ages' ionizing light is
    gone (the sums there come from the older ages only)."""
    from oracle.oracle import Oracle
    n = 3
    rng = np.random.default_rng(951)
    wz = rng.dirichlet(np.ones(107 * 12), size=n).reshape(n, 12, 107)
    on, off = Oracle(data, nbands=20), Oracle(data, nbands=20, add_neb=False)
    whl = on.whlylim
    a = on.csp_batch({"frac_obrun": np.ones(n)}, wz, young=True)
    b = off.csp_batch({"frac_obrun": np.ones(n)}, wz, young=True)
    np.testing.assert_allclose(a["young"][:, :whl], b["young"][:, :whl], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(a["old"][:, :whl], b["old"][:, :whl], rtol=1e-13, atol=1e-300)
    c = on.csp_batch({"frac_obrun": np.zeros(n)}, wz, young=True)
    wo = wz.copy()
    wo[:, :, :on.nt_neb] = 0.0
    d = off.csp_batch({"frac_obrun": np.zeros(n)}, wo, young=True)
    np.testing.assert_allclose(c["young"][:, :whl] + c["old"][:, :whl], d["young"][:, :whl] + d["old"][:, :whl],
                               rtol=1e-13, atol=1e-300)


def test_oracle_nebular_continuum_closed_form(data):
    """The oracle's CLOUDY continuum loop (intervals, geometric steps, the normalisation by the largest weight) on a
    table constant over log Z, age and log U: the continuum is then 10^T(lambda) times sum_t C(t), C(t) the weights
    times |1 - frac_obrun| times the ionizing photon rate of each nebular age's SSPs (computed here directly)."""
    from oracle.oracle import Oracle
    lam = data["lambda"]
    T = -60.4 + 0.3 * np.sin(np.log(lam))
    neb = {"cont": np.broadcast_to(T, (7, 10, 11, lam.size)).copy(), "logz": np.linspace(-2.0, 0.2, 11),
           "lage": np.log10(np.array([0.5, 1, 2, 3, 4, 5, 6, 7, 8, 10]) * 1e6), "logu": np.linspace(-4, -1, 7)}
    n = 3
    rng = np.random.default_rng(5)
    wz = rng.dirichlet(np.ones(107), size=(n, 12)) / 12.0
    params = {"frac_obrun": np.array([0.0, 0.3, 0.9]), "gas_logz": rng.uniform(-2, 0.2, n),
              "gas_logu": rng.uniform(-4, -1, n)}
    on = Oracle(data, nbands=40, add_igm=False, smooth=False, nebular=neb).csp_batch(params, wz, young=True)
    off = Oracle(data, nbands=40, add_igm=False, smooth=False).csp_batch(params, wz, young=True)
    nn = on_nt = Oracle(data, nbands=40, nebular=neb).nt_neb
    assert nn == 35
    whl = int(np.searchsorted(lam, 912.0, side="right"))
    nu = 2.99792458e18 / lam[:whl]
    ssp = data["ssp_spec"]                           # (nz, nt, ns)
    q0 = 0.5 * np.sum(np.abs(np.diff(nu))[None, None, :] * (ssp[:, :nn, 1:whl] / nu[1:] + ssp[:, :nn, :whl - 1] / nu[:-1]),
                      axis=2) / 6.62607015e-27 * 3.828e33          # (nz, nn)
    for m in range(n):
        c = np.sum(wz[m, :, :nn] * q0, axis=0) * abs(1.0 - params["frac_obrun"][m])
        want = 10.0 ** T * c.sum()
        got = (on["young"][m] + on["old"][m]) - (off["young"][m] + off["old"][m])
        np.testing.assert_allclose(got, want, rtol=1e-10)
