"""The oracle's attenuation curves against the reference's own unit checks of them
(tests/physics/test_opensps_dust.f90:114-367, the same inputs and tolerances): the power law's normalisation and
slope, CCM89's regions, its near-UV continuity at 3030 A, far-UV clamp, bump scaling and infrared extension to 10 um,
Calzetti's junction at 0.63 um, V-band normalisation and extension beyond 0.12-2.2 um, Kriek & Conroy's no-tilt
baseline and no-bump slope, Reddy's UV clamp and 6000 A continuity.
"""
import numpy as np
import pytest

from oracle import oracle as O

EPS = 1.0e-6
SMALL_DELTA = 1.0e-4
LESS_SMALL_DELTA = 1.0e-2


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


def c(dust_type, lam, **kw):
    return O.dust_curve(dust_type, lam, **kw)


def test_power_law():
    assert c(0, [5500.0], dust_index=-0.7)[0] == 1.0
    assert np.all(np.abs(c(0, [1000.0, 2000.0, 5000.0], dust_index=0.0) - 1.0) <= EPS)
    assert abs(c(0, [2750.0], dust_index=-1.0)[0] - 2.0) <= EPS


def test_ccm89():
    kw = dict(mwr=3.1, uvb=1.0)
    r = c(1, [1e4 / 0.7, 1e4 / 2.0, 1e4 / 4.0, 1e4 / 6.5, 1e4 / 9.0], **kw)
    assert np.all(np.isfinite(r)) and np.all(r > 0.0)
    b = c(1, [3030.30, 3030.31], **kw)
    assert abs(b[0] - b[1]) <= SMALL_DELTA
    f = c(1, [800.0, 700.0], **kw)
    assert f[0] == f[1]
    assert c(1, [2175.0], mwr=3.1, uvb=1.0)[0] > c(1, [2175.0], mwr=3.1, uvb=0.0)[0]
    ir = c(1, [3.8e4, 8.0e4, 1.2e5], **kw)
    assert ir[0] > ir[1] > 0.0 and ir[2] == 0.0


def test_ccm89_bilinear_in_inverse_rv_and_uvb():
    """The reference's tables take the curve as T0 + T1 / R_V + T2 uvb + T3 uvb / R_V
    (attenuation_table_row, src/physics/opensps_csp_batch.f90:3525-3560)."""
    lam = np.geomspace(900.0, 9.0e4, 400)
    big = 1.0e30
    f00, f10 = c(1, lam, mwr=big, uvb=0.0), c(1, lam, mwr=1.0, uvb=0.0)
    f01, f11 = c(1, lam, mwr=big, uvb=1.0), c(1, lam, mwr=1.0, uvb=1.0)
    for rv, uvb in [(3.1, 1.0), (2.2, 0.4), (5.0, 1.7)]:
        want = f00 + (f10 - f00) / rv + (f01 - f00) * uvb + (f11 - f10 - f01 + f00) * uvb / rv
        np.testing.assert_allclose(c(1, lam, mwr=rv, uvb=uvb), want, rtol=1e-12, atol=1e-12)


def test_calzetti():
    b = c(2, [6300.000, 6300.001])
    assert abs(b[0] - b[1]) <= LESS_SMALL_DELTA
    assert abs(c(2, [5500.0])[0] - 1.0) <= 1.0e-3
    e = c(2, [21999.0, 22001.0, 1000.0, 25000.0, 35000.0, 1.0e5])
    assert abs(e[0] - e[1]) <= 1.0e-4
    assert e[2] > 2.0 and e[3] > 0.0 and e[4] == 0.0 and e[5] == 0.0


def test_kriek_conroy():
    lam = np.array([1500.0, 2175.0, 5500.0])
    drude = 0.85 * (lam * 350.0) ** 2 / ((lam ** 2 - 2175.0 ** 2) ** 2 + (lam * 350.0) ** 2)
    want = (c(2, lam) * 4.05 + drude) / 4.05
    assert np.all(np.abs(c(4, lam, dust_index=0.0) - want) <= EPS)
    nb = c(2, [2175.0])[0] * (2175.0 / 5500.0) ** 0.447
    assert abs(c(4, [2175.0], dust_index=0.447)[0] - nb) <= 5.0e-4
    assert np.array_equal(c(4, lam, dust_index=-0.2, uvb=0.0), c(4, lam, dust_index=-0.2, uvb=5.0))


def test_reddy():
    u = c(6, [1400.0, 1500.0])
    assert u[0] == u[1]
    b = c(6, [5999.999, 6000.000])
    assert abs(b[0] - b[1]) <= SMALL_DELTA
