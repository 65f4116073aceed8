"""Python driver of the FP64 CPU oracle (opensps_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the tests, the smoke check and the benchmark's CPU-baseline leg, never by
the product. It restates OpenSPS's batched CSP in FP64 on the CPU (see the C file for the reference routines each
function follows) on the same synthetic libraries the product reads.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
PAR_NAMES = ("dust1", "dust2", "dust3", "dust_index", "dust1_index", "frac_nodust", "frac_obrun", "zred",
             "igm_factor", "sigma_smooth", "dust_tesc", "duste_qpah", "duste_umin", "duste_gamma", "fagn", "agn_tau",
             "gas_logz", "gas_logu", "mwr", "uvb")
PAR_DEFAULTS = {"dust1": 0.0, "dust2": 0.0, "dust3": 0.0, "dust_index": -0.7, "dust1_index": -1.0,
                "frac_nodust": 0.0, "frac_obrun": 0.0, "zred": 0.0, "igm_factor": 1.0, "sigma_smooth": 0.0,
                "dust_tesc": 7.0, "duste_qpah": 3.5, "duste_umin": 1.0, "duste_gamma": 0.01, "fagn": 0.0,
                "agn_tau": 10.0, "gas_logz": 0.0, "gas_logu": -2.0, "mwr": 3.1, "uvb": 1.0}
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build() -> Path:
    srcs = [HERE / "opensps_oracle.c", HERE / "sfh_oracle.c", HERE / "ops_oracle.c"]
    if not LIB.exists() or any(LIB.stat().st_mtime < s.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


class _Grid(C.Structure):
    _fields_ = [("nspec", C.c_int), ("nt", C.c_int), ("nz", C.c_int), ("nbands", C.c_int),
                ("lam", _dp), ("log_age", _dp), ("basis", _dp), ("mass", _dp), ("lbol", _dp), ("bands", _dp),
                ("zt", _dp), ("dl", _dp), ("nline", C.c_int), ("line_lum", _dp), ("add_igm", C.c_int),
                ("smooth", C.c_int), ("min_wave_smooth", C.c_double), ("max_wave_smooth", C.c_double),
                ("nqpah", C.c_int), ("numin", C.c_int), ("qpah", _dp), ("umin", _dp), ("dustem", _dp),
                ("ntau", C.c_int), ("agn_tau", _dp), ("agn_spec", _dp), ("ssp_ion", _dp), ("nt_neb", C.c_int),
                ("whlylim", C.c_int), ("neb_cont", _dp), ("neb_logz", _dp), ("neb_lage", _dp), ("neb_logu", _dp),
                ("dust_type", C.c_int), ("att_curve", _dp)]


class _OpsT(C.Structure):
    _fields_ = [("nspec", C.c_int), ("nt", C.c_int), ("nz", C.c_int), ("npt", C.c_int), ("ntempl", C.c_int),
                ("lib", C.POINTER(C.c_float)), ("mini", _dp), ("idx", C.POINTER(C.c_int)), ("coef", _dp),
                ("mcur", _dp), ("lum", _dp), ("lower_bound", C.c_double), ("lim_lo", C.c_double),
                ("lim_hi", C.c_double), ("imf_type", C.c_int), ("nuser", C.c_int), ("user", _dp)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        _lib.oracle_imf_integral.restype = C.c_double
        _lib.oracle_imf_integral.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_int]
        _lib.oracle_user_imf_integral.restype = C.c_double
        _lib.oracle_user_imf_integral.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_int]
        _lib.oracle_dust_curve.restype = C.c_double
        _lib.oracle_dust_curve.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
        _lib.oracle_find_interval.restype = C.c_int
        _lib.oracle_find_interval.argtypes = [_dp, C.c_int, C.c_double]
        _lib.oracle_line_basis.argtypes = [C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, _dp, C.c_double, _dp, _dp]
        _lib.oracle_neb_ranges.argtypes = [C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, _ip, _ip]
        _lib.oracle_cosmo_table.argtypes = [C.c_double, C.c_double, C.c_double, _dp, _dp]
        _lib.oracle_distance_term.restype = C.c_double
        _lib.oracle_distance_term.argtypes = [_dp, _dp, C.c_double]
        _lib.oracle_igm_pixel_terms.argtypes = [C.c_double, _dp]
        _lib.oracle_igm_z_terms.argtypes = [C.c_double, _dp]
        _lib.oracle_velocity_row.restype = C.c_int
        _lib.oracle_velocity_row.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double, C.c_int,
                                             C.POINTER(C.c_int), _dp, C.c_int]
        _lib.oracle_csp_batch.argtypes = [C.POINTER(_Grid), C.c_int, _dp, _dp] + [_dp] * 8
        _lib.oracle_npar.restype = C.c_int
        _lib.oracle_expi.restype = C.c_double
        _lib.oracle_expi.argtypes = [C.c_double]
        _lib.oracle_sfh_batch.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        _lib.oracle_csp_from_parts.argtypes = [C.POINTER(_Grid), C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        _lib.oracle_ops_csp.argtypes = [C.POINTER(_OpsT), C.c_int, _dp, _dp, C.c_int, _dp, _dp, _dp, _dp]
        _lib.oracle_kroupa_integral.restype = C.c_double
        _lib.oracle_kroupa_integral.argtypes = [_dp, C.c_double, C.c_double, C.c_int]
        _lib.oracle_abs_mag_zeropoint_log.restype = C.c_double
        _lib.oracle_lum_distance.restype = C.c_double
        _lib.oracle_lum_distance.argtypes = [C.c_double] * 4
        _lib.oracle_observed_frame.argtypes = [C.c_int, _dp, C.c_double, _dp, _dp]
        _lib.oracle_band_fluxes.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip, _ip, _dp, _dp, _dp, _dp]
        _lib.oracle_ssp_weights_raw.argtypes = [_dp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double,
                                                C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                                C.c_int, C.c_int, C.c_int, _dp]
        _lib.oracle_sfh_props.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_double, _dp]
        _lib.oracle_sfh_tab_batch.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_int, _dp, _dp, _dp, _dp]
        _lib.oracle_sfh_tab_sfr.restype = C.c_double
        _lib.oracle_sfh_tab_sfr.argtypes = [C.c_double, C.c_int, _dp, _dp]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


SFH_NAMES = ("tage", "tau", "const", "fburst", "tburst", "sf_start", "sf_trunc", "sf_slope")
SFH_DEFAULTS = {"tage": 0.0, "tau": 1.0, "const": 0.0, "fburst": 0.0, "tburst": 11.0, "sf_start": 0.0,
                "sf_trunc": 0.0, "sf_slope": 0.0}


def sfh_weights(log_age: np.ndarray, sfh: int, params: dict, n: int, table=None):
    """The SFH weights over the ages (n, nt) and the current SFR per unit mass formed (n,) of SFH type sfh (0, 1, 4,
    5) for per-model parameters, or of the tabular SFHs (sfh 2, 3) for table = (age [Gyr], sfr [M_sun / yr]) at the
    models' tage: masses formed and the table's SFR (sfh_oracle.c)."""
    tf = np.ascontiguousarray(log_age, dtype=np.float64)
    if sfh in (2, 3):
        tt = np.ascontiguousarray(np.asarray(table[0], dtype=np.float64) * 1.0e9)
        ts = np.ascontiguousarray(table[1], dtype=np.float64)
        tage = np.ascontiguousarray(np.broadcast_to(np.asarray(params["tage"], dtype=np.float64), (n,)))
        w = np.empty((n, tf.size))
        sfr = np.empty(n)
        lib().oracle_sfh_tab_batch(_p(tf), tf.size, n, _p(tage), tt.size, _p(tt), _p(ts), _p(w), _p(sfr))
        return w, sfr
    p = np.empty((n, len(SFH_NAMES)))
    for i, k in enumerate(SFH_NAMES):
        p[:, i] = np.broadcast_to(np.asarray(params.get(k, SFH_DEFAULTS[k]), dtype=np.float64), (n,))
    w = np.empty((n, tf.size))
    sfr = np.empty(n)
    lib().oracle_sfh_batch(_p(tf), tf.size, int(sfh), n, _p(p), _p(w), _p(sfr))
    return w, sfr


def blend_at_logzsol(data: dict, w: np.ndarray, logzsol: np.ndarray):
    """Weights over ages (n, nt) blended between the two metallicities bracketing logzsol (not clamped), and the
    log-blended L_bol (total, young ages <= 7.0 dex, old) of the model_sums MSUMS_BLEND form
    (src/physics/opensps_csp_batch.f90:2129-2176, the batch's ssp_weights with logzsol)."""
    n, nt = w.shape
    lz = np.log10(data["zlegend"] / 0.0142)
    nz = lz.size
    wz = np.zeros((n, nz, nt))
    lb = np.zeros((n, 3))
    young = data["log_age"] <= 7.0
    for m in range(n):
        zlo = min(max(np.searchsorted(lz, logzsol[m], side="right") - 1, 0), nz - 2)
        dz = (logzsol[m] - lz[zlo]) / (lz[zlo + 1] - lz[zlo])
        wz[m, zlo] = (1 - dz) * w[m]
        wz[m, zlo + 1] = dz * w[m]
        lk = np.where(w[m] > 0, w[m] * 10.0 ** ((1 - dz) * data["ssp_lbol"][zlo] + dz * data["ssp_lbol"][zlo + 1]), 0.0)
        lb[m] = [lk.sum(), lk[young].sum(), lk[~young].sum()]
    return wz, lb


def lum_distance(h0: float, om0: float, ol0: float, z: float) -> float:
    """The luminosity distance [pc] of the oracle's cosmology table (get_luminosity_distance's trapezoid)."""
    return lib().oracle_lum_distance(float(h0), float(om0), float(ol0), float(z))


def observed_frame(lam: np.ndarray, z: float, spec: np.ndarray) -> np.ndarray:
    """observed_frame_z for one rest-frame spectrum: the observed f_lambda / lambda at the grid's pixels."""
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    fin = np.ascontiguousarray(spec, dtype=np.float64)
    out = np.empty_like(lam)
    lib().oracle_observed_frame(lam.size, _p(lam), float(z), _p(fin), _p(out))
    return out


def band_fluxes(bands: np.ndarray, jlo, jhi, do_band, wt: np.ndarray | None, lam: np.ndarray | None,
                fobs: np.ndarray) -> np.ndarray:
    """band_fluxes for one model: bands (nb, ns), 1-based supports jlo / jhi, do_band flags, weights wt (ns) or the
    trapezoid's from lam."""
    b = np.ascontiguousarray(bands, dtype=np.float64)
    nb, ns = b.shape
    jl = np.ascontiguousarray(jlo, dtype=np.int32)
    jh = np.ascontiguousarray(jhi, dtype=np.int32)
    db = np.ascontiguousarray(do_band, dtype=np.int32)
    w = None if wt is None else np.ascontiguousarray(wt, dtype=np.float64)
    lm = None if lam is None else np.ascontiguousarray(lam, dtype=np.float64)
    f = np.ascontiguousarray(fobs, dtype=np.float64)
    out = np.empty(nb)
    ip = C.POINTER(C.c_int)
    lib().oracle_band_fluxes(ns, nb, _p(b), jl.ctypes.data_as(ip), jh.ctypes.data_as(ip), db.ctypes.data_as(ip),
                             _p(w), _p(lm), _p(f), _p(out))
    return out


def ssp_weights_raw(log_t: np.ndarray, sfh_type: int, tage: float, tau: float, idx_min: int, idx_max: int,
                    tiny_logt: float = 0.0, tq: float = 0.0, tb: float = 0.0, trunc: float = 0.0, slope: float = 0.0,
                    t0: float = 0.0, simha: bool = False) -> np.ndarray:
    """compute_ssp_weights alone: the hat-kernel mass of SFH type -1/0/1/4/5 (times in years, slope per year in
    lookback time; simha integrates over [t0, tq]) on the log-age nodes."""
    tf = np.ascontiguousarray(log_t, dtype=np.float64)
    w = np.empty(tf.size)
    lib().oracle_ssp_weights_raw(_p(tf), tf.size, float(tiny_logt), int(sfh_type), float(tage), float(tau), float(tq),
                                 float(tb), float(trunc), float(slope), float(t0), int(bool(simha)), int(idx_min),
                                 int(idx_max), _p(w))
    return w


def sfh_properties(log_age: np.ndarray, sfh: int, params: dict, age: float):
    """get_sfh_properties_at_age at age (Gyr) for one model: the mass fraction formed, the normalised SFR (per Gyr,
    before the unit change and the division by the mass fraction) and the linear (ramp) mass fraction of sfh 5."""
    tf = np.ascontiguousarray(log_age, dtype=np.float64)
    p = np.array([float(params.get(k, SFH_DEFAULTS[k])) for k in SFH_NAMES])
    out = np.empty(3)
    lib().oracle_sfh_props(_p(tf), tf.size, int(sfh), _p(p), float(age), _p(out))
    return float(out[0]), float(out[1]), float(out[2])


def smooth_velocity_direct(lam: np.ndarray, spec: np.ndarray, sigma: float, minl: float, maxl: float) -> np.ndarray:
    """The velocity smoothing as a direct integral (convolve_variable_resolution, the path of smooth_velocity,
    src/spectra/opensps_smoothing.f90:132-139,365-546): per pixel inside [minl, maxl] the +-4 sigma window found by the
    same hunting search, weights exp(-(ln lam_i - ln lam_j)^2 / (2 (sigma/c)^2)) / lam_j, the trapezoid integrals of
    weights and weighted flux over the window, their ratio. Pixels outside, or with fewer than two window pixels,
    keep their value. Plain loops: small grids only."""
    lam = np.asarray(lam, dtype=np.float64)
    spec = np.asarray(spec, dtype=np.float64)
    n = lam.size
    out = spec.copy()
    if n < 2 or sigma <= np.finfo(np.float64).tiny:
        return out
    c_kms = 2.99792458e18 * 1.0e-13
    sig_beta = sigma / c_kms
    inv2 = 0.5 * (1.0 / sig_beta) ** 2
    fb, fr = np.exp(-4.0 * sig_beta), np.exp(4.0 * sig_beta)
    loglam = np.log(lam)
    dl = lam[1:] - lam[:-1]
    il = ih = 0                                       # 0-based window bounds
    for i in range(n):
        if lam[i] < minl or lam[i] > maxl:
            continue
        vl, vh = lam[i] * fb, lam[i] * fr
        while il > 0 and lam[il] > vl:
            il -= 1
        while il < n - 1 and lam[il] < vl:
            il += 1
        if il > 0 and lam[il] > vl:
            il -= 1
        if ih < il:
            ih = il
        while ih > il and lam[ih] > vh:
            ih -= 1
        while ih < n - 1 and lam[ih] < vh:
            ih += 1
        if ih - il + 1 < 2:
            continue
        w = np.exp(-inv2 * (loglam[i] - loglam[il:ih + 1]) ** 2) / lam[il:ih + 1]
        tw = 0.5 * np.dot(w[:-1] + w[1:], dl[il:ih])
        if tw <= np.finfo(np.float64).tiny:
            continue
        wf = w * spec[il:ih + 1]
        out[i] = 0.5 * np.dot(wf[:-1] + wf[1:], dl[il:ih]) / tw
    return out


def smooth_velocity_kernel(lam: np.ndarray, spec: np.ndarray, sigma: float, minl: float, maxl: float) -> np.ndarray:
    """The same smoothing through the oracle's sparse velocity operator (build_velocity_kernel /
    apply_velocity_kernel, opensps_smoothing.f90:553-651): rows of normalised trapezoid coefficients."""
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    spec = np.asarray(spec, dtype=np.float64)
    out = spec.copy()
    lo = C.c_int(0)
    coef = np.empty(lam.size)
    for i in range(lam.size):
        nt = lib().oracle_velocity_row(lam.size, _p(lam), float(sigma), float(minl), float(maxl), i, C.byref(lo),
                                       _p(coef), lam.size)
        if nt > 0:
            out[i] = np.dot(coef[:nt], spec[lo.value:lo.value + nt])
    return out


def expi(x: float) -> float:
    return lib().oracle_expi(float(x))


def dust_curve(dust_type: int, lam, dust_index: float = -0.7, mwr: float = 3.1, uvb: float = 1.0) -> np.ndarray:
    """The oracle's attenuation curve A_lambda / A_V (dust_type 0, 1, 2, 4, 6) at the wavelengths lam [A]."""
    L = lib()
    lam = np.atleast_1d(np.asarray(lam, dtype=np.float64))
    return np.array([L.oracle_dust_curve(int(dust_type), float(x), float(dust_index), float(mwr), float(uvb))
                     for x in lam])


class Oracle:
    """The oracle over one synthetic library and filter set, with a context's batch-wide settings."""

    def __init__(self, data: dict, nbands: int = 40, add_neb: bool = True, add_igm: bool = True,
                 smooth: bool = True, min_wave_smooth: float = 1.0e3, max_wave_smooth: float = 1.0e4,
                 line_sigma: float = 0.0, h0: float = 72.0, om0: float = 0.27, ol0: float = 0.73,
                 dust_emission: dict | None = None, agn: dict | None = None, nebular: dict | None = None,
                 dust_type: int = 0, att_curve: np.ndarray | None = None):
        L = lib()
        self.d = data
        self.lam = np.ascontiguousarray(data["lambda"])
        self.log_age = np.ascontiguousarray(data["log_age"])
        ns, nt, nz = self.lam.size, self.log_age.size, data["zlegend"].size
        self.nspec, self.nt, self.nz = ns, nt, nz
        ssp = np.ascontiguousarray(data["ssp_spec"])          # (nz, nt, ns)
        self.line_lum = np.ascontiguousarray(data["line_lum"])
        nl = data["line_lambda"].size
        if add_neb:
            self.basis = np.empty_like(ssp)
            L.oracle_line_basis(ns, nt, nz, _p(self.lam), nl, _p(np.ascontiguousarray(data["line_lambda"])),
                                _p(self.line_lum), float(line_sigma), _p(ssp), _p(self.basis))
        else:
            self.basis = ssp
        self.mass = np.ascontiguousarray(data["ssp_mass"])
        self.lbol = np.ascontiguousarray(data["ssp_lbol"])
        self.bands = np.ascontiguousarray(data[f"filters_{nbands}"])
        self.nbands = nbands
        self.zt, self.dl = np.empty(500), np.empty(500)
        L.oracle_cosmo_table(h0, om0, ol0, _p(self.zt), _p(self.dl))
        g = _Grid()
        g.nspec, g.nt, g.nz, g.nbands = ns, nt, nz, nbands
        g.lam, g.log_age, g.basis = _p(self.lam), _p(self.log_age), _p(self.basis)
        g.mass, g.lbol, g.bands = _p(self.mass), _p(self.lbol), _p(self.bands)
        g.zt, g.dl = _p(self.zt), _p(self.dl)
        g.nline = nl
        g.line_lum = _p(self.line_lum) if add_neb else None
        g.ssp_ion = None
        if add_neb:
            self._ssp = ssp
            a, b = C.c_int(0), C.c_int(0)
            L.oracle_neb_ranges(ns, nt, nz, _p(self.lam), nl, _p(self.line_lum), C.byref(a), C.byref(b))
            g.ssp_ion, g.nt_neb, g.whlylim = _p(ssp), a.value, b.value
            self.nt_neb, self.whlylim = a.value, b.value
        g.add_igm, g.smooth = int(add_igm), int(smooth)
        g.dust_type = int(dust_type)
        # dust_type 3, 5: the table lookup's curve on the grid (nspec)
        self._att = None if att_curve is None else np.ascontiguousarray(att_curve, dtype=np.float64)
        g.att_curve = _p(self._att) if self._att is not None else None
        g.min_wave_smooth, g.max_wave_smooth = min_wave_smooth, max_wave_smooth
        g.dustem = None
        if dust_emission is not None:
            # the Draine & Li grid (synth_dust.load()): templates (2 numin, nqpah, nspec) C order
            self._dq = np.ascontiguousarray(dust_emission["qpah"], dtype=np.float64)
            self._du = np.ascontiguousarray(dust_emission["umin"], dtype=np.float64)
            self._dt = np.ascontiguousarray(dust_emission["dustem"], dtype=np.float64)
            g.nqpah, g.numin = self._dq.size, self._du.size
            g.qpah, g.umin, g.dustem = _p(self._dq), _p(self._du), _p(self._dt)
        g.agn_spec = None
        if agn is not None:
            # the AGN torus templates (synth_dust.load_agn()): (ntau, nspec)
            self._at = np.ascontiguousarray(agn["tau"], dtype=np.float64)
            self._as = np.ascontiguousarray(agn["agnspec"], dtype=np.float64)
            g.ntau, g.agn_tau, g.agn_spec = self._at.size, _p(self._at), _p(self._as)
        g.neb_cont = None
        if nebular is not None and add_neb:
            # the CLOUDY continuum (stdformat.nebular()); its last age sets the nebular ages:
            # nt_neb = find_interval(time_full, nebem_age(NEBNAGE)) (batch_nebular_indices :1643-1644)
            self._nc = np.ascontiguousarray(nebular["cont"], dtype=np.float64)
            self._nz = np.ascontiguousarray(nebular["logz"], dtype=np.float64)
            self._na = np.ascontiguousarray(nebular["lage"], dtype=np.float64)
            self._nu = np.ascontiguousarray(nebular["logu"], dtype=np.float64)
            g.neb_cont, g.neb_logz, g.neb_lage, g.neb_logu = _p(self._nc), _p(self._nz), _p(self._na), _p(self._nu)
            k = L.oracle_find_interval(_p(self.log_age), nt, float(self._na[-1]))
            g.nt_neb = max(0, min(k, nt))
            self.nt_neb = g.nt_neb
        self.grid = g
        self.nline = nl

    def pack_params(self, params: dict, n: int) -> np.ndarray:
        out = np.empty((n, len(PAR_NAMES)))
        for i, k in enumerate(PAR_NAMES):
            out[:, i] = np.broadcast_to(np.asarray(params.get(k, PAR_DEFAULTS[k]), dtype=np.float64), (n,))
        return np.ascontiguousarray(out)

    def csp_batch(self, params: dict, wz: np.ndarray, spec=True, young=False, fband=False, emlines=False) -> dict:
        """wz: (n, nz, nt) weights over metallicities and ages."""
        wz = np.ascontiguousarray(wz, dtype=np.float64)
        n = wz.shape[0]
        par = self.pack_params(params, n)
        out = {"mags": np.empty((n, self.nbands)), "mass": np.empty(n), "lbol": np.empty(n)}
        if spec: out["spec"] = np.empty((n, self.nspec))
        if young:
            out["young"] = np.empty((n, self.nspec))
            out["old"] = np.empty((n, self.nspec))
        if fband: out["fband"] = np.empty((n, self.nbands))
        if emlines: out["emlines"] = np.empty((n, self.nline))
        lib().oracle_csp_batch(C.byref(self.grid), n, _p(wz), _p(par), _p(out.get("spec")), _p(out["mags"]),
                               _p(out["mass"]), _p(out["lbol"]), _p(out.get("emlines")), _p(out.get("young")),
                               _p(out.get("old")), _p(out.get("fband")))
        return out

    def csp_from_parts(self, params: dict, young: np.ndarray, old: np.ndarray, lsum: np.ndarray | None = None) -> dict:
        """The batch's stages after the age sums (attenuation, dust emission, IGM, AGN, smoothing, magnitudes) from
        given young and old spectra (n, nspec); lsum (n,): the models' linear L_bol (the AGN's scale)."""
        y = np.ascontiguousarray(young, dtype=np.float64)
        o = np.ascontiguousarray(old, dtype=np.float64)
        n = y.shape[0]
        par = self.pack_params(params, n)
        ls = None if lsum is None else np.ascontiguousarray(lsum, dtype=np.float64)
        out = {"mags": np.empty((n, self.nbands)), "spec": np.empty((n, self.nspec)), "fband": np.empty((n, self.nbands))}
        lib().oracle_csp_from_parts(C.byref(self.grid), n, _p(y), _p(o), _p(par), _p(ls), _p(out["spec"]),
                                    _p(out["mags"]), _p(out["fband"]))
        return out

    def velocity_row(self, sigma: float, i: int, minl: float = 1.0e3, maxl: float = 1.0e4):
        lo, coef = C.c_int(0), np.zeros(64)
        nt = lib().oracle_velocity_row(self.nspec, _p(self.lam), sigma, minl, maxl, i, C.byref(lo), _p(coef), 64)
        return lo.value, coef[:nt].copy()

    def distance_term(self, z: float) -> float:
        return lib().oracle_distance_term(_p(self.zt), _p(self.dl), z)


class OpsOracle:
    """The SSP operator applied to per-model IMFs (ops_oracle.c) over the operator dataset (synth_ops): imf_type 2
    Kroupa (alpha per model: imf1-3), 0 Salpeter, 1 Chabrier, 3 van Dokkum (alpha[:, 0] = vdmc), 4 Dave (alpha =
    imf1, imf2, mdave), 5 the user's segments (user: rows of lower mass, upper mass, slope; the limits become its
    first lower and last upper mass). lower_bound: the lower edge of each age's first bin (the dataset's when None)."""

    def __init__(self, ops: dict, lim_lo: float = 0.08, lim_hi: float = 120.0, imf_type: int = 2, user=None,
                 lower_bound=None):
        self.ops = ops
        man = ops["manifest"]
        self.nspec, self.nt, self.nz, self.npt, self.ntempl = man["nspec"], man["nt"], man["nz"], man["npt"], man["ntempl"]
        self._keep = [np.ascontiguousarray(ops[k]) for k in ("lib", "mini", "idx", "coef", "mcur", "lum")]
        lb, mi, ix, co, mc, lu = self._keep
        t = _OpsT()
        t.nspec, t.nt, t.nz, t.npt, t.ntempl = self.nspec, self.nt, self.nz, self.npt, self.ntempl
        t.lib = lb.ctypes.data_as(C.POINTER(C.c_float))
        t.mini, t.coef, t.mcur, t.lum = _p(mi), _p(co), _p(mc), _p(lu)
        t.idx = ix.ctypes.data_as(C.POINTER(C.c_int))
        t.lower_bound, t.lim_lo, t.lim_hi = man["imf_lower_bound"] if lower_bound is None else lower_bound, lim_lo, lim_hi
        t.imf_type = int(imf_type)
        if user is not None:
            u = np.ascontiguousarray(user, dtype=np.float64).reshape(-1, 3)
            self._keep.append(u)
            t.nuser, t.user = u.shape[0], _p(u)
            if imf_type == 5:
                t.lim_lo, t.lim_hi = float(u[0, 0]), float(u[-1, 1])
        self.t = t

    def parts(self, alpha: np.ndarray, wz: np.ndarray, itesc: int):
        """alpha (n, 3) Kroupa slopes, wz (n, nz, nt): young, old (n, nspec), mass and linear L_bol (n,)."""
        a = np.ascontiguousarray(alpha, dtype=np.float64)
        w = np.ascontiguousarray(wz, dtype=np.float64)
        n = a.shape[0]
        y, o = np.empty((n, self.nspec)), np.empty((n, self.nspec))
        mass, ls = np.empty(n), np.empty(n)
        lib().oracle_ops_csp(C.byref(self.t), n, _p(a), _p(w), int(itesc), _p(y), _p(o), _p(mass), _p(ls))
        return y, o, mass, ls


def imf_integral(imf_type: int, m1: float, m2: float, mass_weighted: bool, alpha=(1.3, 2.3, 2.3)) -> float:
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    return lib().oracle_imf_integral(int(imf_type), _p(a), float(m1), float(m2), int(mass_weighted))


def user_imf_integral(user, m1: float, m2: float, mass_weighted: bool) -> float:
    u = np.ascontiguousarray(user, dtype=np.float64).reshape(-1, 3)
    return lib().oracle_user_imf_integral(u.shape[0], _p(u), float(m1), float(m2), int(mass_weighted))


def kroupa_integral(alpha, m1: float, m2: float, mass_weighted: bool) -> float:
    a = np.ascontiguousarray(alpha, dtype=np.float64)
    return lib().oracle_kroupa_integral(_p(a), float(m1), float(m2), int(mass_weighted))
