"""Seeded synthetic inputs of the benchmark workloads (the batched-CSP configurations).

* ``mixed_csp``: the mixed-precision batched CSP workload: per model a weight matrix over 107 ages x 12
  metallicities (a Dirichlet(1) star formation history over the ages times a Gaussian in log Z with a centre
  uniform over the grid and a width uniform in 0.1-0.5 dex, normalised to one solar mass formed), diffuse dust
  tau_V uniform in 0-3 (power law, index -0.7), redshift uniform in 0-6 (with the IGM), velocity smoothing sigma
  uniform in 50-300 km/s; nebular lines and 40 filters on the context.
* ``adjoint_cotangents``: N(0, 1) cotangents on the 40 magnitudes and on 512 log-uniformly spaced spectral pixels.
"""
from __future__ import annotations

import numpy as np

NT, NZ = 107, 12


def mixed_csp(n: int, seed: int = 0, nt: int = NT, nz: int = NZ, out: np.ndarray | None = None):
    """Returns (wz, params): wz (n, nz, nt) float64 (written into ``out`` when given), params dict of (n,) arrays."""
    rng = np.random.default_rng(seed)
    logz = np.linspace(-2.0, 0.5, nz)
    wz = out if out is not None else np.empty((n, nz, nt))
    chunk = 8192
    for m0 in range(0, n, chunk):
        m1 = min(n, m0 + chunk)
        k = m1 - m0
        sfh = rng.dirichlet(np.ones(nt), size=k)
        cen = rng.uniform(-2.0, 0.5, size=k)
        sig = rng.uniform(0.1, 0.5, size=k)
        zw = np.exp(-0.5 * ((logz[None, :] - cen[:, None]) / sig[:, None]) ** 2)
        zw /= zw.sum(axis=1, keepdims=True)
        wz[m0:m1] = sfh[:, None, :] * zw[:, :, None]
    params = {"dust2": rng.uniform(0.0, 3.0, n), "zred": rng.uniform(0.0, 6.0, n),
              "sigma_smooth": rng.uniform(50.0, 300.0, n)}
    return wz, params


DEVICE_PARAM_ORDER = ("dust1", "dust2", "dust3", "dust_index", "dust1_index", "frac_nodust", "frac_obrun", "zred",
                      "igm_factor", "sigma_smooth", "dust_tesc", "mwr", "uvb")
DEVICE_PARAM_DEFAULTS = {"dust1": 0.0, "dust2": 0.0, "dust3": 0.0, "dust_index": -0.7, "dust1_index": -1.0,
                         "frac_nodust": 0.0, "frac_obrun": 0.0, "zred": 0.0, "igm_factor": 1.0, "sigma_smooth": 0.0,
                         "dust_tesc": 7.0, "mwr": 3.1, "uvb": 1.0}


def device_param_table(params: dict, n: int) -> np.ndarray:
    """The (n, 13) float64 per-model table of opensps_gb300_batch_device (column-major 13 x n)."""
    out = np.empty((n, len(DEVICE_PARAM_ORDER)))
    for i, k in enumerate(DEVICE_PARAM_ORDER):
        out[:, i] = np.broadcast_to(np.asarray(params.get(k, DEVICE_PARAM_DEFAULTS[k]), dtype=np.float64), (n,))
    return out


def adjoint_cotangents(n: int, nspec: int, nbands: int, seed: int = 4, nbins: int = 512):
    rng = np.random.default_rng(seed)
    mags_bar = rng.standard_normal((n, nbands)).astype(np.float32).astype(np.float64)
    spec_bar = np.zeros((n, nspec))
    pix = np.unique(np.round(np.linspace(0, nspec - 1, nbins)).astype(int))
    spec_bar[:, pix] = rng.standard_normal((n, pix.size)).astype(np.float32)
    return mags_bar, spec_bar
