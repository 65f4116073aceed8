import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def data():
    from libopensps_gb300 import synthdata
    root = synthdata.default_root()
    synthdata.generate(root)
    os.environ["OPENSPS_DATA_HOME"] = str(root)
    return synthdata.load(root)


@pytest.fixture(scope="session")
def built_lib():
    from libopensps_gb300 import build
    return build.build()


def config3_inputs(n: int, seed: int = 3, nt: int = 107, nz: int = 12):
    """Config-3-style inputs: Dirichlet(1) SFH over ages x a Gaussian in log Z, dust, z, sigma (seeded)."""
    rng = np.random.default_rng(seed)
    logz = np.linspace(-2.0, 0.5, nz)
    sfh = rng.dirichlet(np.ones(nt), size=n)
    cen = rng.uniform(-2.0, 0.5, size=n)
    sig = rng.uniform(0.1, 0.5, size=n)
    zw = np.exp(-0.5 * ((logz[None, :] - cen[:, None]) / sig[:, None]) ** 2)
    zw /= zw.sum(axis=1, keepdims=True)
    wz = sfh[:, None, :] * zw[:, :, None]            # (n, nz, nt)
    params = {"dust2": rng.uniform(0.0, 3.0, n), "zred": rng.uniform(0.0, 6.0, n),
              "sigma_smooth": rng.uniform(50.0, 300.0, n)}
    return wz, params


def rel_err_spec(got: np.ndarray, ref: np.ndarray, floor: float = 1e-6) -> float:
    """Max relative error over the pixels above floor x the model's peak (the reference's exclusion rule)."""
    peak = np.max(np.abs(ref), axis=1, keepdims=True)
    mask = np.abs(ref) >= floor * peak
    err = np.abs(got - ref) / np.where(mask, np.abs(ref), 1.0)
    return float(np.max(np.where(mask, err, 0.0)))


def blend_at_logzsol(data, w, logzsol):
    """The oracle's metallicity blend (oracle.oracle.blend_at_logzsol)."""
    from oracle.oracle import blend_at_logzsol as blend
    return blend(data, w, logzsol)


def oracle_sfh_csp(oracle, data, sfh, params, table=None):
    """The oracle's batch for SFH parameters: its SFH weights, blended at logzsol, through its CSP; L_bol
    log-blended; the SFR per unit mass formed (the tabular SFHs, sfh 2 and 3: of table = (age [Gyr], sfr))."""
    from oracle.oracle import SFH_NAMES, sfh_weights
    n = len(np.atleast_1d(params["tage"]))
    w, sfr = sfh_weights(data["log_age"], sfh, params, n, table=table)
    logzsol = np.broadcast_to(np.asarray(params.get("logzsol", 0.0), dtype=np.float64), (n,))
    wz, lb = blend_at_logzsol(data, w, logzsol)
    out = oracle.csp_batch({k: v for k, v in params.items() if k not in SFH_NAMES and k != "logzsol"}, wz)
    out["lbol"] = np.log10(lb[:, 0])
    out["sfr"] = sfr
    out["w"] = w
    out["wz"] = wz
    return out
