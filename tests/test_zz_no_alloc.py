"""opensps_gb300_spec_mags_noalloc (through the C ABI) against the batch entry point's magnitudes of the same spectra.

The entry point serves callers that may not allocate device memory: a framework's custom-call handler gets its
buffers from a framework that has preallocated most of the device, where a cudaMalloc can fail and a cudaFree
synchronises the device under the framework's stream. Its scratch is a fixed device array of the library.

The batch (opensps_context_compute_csp_batch_grad with no cotangents) gives the magnitudes and leaves its FP32
spectra on the device (opensps_context_batch_spec_device); the no-allocation entry point forms the magnitudes of
those spectra at the same redshifts. Two calls in a row with different batches, each within the parity tests'
magnitude tolerance (1e-3 mag) and with the same NaN pattern (bands not computed); the first also against the FP64
oracle's magnitudes of the same models (1e-3 mag). A fresh process checks that the first call after the context's
set-up changes no device memory (its kernels and array were loaded by the set-up).
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import config3_inputs

pytestmark = pytest.mark.gpu

MAG_TOL = 1e-3
ROOT = Path(__file__).resolve().parent.parent


def _check_against_batch(ctx, torch, n, seed, mask=None, oracle_data=None):
    wz, params = config3_inputs(n, seed=seed)
    ref = ctx.csp_batch(params, ssp_weights_z=wz, spec=False)
    p, ns, nlast, nbytes = ctx.spec_device()
    assert nlast == n and nbytes == 4 and ns == ctx.nspec and p
    zred = torch.tensor(params["zred"], dtype=torch.float64, device="cuda")
    mags = torch.full((n, ctx.nbands), 7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.spec_mags_noalloc(n, p, zred.data_ptr(), mags.data_ptr(), sync=True)
    got = mags.cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(ref["mags"]))
    err = float(np.nanmax(np.abs(got - ref["mags"])))
    assert err <= MAG_TOL, err
    if oracle_data is not None:
        from oracle.oracle import Oracle
        want = Oracle(oracle_data, nbands=ctx.nbands).csp_batch(params, wz)["mags"]
        assert np.array_equal(np.isnan(got), np.isnan(want))
        err = float(np.nanmax(np.abs(got - want)))
        assert err <= MAG_TOL, err
    return got


def test_noalloc_mags_match_batch_entry_point(data, built_lib):
    torch = pytest.importorskip("torch")
    from libopensps_gb300.capi import Context
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    _check_against_batch(c, torch, 300, seed=501, oracle_data=data)
    # a second call, fewer models, on the scratch the first one left behind
    _check_against_batch(c, torch, 37, seed=502)
    c.close()


_FIRST_CALL = r"""
import sys, torch
sys.path.insert(0, sys.argv[1])
from libopensps_gb300.capi import Context
torch.cuda.set_device(0)
c = Context()                      # set-up: loads the entry point's kernels and its array
n = 256
spec = torch.rand((n, c.nspec), dtype=torch.float32, device="cuda") + 0.5
zred = torch.linspace(0.1, 5.0, n, dtype=torch.float64, device="cuda")
mags = torch.empty((n, c.nbands), dtype=torch.float64, device="cuda")
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info()[0]
c.spec_mags_noalloc(n, spec.data_ptr(), zred.data_ptr(), mags.data_ptr(), sync=True)
free1 = torch.cuda.mem_get_info()[0]
assert torch.isfinite(mags).all().item()
print("FREE", free0, free1)
c.close()
"""


def test_first_call_changes_no_device_memory(data, built_lib):
    """In a fresh process, the device's free memory is the same before and after the first call."""
    r = subprocess.run([sys.executable, "-c", _FIRST_CALL, str(ROOT)], capture_output=True, text=True,
                       timeout=300, env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FREE")][-1]
    free0, free1 = (int(x) for x in line.split()[1:])
    assert free0 == free1, (free0, free1)


def test_noalloc_rejects_batches_beyond_its_maximum(data, built_lib):
    from libopensps_gb300.capi import Context, OpenSPSError
    c = Context()
    with pytest.raises(OpenSPSError) as e:
        c.spec_mags_noalloc(65537, 16, 16, 16)   # rejected before any pointer is used
    assert e.value.status == 3 and "65536" in e.value.message
    c.close()
