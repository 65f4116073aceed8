"""opensps_gb300_spec_mags_noalloc (through the C ABI) against the batch entry point's magnitudes of the same spectra.

The batch (opensps_context_compute_csp_batch_grad with no cotangents) gives the magnitudes and leaves its FP32
spectra on the device (opensps_context_batch_spec_device); the no-allocation entry point forms the magnitudes of
those spectra at the same redshifts. Two calls in a row with different batches, each within the parity tests'
magnitude tolerance (1e-3 mag) and with the same NaN pattern (bands not computed).
"""
import numpy as np
import pytest

from conftest import config3_inputs

pytestmark = pytest.mark.gpu

MAG_TOL = 1e-3


def _check_against_batch(ctx, torch, n, seed, mask=None):
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
    return got


def test_noalloc_mags_match_batch_entry_point(data, built_lib):
    torch = pytest.importorskip("torch")
    from libopensps_gb300.capi import Context
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    _check_against_batch(c, torch, 300, seed=501)
    # a second call, fewer models, on the scratch the first one left behind
    _check_against_batch(c, torch, 37, seed=502)
    c.close()


def test_noalloc_rejects_batches_beyond_its_maximum(data, built_lib):
    from libopensps_gb300.capi import Context, OpenSPSError
    c = Context()
    with pytest.raises(OpenSPSError) as e:
        c.spec_mags_noalloc(65537, 16, 16, 16)   # rejected before any pointer is used
    assert e.value.status == 3 and "65536" in e.value.message
    c.close()
