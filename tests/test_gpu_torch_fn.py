"""The torch.autograd.Function over the batch: its gradients are the C API's reverse pass for the same cotangents
(bit for bit: the same library call), and unused outputs send no cotangent."""
import numpy as np
import pytest

from conftest import config3_inputs

pytestmark = pytest.mark.gpu


def test_autograd_matches_the_c_api_reverse_pass(data, built_lib):
    torch = pytest.importorskip("torch")
    from libopensps_gb300.capi import Context
    from libopensps_gb300.torch_fn import GRAD_ROWS, csp_batch
    c = Context()
    c.set_int("add_neb_emission", 1)
    c.set_int("add_igm_absorption", 1)
    n = 12
    wz, params = config3_inputs(n, seed=71)
    rng = np.random.default_rng(72)
    params = dict(params, dust1=rng.uniform(0.1, 1.0, n))
    w_t = torch.tensor(wz, dtype=torch.float64, device="cuda", requires_grad=True)
    p_t = {k: torch.tensor(v, dtype=torch.float64, device="cuda", requires_grad=True) for k, v in params.items()}
    mags, spec, mass, lbol = csp_batch(c, w_t, p_t)
    assert mags.device.type == "cuda" and spec.shape == (n, c.nspec)
    wm = torch.tensor(rng.standard_normal((n, c.nbands)), device="cuda")
    ws = torch.zeros((n, c.nspec), dtype=torch.float64, device="cuda")
    ws[:, ::37] = torch.tensor(rng.standard_normal((n, len(range(0, c.nspec, 37)))), device="cuda")
    loss = (torch.nan_to_num(mags) * wm).sum() + (spec * ws).sum() + 0.5 * lbol.sum()
    loss.backward()
    ref = c.csp_batch_grad(params, wz, mags_bar=wm.cpu().numpy(), spec_bar=ws.cpu().numpy(),
                           lbol_bar=np.full(n, 0.5), spec=False)
    np.testing.assert_array_equal(w_t.grad.cpu().numpy(), ref["weights_z_bar"])
    for k, v in p_t.items():
        np.testing.assert_array_equal(v.grad.cpu().numpy(), ref["params_bar"][:, GRAD_ROWS[k]])
    c.close()
