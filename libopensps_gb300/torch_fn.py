"""torch.autograd.Function over the batched CSP: the forward is compute_csp_batch_grad with no cotangents, the
backward is compute_csp_batch_grad_rows with the incoming cotangents of the magnitudes and spectra (the reverse pass
recomputes the forward on the device, as OpenSPS's batch_backward does).

    from libopensps_gb300.capi import Context
    from libopensps_gb300.torch_fn import csp_batch
    mags, spec, mass, lbol = csp_batch(ctx, wz, {"dust2": d2, "zred": z})   # wz (n, nz, nt), values (n,) tensors
    loss = (mags * w).sum() + (spec * v).sum()
    loss.backward()                                                      # wz.grad, d2.grad, z.grad

Inputs may live on any device; the C API takes host arrays, so they are copied to the host (float64) and the
outputs come back on the device of ``wz``. Parameters without a gradient row on this path (see
``GRAD_ROWS``) receive a zero gradient, as the library writes them.
"""
from __future__ import annotations

import numpy as np
import torch

from .capi import Context

# params_bar rows of the per-model parameters this path varies (opensps.h OPENSPS_BGRAD_*)
GRAD_ROWS = {"dust1": 1, "dust2": 2, "dust3": 3, "dust_index": 4, "dust1_index": 5, "frac_obrun": 6,
             "frac_nodust": 7, "zred": 22, "sigma_smooth": 23, "igm_factor": 32}


def _host(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


class _CSPBatch(torch.autograd.Function):
    @staticmethod
    def forward(fctx, context: Context, names: tuple, wz: torch.Tensor, *values: torch.Tensor):
        fctx.set_materialize_grads(False)   # outputs the loss does not use get no cotangent (None)
        w = _host(wz)
        params = {k: _host(v) for k, v in zip(names, values)}
        out = context.csp_batch(params, ssp_weights_z=w)
        fctx.context, fctx.names, fctx.w, fctx.params = context, names, w, params
        fctx.device = wz.device
        dev = wz.device
        return tuple(torch.from_numpy(out[k]).to(dev) for k in ("mags", "spec", "mass", "lbol"))

    @staticmethod
    def backward(fctx, g_mags, g_spec, g_mass, g_lbol):
        cot = {}
        for key, g in (("mags_bar", g_mags), ("spec_bar", g_spec), ("mass_bar", g_mass), ("lbol_bar", g_lbol)):
            cot[key] = None if g is None else _host(g)
        need_w = fctx.needs_input_grad[2]
        res = fctx.context.csp_batch_grad(fctx.params, fctx.w, weights_z_bar=need_w, spec=False, **cot)
        dev = fctx.device
        g_w = torch.from_numpy(res["weights_z_bar"]).to(dev) if need_w else None
        g_vals = []
        for i, k in enumerate(fctx.names):
            if not fctx.needs_input_grad[3 + i]:
                g_vals.append(None)
                continue
            row = GRAD_ROWS.get(k)
            g = res["params_bar"][:, row] if row is not None else np.zeros(fctx.w.shape[0])
            g_vals.append(torch.from_numpy(np.ascontiguousarray(g)).to(dev))
        return (None, None, g_w, *g_vals)


def csp_batch(context: Context, wz: torch.Tensor, params: dict[str, torch.Tensor]):
    """Differentiable batch: (mags (n, nbands), spec (n, nspec), mass (n,), lbol (n,)) as float64 tensors."""
    names = tuple(params)
    return _CSPBatch.apply(context, names, wz, *[params[k] for k in names])
