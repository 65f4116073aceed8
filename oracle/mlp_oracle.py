"""CPU restatement (numpy, FP64) of the emulator's MLP ensemble: the forward pass, the loss and the reverse pass,
with the device path's roundings: f16 inputs (hi + lo parts), weights and activations in the forward pass, bf16
cotangents, transposed weights and layer inputs in the reverse pass. Test infrastructure: the checker of the
emulator's training and inference kernels (libopensps_gb300/csrc/emulator_train.cu, emulator.cu), never part of the
product.

OpenSPS has no emulator of its CSP; its one network, the cue nebular MLP (src/physics/opensps_cue.f90; HIP
cue_dense_act_kernel / cue_dense_back_kernel in src/accel/hip/opensps_hip_kernels.hip:3669-3811), fuses bias and
activation into each dense layer and back-propagates through the transposed weights, as here.

Parameters, one flat FP32 vector: w0 [5][512][64] (columns 0..11 used: the twelve features) | wh [3][5][512][512] | w4 [5][128][512] |
bias [5][2176] (bias of member g: four hidden layers of 512, then the 128 outputs). SiLU(z) = z sigmoid(z) (the
device evaluates sigmoid through tanh: 1/2 + tanh(z/2)/2).
"""
from __future__ import annotations

import numpy as np

NIN, NFEAT, KIN, H, NOUT, NPC, MEMBERS = 10, 12, 64, 512, 128, 64, 5
NBIAS = 4 * H + NOUT


def bf16(x) -> np.ndarray:
    """Round to the nearest bf16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def f16(x) -> np.ndarray:
    """Round to the nearest f16 (ties to even), returned as float64."""
    return np.asarray(x, dtype=np.float32).astype(np.float16).astype(np.float64)


def unpack(p: np.ndarray):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    w0 = p[o:o + MEMBERS * H * KIN].reshape(MEMBERS, H, KIN); o += MEMBERS * H * KIN
    wh = p[o:o + 3 * MEMBERS * H * H].reshape(3, MEMBERS, H, H); o += 3 * MEMBERS * H * H
    w4 = p[o:o + MEMBERS * NOUT * H].reshape(MEMBERS, NOUT, H); o += MEMBERS * NOUT * H
    b = p[o:o + MEMBERS * NBIAS].reshape(MEMBERS, NBIAS); o += MEMBERS * NBIAS
    assert o == p.size
    return w0, wh, w4, b


def silu(z):
    return z * (0.5 + 0.5 * np.tanh(0.5 * z))


def silu_grad(z):
    s = 0.5 + 0.5 * np.tanh(0.5 * z)
    return s + z * s * (1.0 - s)


def forward(p: np.ndarray, x_std: np.ndarray, member: int):
    """Member `member` on standardised features (n x 12): the reverse pass's layer inputs (bf16), the pre-activations
    Z_L and the outputs (n x 128)."""
    w0, wh, w4, b = unpack(p)
    x32 = np.asarray(x_std, dtype=np.float32).astype(np.float64)
    hi = f16(x32)
    a = hi + f16(x32 - hi)                      # the inputs' hi and lo parts against the same f16 weights
    A_rev = [np.zeros((x32.shape[0], KIN))]
    A_rev[0][:, :NFEAT] = bf16(x32)
    A, Z = a, []
    for L in range(4):
        W = f16(w0[member][:, :NFEAT]) if L == 0 else f16(wh[L - 1, member])
        z = A @ W.T + b[member, L * H:(L + 1) * H]
        Z.append(z)
        h = silu(z)
        A = f16(h)
        A_rev.append(bf16(h))
    out = A @ f16(w4[member]).T + b[member, 4 * H:]
    return A_rev, Z, out


def loss_and_grads(p: np.ndarray, x_std: np.ndarray, y_std: np.ndarray, lossw: np.ndarray):
    """The training step's loss per member (sum_k w_k (out - y)^2 / (n sum_k w_k)) and gradients, in the flat layout."""
    w0, wh, w4, b = unpack(p)
    n = x_std.shape[0]
    g0, gh, g4, gb = np.zeros_like(w0), np.zeros_like(wh), np.zeros_like(w4), np.zeros_like(b)
    loss = np.zeros(MEMBERS)
    scale = 2.0 / (n * lossw.sum())
    for g in range(MEMBERS):
        A, Z, out = forward(p, x_std, g)
        diff = out - y_std
        loss[g] = (lossw * diff * diff).sum() / (n * lossw.sum())
        dz = bf16(scale * lossw * diff)
        g4[g] = dz.T @ A[4]
        gb[g, 4 * H:] = dz.sum(0)
        dh = dz @ bf16(w4[g])
        for L in range(3, -1, -1):
            dz = bf16(dh * silu_grad(Z[L]))
            gb[g, L * H:(L + 1) * H] = dz.sum(0)
            if L > 0:
                gh[L - 1, g] = dz.T @ A[L]
                dh = dz @ bf16(wh[L - 1, g])
            else:
                g0[g] = dz.T @ A[0]
    return loss, np.concatenate([g0.ravel(), gh.ravel(), g4.ravel(), gb.ravel()])


def ensemble(p: np.ndarray, x_std: np.ndarray):
    """The members' outputs (5 x n x 128)."""
    return np.stack([forward(p, x_std, g)[2] for g in range(MEMBERS)])
