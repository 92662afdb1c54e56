"""CPU restatement of the learned warm-start MLP (test infrastructure only).

The checker for the GPU kernels of kizuriphysics3d_gb300/csrc/kzg_mlp.cu: the same network
(24 -> 64 -> 64 -> 3, ReLU), the same standardisation, the same BF16 rounding points (inputs,
weights, hidden activations, and the backward operands dY, dZ2, dZ1), evaluated in float64 so that
only the GPU's FP32 accumulation order differs.  With ``bf=False`` every rounding is skipped, which
gives the exact float64 function used for finite-difference checks of the backward formulas.

Only tests/ use this module; the product never imports it.
"""
from __future__ import annotations

import numpy as np

F, H, O = 24, 64, 3
P = H * F + H + H * H + H + O * H + O
LOG_FLOATS = F + 2 * O


def bf16(x) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    x32 = np.ascontiguousarray(x, np.float32)
    u = x32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(theta):
    t = np.asarray(theta, np.float64)
    o = 0
    W1 = t[o:o + H * F].reshape(H, F); o += H * F
    b1 = t[o:o + H]; o += H
    W2 = t[o:o + H * H].reshape(H, H); o += H * H
    b2 = t[o:o + H]; o += H
    W3 = t[o:o + O * H].reshape(O, H); o += O * H
    b3 = t[o:o + O]; o += O
    return W1, b1, W2, b2, W3, b3


def pack(W1, b1, W2, b2, W3, b3) -> np.ndarray:
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3]).astype(np.float64)


def standardise(x_raw, mean, std, bf=True):
    """(x - mean) * (1 / std) in float32 as the kernels do, then BF16."""
    istd = np.float32(1.0) / np.asarray(std, np.float32)
    xn = (np.asarray(x_raw, np.float32) - np.asarray(mean, np.float32)) * istd
    return bf16(xn) if bf else xn.astype(np.float64)


def forward(theta, mean, std, x_raw, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(theta)
    X = standardise(x_raw, mean, std, bf)
    H1 = r(np.maximum(X @ r(W1).T + b1, 0.0))
    H2 = r(np.maximum(H1 @ r(W2).T + b2, 0.0))
    Y = H2 @ r(W3).T + b3
    return {"X": X, "H1": H1, "H2": H2, "Y": Y}


def loss_and_grad(theta, mean, std, samples, bf=True, tau=0.0):
    """Loss over the valid targets (squared error, or with tau > 0 the pinball loss of quantile
    tau) and its gradient w.r.t. theta."""
    s = np.asarray(samples, np.float64)
    x_raw, tgt, msk = s[:, :F], s[:, F:F + O], s[:, F + O:F + 2 * O]
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(theta)
    f = forward(theta, mean, std, x_raw.astype(np.float32) if bf else x_raw, bf)
    X, H1, H2, Y = f["X"], f["H1"], f["H2"], f["Y"]
    nvalid = msk.sum()
    inv = 1.0 / nvalid if nvalid > 0 else 0.0
    e = Y - tgt
    if tau > 0.0:
        loss = float((msk * np.where(e > 0, (1.0 - tau) * e, -tau * e)).sum() * inv)
        dy = msk * np.where(e > 0, 1.0 - tau, -tau) * inv
    else:
        loss = float((msk * e * e).sum() * inv)
        dy = msk * 2.0 * e * inv
    dYb = r(dy)
    dW3 = dYb.T @ H2
    db3 = dy.sum(0)
    dZ2 = (dYb @ r(W3)) * (H2 > 0)
    dZ2b = r(dZ2)
    dW2 = dZ2b.T @ H1
    db2 = dZ2.sum(0)
    dZ1 = (dZ2b @ r(W2)) * (H1 > 0)
    dZ1b = r(dZ1)
    dW1 = dZ1b.T @ X
    db1 = dZ1.sum(0)
    return loss, pack(dW1, db1, dW2, db2, dW3, db3)
