"""ORACLE — test infrastructure, not part of the product.

CPU restatement (numpy, fp32) of the learned proposal's network
(csrc/gpu/mcbgpu_mlp.cu): h = relu(W1 x + b1), logit = w2 . h + b2, with W1 and w2
rounded to bf16 in the forward pass as the device does, and the gradient of the mean
binary cross-entropy with positives weighted by pos_weight (the rounding treated as
the identity, as the device's master-weight update does).  Used by the tests to
check the device's forward pass and gradients; its own gradient is checked against
finite differences on the CPU.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 16, 64


def bf16_round(a) -> np.ndarray:
    """Round fp32 values to the nearest bf16 (ties to even), returned as fp32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def unpack(params):
    p = np.asarray(params, np.float32)
    k = N_HID * N_IN
    return p[:k].reshape(N_HID, N_IN), p[k:k + N_HID], p[k + N_HID:k + 2 * N_HID], p[-1]


def forward(params, x):
    """(logits, hidden) for features x (count x 16, already bf16 values)."""
    W1, b1, w2, b2 = unpack(params)
    h = np.maximum(x.astype(np.float32) @ bf16_round(W1).T + b1, 0.0).astype(np.float32)
    return (h @ bf16_round(w2) + b2).astype(np.float32), h


def loss_and_grads(params, x, y, pos_weight: float):
    """(mean weighted cross-entropy, gradient of every parameter)."""
    W1, b1, w2, b2 = unpack(params)
    z, h = forward(params, x)
    y = np.asarray(y).astype(bool)
    wt = np.where(y, pos_weight, 1.0).astype(np.float64)
    zz = z.astype(np.float64)
    sp = lambda t: np.maximum(t, 0) + np.log1p(np.exp(-np.abs(t)))  # noqa: E731
    loss = float(np.mean(wt * np.where(y, sp(-zz), sp(zz))))
    s = 1.0 / (1.0 + np.exp(-zz))
    dz = (s - y) * wt / len(z)
    w2r = bf16_round(w2).astype(np.float64)
    dh = np.outer(dz, w2r) * (h > 0)
    gW1 = dh.T @ x.astype(np.float64)
    gb1 = dh.sum(0)
    gw2 = h.astype(np.float64).T @ dz
    gb2 = dz.sum()
    g = np.concatenate([gW1.reshape(-1), gb1, gw2, [gb2]]).astype(np.float32)
    return loss, g
