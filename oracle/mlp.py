"""CPU oracle of the learned tracklet pre-filter (test infrastructure only).

The pre-filter has no counterpart in the reference; this restates the
network the GPU kernels implement, in float64 numpy, so that the
tensor-core inference kernel (logits) and the training kernels (loss and
gradient) can be checked against it:

    x1 = bf16(x)                      12 features
    h1 = bf16(relu(W1' x1 + b1'))     W1' = bf16(W1), b1' = bf16(b1), 64 units
    h2 = relu(W2' h1 + b2')           W2' = bf16(W2), b2' = bf16(b2), 64 units
    z  = b3 + w3' . h2                w3' = bf16(w3), b3 FP32

loss_i = w_i * (softplus(z_i) - y_i z_i); the gradient is taken with the
BF16 roundings treated as the identity (as the training kernels do).
Parameter layout: W1[64][12], b1[64], W2[64][64], b2[64], w3[64], b3.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 12, 64
W1 = 0
B1 = W1 + N_HID * N_IN
W2 = B1 + N_HID
B2 = W2 + N_HID * N_HID
W3 = B2 + N_HID
B3 = W3 + N_HID
N_PARAMS = B3 + 1


def bf16(a) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32)


def unpack(p):
    p = np.asarray(p)
    return (p[W1:B1].reshape(N_HID, N_IN), p[B1:W2], p[W2:B2].reshape(N_HID, N_HID), p[B2:W3], p[W3:B3], p[B3])


def forward(p, x, exact: bool = False):
    """Logits (float64) and the intermediate arrays; exact=True drops the
    BF16 roundings (a smooth function, for finite-difference checks)."""
    r = (lambda a: np.asarray(a, np.float64)) if exact else (lambda a: bf16(np.asarray(a, np.float32)).astype(np.float64))
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x1 = r(np.asarray(x, np.float64 if exact else np.float32).reshape(-1, N_IN))
    a1 = x1 @ r(w1).T + r(b1)
    h1 = np.maximum(a1, 0.0) if exact else bf16(np.maximum(a1, 0.0).astype(np.float32)).astype(np.float64)
    a2 = h1 @ r(w2).T + r(b2)
    h2 = np.maximum(a2, 0.0)
    z = h2 @ r(w3) + float(b3)
    return z, (x1, h1, h2)


def softplus(z):
    return np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))


def sigmoid(z):
    return 0.5 * (1.0 + np.tanh(0.5 * z))


def loss_and_grad(p, x, y, w, exact: bool = False):
    """mean_i w_i * (softplus(z_i) - y_i z_i) and its gradient (float64)."""
    r = (lambda a: np.asarray(a, np.float64)) if exact else (lambda a: bf16(np.asarray(a, np.float32)).astype(np.float64))
    w1, b1, w2, b2, w3, b3 = unpack(p)
    z, (x1, h1, h2) = forward(p, x, exact)
    y = np.asarray(y, np.float64)
    w = np.asarray(w, np.float64)
    n = len(y)
    loss = float(np.sum(w * (softplus(z) - y * z)) / n)
    dz = w * (sigmoid(z) - y) / n
    g = np.zeros(N_PARAMS)
    g[W3:B3] = dz @ h2
    g[B3] = dz.sum()
    d2 = (h2 > 0) * np.outer(dz, r(w3))
    g[W2:B2] = (d2.T @ h1).ravel()
    g[B2:W3] = d2.sum(0)
    d1 = (h1 > 0) * (d2 @ r(w2))
    g[W1:B1] = (d1.T @ x1).ravel()
    g[B1:W2] = d1.sum(0)
    return loss, g


def init_params(seed: int) -> np.ndarray:
    """Random parameters for tests (uniform fan-in scale, small biases)."""
    r = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    p[W1:B1] = r.uniform(-1, 1, N_HID * N_IN) * np.sqrt(6.0 / N_IN)
    p[B1:W2] = r.uniform(-0.1, 0.1, N_HID)
    p[W2:B2] = r.uniform(-1, 1, N_HID * N_HID) * np.sqrt(6.0 / N_HID)
    p[B2:W3] = r.uniform(-0.1, 0.1, N_HID)
    p[W3:B3] = r.uniform(-1, 1, N_HID) * np.sqrt(6.0 / N_HID)
    p[B3] = 0.05
    return p
