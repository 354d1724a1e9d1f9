"""CPU oracle of the learned initial guess's network — TEST INFRASTRUCTURE ONLY.

A float64 numpy restatement of the MLP that the GPU kernels of
``gade_learned.cu`` train and evaluate (no counterpart in the reference): two
hidden ReLU layers, a linear output, mean-squared-error loss, Adam.  The GPU
rounds to BF16 at fixed points (GEMM operands: inputs, weights, hidden
activations, output gradient and backpropagated gradients) and accumulates
in FP32; this oracle rounds at the same points and accumulates in float64,
so GPU gradients agree with it to the FP32 accumulation error except where
a value sits on a BF16 rounding boundary.  Only ``tests/`` import it.

Layout: W1 [din][dh], W2 [dh][dh], W3 [dh][dout] (row = input feature),
b1 [dh], b2 [dh], b3 [dout]; rows of X are samples.
"""
from __future__ import annotations

import numpy as np


def bf16(a) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    if np.any(nan):
        out[nan] = np.nan
    return out


def forward(params: dict, X: np.ndarray) -> dict:
    W1, W2, W3 = (bf16(params[k]) for k in ("W1", "W2", "W3"))
    b1, b2, b3 = (np.asarray(params[k], np.float64) for k in ("b1", "b2", "b3"))
    X16 = bf16(X)
    H1 = np.maximum(X16 @ W1 + b1, 0.0)
    H1_16 = bf16(H1)
    H2 = np.maximum(H1_16 @ W2 + b2, 0.0)
    H2_16 = bf16(H2)
    out = H2_16 @ W3 + b3
    return dict(X16=X16, H1=H1, H1_16=H1_16, H2=H2, H2_16=H2_16, out=out, W=(W1, W2, W3))


def loss_and_grads(params: dict, X: np.ndarray, T: np.ndarray) -> tuple[float, dict]:
    """MSE = mean((out - T)^2) and its gradients with the GPU's rounding points."""
    f = forward(params, X)
    W1, W2, W3 = f["W"]
    M, N = f["out"].shape
    d = f["out"] - T
    loss = float(np.mean(d * d))
    G3 = 2.0 * d / (M * N)
    G3_16 = bf16(G3)
    g = {}
    g["W3"] = f["H2_16"].T @ G3_16
    g["b3"] = G3.sum(axis=0)
    G2 = (G3_16 @ W3.T) * (f["H2"] > 0)
    G2_16 = bf16(G2)
    g["W2"] = f["H1_16"].T @ G2_16
    g["b2"] = G2.sum(axis=0)
    G1 = (G2_16 @ W2.T) * (f["H1"] > 0)
    G1_16 = bf16(G1)
    g["W1"] = f["X16"].T @ G1_16
    g["b1"] = G1.sum(axis=0)
    return loss, g


def loss_and_grads_exact(params: dict, X: np.ndarray, T: np.ndarray) -> tuple[float, dict]:
    """The same network without any rounding (for finite-difference checks)."""
    W1, W2, W3, b1, b2, b3 = (np.asarray(params[k], np.float64) for k in ("W1", "W2", "W3", "b1", "b2", "b3"))
    Z1 = X @ W1 + b1
    H1 = np.maximum(Z1, 0.0)
    Z2 = H1 @ W2 + b2
    H2 = np.maximum(Z2, 0.0)
    out = H2 @ W3 + b3
    M, N = out.shape
    d = out - T
    G3 = 2.0 * d / (M * N)
    g = dict(W3=H2.T @ G3, b3=G3.sum(0))
    G2 = (G3 @ W3.T) * (Z2 > 0)
    g.update(W2=H1.T @ G2, b2=G2.sum(0))
    G1 = (G2 @ W2.T) * (Z1 > 0)
    g.update(W1=X.T @ G1, b1=G1.sum(0))
    return float(np.mean(d * d)), g


def adam(w, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) in float64; returns (w, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v
