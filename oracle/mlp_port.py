"""TEST ORACLE (checker only): numpy restatement of the learned predictor's
forward pass, MSE loss and backward pass (include/sunmlp_gb300.h), with the
GPU kernels' rounding points -- BF16 inputs, weights, hidden activations and
hidden-layer gradients, FP32-or-better accumulation -- so the tensor-core
training kernels can be checked gradient by gradient.  With rounding off
(``bf16=False``) it is the exact float64 gradient, which
tests/test_mlp_oracle.py pins against finite differences.  There is no
reference counterpart: the network is this project's."""
from __future__ import annotations

import numpy as np

IN_PAD, HID, OUT = 144, 64, 64
P_W1, P_B1 = 0, IN_PAD * HID
P_W2 = P_B1 + HID
P_B2 = P_W2 + HID * HID
P_W3 = P_B2 + HID
P_B3 = P_W3 + HID * OUT
NPARAMS = P_B3 + OUT


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def from_bits(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def split(p):
    p = np.asarray(p, np.float64)
    return (p[P_W1:P_B1].reshape(IN_PAD, HID), p[P_B1:P_W2], p[P_W2:P_B2].reshape(HID, HID),
            p[P_B2:P_W3], p[P_W3:P_B3].reshape(HID, OUT), p[P_B3:])


def forward(params, X, rnd=True):
    r = bf16 if rnd else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = split(params)
    W1, W2, W3 = r(W1), r(W2), r(W3)
    X = np.asarray(X, np.float64)
    H1 = r(np.maximum(X @ W1 + b1, 0.0))
    H2 = r(np.maximum(H1 @ W2 + b2, 0.0))
    O = H2 @ W3 + b3
    return O, (X, H1, H2, W1, W2, W3)


def loss_and_grad(params, X, T, rnd=True):
    """Mean-squared error over all outputs and its parameter gradient."""
    r = bf16 if rnd else (lambda a: np.asarray(a, np.float64))
    O, (X, H1, H2, W1, W2, W3) = forward(params, X, rnd)
    m = X.shape[0]
    D = O - np.asarray(T, np.float64)
    loss = float(np.sum(D * D)) / (m * OUT)
    dO = D * (2.0 / (m * OUT))
    G1 = r(dO)
    g = np.zeros(NPARAMS)
    g[P_W3:P_B3] = (H2.T @ G1).reshape(-1)
    g[P_B3:] = dO.sum(axis=0)
    dH2 = r((G1 @ W3.T) * (H2 > 0))
    g[P_W2:P_B2] = (H1.T @ dH2).reshape(-1)
    g[P_B2:P_W3] = dH2.sum(axis=0)
    dH1 = r((dH2 @ W2.T) * (H1 > 0))
    g[P_W1:P_B1] = (X.T @ dH1).reshape(-1)
    g[P_B1:P_W2] = dH1.sum(axis=0)
    return loss, g
