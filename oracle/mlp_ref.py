"""numpy reference of the column-guess MLP (test infrastructure only): forward, mean-square
loss and its gradient in FP64 with the weights rounded to BF16 exactly as the CUDA kernels use
them (straight-through gradient w.r.t. the FP32 master weights).

Network: x (din) -> GELU(W1 x + b1) (h) -> GELU(W2 . + b2) (h) -> W3 . + b3 (dout),
GELU(z) = z/2 (1 + erf(z/sqrt 2)); loss = mean over batch and outputs of (y - t)^2.
Parameters in the library's logical order W1 | b1 | W2 | b2 | W3 | b3.
"""
from __future__ import annotations

import math

import numpy as np

_erf = np.vectorize(math.erf)


def bf16_round(a):
    """float32 -> nearest bfloat16 (ties to even), returned as float64."""
    b = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rnd = 0x7FFF + ((b >> 16) & 1)
    r = ((b + rnd) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unflatten(flat, din, h, dout):
    shapes = [(h, din), (h,), (h, h), (h,), (dout, h), (dout,)]
    out, q = [], 0
    for s in shapes:
        n = int(np.prod(s))
        out.append(np.asarray(flat[q:q + n], dtype=np.float64).reshape(s))
        q += n
    return out


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def loss_grad(flat, X, T, din, h, dout):
    W1, b1, W2, b2, W3, b3 = unflatten(flat, din, h, dout)
    W1r, W2r, W3r = bf16_round(W1), bf16_round(W2), bf16_round(W3)
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    B = X.shape[0]
    Z1 = X @ W1r.T + b1
    A1 = gelu(Z1)
    Z2 = A1 @ W2r.T + b2
    A2 = gelu(Z2)
    Y = A2 @ W3r.T + b3
    E = Y - T
    loss = float(np.mean(E * E))
    dY = 2.0 * E / (B * dout)
    gW3 = dY.T @ A2
    gb3 = dY.sum(0)
    dZ2 = (dY @ W3r) * gelu_d(Z2)
    gW2 = dZ2.T @ A1
    gb2 = dZ2.sum(0)
    dZ1 = (dZ2 @ W2r) * gelu_d(Z1)
    gW1 = dZ1.T @ X
    gb1 = dZ1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g, Y
