"""numpy restatement of the closure MLP (the oracle for its GPU kernels).

TEST INFRASTRUCTURE ONLY.  Mirrors the GPU network of the learned closure
(local-dg_gb300/csrc/ldg_closure.cu, ldg_mlp.cuh): x -> GELU(W1 x + b1) ->
GELU(W2 h + b2) -> W3 h + b3 with BF16 weights, BF16 inputs and
activations, and (here) FP64 accumulation.  Rounding to BF16 happens at the
same points as on the GPU, so the two agree to the FP32-accumulation error
plus rare one-ulp BF16 flips.  Parameters use the flat layout of
ldg_closure_get_params: W1 [H x I], b1 [H], W2 [H x H], b2 [H], W3 [O x H],
b3 [O] (row-major).
"""
from __future__ import annotations

import math

import numpy as np


def bf16(x) -> np.ndarray:
    """Round float values to bfloat16 (nearest even), returned as float64."""
    x = np.asarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def unpack(theta, I, H, O):
    theta = np.asarray(theta, dtype=np.float64)
    o = 0
    W1 = theta[o:o + H * I].reshape(H, I); o += H * I
    b1 = theta[o:o + H]; o += H
    W2 = theta[o:o + H * H].reshape(H, H); o += H * H
    b2 = theta[o:o + H]; o += H
    W3 = theta[o:o + O * H].reshape(O, H); o += O * H
    b3 = theta[o:o + O]; o += O
    assert o == theta.size
    return W1, b1, W2, b2, W3, b3


def forward(theta, x, I, H, O, rounding=True):
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(theta, I, H, O)
    xb = r(x)
    z1 = xb @ r(W1).T + b1
    h1 = r(gelu(z1))
    z2 = h1 @ r(W2).T + b2
    h2 = r(gelu(z2))
    y = h2 @ r(W3).T + b3
    return y, (xb, z1, h1, z2, h2)


def backward(theta, x, dy, I, H, O, rounding=True):
    """Gradient of sum(y * dy) with respect to the flat parameters."""
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(theta, I, H, O)
    _, (xb, z1, h1, z2, h2) = forward(theta, x, I, H, O, rounding)
    dy = np.asarray(dy, dtype=np.float64)
    dyb = r(dy)
    dW3 = dyb.T @ h2
    db3 = dy.sum(axis=0)
    dH2 = dyb @ r(W3)
    dZ2 = dH2 * gelu_grad(z2)
    dZ2b = r(dZ2)
    dW2 = dZ2b.T @ h1
    db2 = dZ2.sum(axis=0)
    dH1 = dZ2b @ r(W2)
    dZ1 = dH1 * gelu_grad(z1)
    dZ1b = r(dZ1)
    dW1 = dZ1b.T @ xb
    db1 = dZ1.sum(axis=0)
    return np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])


def blocks(g, I, H, O):
    """Splits a flat parameter vector into its six named blocks."""
    W1, b1, W2, b2, W3, b3 = unpack(g, I, H, O)
    return {"W1": W1, "b1": b1, "W2": W2, "b2": b2, "W3": W3, "b3": b3}
