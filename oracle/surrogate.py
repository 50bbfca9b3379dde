"""CPU oracle of the learned rank surrogate (test infrastructure only).

The surrogate has no counterpart in the reference: it replaces the fixed
ButterflyRankEstimator sample count (src/ButterflyFactorization/
rankestimation.jl:93-98) whose under-estimates trigger the adaptive
re-sampling of src/ButterflyFactorization/compressors.jl:134-151.  This
module restates the library's network and training arithmetic in NumPy so
that the GPU kernels (bf_surrogate.cu) can be checked against it:

  * weights: FP32 master copy, rounded to BF16 (round to nearest even) in the
    forward pass; gradients pass straight through the rounding;
  * network: x = (f - mu) / sigma, h1 = gelu(W1 x + b1), h2 = gelu(W2 h1 + b2),
    y = w3 . h2 + b3, gelu in its tanh form (Hendrycks & Gimpel 2016);
  * loss: mean over the batch of 0.5 (y - target)^2, target = log(rank);
  * optimiser: Adam (Kingma & Ba 2015) on everything except mu and sigma.

Parity is pinned by central finite differences of an FP64 run of the same
functions (tests/test_surrogate.py).
"""
from __future__ import annotations

import math

import numpy as np

IN, H = 4, 64
NW = 8 + H * IN + H + H * H + H + H + 1  # 4553


def split(w):
    """Views of the weight vector (layout of bf_surrogate.h)."""
    o = 0

    def take(n, shape=None):
        nonlocal o
        v = w[o:o + n]
        o += n
        return v.reshape(shape) if shape else v
    mu = take(4)
    sg = take(4)
    W1 = take(H * IN, (H, IN))
    b1 = take(H)
    W2 = take(H * H, (H, H))
    b2 = take(H)
    W3 = take(H)
    b3 = take(1)
    return mu, sg, W1, b1, W2, b2, W3, b3


def bf16_round(x):
    """Round FP32 values to BF16 (nearest, ties to even), returned as FP32."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    u = ((u + r) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32)


GELU_C = math.sqrt(2.0 / math.pi)
GELU_A = 0.044715


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + GELU_A * x ** 3)))


def gelu_grad(x):
    t = np.tanh(GELU_C * (x + GELU_A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * x * x)


def forward(w, F, round_bf16=True, dtype=np.float32):
    mu, sg, W1, b1, W2, b2, W3, b3 = split(np.asarray(w, dtype))
    rnd = (lambda a: bf16_round(a).astype(dtype)) if round_bf16 else (lambda a: a)
    X = (np.asarray(F, dtype) - mu) / sg
    Z1 = X @ rnd(W1).T + b1
    H1 = gelu(Z1)
    Z2 = H1 @ rnd(W2).T + b2
    H2 = gelu(Z2)
    y = H2 @ rnd(W3) + b3[0]
    return y, (X, Z1, H1, Z2, H2)


def loss_and_grad(w, F, T, round_bf16=True, dtype=np.float32):
    """Mean 0.5 (y - T)^2 and its gradient w.r.t. the weight vector (mu, sigma: 0)."""
    w = np.asarray(w, dtype)
    mu, sg, W1, b1, W2, b2, W3, b3 = split(w)
    rnd = (lambda a: bf16_round(a).astype(dtype)) if round_bf16 else (lambda a: a)
    y, (X, Z1, H1, Z2, H2) = forward(w, F, round_bf16, dtype)
    B = len(T)
    r = y - np.asarray(T, dtype)
    loss = 0.5 * float(np.sum(r.astype(np.float64) ** 2)) / B
    dy = r / B
    g = np.zeros(NW, dtype)
    _, _, gW1, gb1, gW2, gb2, gW3, gb3 = split(g)
    gW3[:] = H2.T @ dy
    gb3[0] = dy.sum()
    dZ2 = np.outer(dy, rnd(W3)) * gelu_grad(Z2)
    gW2[:] = dZ2.T @ H1
    gb2[:] = dZ2.sum(0)
    dZ1 = (dZ2 @ rnd(W2)) * gelu_grad(Z1)
    gW1[:] = dZ1.T @ X
    gb1[:] = dZ1.sum(0)
    return loss, g


def init_weights(F, seed):
    """Normalisation from the data, Glorot-uniform layers, zero biases."""
    F = np.asarray(F, np.float64)
    rng = np.random.default_rng(seed)
    w = np.zeros(NW, np.float32)
    mu, sg, W1, b1, W2, b2, W3, b3 = split(w)
    mu[:] = F.mean(0)
    sg[:] = np.maximum(F.std(0), 1e-6)
    for W, fi, fo in ((W1, IN, H), (W2, H, H)):
        a = math.sqrt(6.0 / (fi + fo))
        W[:] = rng.uniform(-a, a, W.shape)
    a = math.sqrt(6.0 / (H + 1))
    W3[:] = rng.uniform(-a, a, H)
    return w


def adam_step(w, g, m, v, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update in place (entries 0..7, the normalisation, stay fixed)."""
    m[8:] = beta1 * m[8:] + (1 - beta1) * g[8:]
    v[8:] = beta2 * v[8:] + (1 - beta2) * g[8:] * g[8:]
    mh = m[8:] / (1 - beta1 ** t)
    vh = v[8:] / (1 - beta2 ** t)
    w[8:] -= lr * mh / (np.sqrt(vh) + eps)
