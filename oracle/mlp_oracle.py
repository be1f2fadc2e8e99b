"""NumPy float64 restatement of the learned treelet predictor's forward pass,
softmax cross-entropy and backward pass.  TEST INFRASTRUCTURE ONLY: the
checker for the library's GPU kernels (tests/ only).

The model has no counterpart in the reference; this oracle is checked by
finite differences of its own loss (tests/test_mlp_cpu.py).  Weights and the
input vector are rounded to BF16 exactly as the kernels use them; everything
else runs in float64, so the GPU gradients (BF16 activations, FP32
accumulation) agree within a relative error of a few 1e-3.

Parameter layout (float32 vector): E[C][16], W1[22][64], b1[64], W2[64][64],
b2[64], W3[64][C], b3[C].
"""
from __future__ import annotations

import math

import numpy as np

H, EMB, XIN = 64, 16, 22

SAMPLE_DTYPE = np.dtype([("origin", "<f4", 3), ("dir", "<f4", 3), ("current", "<u4"), ("target", "<u4")])


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float32 values to BF16 (round to nearest, ties to even), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return (r.astype(np.uint32)).view(np.float32).astype(np.float64)


def unpack(p: np.ndarray, C: int):
    o = 0

    def take(n, shape):
        nonlocal o
        v = p[o:o + n].reshape(shape)
        o += n
        return v

    E = take(C * EMB, (C, EMB))
    W1 = take(XIN * H, (XIN, H))
    b1 = take(H, (H,))
    W2 = take(H * H, (H, H))
    b2 = take(H, (H,))
    W3 = take(H * C, (H, C))
    b3 = take(C, (C,))
    return E, W1, b1, W2, b2, W3, b3


_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def loss_and_grad(params: np.ndarray, samples: np.ndarray, C: int, round_bf16: bool = True):
    """Mean cross-entropy over the samples and its gradient (float64, same layout as params)."""
    p = params.astype(np.float64)
    E, W1, b1, W2, b2, W3, b3 = unpack(p, C)
    if round_bf16:
        Eb, W1b, W2b, W3b = (bf16_round(w.astype(np.float32)) for w in (E, W1, W2, W3))
    else:
        Eb, W1b, W2b, W3b = E, W1, W2, W3
    n = len(samples)
    cur = samples["current"].astype(np.int64)
    tgt = samples["target"].astype(np.int64)
    X = np.concatenate([samples["origin"].astype(np.float64), samples["dir"].astype(np.float64), Eb[cur]], axis=1)
    if round_bf16:
        X = bf16_round(X.astype(np.float32))
    Z1 = X @ W1b + b1
    H1 = gelu(Z1)
    Z2 = H1 @ W2b + b2
    H2 = gelu(Z2)
    Z3 = H2 @ W3b + b3
    m = Z3.max(axis=1, keepdims=True)
    e = np.exp(Z3 - m)
    s = e.sum(axis=1, keepdims=True)
    loss = float(np.mean(np.log(s[:, 0]) + m[:, 0] - Z3[np.arange(n), tgt]))
    dZ3 = e / s
    dZ3[np.arange(n), tgt] -= 1.0
    dZ3 /= n
    gW3 = H2.T @ dZ3
    gb3 = dZ3.sum(axis=0)
    dH2 = dZ3 @ W3b.T
    dZ2 = dH2 * gelu_grad(Z2)
    gW2 = H1.T @ dZ2
    gb2 = dZ2.sum(axis=0)
    dH1 = dZ2 @ W2b.T
    dZ1 = dH1 * gelu_grad(Z1)
    gW1 = X.T @ dZ1
    gb1 = dZ1.sum(axis=0)
    dX = dZ1 @ W1b.T
    gE = np.zeros_like(E)
    np.add.at(gE, cur, dX[:, 6:6 + EMB])
    g = np.concatenate([gE.ravel(), gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def logits(params: np.ndarray, samples: np.ndarray, C: int) -> np.ndarray:
    p = params.astype(np.float64)
    E, W1, b1, W2, b2, W3, b3 = unpack(p, C)
    r = bf16_round
    X = np.concatenate([samples["origin"].astype(np.float64), samples["dir"].astype(np.float64),
                        r(E.astype(np.float32))[samples["current"].astype(np.int64)]], axis=1)
    X = r(X.astype(np.float32))
    H1 = gelu(X @ r(W1.astype(np.float32)) + b1)
    H2 = gelu(H1 @ r(W2.astype(np.float32)) + b2)
    return H2 @ r(W3.astype(np.float32)) + b3
