"""CPU oracle of the order-selection MLP (test infrastructure only).

Restates, in numpy float64, the network the library trains and runs:
16 inputs -> 64 -> 64 -> 64 -> 16 logits (14 used), GELU (tanh form) on the
hidden layers, BF16 weights and BF16 layer inputs, wider accumulation.  The
GPU forward and backward kernels are checked against `forward` and
`backward` here (gradients within the tolerance BF16 storage allows).

Parameter layout (flat float32 vector, the library's order):
W1[64][16], b1[64], W2[64][64], b2[64], W3[64][64], b3[64], W4[16][64], b4[16].
"""
from __future__ import annotations

import numpy as np

SIZES = [(64, 16), (64,), (64, 64), (64,), (64, 64), (64,), (16, 64), (16,)]
N_CLASSES = 14
N_PARAMS = sum(int(np.prod(s)) for s in SIZES)


def bf16(a):
    """Round to BF16 (nearest even) and back to float64."""
    a = np.asarray(a, np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(theta):
    out, o = [], 0
    for s in SIZES:
        n = int(np.prod(s))
        out.append(np.asarray(theta[o:o + n], np.float64).reshape(s))
        o += n
    return out


def gelu(z):
    c = np.sqrt(2.0 / np.pi)
    return 0.5 * z * (1.0 + np.tanh(c * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    c = np.sqrt(2.0 / np.pi)
    u = c * (z + 0.044715 * z ** 3)
    t = np.tanh(u)
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * c * (1.0 + 3 * 0.044715 * z * z)


def forward(theta, x):
    """x: (batch, 16).  Returns logits (batch, 16) and the cache."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(theta)
    W1, W2, W3, W4 = (bf16(w) for w in (W1, W2, W3, W4))
    a0 = bf16(x)
    z1 = a0 @ W1.T + b1
    a1 = bf16(gelu(z1))
    z2 = a1 @ W2.T + b2
    a2 = bf16(gelu(z2))
    z3 = a2 @ W3.T + b3
    a3 = bf16(gelu(z3))
    z4 = a3 @ W4.T + b4
    return z4, (a0, z1, a1, z2, a2, z3, a3, W1, W2, W3, W4)


def loss_and_grad(theta, x, y):
    """Mean cross-entropy over the 14 classes and its gradient with respect
    to the flat parameters (straight through the BF16 roundings)."""
    z4, (a0, z1, a1, z2, a2, z3, a3, W1, W2, W3, W4) = forward(theta, x)
    n = len(y)
    lg = z4[:, :N_CLASSES]
    lg = lg - lg.max(axis=1, keepdims=True)
    p = np.exp(lg)
    p /= p.sum(axis=1, keepdims=True)
    loss = -np.log(p[np.arange(n), y]).mean()
    d4 = np.zeros_like(z4)
    d4[:, :N_CLASSES] = p
    d4[np.arange(n), y] -= 1.0
    d4 /= n
    gW4 = d4.T @ a3
    gb4 = d4.sum(0)
    d3 = (d4 @ W4) * gelu_grad(z3)
    gW3 = d3.T @ a2
    gb3 = d3.sum(0)
    d2 = (d3 @ W3) * gelu_grad(z2)
    gW2 = d2.T @ a1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * gelu_grad(z1)
    gW1 = d1.T @ a0
    gb1 = d1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3, gW4, gb4)])
    return loss, g


def init(seed=0):
    rng = np.random.default_rng(seed)
    parts = []
    for s in SIZES:
        if len(s) == 2:
            parts.append(rng.standard_normal(s).ravel() * np.sqrt(2.0 / s[1]))
        else:
            parts.append(np.zeros(s))
    return np.concatenate(parts).astype(np.float32)
