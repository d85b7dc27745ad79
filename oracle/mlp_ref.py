"""numpy FP64 reference of the learned preconditioner's MLP (test infrastructure only).

Same architecture and parameter packing as quantum_package_gb300/csrc/mlp.cu:
8 -> 64 -> 64 -> 1, exact GELU (x Phi(x)), parameters W1[64][8], b1[64],
W2[64][64], b2[64], W3[64], b3; loss = mean(w (y - g)^2).  Used to check the
CUDA forward pass and the gradients of the CUDA backward pass.
"""
from __future__ import annotations

import math

import numpy as np

IN, H = 8, 64
NPARAM = H * IN + H + H * H + H + H + 1


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * IN].reshape(H, IN); o += H * IN
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, np.float64)
    z1 = X @ W1.T + b1
    a1 = gelu(z1)
    z2 = a1 @ W2.T + b2
    a2 = gelu(z2)
    return a2 @ W3 + b3, (X, z1, a1, z2, a2)


def loss_and_grad(p, X, g, w):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (X, z1, a1, z2, a2) = forward(p, X)
    n = len(y)
    err = y - np.asarray(g, np.float64)
    w = np.asarray(w, np.float64)
    loss = np.sum(w * err * err) / n
    dy = 2.0 * w * err / n
    gW3 = a2.T @ dy
    gb3 = dy.sum()
    dz2 = (dy[:, None] * W3[None, :]) * gelu_grad(z2)
    gW2 = dz2.T @ a1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    gW1 = dz1.T @ X
    gb1 = dz1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, grad
