"""Numpy (float64) restatement of the learned warm start's per-vertex MLP — TEST INFRASTRUCTURE.

Only tests import it, as the checker of the CUDA forward/backward/Adam kernels.  Same network
and flat parameter layout as fastipc_gb300/csrc/mlp.cu: 64 -> 128 -> 128 -> 128 -> 4, GELU
(erf form) after the hidden layers; params = W1 [128][64], b1, W2 [128][128], b2, W3, b3,
W4 [4][128], b4.  There is no reference counterpart (the learned warm start is an addition).
"""
import numpy as np
from math import erf, sqrt, pi

IN, H, OUT = 64, 128, 4
SHAPES = [('W1', (H, IN)), ('b1', (H,)), ('W2', (H, H)), ('b2', (H,)), ('W3', (H, H)), ('b3', (H,)), ('W4', (OUT, H)), ('b4', (OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)

_erf = np.vectorize(erf)


def unpack(p):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = p[o:o + n].reshape(shp)
        o += n
    return out


def gelu(z):
    return 0.5 * z * (1 + _erf(z / sqrt(2)))


def gelu_grad(z):
    return 0.5 * (1 + _erf(z / sqrt(2))) + z * np.exp(-0.5 * z * z) / sqrt(2 * pi)


def forward(p, X):
    w = unpack(np.asarray(p, np.float64))
    X = np.asarray(X, np.float64)
    Z1 = X @ w['W1'].T + w['b1']
    A1 = gelu(Z1)
    Z2 = A1 @ w['W2'].T + w['b2']
    A2 = gelu(Z2)
    Z3 = A2 @ w['W3'].T + w['b3']
    A3 = gelu(Z3)
    out = A3 @ w['W4'].T + w['b4']
    return out, (X, Z1, A1, Z2, A2, Z3, A3)


def backward(p, cache, dout):
    """Parameter gradient (flat) of sum(dout * out)."""
    w = unpack(np.asarray(p, np.float64))
    X, Z1, A1, Z2, A2, Z3, A3 = cache
    g = {}
    g['W4'] = dout.T @ A3
    g['b4'] = dout.sum(0)
    d = (dout @ w['W4']) * gelu_grad(Z3)
    g['W3'], g['b3'] = d.T @ A2, d.sum(0)
    d = (d @ w['W3']) * gelu_grad(Z2)
    g['W2'], g['b2'] = d.T @ A1, d.sum(0)
    d = (d @ w['W2']) * gelu_grad(Z1)
    g['W1'], g['b1'] = d.T @ X, d.sum(0)
    return np.concatenate([g[name].ravel() for name, _ in SHAPES])


def mse(out, target):
    """Loss over the first 3 outputs and its gradient (the kernel's definition)."""
    n = len(out)
    e = np.zeros_like(out)
    e[:, :3] = out[:, :3] - target[:, :3]
    return float((e ** 2).sum() / (3 * n)), 2 * e / (3 * n)


def adam(p, g, m, v, lr, b1, b2, eps, t):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return p, m, v


def init(seed=0):
    """He-style initialisation (the same one the training driver uses)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shp in SHAPES:
        if name.startswith('W'):
            parts.append(rng.normal(size=shp) * np.sqrt(2.0 / shp[1]))
        else:
            parts.append(np.zeros(shp))
    return np.concatenate([a.ravel() for a in parts])
