"""FP64 numpy restatement of the learned closure's network — TEST INFRASTRUCTURE
ONLY (the checker of the tcgen05 convolution kernels; no reference counterpart).

Layout: activations a[nb][nz][ny][nx][16], weights w[27][16 ci][16 co] with
tap t = (dz+1)*9 + (dy+1)*3 + (dx+1), zero padding, GELU(x) = x * Phi(x)."""
from __future__ import annotations

import math

import numpy as np

_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    cdf = 0.5 * (1.0 + _erf(x / math.sqrt(2.0)))
    return cdf + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def _pad(a):
    return np.pad(a, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))


def conv3d(a, w, b=None):
    nb, nz, ny, nx, _ = a.shape
    ap = _pad(a.astype(np.float64))
    out = np.zeros((nb, nz, ny, nx, w.shape[2]))
    t = 0
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                out += ap[:, dz:dz + nz, dy:dy + ny, dx:dx + nx, :] @ w[t].astype(np.float64)
                t += 1
    if b is not None:
        out += b
    return out


def conv3d_data_grad(g, w):
    """d(conv)/d(input) applied to the output gradient g."""
    nb, nz, ny, nx, _ = g.shape
    gp = _pad(g.astype(np.float64))
    out = np.zeros((nb, nz, ny, nx, w.shape[1]))
    t = 0
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                # output voxel p used input p + off(t): input q gets g[q - off(t)]
                out += gp[:, 2 - dz:2 - dz + nz, 2 - dy:2 - dy + ny, 2 - dx:2 - dx + nx, :] @ w[t].T.astype(np.float64)
                t += 1
    return out


def conv3d_weight_grad(a, g):
    nb, nz, ny, nx, _ = a.shape
    ap = _pad(a.astype(np.float64))
    gw = np.zeros((27, a.shape[4], g.shape[4]))
    t = 0
    g2 = g.reshape(-1, g.shape[4]).astype(np.float64)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                gw[t] = ap[:, dz:dz + nz, dy:dy + ny, dx:dx + nx, :].reshape(-1, a.shape[4]).T @ g2
                t += 1
    return gw, g2.sum(axis=0)


def net_forward(x, ws, bs):
    """Layers 1-3 GELU, layer 4 linear. Returns output and the pre-activations."""
    pres, acts = [], [x]
    a = x
    for i in range(4):
        z = conv3d(a, ws[i], bs[i])
        pres.append(z)
        a = gelu(z) if i < 3 else z
        acts.append(a)
    return a, pres, acts


def net_backward(dy, ws, pres, acts):
    gws, gbs = [None] * 4, [None] * 4
    g = dy
    for i in range(3, -1, -1):
        gws[i], gbs[i] = conv3d_weight_grad(acts[i], g)
        if i > 0:
            g = conv3d_data_grad(g, ws[i]) * gelu_grad(pres[i - 1])
    return gws, gbs
