"""CPU FP64 restatement of the warm-start network (test infrastructure: only
the tests import this file).

The reference has no network (its optimiser starts from fixed values,
src/treeator.cpp:612-615); this is the checker of the engine's own MLP
kernels.  Flat parameter layout as the engine's: per layer W[out][in] then
b[out]; ReLU after every layer but the last; loss = mean over batch x outputs
of squared error.

``bf16=True`` mirrors where the kernels round to bfloat16 (round to nearest
even): the network input, the weights the GEMMs read, every hidden
activation, the output gradient and every back-propagated activation
gradient.  Products and sums stay FP64 here (FP32 in the kernels), so the two
differ by accumulation rounding only.
"""
from __future__ import annotations

import numpy as np


def bf16(a) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounded = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, dims):
    """[(W [out, in], b [out]) per layer] from the flat vector."""
    p = np.asarray(params, dtype=np.float64)
    layers, off = [], 0
    for i in range(len(dims) - 1):
        n_in, n_out = dims[i], dims[i + 1]
        W = p[off:off + n_in * n_out].reshape(n_out, n_in)
        off += n_in * n_out
        b = p[off:off + n_out]
        off += n_out
        layers.append((W, b))
    assert off == p.size, "parameter count does not match the layer sizes"
    return layers


def n_params(dims) -> int:
    return sum(dims[i] * dims[i + 1] + dims[i + 1] for i in range(len(dims) - 1))


def forward(params, dims, x, bf16_mirror: bool = False):
    """Network output [batch, n_out] and the per-layer activations."""
    r = bf16 if bf16_mirror else (lambda a: np.asarray(a, dtype=np.float64))
    layers = unpack(params, dims)
    acts = [r(x)]
    pre = []
    for i, (W, b) in enumerate(layers):
        z = acts[-1] @ r(W).T + b
        pre.append(z)
        if i < len(layers) - 1:
            acts.append(r(np.maximum(z, 0.0)))
    return pre[-1], acts, pre


def loss_and_grad(params, dims, x, t, bf16_mirror: bool = False):
    """(loss, flat gradient) by analytic back-propagation."""
    r = bf16 if bf16_mirror else (lambda a: np.asarray(a, dtype=np.float64))
    layers = unpack(params, dims)
    y, acts, pre = forward(params, dims, x, bf16_mirror)
    t = np.asarray(t, dtype=np.float64)
    n = y.size
    loss = float(np.mean((y - t) ** 2))
    dz = r(2.0 * (y - t) / n)
    grads = [None] * len(layers)
    for i in range(len(layers) - 1, -1, -1):
        W, _ = layers[i]
        gW = dz.T @ acts[i]
        gb = dz.sum(axis=0)
        grads[i] = (gW, gb)
        if i > 0:
            da = dz @ r(W)
            dz = r(np.where(acts[i] > 0.0, da, 0.0))
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def finite_difference(params, dims, x, t, idx, h: float = 1e-6) -> np.ndarray:
    """Central differences of the FP64 loss in the parameters listed by idx."""
    p = np.asarray(params, dtype=np.float64).copy()
    out = np.zeros(len(idx))
    for k, j in enumerate(idx):
        old = p[j]
        p[j] = old + h
        lp = np.mean((forward(p, dims, x)[0] - t) ** 2)
        p[j] = old - h
        lm = np.mean((forward(p, dims, x)[0] - t) ** 2)
        p[j] = old
        out[k] = (lp - lm) / (2 * h)
    return out


def adam(p, g, m, v, step: int, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
    """One Adam update (Kingma & Ba 2015) in FP64; returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
