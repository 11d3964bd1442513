"""Fully connected tanh network in numpy, FP64 (TEST INFRASTRUCTURE ONLY).

CPU restatement of the library's network for checking its GPU forward pass, loss and
gradients: layers n_in -> n_hidden (tanh) -> ... -> n_out (linear), parameters per layer
W [out][in] row-major then b [out], loss = mean squared error over all outputs. Gradients
by reverse-mode differentiation written out by hand; the test checks them against central
finite differences before trusting them.
"""
from __future__ import annotations

import numpy as np


def unpack(params, widths):
    out, off = [], 0
    for l in range(len(widths) - 1):
        ni, no = widths[l], widths[l + 1]
        W = params[off:off + ni * no].reshape(no, ni)
        off += ni * no
        b = params[off:off + no]
        off += no
        out.append((W, b))
    assert off == len(params)
    return out


def forward(params, widths, x):
    acts = [x]
    layers = unpack(np.asarray(params, dtype=np.float64), widths)
    a = np.asarray(x, dtype=np.float64)
    for l, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = np.tanh(z) if l + 1 < len(layers) else z
        acts.append(a)
    return a, acts


def loss_grad(params, widths, x, target):
    params = np.asarray(params, dtype=np.float64)
    y, acts = forward(params, widths, x)
    e = y - target
    loss = float(np.mean(e * e))
    layers = unpack(params, widths)
    delta = 2.0 * e / e.size
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        grads.append((delta.T @ acts[l], delta.sum(axis=0)))
        if l > 0:
            delta = (delta @ W) * (1.0 - acts[l] ** 2)
    g = []
    for dW, db in reversed(grads):
        g.append(dW.reshape(-1))
        g.append(db)
    return loss, np.concatenate(g)
