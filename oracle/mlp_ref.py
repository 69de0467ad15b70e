"""CPU oracle of the task-cost MLP (test infrastructure only): forward, loss and gradients in
numpy (float64), with the parameter layout of the device kernels (palial_gb300/csrc/mlp.cu):
[W1 (nin x H) | b1 (H) | W2 (H x H) | b2 (H) | W3 (H x 1) | b3 (1)], row-major, ReLU hidden
layers, loss = mean squared error."""
from __future__ import annotations

import numpy as np


def unpack(p: np.ndarray, nin: int, h: int):
    o = 0
    w1 = p[o:o + nin * h].reshape(nin, h); o += nin * h
    b1 = p[o:o + h]; o += h
    w2 = p[o:o + h * h].reshape(h, h); o += h * h
    b2 = p[o:o + h]; o += h
    w3 = p[o:o + h].reshape(h, 1); o += h
    b3 = p[o:o + 1]
    return w1, b1, w2, b2, w3, b3


def forward(p, x, nin, h):
    w1, b1, w2, b2, w3, b3 = unpack(np.asarray(p, np.float64), nin, h)
    h1 = np.maximum(x @ w1 + b1, 0.0)
    h2 = np.maximum(h1 @ w2 + b2, 0.0)
    return (h2 @ w3 + b3)[:, 0], (h1, h2)


def loss_and_grad(p, x, y, nin, h):
    x = np.asarray(x, np.float64)
    w1, b1, w2, b2, w3, b3 = unpack(np.asarray(p, np.float64), nin, h)
    out, (h1, h2) = forward(p, x, nin, h)
    d = out - y
    loss = float(np.mean(d * d))
    dy = (2.0 * d / len(y))[:, None]
    gw3 = h2.T @ dy
    gb3 = dy.sum(0)
    dh2 = (dy @ w3.T) * (h2 > 0)
    gw2 = h1.T @ dh2
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ w2.T) * (h1 > 0)
    gw1 = x.T @ dh1
    gb1 = dh1.sum(0)
    g = np.concatenate([gw1.ravel(), gb1, gw2.ravel(), gb2, gw3.ravel(), gb3])
    return loss, g
