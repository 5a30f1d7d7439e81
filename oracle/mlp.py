"""FP64 NumPy restatement of the schedule MLP -- TEST INFRASTRUCTURE ONLY.

The checker for the library's MLP kernels (forward, backward, Adam): the same
network D0 -> H -> H -> 1 with ReLU hidden layers and mean squared error, the
same flat parameter layout W1 (H x D0), b1, W2 (H x H), b2, W3 (1 x H), b3,
evaluated in float64 so that the FP32 kernels can be compared against it.
"""
from __future__ import annotations

import numpy as np


def unpack(p, d0, h):
    p = np.asarray(p, np.float64)
    o = 0

    def take(k, shape):
        nonlocal o
        a = p[o:o + k].reshape(shape)
        o += k
        return a

    W1 = take(h * d0, (h, d0)); b1 = take(h, (h,))
    W2 = take(h * h, (h, h)); b2 = take(h, (h,))
    W3 = take(h, (1, h)); b3 = take(1, (1,))
    return W1, b1, W2, b2, W3, b3


def forward(p, x, d0, h):
    W1, b1, W2, b2, W3, b3 = unpack(p, d0, h)
    x = np.asarray(x, np.float64)
    a1 = np.maximum(x @ W1.T + b1, 0.0)
    a2 = np.maximum(a1 @ W2.T + b2, 0.0)
    return (a2 @ W3.T + b3)[:, 0], (x, a1, a2)


def loss_grad(p, x, y, d0, h):
    """Mean squared error and its gradient with respect to the flat p."""
    W1, b1, W2, b2, W3, b3 = unpack(p, d0, h)
    yhat, (x, a1, a2) = forward(p, x, d0, h)
    B = x.shape[0]
    r = yhat - np.asarray(y, np.float64)
    loss = float(r @ r / B)
    d3 = (2.0 / B) * r[:, None]                 # B x 1
    gW3 = d3.T @ a2; gb3 = d3.sum(0)
    d2 = (d3 @ W3) * (a2 > 0)
    gW2 = d2.T @ a1; gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    gW1 = d1.T @ x; gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def adam_train(p, x, y, d0, h, epochs, lr, b1=0.9, b2=0.999, eps=1e-8):
    """Full-batch Adam, the update rule of the library's training loop."""
    p = np.array(p, np.float64)
    m = np.zeros_like(p); v = np.zeros_like(p)
    for t in range(1, epochs + 1):
        _, g = loss_grad(p, x, y, d0, h)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p -= lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return p, loss_grad(p, x, y, d0, h)[0]
