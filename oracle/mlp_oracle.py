"""CPU oracle of the learned start vector's network (test infrastructure only:
imported by tests/, never by the product).

A numpy restatement, in float64, of what carcassonne_gb300/learned.py runs
through the CUDA kernels of csrc/mlp.cu: hidden layers Y = relu(X W^T + b),
a linear output layer, the loss sum (Y - T)^2 / (2 B) and its gradients by
backpropagation.  The reference has no such network (its start vector is the
previous center, system/_2d.py:435-439, :491-492), so this oracle is pinned
by finite differences (tests/test_mlp_oracle.py), not by reference vectors.
"""
from __future__ import annotations

import numpy as np


def forward(params, X):
    """params: [(W, b), ...] with W (out, in); returns the list of layer outputs."""
    acts = [np.asarray(X, np.float64)]
    for i, (W, b) in enumerate(params):
        z = acts[-1] @ np.asarray(W, np.float64).T + np.asarray(b, np.float64)
        acts.append(np.maximum(z, 0.0) if i + 1 < len(params) else z)
    return acts


def loss_and_grads(params, X, T):
    acts = forward(params, X)
    B = X.shape[0]
    d = acts[-1] - np.asarray(T, np.float64)
    loss = 0.5 * np.sum(d * d) / B
    g = d / B
    grads = [None] * len(params)
    for i in range(len(params) - 1, -1, -1):
        W, _ = params[i]
        if i + 1 < len(params):
            g = g * (acts[i + 1] > 0)
        grads[i] = (g.T @ acts[i], g.sum(axis=0))
        g = g @ np.asarray(W, np.float64)
    return loss, grads


def adam(p, g, m, v, lr, b1, b2, eps, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v
