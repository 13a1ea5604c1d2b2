"""NumPy FP64 restatement of the surrogate MLP's forward and backward pass --
TEST INFRASTRUCTURE (the GPU kernels' gradients are checked against it).

Layers: Z_i = H_{i-1} W_i^T + b_i; H_i = GELU(Z_i) for hidden layers; the
last layer gives logits; loss = mean over samples and cells of
BCE(logits, y) with y in {0, 1}.
"""
import math

import numpy as np


def _erf(x):
    return np.vectorize(math.erf)(x)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def forward_backward(X, weights, biases, Y):
    """X [B][in], weights [W_i [out][in]], biases [b_i], Y [B][ncells] in {0,1}.
    Returns (loss, [dW_i], [db_i])."""
    H = [X]
    Z = []
    n = len(weights)
    for i, (W, b) in enumerate(zip(weights, biases)):
        z = H[-1] @ W.T + b
        Z.append(z)
        H.append(gelu(z) if i < n - 1 else z)
    logits = H[-1]
    B, nc = logits.shape
    loss = np.mean(np.maximum(logits, 0) - logits * Y + np.log1p(np.exp(-np.abs(logits))))
    d = (1.0 / (1.0 + np.exp(-logits)) - Y) / (B * nc)
    dW, db = [None] * n, [None] * n
    for i in range(n - 1, -1, -1):
        dW[i] = d.T @ H[i]
        db[i] = d.sum(axis=0)
        if i > 0:
            d = (d @ weights[i]) * gelu_grad(Z[i - 1])
    return loss, dW, db


def adamw(w, m, v, g, lr, b1, b2, eps, wd, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    upd = (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return w - lr * (upd + wd * w), m, v
