"""FP64 CPU restatement of the learned-warm-start network, for checking.

Test infrastructure only: imported by tests/ (and the evaluation leg of
bench.py), never by the product.  The reference has no learned component; this
oracle restates the network the library defines (parameter layout in
include/gbode.h, gbodeMlpParamCount) and its mean-squared-error loss, with the
backward pass written out by hand, and is itself pinned by central finite
differences in tests/test_mlp_oracle.py.
"""
from __future__ import annotations

import numpy as np

NI, NH, NO = 12, 128, 3
NPARAMS = 2 * NI + NH * NI + NH + 2 * (NH * NH + NH) + NO * NH + NO


def unpack(p):
    p = np.asarray(p, np.float64)
    assert p.size == NPARAMS
    o = 0

    def take(n, shape=None):
        nonlocal o
        a = p[o:o + n]
        o += n
        return a.reshape(shape) if shape else a
    mean, std = take(NI), take(NI)
    W1, b1 = take(NH * NI, (NH, NI)), take(NH)
    W2, b2 = take(NH * NH, (NH, NH)), take(NH)
    W3, b3 = take(NH * NH, (NH, NH)), take(NH)
    W4, b4 = take(NO * NH, (NO, NH)), take(NO)
    return mean, std, [(W1, b1), (W2, b2), (W3, b3), (W4, b4)]


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X):
    """Outputs Y[n][3] of the network on raw features X[n][12] (FP64)."""
    mean, std, layers = unpack(p)
    a = (np.asarray(X, np.float64) - mean) / std
    for i, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = silu(z) if i < 3 else z
    return a


def loss_grad(p, X, Y):
    """Mean squared error over n x 3 outputs and its gradient (FP64); the
    standardisation entries get zero gradient (they are fixed)."""
    mean, std, layers = unpack(p)
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    n = X.shape[0]
    acts = [(X - mean) / std]
    zs = []
    a = acts[0]
    for i, (W, b) in enumerate(layers):
        z = a @ W.T + b
        zs.append(z)
        a = silu(z) if i < 3 else z
        acts.append(a)
    e = acts[-1] - Y
    loss = float((e * e).sum() / (3 * n))
    d = 2.0 * e / (3 * n)
    grads = []
    for i in range(3, -1, -1):
        W, b = layers[i]
        if i < 3:
            d = d * silu_grad(zs[i])
        grads.append((d.T @ acts[i], d.sum(axis=0)))
        d = d @ W
    grads.reverse()
    g = [np.zeros(NI), np.zeros(NI)]
    for gW, gb in grads:
        g += [gW.ravel(), gb]
    return loss, np.concatenate(g)


def init_params(seed: int, mean=None, std=None):
    """He-style initial weights (uniform, scaled by fan-in), zero biases."""
    rng = np.random.default_rng(seed)
    parts = [np.zeros(NI) if mean is None else np.asarray(mean, np.float64),
             np.ones(NI) if std is None else np.asarray(std, np.float64)]
    for fan_in, fan_out in ((NI, NH), (NH, NH), (NH, NH), (NH, NO)):
        lim = np.sqrt(6.0 / fan_in) * (0.5 if fan_out == NO else 1.0)
        parts += [rng.uniform(-lim, lim, fan_in * fan_out), np.zeros(fan_out)]
    return np.concatenate(parts).astype(np.float32)
