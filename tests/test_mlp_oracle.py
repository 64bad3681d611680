"""The FP64 network oracle (oracle/mlp_ref.py) pinned by finite differences,
and the C ABI's parameter count against it.  CPU only."""
from __future__ import annotations

import numpy as np

from oracle import mlp_ref


def test_param_count_matches_header():
    from ode_gb300 import ode
    assert mlp_ref.NPARAMS == ode.GBODE_MLP_NPARAMS == 35099


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = mlp_ref.init_params(1, mean=rng.normal(size=12), std=rng.uniform(0.5, 2.0, 12)).astype(np.float64)
    X = rng.normal(size=(7, 12))
    Y = rng.normal(size=(7, 3))
    loss, g = mlp_ref.loss_grad(p, X, Y)
    assert np.isclose(loss, ((mlp_ref.forward(p, X) - Y) ** 2).mean())
    idx = np.concatenate([rng.choice(np.arange(24, mlp_ref.NPARAMS), 200, replace=False),
                          np.arange(mlp_ref.NPARAMS - 3, mlp_ref.NPARAMS)])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp_ref.loss_grad(pp, X, Y)[0] - mlp_ref.loss_grad(pm, X, Y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(fd), (i, fd, g[i])
    assert np.all(g[:24] == 0)
