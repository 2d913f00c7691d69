"""The float64 MLP oracle's own gradient, checked by finite differences."""
import numpy as np

from oracle import mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = mlp.init_params(1) + rng.normal(0, 0.05, mlp.NPARAM)
    X = rng.normal(size=(37, 9))
    T = rng.normal(size=37)
    loss, g = mlp.loss_grad(p, X, T)
    idx = rng.choice(mlp.NPARAM, 60, replace=False)
    idx = np.concatenate([idx, [mlp.NPARAM - 1, 0, 600]])
    for i in idx:
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (mlp.loss_grad(p + e, X, T)[0] - mlp.loss_grad(p - e, X, T)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
    assert mlp.NPARAM == 4865
