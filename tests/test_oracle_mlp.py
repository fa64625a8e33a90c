"""The CPU MLP oracle's analytic gradient agrees with central finite differences."""
import numpy as np

from oracle import mlp


def test_analytic_gradient_matches_finite_differences():
    H = 8
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.5, mlp.nparams(H))
    X = rng.uniform(-1, 1, (64, 2))
    T = rng.normal(0, 1, 64)
    g, _ = mlp.gradients(p, H, X, T)
    fd = mlp.fd_gradients(p, H, X, T)
    for k, v in fd.items():
        assert abs(g[k] - v) <= 1e-7 * max(1.0, abs(v)), k
