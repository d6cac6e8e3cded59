"""The oracle of the learned-remainder network (oracle/mlp.py) against
central finite differences (float64), so that it can judge the CUDA
backward kernels."""

import numpy as np

from oracle import mlp as O


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_in, n_layers, n_out = 2, 2, 6
    _, count = O.layout(n_in, n_layers, n_out)
    p = rng.standard_normal(count) * 0.3
    X = rng.uniform(-1, 1, (17, n_in))
    Y = rng.standard_normal((17, n_out))
    loss, g = O.loss_grad(p, X, Y, n_layers)
    idx = rng.choice(count, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros(count)
        e[i] = h
        fd = (O.loss_grad(p + e, X, Y, n_layers)[0] - O.loss_grad(p - e, X, Y, n_layers)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 * max(1.0, abs(g[i])), (i, fd, g[i])
    assert np.isclose(loss, np.mean((O.forward(p, X, n_layers, n_out)[0] - Y) ** 2))


def test_oracle_layout_counts():
    lay, count = O.layout(2, 3, 6)
    assert count == (2 * 64 + 64) + 2 * (64 * 64 + 64) + (6 * 64 + 6)
    assert [l[1:] for l in lay] == [(64, 2), (64, 64), (64, 64), (6, 64)]
