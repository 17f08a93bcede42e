"""The CPU reference of the learned proposal's network against finite
differences (it is the checker of the device's tensor-core gradients)."""

import numpy as np

from mlp_reference import IN, TOTAL, init, loss_and_grad


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = init(3).astype(np.float64)
    n = 64
    samples = np.column_stack([rng.uniform(-1, 1, (n, IN)), rng.integers(0, 16, n), rng.normal(0, 2, n)])
    tau = 0.9
    loss, g = loss_and_grad(p, samples, tau, emulate=False)
    idx = rng.choice(TOTAL, 60, replace=False)
    for i in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (loss_and_grad(pp, samples, tau, emulate=False)[0] - loss_and_grad(pm, samples, tau, emulate=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])
