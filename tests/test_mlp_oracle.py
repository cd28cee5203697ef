"""The CPU oracle of the learned-proposal network: its hand-written
backpropagation against central finite differences (unrounded weights,
float64), and its BF16 rounding against exact values."""
import numpy as np

import mlp_ref


def test_bf16_rounding():
    v = mlp_ref.bf16(np.float32([1.0, 1.00390625, 1.01171875, -3.0, 0.0]))
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties to even -> 1
    assert np.array_equal(v, [1.0, 1.0, 1.015625, -3.0, 0.0])


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    n = 40
    X = rng.normal(size=(n, mlp_ref.F))
    y = (rng.random(n) < 0.3).astype(np.uint8)
    p = np.concatenate([rng.normal(0, 0.3, s) for _, s in mlp_ref.SIZES]).astype(np.float64)
    loss, g = mlp_ref.loss_grad(p, X, y, 2.5, rounded=False)
    idx = rng.choice(len(p), 60, replace=False)
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp_ref.loss_grad(pp, X, y, 2.5, rounded=False)[0] - mlp_ref.loss_grad(pm, X, y, 2.5, rounded=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])
