"""CPU checks of the FP64 network oracle (oracle/mlp_oracle.py): its gradient
agrees with central finite differences, and BF16 rounding matches the
round-to-nearest-even definition."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_round():
    x = np.array([1.0, 1.00390625, 1.0 + 2 ** -8 + 2 ** -9, -3.14159, 65504.0], np.float32)
    r = mo.bf16_round(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # tie: rounds to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    F, B = 10, 16
    n = mo.H * F + mo.H * mo.H + 3 * mo.H + 1
    # bf16-representable weights so that rounding does not move under +-h
    p = mo.bf16_round(rng.normal(0, 0.1, n).astype(np.float32))
    X = rng.integers(0, 2, (B, F)).astype(np.float64)
    X[:, -1] = 1.0
    t = rng.normal(0, 1, B)
    loss, g, _ = mo.loss_and_grad(p, X, t)
    W_end = mo.H * F + mo.H * mo.H
    for k in list(rng.choice(np.arange(W_end, n), 12, replace=False)):  # biases and w3 (not rounded)
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mo.loss_and_grad(pp, X, t)[0] - mo.loss_and_grad(pm, X, t)[0]) / (2 * h)
        assert abs(fd - g[k]) < 1e-6 + 1e-5 * abs(fd)
    # weight entries: perturb by exactly one bf16 step around a representable value
    for k in list(rng.choice(np.arange(0, W_end), 6, replace=False)):
        v = p[k]
        step = 2.0 ** (np.floor(np.log2(abs(v))) - 7) if v != 0 else 2.0 ** -20
        pp, pm = p.copy(), p.copy()
        pp[k] = v + step
        pm[k] = v - step
        fd = (mo.loss_and_grad(pp, X, t)[0] - mo.loss_and_grad(pm, X, t)[0]) / (2 * step)
        assert abs(fd - g[k]) < 1e-3 * (1 + abs(fd))
