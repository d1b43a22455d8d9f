"""The surrogate network's CPU oracle (oracle/mlp_oracle.py), without a GPU:
its FP64 gradient against central finite differences, its BF16 rounding
against exact cases, and its Adam step against the textbook update."""
import numpy as np

from oracle import mlp_oracle as mo


def test_parameter_count_matches_header():
    assert mo.NPARAMS == 34308


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 3.0e38])
    got = mo.to_bf16(x)
    # ties to even: 1 + 2^-8 -> 1, 1 + 3 * 2^-8 -> 1 + 2^-6
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -7 and got[3] == 1.0 + 2 ** -6
    assert got[4] == -2.5 and got[5] == 0.0
    assert np.all(np.abs(got[:6] - x[:6]) <= np.abs(x[:6]) * 2 ** -8)


def test_fp64_gradient_against_finite_differences():
    rng = np.random.default_rng(0)
    flat = mo.init_params(1)
    flat = flat + rng.normal(0.0, 0.05, flat.size)  # non-zero biases too
    x = rng.normal(size=(16, 5))
    t = rng.normal(size=(16, 4))
    w = np.array([1.0, 0.5, 2.0, 1.5])
    loss, g = mo.loss_and_gradient(flat, x, t, w, bf16=False)
    assert np.isfinite(loss)
    idx = rng.choice(flat.size, 60, replace=False)
    idx = np.concatenate([idx, [0, 639, 640, 767, 34303, 34307]])  # W1, b1 ends, W4, b4
    h = 1e-6
    for i in idx:
        e = np.zeros_like(flat)
        e[i] = h
        lp, _ = mo.loss_and_gradient(flat + e, x, t, w, bf16=False)
        lm, _ = mo.loss_and_gradient(flat - e, x, t, w, bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_gradient_close_to_fp64():
    rng = np.random.default_rng(2)
    flat = mo.init_params(3)
    x = rng.normal(size=(256, 5))
    t = rng.normal(size=(256, 4))
    _, g64 = mo.loss_and_gradient(flat, x, t, bf16=False)
    _, g16 = mo.loss_and_gradient(flat, x, t, bf16=True)
    assert np.linalg.norm(g16 - g64) <= 0.05 * np.linalg.norm(g64)


def test_adam_step():
    p = np.array([1.0, -2.0])
    g = np.array([0.5, -0.25])
    p1, m1, m2 = mo.adam_step(p, g, np.zeros(2), np.zeros(2), 1, 0.1)
    # first step: m_hat = g, v_hat = g^2 -> step = lr * sign(g)
    np.testing.assert_allclose(p1, p - 0.1 * np.sign(g) * np.abs(g) / (np.abs(g) + 1e-8), rtol=1e-12)
