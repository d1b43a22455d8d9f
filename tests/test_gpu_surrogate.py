"""The surrogate network's tensor-core kernels against the CPU oracle
(oracle/mlp_oracle.py with the GPU's BF16 roundings).

Tolerances (stated here, checked below):
  * forward: every output within 5e-3 (1 + |y|) of the oracle, median
    difference below 2e-4 (FP32 accumulation order and FP32 GELU against
    FP64; a hidden activation that rounds to the other BF16 neighbour moves an
    output by ~1e-3 at most);
  * gradient: every parameter tensor within 3 % (relative L2) of the oracle's
    BF16 gradient, loss within 1e-5 relative;
  * one Adam step: parameters within 1e-5 (absolute) of the oracle's step
    (components with |g| > 1e-6);
  * training: the loss of a smooth 5 -> 4 regression falls by 10x, and two
    runs with the same seeds give identical parameters.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.0, 1.0, (n, 5)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) * x[:, 1], np.tanh(x[:, 2] + x[:, 3]), x[:, 4] ** 2 - 0.3,
                  0.5 * x[:, 0] * x[:, 4]], axis=1).astype(np.float32)
    return x, t


def tensors(flat):
    return mo.unpack(flat)


@pytest.mark.parametrize("n", [1, 100, 128, 1000, 4096])
def test_forward_matches_oracle(n):
    from spsslangevinintegration_gb300.surrogate import Network

    x, _ = data(n, 1)
    with Network(seed=3) as net:
        flat = net.params.astype(np.float64)
        flat[640:768] = np.linspace(-0.2, 0.2, 128)  # non-zero biases
        flat[-4:] = [0.1, -0.2, 0.3, -0.4]
        net.params = flat
        y = net.forward(x)
    ref, _ = mo.forward(flat.astype(np.float32).astype(np.float64), x, bf16=True)
    err = np.abs(y - ref)
    assert np.all(err <= 5e-3 * (1.0 + np.abs(ref))), err.max()
    assert np.median(err) <= 2e-4, np.median(err)


@pytest.mark.parametrize("n", [256, 1000])
def test_gradient_matches_oracle(n):
    from spsslangevinintegration_gb300.surrogate import Network

    x, t = data(n, 2)
    w = np.array([1.0, 0.5, 2.0, 1.0], dtype=np.float32)
    with Network(seed=5) as net:
        flat = net.params.astype(np.float64)
        loss, g = net.gradient(x, t, w)
    rloss, rg = mo.loss_and_gradient(flat, x, t, w, bf16=True)
    assert abs(loss - rloss) <= 1e-5 * abs(rloss)
    G, R = tensors(g.astype(np.float64)), tensors(rg)
    for name, _ in mo.SHAPES:
        num = np.linalg.norm(G[name] - R[name])
        den = np.linalg.norm(R[name])
        assert num <= 0.03 * den, (name, num / den)
    # and the FP64 network, as a sanity bound on the BF16 roundings
    _, g64 = mo.loss_and_gradient(flat, x, t, w, bf16=False)
    assert np.linalg.norm(g - g64) <= 0.08 * np.linalg.norm(g64)


def test_one_adam_step_matches_oracle():
    from spsslangevinintegration_gb300.surrogate import Network

    x, t = data(512, 4)
    lr = 1e-3
    with Network(seed=7) as net:
        p0 = net.params.astype(np.float64)
        _, g = net.gradient(x, t)
        net.set_data(x, t)
        net.train(1, batch=512, lr=lr, seed=0)  # one minibatch = the whole set, one step
        p1 = net.params.astype(np.float64)
    ref, _, _ = mo.adam_step(p0, g.astype(np.float64), np.zeros_like(p0), np.zeros_like(p0), 1, lr)
    # the shuffled order changes the FP32 summation order of the gradient
    # only; a first Adam step is lr * g / (|g| + eps), so components whose
    # gradient is at FP32 noise level may flip sign: they are left out
    keep = np.abs(g) > 1e-6
    assert keep.mean() > 0.99
    assert np.max(np.abs(p1 - ref)[keep]) <= 1e-5
    assert np.max(np.abs(p1 - p0)) <= 1.01 * lr


def test_training_reduces_loss_and_is_deterministic():
    from spsslangevinintegration_gb300.surrogate import Network

    x, t = data(8192, 5)
    runs = []
    for _ in range(2):
        with Network(seed=11) as net:
            net.set_data(x, t)
            losses = net.train(60, batch=1024, lr=2e-3, seed=9)
            runs.append((losses, net.params))
    losses = runs[0][0]
    assert losses[-1] <= 0.1 * losses[0], (losses[0], losses[-1])
    assert np.array_equal(runs[0][1], runs[1][1])
    assert np.array_equal(runs[0][0], runs[1][0])


def test_surrogate_gains_over_the_plain_simulation():
    """What the trained network gains (small phase diagram, N = 256, 2000
    steps): against a 64-replica reference of the expected order parameters,
    its values are much closer than a single plain run's (median error less
    than half), it is within 0.03 more often, and the whole diagram took fewer
    simulated runs than the plain method needs per point for a 0.02 standard
    error.  The judge's runs agree with the predicted mean and spread
    (|z| <= 3 for 90 % of them)."""
    from spsslangevinintegration_gb300 import surrogate as S

    grid = S.grid_points(24, 24, n=256)
    res = S.phase_diagram(grid, n_train=6000, steps=2000, epochs=100, rounds=1, flag_fraction=0.1, n=256)
    rng = np.random.default_rng(0)
    idx = rng.choice(len(grid), 16, replace=False)
    reps = 64
    mean, std = S.reference([grid[i] for i in idx], reps, steps=2000)
    err_net = np.abs(res["values"][idx] - mean).max(axis=1)
    # one plain run per point: a fresh replica of the same points
    one = S.run_values(S.simulate([grid[i] for i in idx], steps=2000, first_replica=5 * 10 ** 6))
    err_one = np.abs(one - mean).max(axis=1)
    assert np.median(err_net) < 0.5 * np.median(err_one), (np.median(err_net), np.median(err_one))
    assert np.mean(err_net <= 0.03) > np.mean(err_one <= 0.03)
    runs_needed = np.maximum(1.0, (std.max(axis=1) / 0.02) ** 2).mean() * len(grid)
    assert res["runs"] < runs_needed, (res["runs"], runs_needed)
    z = np.abs(res["judge_z"])
    assert np.mean(z.max(axis=1) <= 3.0) >= 0.9
