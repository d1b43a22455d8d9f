"""Strong order of the stochastic Runge-Kutta (order 1.5 stochastic Taylor)
steppers, measured on the FP64 oracle.

The second-order model's SRK scheme has no reference code: it is derived for
additive noise from Kloeden & Platen sec. 10.4 (the source the reference's
first-order scheme cites, Steppers/StochasticRungeKuttaStepperPtr.hpp:17-20)
in oracle/spss_oracle.c (spo_srk_step).  Matching a transcription of the same
derivation proves nothing about the scheme, so this test measures its order:
strong error at T against a solution with dt/16 on the SAME Brownian path,
over four halvings of dt, with every pair inside the interaction radius so
the drift is smooth (a particle entering or leaving the radius makes the
drift jump and caps any scheme at a lower order).

Brownian path: the fine steps draw (U1, U2) per noise component; two
consecutive steps of length h combine into one of length 2h by
    dW = dW_a + dW_b,   dZ = dZ_a + dZ_b + h dW_a
(dZ = int (W(s) - W(t_n)) ds over the step), and (U1, U2) of the coarse step
follow from dW = U1 sqrt(2h), dZ = (2h)^1.5 (U1 + U2 / sqrt 3) / 2.

Stated bars: the fitted slope of log error against log dt is >= 1.3 for the
SRK scheme of both models (the reference's first-order scheme,
StochasticRungeKuttaStepperPtr.hpp:52-71, is the control), and the
Euler-Maruyama scheme on the same paths shows order 1 (slope within
[0.8, 1.2]); a scheme missing the dt^2 / 2 drift correction, planted on the
CPU by zeroing the complementary force, falls to order 1 as well.
"""
import numpy as np
import pytest

from oracle import binding as ob

T = 0.5
LEVELS = 4          # dt = T/8, T/16, T/32, T/64; reference T/128
COARSE = 8


def _system(model, n):
    rho = 0.75  # > sqrt(2)/2: every pair of the unit box is in range
    if model == 1:
        return ob.System(1, n, rho, v0=0.5, xi=0.5, sigma=2.0, D_phi=0.5, alpha=0.3, flavor=1)
    return ob.System(2, n, rho, v0=0.5, xi_r=1.0, D_r=0.05, xi_phi=1.0, D_phi=0.5, sigma=2.0, alpha=0.3, flavor=1)


def _initial(model, n, seed):
    rng = np.random.default_rng(seed)
    s = 4 if model == 1 else 6
    x = np.zeros((n, s))
    x[:, 0], x[:, 1] = rng.random(n), rng.random(n)
    if model == 1:
        x[:, 2], x[:, 3] = rng.uniform(-np.pi, np.pi, n), rng.normal(0.0, 1.0, n)
    else:
        x[:, 2], x[:, 3] = rng.normal(0.0, 0.3, n), rng.normal(0.0, 0.3, n)
        x[:, 4], x[:, 5] = rng.uniform(-np.pi, np.pi, n), rng.normal(0.0, 1.0, n)
    return x.reshape(-1)


def _coarsen(u, h):
    """(steps, n, k, 2) normals of steps of length h -> (steps/2, n, k, 2) of length 2h."""
    w = u[..., 0] * np.sqrt(h)
    z = 0.5 * h ** 1.5 * (u[..., 0] + u[..., 1] / np.sqrt(3.0))
    W = w[0::2] + w[1::2]
    Z = z[0::2] + z[1::2] + h * w[0::2]
    H = 2.0 * h
    U1 = W / np.sqrt(H)
    U2 = np.sqrt(3.0) * (2.0 * Z / H ** 1.5 - U1)
    return np.stack([U1, U2], axis=-1)


def _paths(model, n, seed):
    """Normals of every level, finest (reference) first."""
    k = 1 if model == 1 else 3
    steps = COARSE * 2 ** LEVELS
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(steps, n, k, 2))
    out = [u]
    h = T / steps
    for _ in range(LEVELS):
        u = _coarsen(u, h)
        h *= 2.0
        out.append(u)
    return out  # out[j]: steps / 2^j steps of length T / steps * 2^j


def _integrate(model, n, x0, normals, stepper, plant_no_correction=False):
    sys = _system(model, n)
    x = x0.copy()
    steps = normals.shape[0]
    dt = T / steps
    for m in range(steps):
        u = normals[m]
        if stepper == ob.SE:
            # Euler-Maruyama on the same path: one normal per component, U1.
            flat = u[..., 0].reshape(-1)
            if model == 2:
                flat = np.stack([u[:, 0, 0], u[:, 1, 0], u[:, 2, 0]], axis=1).reshape(-1)
            sys.step(ob.SE, ob.ALL_PAIRS, x, (m + 1) * dt, dt, flat)
        else:
            if plant_no_correction:
                _srk_without_complementary_force(sys, model, x, dt, u)
            else:
                sys.step(ob.SRK, ob.ALL_PAIRS, x, (m + 1) * dt, dt, u.reshape(-1))
        if model == 2:
            # The second-order engine wraps positions after every step
            # (SimulationEngineSecondOrder.cpp:136); its ClassA distance
            # (PeriodicBoundaryConditions.cpp:26-38) assumes wrapped positions.
            ob.apply_pbc(2, x)
    sys.close()
    return x


def _srk_without_complementary_force(sys, model, x, dt, u):
    """The SRK step with the complementary force C left out of the dt^2/2
    drift correction of omega: the oracle's step minus (C dt^2 / 2)."""
    s = 4 if model == 1 else 6
    sys.step(ob.SRK, ob.ALL_PAIRS, x, 0.0, dt, u.reshape(-1))
    c = sys.complementary_force()
    x.reshape(-1, s)[:, s - 1] -= 0.5 * c * dt * dt


def _slope(model, stepper, plant=False, n=48, paths=4):
    errs = np.zeros(LEVELS)
    for p in range(paths):
        x0 = _initial(model, n, 10 + p)
        normals = _paths(model, n, 100 + p)
        ref = _integrate(model, n, x0, normals[0], ob.SRK)
        for j in range(1, LEVELS + 1):
            got = _integrate(model, n, x0, normals[j], stepper, plant)
            d = (got - ref).reshape(n, -1)
            d[:, :2] -= np.round(d[:, :2])
            errs[j - 1] += np.mean(d ** 2)
    errs = np.sqrt(errs / paths)
    dts = T / (COARSE * 2 ** LEVELS) * 2.0 ** np.arange(1, LEVELS + 1)
    slope = np.polyfit(np.log(dts), np.log(errs), 1)[0]
    return slope, errs


@pytest.mark.parametrize("model", [1, 2])
def test_srk_strong_order_at_least_1_3(model):
    slope, errs = _slope(model, ob.SRK)
    assert slope >= 1.3, (slope, errs)
    assert np.all(np.diff(errs) > 0), errs  # the error grows with dt at every level


@pytest.mark.parametrize("model", [1, 2])
def test_euler_maruyama_on_the_same_paths_is_order_one(model):
    slope, errs = _slope(model, ob.SE)
    assert 0.8 <= slope <= 1.2, (slope, errs)


@pytest.mark.parametrize("model", [1, 2])
def test_planted_missing_correction_drops_to_order_one(model):
    slope, errs = _slope(model, ob.SRK, plant=True)
    assert slope <= 1.2, (slope, errs)
