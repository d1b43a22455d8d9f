"""The GPU's stochastic Runge-Kutta steppers are the scheme whose strong order
tests/test_srk_strong_order.py measures on the oracle: at every step size of
that test (dt = T/8 .. T/64, T = 0.5; all pairs in range), a run on the GPU
matches the oracle replaying the GPU's normals — FP64 path within 1e-12
relative per component, FP32 path within 1e-6 — with positions wrapped on
the GPU after every step by spss_apply_pbc, as the second-order engine wraps
them (SimulationEngineSecondOrder.cpp:136,
PeriodicBoundaryConditions.cpp:127-135)."""
import numpy as np
import pytest

from helpers import state_err

pytestmark = pytest.mark.gpu

T = 0.5
SRK, ALL_PAIRS = 2, 1


def _params(model):
    if model == 1:
        return dict(v0=0.5, xi=0.5, sigma=2.0, D_phi=0.5, alpha=0.3)
    return dict(v0=0.5, xi_r=1.0, D_r=0.05, xi_phi=1.0, D_phi=0.5, sigma=2.0, alpha=0.3)


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


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)])
@pytest.mark.parametrize("model", [1, 2])
def test_gpu_srk_matches_oracle_at_every_step_size(model, precision, tol):
    from oracle import binding as ob
    from spsslangevinintegration_gb300 import Context

    n, s = 48, 4 if model == 1 else 6
    x0 = _initial(model, n, 3)
    for steps in (8, 16, 32, 64):
        dt = T / steps
        x = x0.copy()
        orc = ob.System(model, n, 0.75, flavor=1, **_params(model))
        with Context(model, n, 0.75, precision=precision, variant=ALL_PAIRS, flavor=1, seed=9, **_params(model)) as ctx:
            ctx.set_state(x0)
            for k in range(steps):
                normals = ctx.noise(SRK, k)
                ctx.step(SRK, (k + 1) * dt, dt)
                orc.step(SRK, ALL_PAIRS, x, (k + 1) * dt, dt, normals)
                if model == 2:
                    ctx.apply_pbc()
                    ob.apply_pbc(2, x)
            got = ctx.get_state()
        orc.close()
        err = state_err(got, x, s).max()
        print("SRK model %d precision %d, %d steps: error %.3e" % (model, precision, steps, err))
        assert err <= tol, (steps, err)
        if model == 2:
            pos = got.reshape(n, s)[:, :2]
            assert np.all((pos >= 0.0) & (pos < 1.0))
