"""Adaptive Dormand-Prince 5(4) with dense output (the reference's odeint
path) on the GPU against the same method over the FP64 oracle's right-hand
side (oracle/dopri5_oracle.py): the same number of accepted steps and the
observer states within 1e-9 relative (the right-hand sides agree to 1e-12;
the step sequence is identical unless an error norm lands within rounding of
the acceptance bound)."""
import numpy as np
import pytest

from helpers import gpu_context, initial, oracle_system, per_component_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rho,variant", [(0.8, 0), (0.3, 1)])
def test_dopri5_matches_oracle(rho, variant):
    from oracle import dopri5_oracle as dp

    n = 300
    p = dict(model=1, n=n, rho=rho, flavor="ptr", v0=0.02, xi=0.1, sigma=1.0, alpha=0.3)
    x0 = initial(1, n, 17, omega=0.8)
    got = []
    with gpu_context(p, precision=0, variant=variant) as ctx:
        ctx.set_state(x0)
        steps = ctx.integrate_dopri5(0.0, 2.0, 0.1, 1e-6, 1e-6, observer=lambda x, t: got.append((t, x)))
        final = ctx.get_state()
    orc = oracle_system(p)
    times, states, ref_steps = dp.integrate(orc, variant, x0, 0.0, 2.0, 0.1, 1e-6, 1e-6)
    orc.close()
    assert steps == ref_steps
    assert len(got) == len(times) == 21
    for (t, x), tr, xr in zip(got, times, states):
        assert abs(t - tr) <= 1e-12
        per_component_close(x, xr, 4, 1e-9, "dopri5 at t=%g" % t)
    per_component_close(final, states[-1], 4, 1e-9, "dopri5 end state")


def test_dopri5_observer_can_stop():
    p = dict(model=1, n=200, rho=0.8, flavor="ptr", v0=0.02, xi=0.1, sigma=1.0)
    seen = []
    with gpu_context(p, precision=0) as ctx:
        ctx.set_state(initial(1, 200, 3))
        ctx.integrate_dopri5(0.0, 5.0, 0.5, observer=lambda x, t: seen.append(t) or t >= 1.0)
    assert seen == [0.0, 0.5, 1.0]


def test_dopri5_on_a_closed_form_solution():
    """The GPU integrator on uncoupled particles without friction, whose
    trajectories are known in closed form (tests/test_dopri5_method.py):
    within 10 x the requested tolerance at every observer time."""
    from test_dopri5_method import _closed_form, closed_form_case

    p, x0 = closed_form_case()
    got = []
    with gpu_context(p, precision=0, variant=1) as ctx:
        ctx.set_state(x0)
        ctx.integrate_dopri5(0.0, 3.0, 0.25, 1e-8, 1e-8, observer=lambda x, t: got.append((t, x)))
    assert len(got) == 13
    for t, x in got:
        exact = _closed_form(x0, t, p["v0"])
        assert np.max(np.abs(x - exact) / (1.0 + np.abs(exact))) <= 1e-7, t
