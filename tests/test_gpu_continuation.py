"""Parameter continuation (SimulationEngineFirstOrderPtr.cpp:167-217).

* One system, the reference's own setting (first order, global field by the
  dispatch rule, RK4, FP64): three stages in alpha, each from the previous
  stage's end state, against the FP64 oracle run through the same stages
  (1e-9 relative after 150 steps).
* Replicas batched on the GPU path: every replica's end states equal the same
  replica continued alone (bit for bit: cell lists), and the stage statistics
  count the samples of each stage.
"""
import numpy as np
import pytest

from helpers import initial, oracle_system, params, per_component_close

pytestmark = pytest.mark.gpu


def test_single_system_continuation_matches_oracle():
    from spsslangevinintegration_gb300 import continuation as C

    n, dt, span = 300, 0.01, 0.5
    base = dict(model=1, n=n, rho=0.8, precision=0, variant=0, flavor=1, v0=0.01, xi=0.1, sigma=1.0, D_phi=0.0)
    alphas = (0.55, 0.5, 0.45)
    stages = [dict(base, alpha=a) for a in alphas]
    x0 = initial(1, n, 31)
    ends, series = C.continuation(x0, stages, span, dt, stepper=0, record_every=10)
    assert len(ends) == 3 and all(len(s) == 5 for s in series)
    x = x0.copy()
    for a, end in zip(alphas, ends):
        orc = oracle_system(dict(model=1, n=n, rho=0.8, flavor=1, v0=0.01, xi=0.1, sigma=1.0, alpha=a))
        t = 0.0
        for _ in range(int(round(span / dt))):
            t += dt
            orc.step(0, 0, x, t, dt)
        orc.close()
        per_component_close(end, x, 4, 1e-9, "continuation stage alpha=%g" % a)


def test_replica_continuation_equals_single_runs():
    from spsslangevinintegration_gb300 import continuation as C

    n = 2048
    p = params(2, n)
    kw = {k: p[k] for k in ("v0", "xi_r", "D_r", "xi_phi", "D_phi", "sigma") if k in p}
    base = dict(model=2, n=n, rho=p["rho"], precision=1, variant=2, seed=9, **kw)
    stages = [dict(base, alpha=a) for a in (0.0, 0.2)]
    states = [initial(2, n, 40 + r) for r in range(3)]
    ends, stats = C.continuation_replicas(states, stages, 0.1, 0.005, stepper=1, sample_every=5, burn_in=5)
    assert len(ends) == 2 and stats[0].shape == (3, 5)
    assert np.all(stats[0][:, 4] == 4) and np.all(stats[1][:, 4] == 4)
    for r in range(3):
        single, _ = C.continuation(states[r], [dict(s, replica=r) for s in stages], 0.1, 0.005, stepper=1,
                                   record_every=20)
        for k in range(2):
            assert np.array_equal(ends[k][r], single[k])
