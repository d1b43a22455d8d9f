"""Long runs: the GB300 path's time-averaged order parameter against the FP64
oracle's, statistically.

Over long horizons two trajectories of these systems separate (a neighbour
entering the interaction radius one step earlier is enough), so long runs
are compared as ensembles: for one first-order and one second-order point,
16 independent runs on each side (the GPU with its own noise stream, the
oracle with an independent Philox stream of full 32-bit uniforms), each run's
phase order parameter |<e^{i phi}>| (BinaryObserverSecondOrder.cpp:121-138,
BinaryObserverFirstOrder.cpp:125-142) averaged over the second half of the
run.  Tolerance: the two ensemble means agree within two standard errors of
their difference.  The runs are at a reduced size (N = 1024, density 2,
R = 1), long enough for the angular velocities to relax many times over
(1 / xi_phi = 200 steps for the second-order point, 1 / xi = 2000 steps for
the first-order point).
"""
import concurrent.futures

import numpy as np
import pytest

from helpers import config_initial, config_system, oracle_system

pytestmark = pytest.mark.gpu

SEEDS = 16
N = 1024
DT = 0.005
SE, SRK = 1, 2
LINKED_LIST, LLVERLET = 2, 4


def _oracle_run(p, variant, stepper, x0, steps, seed, sample_every, sample_from, extra):
    from oracle import binding as ob

    orc = oracle_system(p, **extra)
    per = ob.normals_per_particle(p["model"], stepper)
    x = x0.copy()
    samples = []
    for k in range(steps):
        normals = ob.philox_normals(seed, k, 0, p["n"] * per)
        orc.step(stepper, variant, x, (k + 1) * DT, DT, normals)
        if (k + 1) % sample_every == 0 and k + 1 >= sample_from:
            samples.append(ob.order_parameters(p["model"], x)[0])
    orc.close()
    return float(np.mean(samples))


def _compare(model, variant, stepper, steps, extra_gpu, extra_orc):
    from oracle import binding as ob
    from spsslangevinintegration_gb300 import Batch, PRECISION_F32

    p, L = config_system(model, N, density=2.0)
    sample_every, sample_from = 10, steps // 2
    x0 = [config_initial(model, N, L, seed=100 + r) for r in range(SEEDS)]

    systems = []
    for r in range(SEEDS):
        kw = {k: v for k, v in p.items() if k != "flavor"}
        kw.update(precision=PRECISION_F32, variant=variant, flavor=1, seed=7, replica=r, **extra_gpu)
        systems.append(kw)
    with Batch(systems) as b:
        b.set_state(np.concatenate(x0))
        b.run(stepper, 0.0, DT, steps, sample_every=sample_every, sample_from=sample_from)
        st = b.stats()
    gpu = st[:, 0]
    assert np.all(st[:, 4] == (steps - sample_from) // sample_every + 1)

    ob.set_threads(1)
    with concurrent.futures.ThreadPoolExecutor(max_workers=SEEDS) as ex:
        futs = [ex.submit(_oracle_run, p, variant, stepper, x0[r], steps, 5000 + r, sample_every, sample_from,
                          extra_orc) for r in range(SEEDS)]
        orc = np.array([f.result() for f in futs])

    se = np.sqrt(gpu.var(ddof=1) / SEEDS + orc.var(ddof=1) / SEEDS)
    diff = gpu.mean() - orc.mean()
    print("long run model %d: GPU %.4f +- %.4f, oracle %.4f +- %.4f, difference %.4f (2 SE %.4f)" % (
        model, gpu.mean(), gpu.std(ddof=1) / np.sqrt(SEEDS), orc.mean(), orc.std(ddof=1) / np.sqrt(SEEDS), diff,
        2.0 * se))
    assert abs(diff) <= 2.0 * se, (gpu.mean(), orc.mean(), se)
    return gpu, orc


def test_second_order_cell_list_stochastic_euler():
    """Configuration 2's point (second order, density 2, D = 0.1, m = 1,
    v0 = 0.5, sigma = 1, cell list, SE) over 4000 steps."""
    _compare(2, LINKED_LIST, SE, 4000, {}, {})


def test_first_order_verlet_stochastic_runge_kutta():
    """First order (xi = 0.1, sigma = 1, D = 0.1, v0 = 0.5, density 2),
    linked list + Verlet (skin 0.3 R), the strong order 1.5 SRK stepper with
    the complementary force, over 8000 steps."""
    p, _ = config_system(1, N, density=2.0)
    r_max = 1.3 * p["rho"]
    extra = dict(r_max=r_max, nc_verlet=int(1.0 / r_max))
    _compare(1, LLVERLET, SRK, 8000, extra, extra)
