"""Parity at the benchmark workloads' own sizes, against the FP64 oracle on
identical noise (the oracle replays the normals the GPU drew).

Tolerances (stated here, checked below):
  * the large system (second order, N = 4,194,304, density 2, Verlet skin
    0.3 R, SRK, dt = 0.005): one step of the FP32 path from every state of a
    20-step FP64 trajectory agrees with the oracle's step in EVERY component
    of every particle within 1e-5 relative (floor 1e-5 of the component's
    largest magnitude); the free-running 40-step FP32 trajectory (one Verlet
    rebuild on each side's own trigger): median per-particle error <= 1e-6,
    99.9 % <= 1e-5, at most 64 particles (0.0015 %) above 1e-4 and none above
    5e-2 (the tail bound is derived in test_n4m_srk_verlet_forty_free_steps), and
    the same Verlet rebuild steps;
  * the cell-list system (second order, N = 65,536, density 2, cell list, SE):
    100 steps, every particle within 1e-3 relative, median <= 1e-5;
  * the all-pairs system (first order, N = 1000, density 1, all pairs, RK4, FP64):
    the full 1000 steps against the oracle within 1e-12 relative per
    component (floor 1e-12 of the component's scale), also after 100 steps.
"""
import os

import numpy as np
import pytest

from helpers import config_initial, config_system, gpu_context, oracle_system, state_err

pytestmark = pytest.mark.gpu

F32, F64 = 1, 0
RK4, SE, SRK = 0, 1, 2
ALL_PAIRS, LINKED_LIST, LLVERLET = 1, 2, 4
DT = 0.005


def _threads():
    from oracle import binding as ob

    ob.set_threads(os.cpu_count() or 1)


def _n4m_srk_verlet(n=4194304):
    p, L = config_system(2, n, density=2.0)
    r_max = 1.3 * p["rho"]
    return p, L, r_max, int(1.0 / r_max)


def test_n4m_srk_verlet_each_step_matches_fp64_oracle_everywhere():
    """Along a 20-step FP64 oracle trajectory of the benchmark system, the
    FP32 step from the oracle's state agrees with the oracle's step for every
    particle (Verlet lists at capacity 40 with 16-bit offsets, the overflow
    fallback, tile staging at the real density): max error <= 1e-5."""
    _threads()
    p, L, r_max, nc_v = _n4m_srk_verlet()
    n = p["n"]
    x = config_initial(2, n, L, seed=0)
    orc = oracle_system(p, r_max=r_max, nc_verlet=nc_v)
    worst = []
    with gpu_context(p, precision=F32, variant=LLVERLET, r_max=r_max, nc_verlet=nc_v, seed=0) as ctx:
        for k in range(20):
            ctx.set_state(x)
            ctx.step_counter = k
            normals = ctx.noise(SRK, k)
            ctx.step(SRK, (k + 1) * DT, DT)
            got = ctx.get_state()
            orc.step(SRK, LLVERLET, x, (k + 1) * DT, DT, normals)
            err = state_err(got, x, 6)
            worst.append(float(err.max()))
            assert np.all(np.isfinite(got))
    print("N=4194304 SRK Verlet, one step from each oracle state: worst error per step", worst)
    assert max(worst) <= 1e-5, worst


def test_n4m_srk_verlet_forty_free_steps():
    """The free-running FP32 trajectory of the benchmark system against the
    FP64 oracle on the same normals, 40 steps, lists rebuilt on each side's
    own displacement trigger (the first trigger fires after about 31 steps).

    Tail bound: the two trajectories differ by ~1e-12 of the box in position
    after 40 steps, so a pair whose separation crosses the cutoff within that
    distance of a step boundary is in range on one side and out on the other
    for one step (~1e-6 of the ~9e4 cutoff crossings per step).  That moves
    the angular velocity of its two particles by at most dt sigma / N_i
    (<= 5e-3 with the zero-filled derivative of an isolated particle), i.e.
    a relative error below 5e-2 of the angular velocity's scale; the pair
    sum of a neighbour then moves by O(dt) of that.  A handful of such
    events is expected in 40 steps, each touching a few particles."""
    _threads()
    p, L, r_max, nc_v = _n4m_srk_verlet()
    n = p["n"]
    x0 = config_initial(2, n, L, seed=0)
    x = x0.copy()
    orc = oracle_system(p, r_max=r_max, nc_verlet=nc_v)
    rebuild_gpu, rebuild_orc = [], []
    with gpu_context(p, precision=F32, variant=LLVERLET, r_max=r_max, nc_verlet=nc_v, seed=0) as ctx:
        ctx.set_state(x0)
        for k in range(40):
            normals = ctx.noise(SRK, k)
            ctx.step(SRK, (k + 1) * DT, DT)
            orc.step(SRK, LLVERLET, x, (k + 1) * DT, DT, normals)
            acc_g, flag_g, _ = ctx.verlet_state()
            rebuild_gpu.append(flag_g)
            rebuild_orc.append(orc.should_update_lists)
            assert acc_g == pytest.approx(orc.accumulated_displacement, rel=1e-5, abs=1e-12)
        got = ctx.get_state()
    err = state_err(got, x, 6).max(axis=1)
    print("N=4194304 SRK Verlet, 40 free steps: median %.3e, 99.9%% %.3e, max %.3e, above 1e-4: %d, rebuild flags %s / %s" % (
        np.median(err), np.quantile(err, 0.999), err.max(), np.count_nonzero(err > 1e-4), rebuild_gpu, rebuild_orc))
    assert rebuild_gpu == rebuild_orc
    assert any(rebuild_gpu)
    assert np.median(err) <= 1e-6
    assert np.quantile(err, 0.999) <= 1e-5
    assert int(np.count_nonzero(err > 1e-4)) <= 64
    assert err.max() <= 5e-2


def test_n65536_cell_list_se_hundred_steps():
    """The cell-list system (N = 65,536, density 2, cell list, SE,
    D = 0.1, m = 1, v0 = 0.5): 100 steps, every particle within 1e-3."""
    _threads()
    n = 65536
    p, L = config_system(2, n, density=2.0)
    x0 = config_initial(2, n, L, seed=0)
    x = x0.copy()
    orc = oracle_system(p)
    with gpu_context(p, precision=F32, variant=LINKED_LIST, seed=0) as ctx:
        ctx.set_state(x0)
        for k in range(100):
            normals = ctx.noise(SE, k)
            ctx.step(SE, (k + 1) * DT, DT)
            orc.step(SE, LINKED_LIST, x, (k + 1) * DT, DT, normals)
        got = ctx.get_state()
    err = state_err(got, x, 6).max(axis=1)
    print("N=65536 cell list SE, 100 steps: median %.3e, max %.3e" % (np.median(err), err.max()))
    assert err.max() <= 1e-3, float(err.max())
    assert np.median(err) <= 1e-5


def test_n1000_all_pairs_rk4_thousand_steps_fp64():
    """The all-pairs system (first order, N = 1000, density 1 -> rho = 1/sqrt(1000)
    of the unit box, all pairs called directly, D = 0, v0 = 0.1, sigma = 1,
    xi = 0.1, RK4, dt = 0.01): the FP64 path over the whole 1000 steps
    against the oracle (the reference's EvaluateInteractionsWithAllPairs,
    ParticleSystemFirstOrder.cpp:162-228, and RungeKutta4Stepper::DoStep,
    RungeKutta4Stepper.cpp:29-64).  The paths differ only in the device
    sin/cos and the all-pairs summation order (ulp-level per step)."""
    _threads()
    n, dt = 1000, 0.01
    p, L = config_system(1, n, density=1.0, v0=0.1, D=0.0)
    x = config_initial(1, n, L, seed=0)
    orc = oracle_system(p)
    with gpu_context(p, precision=F64, variant=ALL_PAIRS, seed=0) as ctx:
        ctx.set_state(x)
        for k in range(1000):
            ctx.step(RK4, (k + 1) * dt, dt)
            orc.step(RK4, ALL_PAIRS, x, (k + 1) * dt, dt)
            if k + 1 == 100:
                err100 = float(state_err(ctx.get_state(), x, 4).max())
        got = ctx.get_state()
    err = float(state_err(got, x, 4).max())
    print("N=1000 all pairs RK4: error after 100 steps %.3e, after 1000 steps %.3e" % (err100, err))
    assert err100 <= 1e-12, err100
    assert err <= 1e-12, err
