"""GB300 fast path (fixed-point positions, FP32 pair and stage arithmetic)
against the FP64 oracle on identical noise (the oracle replays the normals the
GPU drew), plus size-independent properties at the benchmark sizes.

Tolerances (stated here, checked below):
  * one step from the same FP64 state: every component within 1e-5 relative
    (floor: 1e-5 of the component's largest magnitude); the step increments
    themselves within 2e-4 of the component's largest increment;
  * 50 steps: 99.9% of particles within 1e-3 relative (a neighbour crossing
    the cutoff earlier or later on the diverging FP32 trajectory moves single
    particles by more, as it would between two FP64 codes with different
    summation orders);
  * neighbour sets: exact (cutoff decisions inside an FP32 guard band are
    recomputed in FP64 from the 64-bit fixed-point positions).
"""
import numpy as np
import pytest

from helpers import gpu_context, initial, min_image, oracle_system, params

pytestmark = pytest.mark.gpu

F32 = 1


def state_err(got, ref, s):
    got, ref = got.reshape(-1, s), ref.reshape(-1, s)
    d = got - ref
    d[:, :2] = min_image(d[:, :2])
    scale = np.abs(ref).max(axis=0)
    scale[:2] = 1.0
    return np.abs(d) / (np.abs(ref) + scale)


def run_pair(model, variant, stepper, n, steps, seed=3, skin=0.3, **kw):
    p = params(model, n, **kw)
    x0 = initial(model, n, seed, v=p["v0"])
    r_max = (1.0 + skin) * p["rho"]
    nc_v = int(1.0 / r_max)
    ctx = gpu_context(p, precision=F32, variant=variant, r_max=r_max, nc_verlet=nc_v, seed=11)
    orc = oracle_system(p, r_max=r_max, nc_verlet=nc_v)
    ctx.set_state(x0)
    x = x0.copy()
    t, dt = 0.0, 0.005
    for k in range(steps):
        t += dt
        normals = ctx.noise(stepper, k)
        ctx.step(stepper, t, dt)
        orc.step(stepper, variant, x, t, dt, normals)
    got = ctx.get_state()
    ctx.close()
    return x0, got, x


CASES = [(2, 2, 1), (2, 2, 2), (2, 4, 1), (2, 4, 2), (2, 1, 2), (1, 4, 2), (1, 2, 1), (1, 4, 1)]


@pytest.mark.parametrize("model,variant,stepper", CASES)
def test_one_step_matches_fp64_oracle(model, variant, stepper):
    n = 400 if variant == 1 else 8192
    x0, got, ref = run_pair(model, variant, stepper, n, 1)
    s = 4 if model == 1 else 6
    assert state_err(got, ref, s).max() <= 1e-5
    inc_got, inc_ref = (got - x0).reshape(-1, s), (ref - x0).reshape(-1, s)
    inc_got[:, :2], inc_ref[:, :2] = min_image(inc_got[:, :2]), min_image(inc_ref[:, :2])
    for c in range(s):
        scale = np.abs(inc_ref[:, c]).max()
        assert np.abs(inc_got[:, c] - inc_ref[:, c]).max() <= 2e-4 * scale + 1e-12, c


@pytest.mark.parametrize("model,variant,stepper", [(2, 4, 2), (2, 2, 1), (1, 4, 2)])
def test_fifty_steps_track_fp64_oracle(model, variant, stepper):
    x0, got, ref = run_pair(model, variant, stepper, 4096, 50)
    s = 4 if model == 1 else 6
    err = state_err(got, ref, s).max(axis=1)
    assert np.quantile(err, 0.999) <= 1e-3
    assert np.median(err) <= 1e-5


def test_isolated_particle_torque_derivative_is_zero_like_reference():
    """SE/SRK zero-fill the derivative, so a particle without neighbours gets
    omega += noise only (StochasticEulerStepper.hpp:36, StochasticRungeKuttaStepperPtr.hpp:43)."""
    x0, got, ref = run_pair(2, 2, 1, 200, 1, density=0.05)  # sparse: many isolated particles
    assert state_err(got, ref, 6).max() <= 1e-5


def test_graph_steps_equal_single_steps_bitwise():
    p = params(2, 20000)
    x0 = initial(2, 20000, 5, v=p["v0"])
    r_max = 1.3 * p["rho"]
    out = []
    for use_graph in (False, True):
        with gpu_context(p, precision=F32, variant=4, r_max=r_max, nc_verlet=int(1 / r_max), seed=3) as ctx:
            ctx.set_state(x0)
            if use_graph:
                ctx.steps(2, 0.0, 0.005, 120)
            else:
                for k in range(120):
                    ctx.step(2, (k + 1) * 0.005, 0.005)
            out.append((ctx.get_state(), ctx.verlet_state(), ctx.step_counter))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]
    assert out[0][2] == out[1][2] == 120


def test_verlet_equals_linked_list_at_benchmark_size():
    """Benchmark size (N = 4,194,304): the Verlet path (skin 0.3 R, rebuilt on the displacement
    trigger) and the per-step cell list see the same neighbour sets, so the
    trajectories agree to FP32 summation-order differences."""
    n = 4194304
    p = params(2, n)
    x0 = initial(2, n, 9, v=p["v0"])
    r_max = 1.3 * p["rho"]
    res = {}
    for variant in (2, 4):
        with gpu_context(p, precision=F32, variant=variant, r_max=r_max, nc_verlet=int(1 / r_max), seed=5) as ctx:
            ctx.set_state(x0)
            ctx.steps(2, 0.0, 0.005, 20)
            res[variant] = ctx.get_state()
            assert np.all(np.isfinite(res[variant]))
    err = state_err(res[4], res[2], 6).max(axis=1)
    assert np.quantile(err, 0.9999) <= 1e-4


def test_step_host_matches_device_steps():
    p = params(2, 5000)
    x0 = initial(2, 5000, 2, v=p["v0"])
    with gpu_context(p, precision=F32, variant=2, seed=8) as a, gpu_context(p, precision=F32, variant=2, seed=8) as b:
        a.set_state(x0)
        host = x0.copy()
        for k in range(5):
            a.step(1, (k + 1) * 0.005, 0.005)
            b.step_host(1, host, (k + 1) * 0.005, 0.005)
        np.testing.assert_array_equal(a.get_state(), host)


def test_step_host_on_pinned_array_equals_pageable():
    """spss_step_host on a page-locked mapped array (PinnedArray, used in
    place) and on a pageable array (registered by the library) give the same
    bits."""
    from spsslangevinintegration_gb300 import PinnedArray

    p = params(2, 5000)
    x0 = initial(2, 5000, 3, v=p["v0"])
    with gpu_context(p, precision=F32, variant=2, seed=8) as a, gpu_context(p, precision=F32, variant=2, seed=8) as b:
        host = x0.copy()
        with PinnedArray(x0.size) as pin:
            pin.array[:] = x0
            for k in range(4):
                a.step_host(1, host, (k + 1) * 0.005, 0.005)
                b.step_host(1, pin.array, (k + 1) * 0.005, 0.005)
            np.testing.assert_array_equal(pin.array, host)


def test_upload_download_round_trip():
    p = params(2, 3000)
    x0 = initial(2, 3000, 4, v=p["v0"])
    x0[::6] += 3.0  # positions outside the box keep their image
    x0[4::6] += 25.0  # phases beyond 2 pi keep their turns
    with gpu_context(p, precision=F32, variant=2) as ctx:
        ctx.set_state(x0)
        back = ctx.get_state().reshape(-1, 6)
        ref = x0.reshape(-1, 6)
        np.testing.assert_allclose(back[:, :2], ref[:, :2], rtol=0, atol=1e-15 * 8)
        np.testing.assert_allclose(back[:, 4], ref[:, 4], rtol=0, atol=1e-8)
        np.testing.assert_allclose(back[:, [2, 3, 5]], ref[:, [2, 3, 5]], rtol=1e-7)


def test_deterministic_and_noise_reproducible():
    p = params(2, 10000)
    x0 = initial(2, 10000, 6, v=p["v0"])
    r_max = 1.3 * p["rho"]
    outs = []
    for _ in range(2):
        with gpu_context(p, precision=F32, variant=4, r_max=r_max, nc_verlet=int(1 / r_max), seed=21) as ctx:
            ctx.set_state(x0)
            ctx.steps(2, 0.0, 0.005, 30)
            outs.append(ctx.get_state())
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("model,variant,stepper,n,density", [
    (2, 2, 1, 1, 2.0), (2, 2, 1, 2, 2.0), (2, 4, 2, 7, 2.0), (1, 2, 2, 5, 0.5), (1, 4, 1, 40, 2.0),
    (2, 2, 2, 64, 8.0), (1, 4, 2, 64, 2.0)])
def test_tiny_systems_match_fp64_oracle(model, variant, stepper, n, density):
    """Systems of 1 to 64 particles: one to six cells per side, so stencils
    wrap onto the same cells several times (as the reference's do) and Verlet
    lists can exceed their capacity (the step then scans the stencil)."""
    p = params(model, n, density=density)
    x0 = initial(model, n, 31 + n, v=p["v0"])
    r_max = 1.3 * p["rho"]
    nc_v = max(1, int(1.0 / r_max))
    s = 4 if model == 1 else 6
    with gpu_context(p, precision=F32, variant=variant, r_max=r_max, nc_verlet=nc_v, seed=29) as ctx:
        orc = oracle_system(p, r_max=r_max, nc_verlet=nc_v)
        ctx.set_state(x0)
        x = x0.copy()
        for k in range(3):
            normals = ctx.noise(stepper, k)
            ctx.step(stepper, (k + 1) * 0.005, 0.005)
            orc.step(stepper, variant, x, (k + 1) * 0.005, 0.005, normals)
        got = ctx.get_state()
    assert np.all(np.isfinite(got))
    assert state_err(got, x, s).max() <= 1e-5


def band_pairs(model, seed):
    """Isolated pairs at separations rho + m 2^-36 (rho = 2^-6 of the box,
    m = -3..3), along x and along y, inside the box and across its periodic
    edge; every coordinate a multiple of 2^-40, so the separations are exact
    in FP64 and in the 64-bit fixed point alike.  Returns rho, the AoS state
    and, per particle, whether its pair is within rho (m <= 0)."""
    rho = 2.0 ** -6
    pts, inside = [], []
    for k, m in enumerate(range(-3, 4)):
        d = rho + m * 2.0 ** -36
        y = 0.0625 + 0.125 * k
        pts += [(0.25, y), (0.25 + d, y)]                  # along x, inside
        pts += [(1.0 - 2.0 ** -8, y), (d - 2.0 ** -8, y)]  # along x, across the edge
        pts += [(0.5, y), (0.5, y + d)]                    # along y, inside
        x = 0.5625 + 0.0625 * k
        pts += [(x, 1.0 - 2.0 ** -8), (x, d - 2.0 ** -8)]  # along y, across the edge
        inside += [m <= 0] * 8
    pts = np.array(pts)
    n = len(pts)
    rng = np.random.default_rng(seed)
    s = 4 if model == 1 else 6
    x = np.zeros((n, s))
    x[:, :2] = pts
    phi = rng.uniform(-np.pi, np.pi, n)
    if model == 1:
        x[:, 2], x[:, 3] = phi, rng.uniform(-0.5, 0.5, n)
    else:
        x[:, 2], x[:, 3] = 1e-3 * np.cos(phi), 1e-3 * np.sin(phi)
        x[:, 4], x[:, 5] = phi, rng.uniform(-0.5, 0.5, n)
    return rho, x.reshape(-1), np.array(inside)


@pytest.mark.parametrize("model,variant,stepper", [(1, 2, 2), (1, 4, 2), (1, 1, 1), (2, 2, 1), (2, 4, 2)])
def test_cutoff_decisions_in_the_guard_band_match_fp64(model, variant, stepper):
    """Every pair of band_pairs falls inside the FP32 guard band around
    r = rho, so the FP64 decision from the 64-bit positions says whether it
    interacts (m <= 0: in, m > 0: out).  One step equals the FP64 oracle's on
    identical noise (one-step tolerance), and, particle by particle, equals
    the oracle run with every pair in (rho + 2^-30) where m <= 0 and with
    every pair out (rho - 2^-30) where m > 0, while differing from the other:
    a wrong decision changes a neighbour count between 0 and 1."""
    rho, x0, inside = band_pairs(model, 17)
    n = inside.size
    p = dict(model=model, n=n, rho=rho, flavor="ptr", v0=1e-3, sigma=1.0, alpha=0.2)
    if model == 1:
        p.update(xi=0.1, D_phi=0.1)
    else:
        p.update(xi_r=1.0, xi_phi=1.0, D_phi=0.1)
    r_max = 1.3 * rho
    kw = dict(r_max=r_max, nc_verlet=int(1.0 / r_max)) if variant == 4 else {}
    s = 4 if model == 1 else 6
    with gpu_context(p, precision=F32, variant=variant, seed=23, **kw) as ctx:
        ctx.set_state(x0)
        normals = ctx.noise(stepper, 0)
        ctx.step(stepper, 0.005, 0.005)
        got = ctx.get_state()

    def oracle_step(rho_o):
        x = x0.copy()
        oracle_system(dict(p, rho=rho_o), **kw).step(stepper, variant, x, 0.005, 0.005, normals)
        return x

    ref, all_in, all_out = oracle_step(rho), oracle_step(rho + 2.0 ** -30), oracle_step(rho - 2.0 ** -30)
    assert state_err(got, ref, s).max() <= 1e-5
    e_in = state_err(got, all_in, s).max(axis=1)
    e_out = state_err(got, all_out, s).max(axis=1)
    assert np.all(e_in[inside] <= 1e-5) and np.all(e_out[~inside] <= 1e-5)
    assert np.all(e_out[inside] > 5e-5) and np.all(e_in[~inside] > 5e-5)


@pytest.mark.parametrize("model,stepper,per", [(2, 2, 6), (2, 1, 3), (1, 2, 2), (1, 1, 1)])
def test_fast_noise_is_standard_normal_and_independent(model, stepper, per):
    """The fast path's normals (six from one Philox block for second-order SRK,
    Box-Muller pairs otherwise): mean, variance, kurtosis, tail mass, and no
    correlation between a particle's components or their squares."""
    n = 200000
    p = params(model, n)
    r_max = 1.3 * p["rho"]
    with gpu_context(p, precision=F32, variant=4, r_max=r_max, nc_verlet=int(1 / r_max), seed=5) as ctx:
        z = np.concatenate([ctx.noise(stepper, k).reshape(n, per) for k in range(3)])
    m = z.shape[0]
    assert np.abs(z.mean(axis=0)).max() < 5 * np.sqrt(1.0 / m)
    assert np.abs(z.var(axis=0) - 1.0).max() < 5 * np.sqrt(2.0 / m)
    assert np.abs((z ** 4).mean(axis=0) - 3.0).max() < 5 * np.sqrt(96.0 / m)
    tail = (np.abs(z) > 3.0).mean(axis=0)  # 2.6998e-3 for a standard normal
    assert np.abs(tail - 2.6998e-3).max() < 5 * np.sqrt(2.7e-3 / m)
    if per > 1:
        off = ~np.eye(per, dtype=bool)
        assert np.abs(np.corrcoef(z.T)[off]).max() < 5 / np.sqrt(m)
        assert np.abs(np.corrcoef((z ** 2).T)[off]).max() < 5 / np.sqrt(m)


@pytest.mark.parametrize("stepper", [1, 2])
def test_global_field_matches_fp64_oracle(stepper):
    """Global polar order field (first order) with natural frequencies: one and
    ten steps against the FP64 oracle on identical noise, within the one-step
    tolerance (1e-5) and the 50-step tolerance (99.9 % within 1e-3)."""
    n = 4096
    p = params(1, n, sigma=1.5, alpha=0.3)
    x0 = initial(1, n, 21)
    nu = np.random.default_rng(4).normal(0.0, 0.5, n)
    ctx = gpu_context(p, precision=F32, variant=5, seed=13)
    orc = oracle_system(p)
    ctx.set_natural_frequencies(nu)
    orc.set_natural_frequencies(nu)
    ctx.set_state(x0)
    x, t, dt = x0.copy(), 0.0, 0.005
    for k in range(10):
        t += dt
        normals = ctx.noise(stepper, k)
        ctx.step(stepper, t, dt)
        orc.step(stepper, 5, x, t, dt, normals)
        if k == 0:
            assert state_err(ctx.get_state(), x, 4).max() <= 1e-5
    err = state_err(ctx.get_state(), x, 4).max(axis=1)
    ctx.close()
    assert np.quantile(err, 0.999) <= 1e-3
    assert np.median(err) <= 1e-5


@pytest.mark.parametrize("stepper", [1, 2])
@pytest.mark.parametrize("variant", [0, 3])
def test_verlet_radius_over_a_third_runs_all_pairs_with_the_trigger(variant, stepper):
    """The reference's first-order dispatch picks the O(N^2) Verlet list for
    0.25 < rho <= 0.5 (ParticleSystemFirstOrder.cpp:96-111, r_max = rho + 0.05):
    with r_max > 1/3 the fast path evaluates every pair each step and keeps
    the list trigger.  One step within 1e-5 of the oracle's Verlet routine
    (ParticleSystemFirstOrder.cpp:355-477); 20 steps track it with the same
    rebuild steps and accumulated displacement."""
    from helpers import gpu_context, oracle_system

    n, rho = 600, 0.3
    p = dict(model=1, n=n, rho=rho, flavor="ptr", v0=0.5, xi=0.1, sigma=1.0, D_phi=0.1, alpha=0.2)
    x0 = initial(1, n, 4, omega=0.5)
    with gpu_context(p, precision=F32, variant=variant, seed=2) as ctx:
        orc = oracle_system(p)
        assert ctx.verlet_state()[2] == 1
        ctx.set_state(x0)
        x = x0.copy()
        flags_g, flags_o = [], []
        for k in range(20):
            normals = ctx.noise(stepper, k)
            ctx.step(stepper, (k + 1) * 0.005, 0.005)
            orc.step(stepper, 3, x, (k + 1) * 0.005, 0.005, normals)
            acc, flag, uses = ctx.verlet_state()
            assert uses == 1
            assert acc == pytest.approx(orc.accumulated_displacement, rel=1e-5, abs=1e-12)
            flags_g.append(flag)
            flags_o.append(orc.should_update_lists)
            if k == 0:
                assert state_err(ctx.get_state(), x, 4).max() <= 1e-5
        got = ctx.get_state()
    assert flags_g == flags_o and any(flags_o)
    err = state_err(got, x, 4).max(axis=1)
    assert np.quantile(err, 0.999) <= 1e-3
    assert np.median(err) <= 1e-5


def _verlet_context(n, seed=3):
    p = params(2, n)
    r_max = 1.3 * p["rho"]
    return gpu_context(p, precision=F32, variant=4, r_max=r_max, nc_verlet=int(1 / r_max), seed=seed), p


def test_graph_step_whose_trigger_fires_reports_it_like_single_steps():
    """A graph step whose displacement trigger fires rebuilds the lists at once
    (the control kernel tail-launches the rebuild graph); single steps rebuild
    at the start of the next step.  Both report should_update_lists after
    that step, as the reference does, and continue with the same bits."""
    n = 12000
    ctx, p = _verlet_context(n)
    x0 = initial(2, n, 6, v=p["v0"])
    with ctx:
        ctx.set_state(x0)
        ctx.step(2, 0.005, 0.005)  # the first rebuild
        m = 1
        while ctx.verlet_state()[1] == 0 and m < 400:
            ctx.step(2, (m + 1) * 0.005, 0.005)
            m += 1
        assert ctx.verlet_state()[1] == 1, "the trigger should fire within 400 steps"
        eager_flag_state = (ctx.get_state(), ctx.verlet_state())
        for k in range(30):
            ctx.step(2, (m + k + 1) * 0.005, 0.005)
        eager_end = ctx.get_state()
    ctx, _ = _verlet_context(n)
    with ctx:
        ctx.set_state(x0)
        ctx.steps(2, 0.0, 0.005, m)
        builds = ctx.rebuild_count
        np.testing.assert_array_equal(ctx.get_state(), eager_flag_state[0])
        assert ctx.verlet_state() == eager_flag_state[1]
        ctx.steps(2, 0.0, 0.005, 30)
        np.testing.assert_array_equal(ctx.get_state(), eager_end)
        assert ctx.rebuild_count >= builds


def test_host_requested_rebuild_runs_before_the_next_graph_step():
    """spss_set_should_update_lists(1) between graph runs rebuilds the lists
    before the next step; the neighbours within rho are the same, so the run
    differs from the unforced one only in the order of the sums (the slot
    order within cells changes with the extra re-sort)."""
    n = 12000
    ctx, p = _verlet_context(n)
    x0 = initial(2, n, 7, v=p["v0"])
    with ctx:
        ctx.set_state(x0)
        ctx.steps(2, 0.0, 0.005, 5)
        before = ctx.rebuild_count
        ctx.set_should_update_lists(1)
        ctx.steps(2, 0.0, 0.005, 5)
        assert ctx.rebuild_count >= before + 1
        forced = ctx.get_state()
    ctx, _ = _verlet_context(n)
    with ctx:
        ctx.set_state(x0)
        ctx.steps(2, 0.0, 0.005, 10)
        assert state_err(forced, ctx.get_state(), 6).max() <= 1e-5


@pytest.mark.parametrize("variant,stepper", [(4, 2), (2, 1)])
def test_conditional_graph_form_equals_device_rebuild(variant, stepper):
    """The conditional-node step graph (the form for devices that refuse
    device-launched graphs) steps bit for bit as the default form, through
    list rebuilds (Verlet) and per-step cell lists."""
    n = 12000
    p = params(2, n)
    r_max = 1.3 * p["rho"]
    x0 = initial(2, n, 8, v=p["v0"])
    out = []
    for device in (True, False):
        with gpu_context(p, precision=F32, variant=variant, r_max=r_max, nc_verlet=int(1 / r_max), seed=4) as ctx:
            ctx.set_device_rebuild(device)
            ctx.set_state(x0)
            ctx.steps(stepper, 0.0, 0.005, 150)
            out.append((ctx.get_state(), ctx.verlet_state(), ctx.rebuild_count))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]

