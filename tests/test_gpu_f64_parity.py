"""FP64 GPU path against the reference (golden fixtures from its own sources)
and against the oracle replaying the GPU's own Philox noise.

Tolerance: the FP64 path performs the reference's operations in the
reference's order with FMA contraction off; results differ only by the
device sin/cos/atan2 (<= 2 ulp) and the all-pairs sum order, so every float
must agree to 1e-12 relative (plus 1e-12 of the array's magnitude).  Cell ids,
per-cell member lists and Verlet lists must be identical.
"""
import os

import numpy as np
import pytest

from helpers import assert_close, fixtures, gpu_context, load_fixture, oracle_system, per_component_close

pytestmark = pytest.mark.gpu

RTOL = 1e-12
RHS = [f for f in fixtures() if "_rhs_" in os.path.basename(f)]
STEPS = [f for f in fixtures() if "_rhs_" not in os.path.basename(f)]


def _ids(paths):
    return [os.path.basename(p)[:-4] for p in paths]


@pytest.mark.parametrize("path", RHS, ids=_ids(RHS))
def test_rhs_matches_reference(path):
    f = load_fixture(path)
    p = f["params"]
    with gpu_context(p) as ctx:
        if p.get("higher_order"):
            ctx.set_higher_order(True)
        if "freqs" in f:
            ctx.set_natural_frequencies(f["freqs"])
        variant = p.get("variant", 0)
        k = ctx.evaluate_rhs(variant, f["state_in"], f["kprev_in"], f["knext_in"], p["k_coef"], p["dt"])
        per_component_close(k, f["knext_out"], 4 if p["model"] == 1 else 6, RTOL, "k_next")
        # entries the reference leaves untouched keep the sentinel exactly
        untouched = f["knext_out"] == f["knext_in"]
        np.testing.assert_array_equal(k[untouched], f["knext_in"][untouched])
        if p.get("higher_order") and "caf" in f:
            assert_close(ctx.complementary_force(), f["caf"], RTOL, what="complementary force")
        if variant in (2, 4) and "pll" in f:
            np.testing.assert_array_equal(ctx.pre_linked_list(), f["pll"])
            off, mem = ctx.cells()
            np.testing.assert_array_equal(off, f["cells"][: off.size])
            np.testing.assert_array_equal(mem, f["cells"][off.size:])
        if variant in (3, 4) and "verlet" in f:
            off, ent = ctx.verlet_lists()
            n = p["n"]
            np.testing.assert_array_equal(off, f["verlet"][: n + 1])
            np.testing.assert_array_equal(ent, f["verlet"][n + 1:])


DETERMINISTIC = [f for f in STEPS if "_rk4" in os.path.basename(f)]


@pytest.mark.parametrize("path", DETERMINISTIC, ids=_ids(DETERMINISTIC))
def test_rk4_trajectory_matches_reference(path):
    f = load_fixture(path)
    p = f["params"]
    variant = p.get("variant", 0)
    with gpu_context(p, variant=variant) as ctx:
        ctx.set_state(f["state_in"])
        t = 0.0
        for _ in range(p["nsteps"]):
            t += p["dt"]
            ctx.step(0, t, p["dt"])
        s = 4 if p["model"] == 1 else 6
        per_component_close(ctx.get_state(), f["state_out"], s, 1e-11, "state")
        acc, flag, uses = ctx.verlet_state()
        assert flag == int(f["meta"]["should_update_lists"])
        assert abs(acc - f["meta"]["accumulated_displacement"]) <= 1e-12


STOCHASTIC = [f for f in STEPS if "_se_" in os.path.basename(f) or "_srk_" in os.path.basename(f)]


@pytest.mark.parametrize("path", STOCHASTIC, ids=_ids(STOCHASTIC))
def test_stochastic_trajectory_matches_oracle_with_gpu_noise(path):
    """Same initial state; the oracle replays the normals the GPU drew (spss_noise)."""
    from oracle import binding as ob

    f = load_fixture(path)
    p = f["params"]
    stepper = {"se": 1, "srk": 2}[p["stepper"]]
    with gpu_context(p, seed=1234, replica=3) as ctx:
        ctx.set_state(f["state_in"])
        orc = oracle_system(p)
        x = f["state_in"].copy()
        t = 0.0
        for step in range(p["nsteps"]):
            t += p["dt"]
            normals = ctx.noise(stepper, step)
            ctx.step(stepper, t, p["dt"])
            orc.step(stepper, 0, x, t, p["dt"], normals)
        s = 4 if p["model"] == 1 else 6
        per_component_close(ctx.get_state(), x, s, 1e-11, "state")
        acc, flag, uses = ctx.verlet_state()
        assert flag == orc.should_update_lists
        assert abs(acc - orc.accumulated_displacement) <= 1e-12
        assert ctx.step_counter == p["nsteps"]


def test_noise_is_standard_normal_and_counter_based():
    p = dict(model=2, n=20000, rho=0.05, flavor="serial")
    with gpu_context(p, seed=7) as ctx:
        z = ctx.noise(2, 5)
        assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
        np.testing.assert_array_equal(z, ctx.noise(2, 5))  # same counter -> same draws
        assert not np.array_equal(z, ctx.noise(2, 6))
    with gpu_context(p, seed=7, replica=1) as ctx2:
        assert not np.array_equal(z, ctx2.noise(2, 5))


@pytest.mark.parametrize("model,variant,stepper", [(2, 4, 2), (2, 3, 1), (2, 4, 0), (1, 4, 2), (1, 2, 1)])
def test_restated_paths_match_oracle(model, variant, stepper):
    """Paths with no reference code (second-order Verlet, second-order SRK) and
    explicit-variant steppers: GPU FP64 against the oracle restatement."""
    from golden.make_golden import initial_state

    n, rho = 700, 0.06
    p = dict(model=model, n=n, rho=rho, flavor="ptr", v0=0.3, xi=0.1, xi_r=1.0, D_r=0.02, xi_phi=1.0, D_phi=0.1,
             sigma=1.0, alpha=0.2)
    x0 = initial_state(model, n, seed=40 + variant, v0=0.02)
    r_max = rho + 0.3 * rho
    nc_v = int(1.0 / r_max)
    with gpu_context(p, variant=variant, r_max=r_max, nc_verlet=nc_v, seed=99) as ctx:
        ctx.set_state(x0)
        orc = oracle_system(p, r_max=r_max, nc_verlet=nc_v)
        x = x0.copy()
        t, dt = 0.0, 0.01
        for step in range(30):
            t += dt
            normals = ctx.noise(stepper, step) if stepper else None
            ctx.step(stepper, t, dt)
            orc.step(stepper, variant, x, t, dt, normals)
        per_component_close(ctx.get_state(), x, 4 if model == 1 else 6, 1e-10, "state")
        acc, flag, _ = ctx.verlet_state()
        assert flag == orc.should_update_lists
        if variant in (3, 4):
            off, ent = ctx.verlet_lists()
            ooff, oent = orc.verlet()
            np.testing.assert_array_equal(off, ooff)
            np.testing.assert_array_equal(ent, oent)


def test_order_parameters_and_averaging_match_oracle():
    from oracle import binding as ob
    from golden.make_golden import initial_state

    for model in (1, 2):
        p = dict(model=model, n=3000, rho=0.05, flavor="ptr")
        x = initial_state(model, 3000, seed=5 + model, v0=0.1)
        with gpu_context(p) as ctx:
            ctx.set_state(x)
            assert_close(ctx.order_parameters(), ob.order_parameters(model, x), 1e-12, what="order parameters")
            ctx.average_accumulate()
            ctx.set_state(2 * x)
            ctx.average_accumulate()
            mean, cnt = ctx.average()
            assert cnt == 2
            assert_close(mean, 1.5 * x, 1e-15, what="average")


def test_wrapped_coordinate_at_box_edge_is_clamped_like_oracle():
    """x = -tiny wraps to exactly 1.0; the reference would index cell nc (out of range).
    GPU and oracle both clamp it into the last cell."""
    from golden.make_golden import initial_state

    n = 300
    p = dict(model=1, n=n, rho=0.1, flavor="ptr", v0=0.02, xi=0.1, sigma=1.0)
    x = initial_state(1, n, seed=3)
    x[0] = -1e-18
    x[4 + 1] = -1e-18
    orc = oracle_system(p)
    k_ref = np.zeros(4 * n)
    orc.evaluate(2, x, np.zeros(4 * n), k_ref, 0.0, 0.01)
    with gpu_context(p) as ctx:
        k = ctx.evaluate_rhs(2, x, np.zeros(4 * n), np.zeros(4 * n), 0.0, 0.01)
        np.testing.assert_array_equal(ctx.pre_linked_list(), orc.pre_linked_list())
        assert ctx.pre_linked_list()[0] < 100
        per_component_close(k, k_ref, 4, RTOL, "k_next")


def test_invalid_arguments_are_rejected():
    from spsslangevinintegration_gb300 import Context, SpssError

    with pytest.raises(SpssError):
        Context(3, 10, 0.1)
    with pytest.raises(SpssError):
        Context(1, 0, 0.1)
    with gpu_context(dict(model=1, n=10, rho=0.1)) as ctx:
        with pytest.raises(SpssError):
            ctx.set_state(np.zeros(7))
        with pytest.raises(SpssError):
            ctx.step(9, 0.0, 0.01)


@pytest.mark.parametrize("variant,rho", [(1, 0.05), (2, 0.05), (5, 0.8), (0, 0.03)])
def test_rk4_graph_steps_equal_single_steps(variant, rho):
    """spss_steps replays one captured RK4 step as a CUDA graph on the FP64
    path (no noise, no host decision between steps): the state equals that of
    single steps bit for bit, stale torque derivatives included."""
    from helpers import gpu_context, initial

    p = dict(model=1, n=700, rho=rho, flavor="ptr", v0=0.02, xi=0.1, sigma=1.0, alpha=0.3)
    x0 = initial(1, 700, 31, omega=0.8)
    out = []
    for graph in (False, True):
        with gpu_context(p, precision=0, variant=variant) as ctx:
            ctx.set_state(x0)
            if graph:
                ctx.steps(0, 0.0, 0.01, 25)
            else:
                for k in range(25):
                    ctx.step(0, (k + 1) * 0.01, 0.01)
            out.append(ctx.get_state())
    np.testing.assert_array_equal(out[0], out[1])
