"""Batches of independent systems (spss_batch_create), tilings of the
pair-and-update kernel and the autotuner, per-system order parameters and
their time averages.

Checks (exact unless stated):
  * a batch of systems with different sizes and parameters steps every system
    bit for bit as a single-system context with the same parameters does
    (cell lists, rebuilt every step in both), and draws the same noise;
  * Verlet lists in a batch are rebuilt per system, when that system's own
    trigger fires: every system steps bit for bit as alone, through rebuilds
    on different steps;
  * results do not depend on the tiling (cells per tile, persistent launch);
  * spss_autotune leaves the state as it found it: the tuned run equals an
    untuned one bit for bit;
  * per-system order parameters: within 1e-6 of the FP64 reduction of each
    system's downloaded state (the kernel sums the FP32 cos/sin in FP64);
  * time averages: within 1e-12 relative of averaging the per-system order
    parameters sampled step by step on an identical batch.
"""
import numpy as np
import pytest

from helpers import PARAM_KEYS, initial, min_image, params

pytestmark = pytest.mark.gpu

F32 = 1
LINKED_LIST, LINKED_LIST_VERLET = 2, 4
SE, SRK = 1, 2
DT = 0.005


def systems(model=2, variant=LINKED_LIST, sizes=(1024, 3000, 8192), seed=5, skin=0.3):
    out = []
    for r, n in enumerate(sizes):
        m = (1.0, 0.1, 10.0)[r % 3]
        p = params(model, n, m=m, D=(0.1, 0.01, 1.0)[r % 3], sigma=(1.0, 0.5, 2.5)[r % 3],
                   v0=(0.5, 0.83, 0.31)[r % 3])
        kw = {k: p[k] for k in PARAM_KEYS if k in p}
        s = dict(model=model, n=n, rho=p["rho"], precision=F32, variant=variant, seed=seed, replica=r, **kw)
        if variant == LINKED_LIST_VERLET:
            s["r_max"] = p["rho"] * (1.0 + skin)
            s["nc_verlet"] = int(1.0 / s["r_max"])
        out.append(s)
    return out


def states(sys_list, seed=10):
    return [initial(s["model"], s["n"], seed + r) for r, s in enumerate(sys_list)]


def run_single(s, x0, stepper, nsteps, tiling=None):
    from spsslangevinintegration_gb300 import Context

    kw = dict(s)
    with Context(kw.pop("model"), kw.pop("n"), kw.pop("rho"), **kw) as ctx:
        if tiling:
            ctx.set_tiling(*tiling)
        ctx.set_state(x0)
        ctx.steps(stepper, 0.0, DT, nsteps)
        return ctx.get_state()


def run_batch(sys_list, xs, stepper, nsteps, tiling=None):
    from spsslangevinintegration_gb300 import Batch

    with Batch(sys_list) as b:
        if tiling:
            b.set_tiling(*tiling)
        b.set_state(np.concatenate(xs))
        b.steps(stepper, 0.0, DT, nsteps)
        out = b.get_state()
        return [b.system_rows(out, r).copy() for r in range(b.nsys)]


@pytest.mark.parametrize("model,stepper", [(2, SE), (2, SRK), (1, SE), (1, SRK)])
def test_batch_equals_single_contexts_cells(model, stepper):
    sl = systems(model=model)
    xs = states(sl)
    got = run_batch(sl, xs, stepper, 9)
    for r, s in enumerate(sl):
        ref = run_single(s, xs[r], stepper, 9)
        assert np.array_equal(got[r], ref), "system %d differs from its single-context run" % r


def test_batch_noise_is_each_systems_noise():
    from spsslangevinintegration_gb300 import Batch, Context

    sl = systems()
    with Batch(sl) as b:
        for stepper in (SE, SRK):
            z = b.noise(stepper, 17)
            per = z.size // b.n
            for r, s in enumerate(sl):
                kw = dict(s)
                with Context(kw.pop("model"), kw.pop("n"), kw.pop("rho"), **kw) as ctx:
                    ref = ctx.noise(stepper, 17)
                assert np.array_equal(z[per * b.first[r]: per * b.first[r + 1]], ref)


@pytest.mark.parametrize("model,stepper", [(2, SE), (2, SRK), (1, SRK)])
def test_batch_verlet_equals_single_contexts(model, stepper):
    """Each system of a Verlet-list batch rebuilds its lists when its own
    trigger fires, and only then, so it steps bit for bit as it does alone,
    through rebuilds that fall on different steps for different systems."""
    from spsslangevinintegration_gb300 import Batch

    sl = systems(model=model, variant=LINKED_LIST_VERLET, sizes=(4096, 20000, 9000))
    xs = states(sl, seed=20)
    singles = []
    for r, s in enumerate(sl):
        from spsslangevinintegration_gb300 import Context

        kw = dict(s)
        with Context(kw.pop("model"), kw.pop("n"), kw.pop("rho"), **kw) as ctx:
            ctx.set_state(xs[r])
            builds = [ctx.rebuild_count]
            for k in range(20):
                ctx.steps(stepper, 0.0, DT, 20)
                builds.append(ctx.rebuild_count)
            singles.append((ctx.get_state(), builds))
    with Batch(sl) as b:
        b.set_state(np.concatenate(xs))
        b.steps(stepper, 0.0, DT, 400)
        out = b.get_state()
        batch_builds = b.rebuild_count
    for r in range(len(sl)):
        assert np.array_equal(b.system_rows(out, r), singles[r][0]), "system %d differs from its run alone" % r
    # every system rebuilt on its own trigger at least once, and not all on the
    # same steps: the batch's rebuild steps (the union) outnumber each system's
    counts = [sb[1][-1] - sb[1][0] for sb in singles]
    assert min(counts) >= 2
    assert batch_builds > max(counts)


@pytest.mark.parametrize("variant,stepper", [(LINKED_LIST, SE), (LINKED_LIST_VERLET, SRK)])
def test_results_do_not_depend_on_tiling(variant, stepper):
    s = systems(variant=variant, sizes=(30000,))[0]
    x0 = states([s], seed=30)[0]
    ref = run_single(s, x0, stepper, 12)
    for tiling in ((8, True), (16, False), (64, True), (5, False)):
        assert np.array_equal(run_single(s, x0, stepper, 12, tiling=tiling), ref), tiling


def test_batch_tiling_and_persistent_launch():
    sl = systems(variant=LINKED_LIST_VERLET, sizes=(2048, 12000, 5000))
    xs = states(sl, seed=40)
    ref = run_batch(sl, xs, SE, 10)
    got = run_batch(sl, xs, SE, 10, tiling=(16, True))
    for r in range(len(sl)):
        assert np.array_equal(got[r], ref[r])


def test_autotune_restores_state():
    from spsslangevinintegration_gb300 import Batch

    sl = systems(sizes=(4096, 16384))
    xs = states(sl, seed=50)
    ref = run_batch(sl, xs, SE, 8)
    with Batch(sl) as b:
        b.set_state(np.concatenate(xs))
        before = b.get_state()
        ms = b.autotune(SE, DT, steps=2)
        assert ms > 0.0
        tc, pers = b.tiling()
        assert tc in range(16, 65, 4)
        assert np.array_equal(b.get_state(), before)
        assert b.step_counter == 0
        b.steps(SE, 0.0, DT, 8)
        out = b.get_state()
        for r in range(b.nsys):
            assert np.array_equal(b.system_rows(out, r), ref[r])


def order_of(x, model):
    x = x.reshape(-1, 4 if model == 1 else 6)
    phi = x[:, 2] if model == 1 else x[:, 4]
    z = np.mean(np.exp(1j * phi))
    if model == 1:
        return np.array([abs(z), np.angle(z), abs(z), np.angle(z)])
    v = x[:, 2] + 1j * x[:, 3]
    u = np.mean(v / np.abs(v))
    return np.array([abs(z), np.angle(z), abs(u), np.angle(u)])


@pytest.mark.parametrize("model", [1, 2])
def test_system_order_parameters(model):
    from spsslangevinintegration_gb300 import Batch

    sl = systems(model=model)
    xs = states(sl, seed=60)
    with Batch(sl) as b:
        b.set_state(np.concatenate(xs))
        b.steps(SE, 0.0, DT, 5)
        got = b.system_order_parameters()
        out = b.get_state()
        for r in range(b.nsys):
            ref = order_of(b.system_rows(out, r), model)
            assert abs(got[r, 0] - ref[0]) <= 1e-6 and abs(got[r, 2] - ref[2]) <= 1e-6, (r, got[r], ref)
            # angles: compare on the circle
            for k in (1, 3):
                assert abs(np.angle(np.exp(1j * (got[r, k] - ref[k])))) <= 1e-5 / max(ref[k - 1], 1e-3)


def test_time_averages_match_step_by_step_sampling():
    from spsslangevinintegration_gb300 import Batch

    sl = systems(sizes=(2048, 6000, 3000))
    xs = states(sl, seed=70)
    every, start, nsteps = 3, 4, 20
    with Batch(sl) as b:
        b.set_state(np.concatenate(xs))
        b.run(SE, 0.0, DT, nsteps, sample_every=every, sample_from=start)
        st = b.stats()
        final = b.get_state()
    samples = []
    with Batch(sl) as b:
        b.set_state(np.concatenate(xs))
        for k in range(1, nsteps + 1):
            b.steps(SE, 0.0, DT, 1)
            if k % every == 0 and k >= start:
                samples.append(b.system_order_parameters())
        assert np.array_equal(b.get_state(), final)
    samples = np.array(samples)  # (count, nsys, 4)
    assert np.all(st[:, 4] == len(samples))
    for c, k in ((0, 0), (2, 2)):
        mean = samples[:, :, k].mean(axis=0)
        var = np.maximum(0.0, (samples[:, :, k] ** 2).mean(axis=0) - mean ** 2)
        np.testing.assert_allclose(st[:, c], mean, rtol=1e-12, atol=0)
        np.testing.assert_allclose(st[:, c + 1], var, rtol=1e-9, atol=1e-15)
