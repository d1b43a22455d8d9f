"""Inner lists of the Verlet path (spss_set_inner_lists).

A Verlet step walks each particle's inner list: the entries of its Verlet
list (pairs within r_max = rho + skin) that were within rho + buffer when the
inner list was last built, in the Verlet list's order.  The inner lists are
built by a step that walks the whole Verlet lists: the first step after every
rebuild, and the step after the accumulated largest displacement since the
last build passes half the buffer, so no pair left out can have come within
rho.  The pairs within rho and the order in which their contributions are
summed are then those of the whole list, so results must be bit-identical
with the inner lists on or off.

Checks (exact):
  * trajectories over several list rebuilds and many inner-list builds equal
    the whole-list trajectories bit for bit, for the second-order SRK and SE
    steppers and the first-order SRK stepper, in graph-driven and single
    steps, and with the persistent launch;
  * a batch of systems, each building its inner lists on its own trigger,
    equals the batch without inner lists;
  * switching the inner lists off and on between steps changes nothing.
"""
import numpy as np
import pytest

from helpers import PARAM_KEYS, gpu_context, initial, params

pytestmark = pytest.mark.gpu

F32 = 1
VERLET = 4
SE, SRK = 1, 2
DT = 0.005


def context(model, n, seed=3, skin=0.3):
    p = params(model, n)
    r_max = (1.0 + skin) * p["rho"]
    return gpu_context(p, precision=F32, variant=VERLET, r_max=r_max, nc_verlet=int(1.0 / r_max), seed=seed), p


def run(model, stepper, n, nsteps, inner, chunk=None, tiling=None):
    ctx, p = context(model, n)
    with ctx:
        ctx.set_inner_lists(inner)
        assert ctx.inner_lists() == inner
        if tiling:
            ctx.set_tiling(*tiling)
        ctx.set_state(initial(model, n, 7, v=p.get("v0", 0.01)))
        builds0 = ctx.rebuild_count
        if chunk is None:
            ctx.steps(stepper, 0.0, DT, nsteps)
        else:
            for k in range(0, nsteps, chunk):
                for j in range(k, min(nsteps, k + chunk)):
                    ctx.step(stepper, (j + 1) * DT, DT)
        return ctx.get_state(), ctx.verlet_state(), ctx.rebuild_count - builds0


@pytest.mark.parametrize("model,stepper", [(2, SRK), (2, SE), (1, SRK)])
def test_inner_lists_equal_whole_lists_bitwise(model, stepper):
    whole = run(model, stepper, 20000, 240, False)
    inner = run(model, stepper, 20000, 240, True)
    assert whole[2] >= 3, "the run should hold several list rebuilds"
    np.testing.assert_array_equal(inner[0], whole[0])
    assert inner[1] == whole[1]
    assert inner[2] == whole[2]


def test_inner_lists_in_single_steps_and_persistent_launch():
    ref = run(2, SRK, 12000, 90, False)
    np.testing.assert_array_equal(run(2, SRK, 12000, 90, True, chunk=1)[0], ref[0])
    np.testing.assert_array_equal(run(2, SRK, 12000, 90, True, tiling=(16, True))[0], ref[0])


def test_inner_lists_switched_between_steps():
    n = 15000
    ctx_ref, p = context(2, n)
    x0 = initial(2, n, 11, v=p["v0"])
    with ctx_ref:
        ctx_ref.set_inner_lists(False)
        ctx_ref.set_state(x0)
        ctx_ref.steps(SRK, 0.0, DT, 150)
        ref = ctx_ref.get_state()
    ctx, _ = context(2, n)
    with ctx:
        ctx.set_state(x0)
        ctx.steps(SRK, 0.0, DT, 40)
        ctx.set_inner_lists(False)
        ctx.steps(SRK, 0.0, DT, 40)
        ctx.set_inner_lists(True)
        ctx.steps(SRK, 0.0, DT, 70)
        np.testing.assert_array_equal(ctx.get_state(), ref)


def test_batch_inner_lists_equal_whole_lists():
    from spsslangevinintegration_gb300 import Batch

    sl = []
    for r, n in enumerate((4096, 20000, 9000)):
        p = params(2, n, m=(1.0, 0.1, 10.0)[r], D=(0.1, 0.01, 1.0)[r], v0=(0.5, 0.83, 0.31)[r])
        s = dict(model=2, n=n, rho=p["rho"], precision=F32, variant=VERLET, seed=5, replica=r,
                 **{k: p[k] for k in PARAM_KEYS if k in p})
        s["r_max"] = 1.3 * p["rho"]
        s["nc_verlet"] = int(1.0 / s["r_max"])
        sl.append(s)
    x0 = np.concatenate([initial(2, s["n"], 20 + r) for r, s in enumerate(sl)])
    out = {}
    for inner in (False, True):
        with Batch(sl) as b:
            b.set_inner_lists(inner)
            b.set_state(x0)
            b.steps(SE, 0.0, DT, 300)
            out[inner] = (b.get_state(), b.rebuild_count)
    np.testing.assert_array_equal(out[True][0], out[False][0])
    assert out[True][1] == out[False][1]
