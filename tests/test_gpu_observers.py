"""Observer frames computed on the GPU (spss_frame_async) against the
reference's observer arithmetic applied to the same state (bit for bit: the
same float conversion and the same double-rounded wraps), and the Python
trajectory writer end to end: frames in order, summary lines, restart."""
import os
import tempfile

import numpy as np
import pytest

from helpers import initial, params, reference_frame

pytestmark = pytest.mark.gpu


def context(model, precision, n=3000, variant=2):
    from spsslangevinintegration_gb300 import Context

    p = params(model, n)
    kw = {k: p[k] for k in ("v0", "xi", "xi_r", "D_r", "xi_phi", "D_phi", "sigma", "alpha") if k in p}
    return Context(model, n, p["rho"], precision=precision, variant=variant, seed=3, **kw)


@pytest.mark.parametrize("model,precision", [(1, 0), (1, 1), (2, 0), (2, 1)])
def test_frame_matches_reference_observer(model, precision):
    from spsslangevinintegration_gb300.observers import frame

    s = 4 if model == 1 else 6
    with context(model, precision) as ctx:
        x0 = initial(model, ctx.n, 5)
        # phases outside [0, 2 pi) and positions outside the box exercise the wraps
        x0 = x0.reshape(-1, s)
        x0[:, 0] += np.round(np.linspace(-2, 2, ctx.n))
        x0[:, s - 2] += 2 * np.pi * np.round(np.linspace(-3, 3, ctx.n))
        ctx.set_state(x0.reshape(-1))
        stepper = 1 if precision == 1 else 0
        ctx.steps(stepper, 0.0, 0.005, 3)
        state = ctx.get_state()
        for wrapped in (False, True):
            got = frame(ctx, wrapped=wrapped)
            np.testing.assert_array_equal(got, reference_frame(state, s, wrapped))


def test_trajectory_writer_and_restart():
    from spsslangevinintegration_gb300.observers import TrajectoryWriter, read_frames, read_last_frame

    with tempfile.TemporaryDirectory() as d, context(2, 1, n=5000) as ctx:
        ctx.set_state(initial(2, ctx.n, 9))
        traj, summ = os.path.join(d, "t.bin"), os.path.join(d, "s.txt")
        states, t = [], 0.0
        with TrajectoryWriter(ctx, traj, summ, every=3) as w:
            for k in range(10):
                ctx.steps(1, t, 0.005, 1)
                t += 0.005
                if k % 3 == 0:
                    states.append((t, ctx.get_state(), ctx.order_parameters()))
                w(t)
        times, frames = read_frames(traj, ctx.n, 6)
        summary = np.loadtxt(summ)
        t_last, x_last = read_last_frame(traj, ctx.n, 6)
    assert len(frames) == 4 and summary.shape == (4, 3)
    for (tk, xk, rk), tf, fk, line in zip(states, times, frames, summary):
        assert tf == np.float32(tk)
        np.testing.assert_array_equal(fk, reference_frame(xk, 6, wrapped=False))
        np.testing.assert_allclose(line[1:], rk[:2].astype(np.float32), rtol=1e-5, atol=1e-7)
    assert t_last == times[-1]
    np.testing.assert_array_equal(x_last, frames[-1].astype(np.float64))


def test_pinned_array_view_keeps_its_memory():
    """A numpy view of a PinnedArray keeps the page-locked block alive after
    the PinnedArray itself is gone, and the block is freed with the last view."""
    import gc
    import weakref

    from spsslangevinintegration_gb300 import PinnedArray

    pa = PinnedArray(4096)
    owner = weakref.ref(pa._alloc)
    view = pa.array
    del pa
    gc.collect()
    view[:] = 2.5
    assert owner() is not None and float(view.sum()) == 2.5 * 4096
    del view
    gc.collect()
    assert owner() is None
