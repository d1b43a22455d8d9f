"""Parameter continuation (SimulationEngineFirstOrderPtr::RunContinuationMethod,
SimulationEngineFirstOrderPtr.cpp:167-217): a parameter is stepped through a
list of values, each stage integrating from the state the previous stage ended
in, with the order parameter recorded along the way and the end state of every
stage kept (the reference saves it as the stage's last frame).

``continuation`` runs one system on either arithmetic path — the reference's
own use is the first-order model in the global field with RK4 in FP64.
``continuation_replicas`` runs independent replicas of the same continuation
(the reference's commented-out loop over trials) as one batch per stage on the
GPU path: every replica carries its own state from stage to stage and draws
its own noise.
"""
import numpy as np

from . import _native as N
from .context import Batch, Context


def _context(kw):
    kw = dict(kw)
    return Context(kw.pop("model"), kw.pop("n"), kw.pop("rho"), **kw)


def continuation(state, stages, t_span, dt, stepper=N.RK4, record_every=100):
    """`stages`: list of make_params keyword dicts, one per parameter value.
    Returns (end states [stage][s*n], order-parameter series [stage][k][3] =
    (t, |R|, arg R) recorded every `record_every` steps).  The step counter
    (the noise stream) continues across stages."""
    x = np.ascontiguousarray(state, dtype=np.float64).copy()
    nsteps = int(round(t_span / dt))
    ends, series = [], []
    counter = 0
    for kw in stages:
        with _context(kw) as ctx:
            ctx.set_state(x)
            ctx.step_counter = counter
            rec, t = [], 0.0
            done = 0
            while done < nsteps:
                chunk = min(record_every, nsteps - done)
                if ctx.params.precision == N.PRECISION_F64:
                    for _ in range(chunk):
                        t += dt
                        ctx.step(stepper, t, dt)
                else:
                    ctx.steps(stepper, t, dt, chunk)
                    t += chunk * dt
                done += chunk
                r = ctx.order_parameters()
                rec.append((t, r[0], r[1]))
            counter = ctx.step_counter
            x = ctx.get_state()
        ends.append(x.copy())
        series.append(np.array(rec))
    return ends, series


def continuation_replicas(states, stages, t_span, dt, stepper=N.STOCHASTIC_EULER, sample_every=10, burn_in=0):
    """Replicas of one continuation, batched: `states` [r][s*n] initial states,
    `stages` make_params keyword dicts (precision F32; the replica index is set
    here).  Returns (end states [stage][r][s*n], stats [stage][r][5] as
    spss_batch_stats: time averages over the stage after `burn_in` steps)."""
    xs = [np.ascontiguousarray(x, dtype=np.float64).copy() for x in states]
    nsteps = int(round(t_span / dt))
    ends, stats = [], []
    counter = 0
    for kw in stages:
        systems = [dict(kw, replica=r) for r in range(len(xs))]
        with Batch(systems) as b:
            b.set_state(np.concatenate(xs))
            b.step_counter = counter
            b.run(stepper, 0.0, dt, nsteps, sample_every=sample_every, sample_from=counter + max(burn_in, 1))
            stats.append(b.stats())
            out = b.get_state()
            xs = [b.system_rows(out, r).copy() for r in range(b.nsys)]
            counter = b.step_counter
        ends.append([x.copy() for x in xs])
    return ends, stats
