"""One pass over every kernel family of the library at moderate sizes: a
usage tour of the Python handles and a quick check that every path runs.

    python -m spsslangevinintegration_gb300.tour

* GB300 path, second-order model, Verlet skin 0.3 R, StochasticRungeKutta,
  N = 2,097,152 at density 2: upload, list rebuild (cells, binning, slot
  permutation, tile layout, tile list build), three steps, the order
  parameters, one trajectory frame, download;
* GB300 path, a batch of 64 independent second-order systems with cell lists,
  StochasticEuler: two steps with the per-system order-parameter sample;
* GB300 path, first-order model in the global polar order field with natural
  frequencies, StochasticRungeKutta, N = 1,048,576;
* reference arithmetic (FP64): first-order all pairs RK4 at N = 1000 and
  density 1, second-order linked list StochasticEuler at N = 65,536,
  first-order linked list + Verlet StochasticRungeKutta at N = 65,536, one
  right-hand-side evaluation, the max-displacement check, the odeint
  (dopri5) path over a short interval;
* the surrogate network: one training epoch and one forward pass.
"""
import time

import numpy as np

from . import _native as N
from . import observers, sweep
from .context import Context
from .surrogate import Network

RK4, SE, SRK = N.RK4, N.STOCHASTIC_EULER, N.STOCHASTIC_RUNGE_KUTTA
DT = 0.005


def _state(model, n, L, seed):
    """Uniform positions and phases in the unit box; second order: unit
    speed along the phase (in box units), omega = 0."""
    rng = np.random.default_rng(seed)
    s = 4 if model == 1 else 6
    x = np.zeros((n, s))
    x[:, 0] = rng.random(n)
    x[:, 1] = rng.random(n)
    phi = rng.uniform(-np.pi, np.pi, n)
    if model == 1:
        x[:, 2] = phi
    else:
        x[:, 2] = np.cos(phi) / L
        x[:, 3] = np.sin(phi) / L
        x[:, 4] = phi
    return x.reshape(-1)


def fast_verlet(n=2097152):
    L = np.sqrt(n / 2.0)
    rho = 1.0 / L
    r_max = 1.3 * rho
    with Context(2, n, rho, precision=N.PRECISION_F32, variant=N.LINKED_LIST_VERLET, v0=0.5 / L, xi_r=1.0,
                 xi_phi=1.0, D_phi=0.1, sigma=1.0, r_max=r_max, nc_verlet=int(1.0 / r_max), seed=1) as ctx:
        ctx.set_state(_state(2, n, L, 0))
        for k in range(3):
            ctx.step(SRK, (k + 1) * DT, DT)
        r = ctx.order_parameters()
        observers.frame(ctx, wrapped=False)
        x = ctx.get_state()
    return "GB300 path, Verlet SRK, N=%d: |R| = %.4f, finite %s" % (n, r[0], bool(np.all(np.isfinite(x))))


def fast_batch(count=64):
    points = sweep.replica_table(count, seed=0, n_range=(1024, 16384))
    b = sweep.make_batch(points, seed=0)
    b.run(SE, 0.0, DT, 2, sample_every=1, sample_from=0)
    r = b.system_order_parameters()
    b.close()
    return "GB300 path, batch of %d systems (cell lists, SE): mean |R| = %.4f" % (count, float(np.mean(r[:, 0])))


def fast_global(n=1048576):
    with Context(1, n, 1.0, precision=N.PRECISION_F32, variant=N.GLOBAL_FIELD, v0=0.01, xi=0.1, D_phi=0.1,
                 sigma=1.0, seed=2) as ctx:
        ctx.set_natural_frequencies(np.random.default_rng(3).normal(0.0, 0.5, n))
        ctx.set_state(_state(1, n, 1.0, 4))
        for k in range(3):
            ctx.step(SRK, (k + 1) * DT, DT)
        r = ctx.order_parameters()
    return "GB300 path, global field SRK, N=%d: |R| = %.4f" % (n, r[0])


def reference_paths():
    out = []
    n = 1000
    L = np.sqrt(n / 1.0)
    with Context(1, n, 1.0 / L, precision=N.PRECISION_F64, variant=N.ALL_PAIRS, v0=0.1 / L, xi=0.1,
                 sigma=1.0) as ctx:
        x = _state(1, n, L, 5)
        ctx.set_state(x)
        for k in range(2):
            ctx.step(RK4, (k + 1) * 0.01, 0.01)
        k_next = ctx.evaluate_rhs(N.ALL_PAIRS, x, np.zeros_like(x), np.zeros_like(x), 0.0, 0.01)
        times = []
        ctx.set_state(x)
        ctx.integrate_dopri5(0.0, 0.05, 0.01, observer=lambda s, t: times.append(t))
        out.append("FP64 all pairs RK4 + dopri5, N=%d: |k| = %.3e, %d outputs" % (n, np.abs(k_next).max(),
                                                                                len(times)))
    n = 65536
    L = np.sqrt(n / 2.0)
    with Context(2, n, 1.0 / L, precision=N.PRECISION_F64, variant=N.LINKED_LIST, v0=0.5 / L, xi_r=1.0,
                 xi_phi=1.0, D_phi=0.1, sigma=1.0, seed=6) as ctx:
        ctx.set_state(_state(2, n, L, 7))
        for k in range(2):
            ctx.step(SE, (k + 1) * DT, DT)
        out.append("FP64 linked list SE, N=%d: |R| = %.4f" % (n, ctx.order_parameters()[0]))
    r_max = 1.3 / L
    with Context(1, n, 1.0 / L, precision=N.PRECISION_F64, variant=N.LINKED_LIST_VERLET, v0=0.5 / L, xi=0.1,
                 D_phi=0.1, sigma=1.0, r_max=r_max, nc_verlet=int(1.0 / r_max), seed=8) as ctx:
        ctx.set_state(_state(1, n, L, 9))
        for k in range(2):
            ctx.step(SRK, (k + 1) * DT, DT)
        acc, flag, _ = ctx.verlet_state()
        out.append("FP64 linked list + Verlet SRK, N=%d: accumulated displacement %.3e" % (n, acc))
    return out


def network():
    rng = np.random.default_rng(10)
    x = rng.normal(size=(4096, N.MLP_INPUTS)).astype(np.float32)
    t = rng.normal(size=(4096, N.MLP_OUTPUTS)).astype(np.float32)
    with Network(seed=11) as net:
        net.set_data(x, t)
        loss = net.train(1, batch=1024)
        y = net.forward(x)
    return "surrogate network: epoch loss %.4f, forward %s" % (float(loss[-1]), y.shape)


def main():
    t0 = time.perf_counter()
    lines = [fast_verlet(), fast_batch(), fast_global()] + reference_paths() + [network()]
    for line in lines:
        print(line)
    print("tour done in %.1f s" % (time.perf_counter() - t0))


if __name__ == "__main__":
    main()
