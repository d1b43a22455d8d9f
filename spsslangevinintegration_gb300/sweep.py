"""Parameter sweeps: many independent systems stepped as one batch.

The reference scans parameters by giving each MPI rank its own parameter
point (MPI_PARAMETER_SCAN in the SimulationEngine*Ptr engines) and keeps time
averages of the observers' order parameters.  Here a sweep is one batch
context (spss_batch_create): all systems advance together, every step is one
CUDA graph, and the per-system phase / velocity-direction order parameters
are averaged on the GPU.

Physical points are given in the units of the model
    m dv/dt = -v + v0 e(phi) + sqrt(2 D_r) xi,   m domega/dt = -omega + sigma F + sqrt(2 D) eta
(density, interaction radius R, self-propulsion speed v0, coupling sigma,
noise D, inertia m) and mapped to the reference's unit box: L = sqrt(N /
density), rho = R / L, v0 -> v0 / L, xi_r = xi_phi = 1 / m, sigma -> sigma / m,
D_phi = D / m^2, D_r = D_r / (m^2 L^2).
"""
import numpy as np

from . import _native as N
from .context import Batch


def replica_table(count=512, seed=0, n_range=(1024, 65536), sigma_range=(0.0, 3.0), d_range=(0.01, 1.0),
                  masses=(0.1, 1.0, 10.0), density=2.0, radius=1.0, v0=0.5):
    """Seeded random parameter points: N and D log-uniform, sigma uniform, m
    drawn from `masses`."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]), count)).astype(np.int64)
    sigma = rng.uniform(sigma_range[0], sigma_range[1], count)
    d = np.exp(rng.uniform(np.log(d_range[0]), np.log(d_range[1]), count))
    m = rng.choice(np.asarray(masses, dtype=np.float64), count)
    return [dict(n=int(n[i]), sigma=float(sigma[i]), D=float(d[i]), m=float(m[i]), density=density, R=radius, v0=v0)
            for i in range(count)]


def system_params(point, variant=N.LINKED_LIST, seed=0, replica=0, skin=0.0, D_r=0.0):
    """make_params keywords of one physical point (second-order model, F32)."""
    n, m = point["n"], point["m"]
    L = np.sqrt(n / point["density"])
    rho = point["R"] / L
    kw = dict(model=2, n=n, rho=rho, precision=N.PRECISION_F32, variant=variant, v0=point["v0"] / L,
              xi_r=1.0 / m, xi_phi=1.0 / m, D_r=D_r / (m * m * L * L), D_phi=point["D"] / (m * m),
              sigma=point["sigma"] / m, seed=seed, replica=replica)
    if skin > 0.0:
        kw["r_max"] = rho * (1.0 + skin)
        kw["nc_verlet"] = int(1.0 / kw["r_max"])
    return kw


def initial_state(n, L, seed):
    """Uniform positions, phases uniform in [-pi, pi), velocity a unit vector
    along phi (divided by L), omega = 0 (SimulationEngineSecondOrder.cpp:46-50)."""
    rng = np.random.default_rng(seed)
    x = np.empty((n, 6))
    x[:, 0] = rng.random(n)
    x[:, 1] = rng.random(n)
    phi = rng.uniform(-np.pi, np.pi, n)
    x[:, 2] = np.cos(phi) / L
    x[:, 3] = np.sin(phi) / L
    x[:, 4] = phi
    x[:, 5] = 0.0
    return x.reshape(-1)


def make_batch(points, variant=N.LINKED_LIST, seed=0, skin=0.0, state_seed=1, first_replica=0):
    """A batch context for `points` with its seeded initial state loaded."""
    systems = [system_params(p, variant=variant, seed=seed, replica=first_replica + i, skin=skin)
               for i, p in enumerate(points)]
    b = Batch(systems)
    xs = [initial_state(p["n"], np.sqrt(p["n"] / p["density"]), state_seed * 1000003 + first_replica + i)
          for i, p in enumerate(points)]
    b.set_state(np.concatenate(xs))
    return b


def run_sweep(points, steps=20000, dt=0.005, sample_every=10, burn_in=None, variant=N.LINKED_LIST, seed=0,
              skin=0.0, autotune=True, stepper=N.STOCHASTIC_EULER, first_replica=0):
    """Time-averaged order parameters of every point: array (len(points), 5) =
    mean and variance of the phase order, mean and variance of the
    velocity-direction order, number of samples.  Samples every
    `sample_every` steps after `burn_in` steps (default: half the run)."""
    if burn_in is None:
        burn_in = steps // 2
    b = make_batch(points, variant=variant, seed=seed, skin=skin, first_replica=first_replica)
    try:
        if autotune:
            b.autotune(stepper, dt, steps=3)
        b.run(stepper, 0.0, dt, steps, sample_every=sample_every, sample_from=max(burn_in, 1))
        return b.stats()
    finally:
        b.close()
