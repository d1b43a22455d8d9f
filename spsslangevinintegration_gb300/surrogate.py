"""Learned surrogate of the stationary order parameters (include/spss_surrogate.h).

``Network`` is the handle on the GPU network (tcgen05 kernels in
csrc/surrogate.cu).  ``Surrogate`` adds the feature and target transforms:
inputs are the physical point (sigma, D, density, m, v0); outputs are the
expected time-averaged phase and velocity order parameters of one run and
their run-to-run variances.  A run's time average varies from run to run
(coarsening and multistable locked states make it depend on the initial
field and the noise), so the network is fitted in two stages on single runs:
the means by least squares, then the squared residuals of those means, whose
least-squares fit is the conditional variance.  ``active_sweep`` maps a
(sigma, D) grid: the network predicts every point, points whose predicted
variance is above a threshold calibrated on held-out runs are simulated with
the plain batched simulation, which stays the judge.
"""
import ctypes
import time

import numpy as np

from . import _native as N


class Network:
    """5 -> 128 -> 128 -> 128 -> 4 GELU network trained and evaluated on the GPU."""

    def __init__(self, seed=0):
        self.L = N.lib()
        h = ctypes.c_void_p()
        N.check(self.L.spss_mlp_create(int(seed), ctypes.byref(h)), "spss_mlp_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.spss_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def params(self):
        out = np.empty(N.MLP_PARAMS, dtype=np.float32)
        N.check(self.L.spss_mlp_get_params(self.h, N.fptr(out), out.size), "spss_mlp_get_params")
        return out

    @params.setter
    def params(self, flat):
        flat = np.ascontiguousarray(flat, dtype=np.float32)
        N.check(self.L.spss_mlp_set_params(self.h, N.fptr(flat), flat.size), "spss_mlp_set_params")

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N.MLP_INPUTS)
        y = np.empty((x.shape[0], N.MLP_OUTPUTS), dtype=np.float32)
        N.check(self.L.spss_mlp_forward(self.h, N.fptr(x), x.shape[0], N.fptr(y)), "spss_mlp_forward")
        return y

    def gradient(self, x, t, w=None):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N.MLP_INPUTS)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, N.MLP_OUTPUTS)
        wp = None if w is None else N.fptr(np.ascontiguousarray(w, dtype=np.float32))
        g = np.empty(N.MLP_PARAMS, dtype=np.float32)
        loss = ctypes.c_double()
        N.check(self.L.spss_mlp_gradient(self.h, N.fptr(x), N.fptr(t), wp, x.shape[0], N.fptr(g),
                                         ctypes.byref(loss)), "spss_mlp_gradient")
        return loss.value, g

    def set_data(self, x, t):
        self._x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N.MLP_INPUTS)
        self._t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, N.MLP_OUTPUTS)
        N.check(self.L.spss_mlp_set_data(self.h, N.fptr(self._x), N.fptr(self._t), self._x.shape[0]),
                "spss_mlp_set_data")

    def train(self, epochs, batch=1024, lr=1e-3, w=None, seed=0):
        """Minibatch Adam on the resident data; returns the loss of every epoch."""
        losses = np.empty(max(epochs, 1), dtype=np.float32)
        wp = None if w is None else N.fptr(np.ascontiguousarray(w, dtype=np.float32))
        N.check(self.L.spss_mlp_train(self.h, int(epochs), int(batch), float(lr), wp, int(seed), N.fptr(losses)),
                "spss_mlp_train")
        return losses[:epochs]

    @property
    def kernel_launches(self):
        c = ctypes.c_ulonglong()
        N.check(self.L.spss_mlp_kernel_launches(self.h, ctypes.byref(c)), "spss_mlp_kernel_launches")
        return c.value


# ---------------------------------------------------------------- workflow

FEATURES = ("sigma", "log10 D", "density", "log10 m", "v0")
TARGETS = ("phase order", "velocity order", "run-to-run variance of the phase order",
           "run-to-run variance of the velocity order")


def point_features(points):
    """Network inputs of physical points (before standardisation)."""
    return np.array([[p["sigma"], np.log10(p["D"]), p["density"], np.log10(p["m"]), p["v0"]] for p in points],
                    dtype=np.float64)


def run_values(stats):
    """Time-averaged phase and velocity order parameters of spss_batch_stats rows."""
    st = np.asarray(stats, dtype=np.float64)
    return np.stack([st[:, 0], st[:, 2]], axis=1)


def simulate(points, steps=2000, sample_every=10, burn_in=None, max_systems=8192, seed=0, first_replica=0,
             variant=N.LINKED_LIST_VERLET, skin=0.3, autotune=True):
    """Plain batched simulation of every point (the judge): spss_batch_stats
    rows, in the order of `points`.  Points go in batches of at most
    `max_systems` systems, each batch one context stepped as one graph per
    step.  By default every system runs the reference's linked list + Verlet
    routine with skin 0.3 R, its lists rebuilt on its own displacement
    trigger (the same neighbour sets within R as a cell list, at about half
    the candidates)."""
    from .sweep import run_sweep

    out = []
    for b0 in range(0, len(points), max_systems):
        chunk = points[b0:b0 + max_systems]
        out.append(run_sweep(chunk, steps=steps, sample_every=sample_every, burn_in=burn_in, variant=variant,
                             seed=seed, autotune=autotune, first_replica=first_replica + b0,
                             skin=skin if variant == N.LINKED_LIST_VERLET else 0.0))
    return np.concatenate(out, axis=0) if out else np.zeros((0, N.STATS_PER_SYSTEM))


class Surrogate:
    """The network with standardised features and targets and a calibrated
    threshold on the predicted fluctuation (where to trust it)."""

    def __init__(self, seed=0):
        self.net = Network(seed)
        self.threshold = np.inf

    def close(self):
        self.net.close()

    def fit(self, points, stats, epochs=200, batch=1024, lr=2e-3, seed=0):
        """Stage 1: the two means (variance outputs weighted 0); stage 2: all
        four outputs, the variance targets being the squared stage-1
        residuals.  Returns the per-epoch losses of both stages."""
        x = point_features(points)
        v = run_values(stats)
        self.x_mean, self.x_std = x.mean(axis=0), np.maximum(x.std(axis=0), 1e-6)
        xs = (x - self.x_mean) / self.x_std
        self.t_mean = np.zeros(4)
        self.t_std = np.ones(4)
        self.t_mean[:2], self.t_std[:2] = v.mean(axis=0), np.maximum(v.std(axis=0), 1e-6)
        t = np.zeros((len(points), 4))
        t[:, :2] = (v - self.t_mean[:2]) / self.t_std[:2]
        self.net.set_data(xs, t)
        l1 = self.net.train(epochs, batch=batch, lr=lr, w=[1.0, 1.0, 0.0, 0.0], seed=seed)
        res2 = (v - self.predict(points)[:, :2]) ** 2
        self.t_mean[2:], self.t_std[2:] = res2.mean(axis=0), np.maximum(res2.std(axis=0), 1e-12)
        t[:, 2:] = (res2 - self.t_mean[2:]) / self.t_std[2:]
        self.net.set_data(xs, t)
        l2 = self.net.train(max(1, epochs // 2), batch=batch, lr=0.5 * lr, seed=seed + 1)
        return np.concatenate([l1, l2])

    def predict(self, points):
        """Predicted outputs (unstandardised, columns as TARGETS; variances
        clipped at zero)."""
        x = (point_features(points) - self.x_mean) / self.x_std
        out = self.net.forward(x).astype(np.float64) * self.t_std + self.t_mean
        out[:, 2:] = np.maximum(out[:, 2:], 0.0)
        return out

    @staticmethod
    def score(pred):
        """Uncertainty score of a prediction: the larger predicted run-to-run variance."""
        return np.maximum(pred[:, 2], pred[:, 3])

    @staticmethod
    def error(pred, stats):
        """Largest absolute error of the two predicted order parameters."""
        st = np.asarray(stats)
        return np.maximum(np.abs(pred[:, 0] - st[:, 0]), np.abs(pred[:, 1] - st[:, 2]))

    def calibrate(self, points, stats, tol=0.02, coverage=0.99):
        """Largest threshold on the fluctuation score such that, on these
        held-out points, at least `coverage` of the points scored below it are
        predicted within `tol`."""
        pred = self.predict(points)
        s = self.score(pred)
        ok = self.error(pred, stats) <= tol
        order = np.argsort(s)
        good = np.cumsum(ok[order])
        k = np.arange(1, len(order) + 1)
        fine = np.nonzero(good >= coverage * k)[0]
        self.threshold = float(s[order][fine[-1]]) if len(fine) else -np.inf
        return self.threshold


def grid_points(nsigma=256, nd=256, sigma_range=(0.0, 3.0), d_range=(0.01, 1.0), n=1024, m=1.0, density=2.0,
                v0=0.5, radius=1.0):
    """The (sigma, D) phase-diagram grid: sigma uniform, D logarithmic."""
    sig = np.linspace(sigma_range[0], sigma_range[1], nsigma)
    dd = np.exp(np.linspace(np.log(d_range[0]), np.log(d_range[1]), nd))
    return [dict(n=n, sigma=float(s), D=float(d), m=m, density=density, R=radius, v0=v0) for d in dd for s in sig]


def training_points(count, seed=0, n=1024, masses=(0.1, 1.0, 10.0), density=2.0, v0=0.5):
    """Random points of the batched sweep (sigma uniform in [0, 3], D
    log-uniform in [0.01, 1], m from `masses`) at a fixed system size."""
    rng = np.random.default_rng(seed)
    sig = rng.uniform(0.0, 3.0, count)
    d = np.exp(rng.uniform(np.log(0.01), np.log(1.0), count))
    m = rng.choice(np.asarray(masses, dtype=np.float64), count)
    return [dict(n=n, sigma=float(sig[i]), D=float(d[i]), m=float(m[i]), density=density, R=1.0, v0=v0)
            for i in range(count)]


def active_sweep(sur, points, steps=2000, sample_every=10, seed=0, first_replica=0):
    """Phase diagram of `points`: the network predicts every point, points
    scored above the calibrated threshold are simulated (the judge) and their
    simulated values replace the prediction.  Returns (values [k][2] = phase
    and velocity order, simulated mask, seconds spent predicting, seconds
    spent simulating)."""
    import torch

    t0 = time.perf_counter()
    pred = sur.predict(points)
    flagged = sur.score(pred) > sur.threshold
    t1 = time.perf_counter()
    values = pred[:, :2].copy()
    idx = np.nonzero(flagged)[0]
    if len(idx):
        st = simulate([points[i] for i in idx], steps=steps, sample_every=sample_every, seed=seed,
                      first_replica=first_replica)
        values[idx, 0] = st[:, 0]
        values[idx, 1] = st[:, 2]
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return values, flagged, t1 - t0, t2 - t1


def reference(points, replicas, steps=4000, sample_every=10, seed=0, first_replica=10 ** 7):
    """High-replica estimate of the expected order parameters of `points`:
    (mean [k][2], standard deviation of one run [k][2])."""
    pts = [p for p in points for _ in range(replicas)]
    v = run_values(simulate(pts, steps=steps, sample_every=sample_every, seed=seed, first_replica=first_replica))
    v = v.reshape(len(points), replicas, 2)
    return v.mean(axis=1), v.std(axis=1, ddof=1)


def phase_diagram(grid, n_train=50000, steps=4000, epochs=100, rounds=1, flag_fraction=0.1, sample_every=10,
                  seed=0, train_seed=1, n=1024, masses=(0.1, 1.0, 10.0)):
    """Expected phase and velocity order parameters over `grid` from the
    surrogate with active learning:

    1. one plain run at each of `n_train` random points of the sweep's
       parameter space (sigma, D, m; batched simulation);
    2. fit the network (means and run-to-run variances);
    3. each round: the `flag_fraction` of grid points with the largest
       predicted variance are simulated (one plain run each, the judge); the
       runs are compared with the prediction (z = (run - mean) / std) and
       added to the training set, and the network is refitted;
    4. the network predicts every grid point.

    Returns a dict: values [k][2], std [k][2] (predicted run-to-run standard
    deviation), flagged mask, judge z-scores, run count and seconds per phase."""
    import torch

    t = {}
    t0 = time.perf_counter()
    tp = training_points(n_train, seed=train_seed, n=n, masses=masses)
    st = simulate(tp, steps=steps, sample_every=sample_every, seed=seed, first_replica=0)
    t["simulate_training"] = time.perf_counter() - t0
    sur = Surrogate(seed=seed)
    t0 = time.perf_counter()
    sur.fit(tp, st, epochs=epochs)
    t["fit"] = time.perf_counter() - t0
    flagged = np.zeros(len(grid), dtype=bool)
    z_all = []
    runs = n_train
    t["judge"] = 0.0
    for r in range(rounds):
        t0 = time.perf_counter()
        pred = sur.predict(grid)
        score = Surrogate.score(pred)
        score[flagged] = -np.inf  # judge a point once
        k = int(round(flag_fraction * len(grid)))
        idx = np.argsort(-score)[:k]
        flagged[idx] = True
        pts = [grid[i] for i in idx]
        sj = simulate(pts, steps=steps, sample_every=sample_every, seed=seed, first_replica=n_train + r * len(grid))
        vj = run_values(sj)
        z_all.append((vj - pred[idx, :2]) / np.sqrt(np.maximum(pred[idx, 2:], 1e-12)))
        runs += len(idx)
        tp = tp + pts
        st = np.concatenate([st, sj], axis=0)
        t["judge"] += time.perf_counter() - t0
        sur.close()
        sur = Surrogate(seed=seed)
        t0 = time.perf_counter()
        sur.fit(tp, st, epochs=epochs)
        t["fit"] += time.perf_counter() - t0
    t0 = time.perf_counter()
    pred = sur.predict(grid)
    torch.cuda.synchronize()
    t["predict"] = time.perf_counter() - t0
    launches = sur.net.kernel_launches
    sur.close()
    return {"values": pred[:, :2], "std": np.sqrt(pred[:, 2:]), "flagged": flagged,
            "judge_z": np.concatenate(z_all) if z_all else np.zeros((0, 2)), "runs": runs, "seconds": t,
            "network_kernel_launches": launches}
