"""Shared helpers for the parity tests: fixtures, oracle and GPU contexts from
the same parameter dictionary, and tolerance checks."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARAM_KEYS = ("v0", "xi", "xi_r", "D_r", "xi_phi", "D_phi", "sigma", "alpha")


def fixtures(pattern="*.npz"):
    return sorted(glob.glob(os.path.join(GOLDEN, pattern)))


def load_fixture(path):
    z = np.load(path)
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    d["meta"] = json.loads(str(d["meta"]))
    return d


def oracle_system(p, **kw):
    from oracle import binding as ob

    args = {k: p.get(k, 0.0) for k in PARAM_KEYS}
    args.update(kw)
    flavor = p.get("flavor", "ptr")
    return ob.System(p["model"], p["n"], p["rho"], flavor=1 if flavor in ("ptr", 1) else 0, **args)


def gpu_context(p, precision=0, variant=0, **kw):
    from spsslangevinintegration_gb300 import Context

    args = {k: p.get(k, 0.0) for k in PARAM_KEYS}
    args.update(kw)
    flavor = p.get("flavor", "ptr")
    return Context(p["model"], p["n"], p["rho"], precision=precision, variant=variant,
                   flavor=1 if flavor in ("ptr", 1) else 0, **args)


def assert_close(got, ref, rtol, atol_scale=None, what=""):
    """|got - ref| <= rtol * |ref| + rtol * scale, scale = max |ref| (per call)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    scale = np.max(np.abs(ref)) if atol_scale is None else atol_scale
    err = np.abs(got - ref)
    bound = rtol * np.abs(ref) + rtol * scale
    bad = err > bound
    if np.any(bad):
        i = int(np.argmax(err - bound))
        raise AssertionError("%s: %d/%d entries off; worst at %d: got %r ref %r (err %.3e, bound %.3e)" % (
            what, int(bad.sum()), bad.size, i, got.flat[i], ref.flat[i], err.flat[i], bound.flat[i]))


def per_component_close(got, ref, s, rtol, what=""):
    got = np.asarray(got).reshape(-1, s)
    ref = np.asarray(ref).reshape(-1, s)
    for c in range(s):
        assert_close(got[:, c], ref[:, c], rtol, what="%s component %d" % (what, c))


def min_image(d):
    return d - np.round(d)


def initial(model, n, seed, v=0.01, omega=0.5):
    rng = np.random.default_rng(seed)
    s = 4 if model == 1 else 6
    x = np.zeros((n, s))
    x[:, 0], x[:, 1] = rng.random(n), rng.random(n)
    phi = rng.uniform(-np.pi, np.pi, n)
    if model == 1:
        x[:, 2], x[:, 3] = phi, rng.uniform(-omega, omega, n)
    else:
        x[:, 2], x[:, 3] = v * np.cos(phi), v * np.sin(phi)
        x[:, 4], x[:, 5] = phi, rng.uniform(-omega, omega, n)
    return x.reshape(-1)


def params(model, n, density=2.0, R=1.0, v0=0.5, m=1.0, D=0.1, sigma=1.0, alpha=0.0):
    """Physical parameters mapped to the reference's unit box (L = sqrt(N/density))."""
    L = np.sqrt(n / density)
    p = dict(model=model, n=n, rho=R / L, flavor="ptr", v0=v0 / L, sigma=sigma / m, alpha=alpha)
    if model == 1:
        p.update(xi=0.1, D_phi=D)
    else:
        p.update(xi_r=1.0 / m, xi_phi=1.0 / m, D_r=1e-3 / L ** 2, D_phi=D / m ** 2)
    return p


def reference_frame(x, s, wrapped):
    """The frame a reference binary observer writes for the FP64 AoS state x:
    float conversion, then (wrapped, first-order observer) the unit-box wrap
    and the phase wrap evaluated in double on the float value and rounded back
    (BinaryObserverFirstOrder.cpp:111-117, PeriodicBoundaryConditions.cpp:137-145)."""
    f = np.asarray(x, dtype=np.float64).astype(np.float32).reshape(-1, s)
    if wrapped:
        out = f.copy()
        for k in (0, 1):
            d = f[:, k].astype(np.float64)
            out[:, k] = (d - np.floor(d * 1.0) * 1.0).astype(np.float32)
        ip = 2 if s == 4 else 4
        d = f[:, ip].astype(np.float64)
        two_pi = 6.283185307179586
        out[:, ip] = (d - np.floor(d / two_pi) * two_pi).astype(np.float32)
        f = out
    return f.reshape(-1)


def config_system(model, n, density, R=1.0, v0=0.5, m=1.0, D=0.1, sigma=1.0, alpha=0.0, xi=0.1):
    """The benchmark configurations' physical parameters in the reference's
    unit box: L = sqrt(N / density), rho = R / L, v0 -> v0 / L; second order
    xi_r = xi_phi = 1 / m, sigma -> sigma / m, D_phi = D / m^2, D_r = 0;
    first order the reference's default friction xi = 0.1 and D_phi = D."""
    L = np.sqrt(n / density)
    p = dict(model=model, n=n, rho=R / L, flavor="ptr", v0=v0 / L, alpha=alpha)
    if model == 1:
        p.update(xi=xi, sigma=sigma, D_phi=D)
    else:
        p.update(xi_r=1.0 / m, xi_phi=1.0 / m, D_r=0.0, D_phi=D / m ** 2, sigma=sigma / m)
    return p, L


def config_initial(model, n, L, seed):
    """Uniform positions in the unit box, phases uniform in [-pi, pi),
    omega = 0; second order: velocity the unit vector along phi divided by L
    (SimulationEngineSecondOrder.cpp:46-50)."""
    rng = np.random.default_rng(seed)
    s = 4 if model == 1 else 6
    x = np.zeros((n, s))
    x[:, 0], x[:, 1] = rng.random(n), rng.random(n)
    phi = rng.uniform(-np.pi, np.pi, n)
    if model == 1:
        x[:, 2] = phi
    else:
        x[:, 2], x[:, 3], x[:, 4] = np.cos(phi) / L, np.sin(phi) / L, phi
    return x.reshape(-1)


def state_err(got, ref, s):
    """Per-component error |got - ref| / (|ref| + max |ref| of the component),
    positions under the minimum image with unit scale."""
    got, ref = np.asarray(got).reshape(-1, s), np.asarray(ref).reshape(-1, s)
    d = got - ref
    d[:, :2] = min_image(d[:, :2])
    scale = np.abs(ref).max(axis=0)
    scale[:2] = 1.0
    return np.abs(d) / (np.abs(ref) + scale)
