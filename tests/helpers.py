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
