"""Generate the golden fixtures in this directory from the reference itself.

Run with the path of the reference source tree (or SPSS_REFERENCE set):

    python tests/golden/make_golden.py --ref /path/to/reference

It compiles the reference's own hot-path sources unmodified (``make ref`` in
``oracle/``: single-rank MPI stand-in, noise-replay shim, -ffp-contract=off),
runs each case below through ``oracle/_ref/spss_ref`` in its own process (the
reference keeps function-local static buffers sized at their first call) and
stores inputs and outputs as ``<case>.npz``.  The reference has no tests,
fixtures or golden vectors of its own, so these runs are what pins the CPU
restatement in ``oracle/spss_oracle.c``.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")
REF_BIN = os.path.join(ORACLE, "_ref", "spss_ref")


def initial_state(model, n, seed, v0=0.1, omega_scale=0.5, outside=0):
    """Uniform positions and phases; `outside` particles nudged just out of the box."""
    rng = np.random.default_rng(seed)
    s = 4 if model == 1 else 6
    x = np.zeros((n, s))
    x[:, 0] = rng.random(n)
    x[:, 1] = rng.random(n)
    phi = rng.uniform(-np.pi, np.pi, n)
    if model == 1:
        x[:, 2] = phi
        x[:, 3] = rng.uniform(-omega_scale, omega_scale, n)
    else:
        x[:, 2] = v0 * np.cos(phi) * rng.uniform(0.5, 1.5, n)
        x[:, 3] = v0 * np.sin(phi) * rng.uniform(0.5, 1.5, n)
        x[:, 4] = phi
        x[:, 5] = rng.uniform(-omega_scale, omega_scale, n)
    if outside:
        idx = rng.choice(n, outside, replace=False)
        for q, i in enumerate(idx):
            c = q % 2
            x[i, c] = -rng.uniform(1e-4, 2e-3) if (q // 2) % 2 == 0 else 1.0 + rng.uniform(0.0, 2e-3)
    return x.reshape(-1)


CASES = []


def case(name, **kw):
    CASES.append(dict(name=name, **kw))


# ---- first order, single RHS evaluations ------------------------------------
P1 = dict(v0=0.02, xi=0.1, sigma=1.0, alpha=0.3, D_phi=0.05)
case("fo_rhs_allpairs_serial", model=1, flavor="serial", mode="rhs", variant=1, n=200, rho=0.12, k_coef=0.5,
     dt=0.01, seed=1, **P1)
case("fo_rhs_allpairs_ptr", model=1, flavor="ptr", mode="rhs", variant=1, n=200, rho=0.12, k_coef=0.5, dt=0.01,
     seed=2, higher_order=1, outside=6, **P1)
case("fo_rhs_allpairs_n1000", model=1, flavor="serial", mode="rhs", variant=1, n=1000, rho=1 / np.sqrt(1000.0),
     k_coef=0.0, dt=0.01, seed=3, v0=0.1 / np.sqrt(1000.0), xi=0.1, sigma=1.0, alpha=0.0, D_phi=0.0)
case("fo_rhs_linkedlist_serial", model=1, flavor="serial", mode="rhs", variant=2, n=400, rho=0.08, k_coef=0.5,
     dt=0.01, seed=4, outside=8, **P1)
case("fo_rhs_linkedlist_ptr", model=1, flavor="ptr", mode="rhs", variant=2, n=400, rho=0.08, k_coef=1.0, dt=0.01,
     seed=5, higher_order=1, outside=8, **P1)
case("fo_rhs_verlet_ptr", model=1, flavor="ptr", mode="rhs", variant=3, n=300, rho=0.3, k_coef=0.5, dt=0.01,
     seed=6, higher_order=1, **P1)
case("fo_rhs_llverlet_ptr", model=1, flavor="ptr", mode="rhs", variant=4, n=600, rho=0.06, k_coef=0.5, dt=0.01,
     seed=7, higher_order=1, outside=10, **P1)
case("fo_rhs_llverlet_serial", model=1, flavor="serial", mode="rhs", variant=4, n=600, rho=0.06, k_coef=0.0,
     dt=0.01, seed=8, **P1)
case("fo_rhs_global_serial", model=1, flavor="serial", mode="rhs", variant=5, n=300, rho=0.8, k_coef=0.5, dt=0.01,
     seed=9, freqs=True, **P1)
case("fo_rhs_global_ptr", model=1, flavor="ptr", mode="rhs", variant=5, n=300, rho=0.8, k_coef=0.5, dt=0.01,
     seed=10, freqs=True, higher_order=1, **P1)

# ---- first order, steppers (reference dispatch on rho) ----------------------
P1s = dict(v0=0.3, xi=0.1, sigma=1.0, alpha=0.2, D_phi=0.1)
case("fo_rk4_llverlet_ptr", model=1, flavor="ptr", mode="step", stepper="rk4", n=400, rho=0.1, dt=0.01, nsteps=25,
     seed=11, **P1s)
case("fo_rk4_llverlet_serial", model=1, flavor="serial", mode="step", stepper="rk4", n=400, rho=0.1, dt=0.01,
     nsteps=25, seed=12, **P1s)
case("fo_rk4_verlet_serial", model=1, flavor="serial", mode="step", stepper="rk4", n=200, rho=0.3, dt=0.01,
     nsteps=10, seed=13, **P1s)
case("fo_rk4_allpairs_serial", model=1, flavor="serial", mode="step", stepper="rk4", n=150, rho=0.6, dt=0.01,
     nsteps=5, seed=14, **P1s)
case("fo_rk4direct_allpairs_n1000", model=1, flavor="serial", mode="step", stepper="rk4_direct", variant=1,
     n=1000, rho=1 / np.sqrt(1000.0), dt=0.01, nsteps=3, seed=15, v0=0.1 / np.sqrt(1000.0), xi=0.1, sigma=1.0,
     alpha=0.0, D_phi=0.0)
case("fo_se_llverlet_ptr", model=1, flavor="ptr", mode="step", stepper="se", n=400, rho=0.1, dt=0.01, nsteps=25,
     seed=16, noise=True, **P1s)
case("fo_srk_llverlet_ptr", model=1, flavor="ptr", mode="step", stepper="srk", n=400, rho=0.1, dt=0.01, nsteps=25,
     seed=17, noise=True, **P1s)
case("fo_srk_allpairs_ptr", model=1, flavor="ptr", mode="step", stepper="srk", n=150, rho=0.6, dt=0.01, nsteps=5,
     seed=18, noise=True, **P1s)
case("fo_srk_global_ptr", model=1, flavor="ptr", mode="step", stepper="srk", n=150, rho=0.8, dt=0.01, nsteps=5,
     seed=19, noise=True, **P1s)

# ---- second order, single RHS evaluations -----------------------------------
P2 = dict(v0=0.05, xi_r=1.0, D_r=0.01, xi_phi=1.0, D_phi=0.1, sigma=1.0, alpha=0.4)
case("so_rhs_allpairs_serial", model=2, flavor="serial", mode="rhs", variant=1, n=200, rho=0.12, k_coef=0.5,
     dt=0.01, seed=21, outside=6, **P2)
case("so_rhs_allpairs_ptr", model=2, flavor="ptr", mode="rhs", variant=1, n=200, rho=0.12, k_coef=0.5, dt=0.01,
     seed=22, **P2)
case("so_rhs_linkedlist_serial", model=2, flavor="serial", mode="rhs", variant=2, n=500, rho=0.07, k_coef=0.5,
     dt=0.01, seed=23, outside=10, **P2)
case("so_rhs_linkedlist_ptr", model=2, flavor="ptr", mode="rhs", variant=2, n=500, rho=0.07, k_coef=1.0, dt=0.01,
     seed=24, outside=10, **P2)

# ---- second order, steppers ---------------------------------------------------
P2s = dict(v0=0.5, xi_r=1.0, D_r=0.02, xi_phi=1.0, D_phi=0.1, sigma=1.0, alpha=0.0)
case("so_se_linkedlist_serial", model=2, flavor="serial", mode="step", stepper="se", n=500, rho=0.07, dt=0.005,
     nsteps=20, seed=25, noise=True, **P2s)
case("so_rk4_linkedlist_serial", model=2, flavor="serial", mode="step", stepper="rk4", n=400, rho=0.08, dt=0.005,
     nsteps=10, seed=26, **P2s)
case("so_rk4_allpairs_ptr", model=2, flavor="ptr", mode="step", stepper="rk4", n=150, rho=0.3, dt=0.005, nsteps=5,
     seed=27, **P2s)
case("so_se_allpairs_serial", model=2, flavor="serial", mode="step", stepper="se", n=150, rho=0.3, dt=0.005,
     nsteps=10, seed=28, noise=True, **P2s)

# ---- sparse systems: many isolated particles (RHS leaves k[..+3] / k[..+5] unwritten)
case("fo_rk4_sparse_serial", model=1, flavor="serial", mode="step", stepper="rk4", n=100, rho=0.05, dt=0.01,
     nsteps=12, seed=31, **P1s)
case("fo_srk_sparse_ptr", model=1, flavor="ptr", mode="step", stepper="srk", n=100, rho=0.05, dt=0.01, nsteps=12,
     seed=32, noise=True, **P1s)
case("so_rk4_sparse_serial", model=2, flavor="serial", mode="step", stepper="rk4", n=100, rho=0.05, dt=0.005,
     nsteps=12, seed=33, **P2s)
case("so_se_sparse_serial", model=2, flavor="serial", mode="step", stepper="se", n=100, rho=0.05, dt=0.005,
     nsteps=12, seed=34, noise=True, **P2s)

NORMALS = {("step", 1, "se"): 1, ("step", 1, "srk"): 2, ("step", 2, "se"): 3}


def run_case(c, tmp):
    model, n = c["model"], c["n"]
    s = 4 if model == 1 else 6
    state = initial_state(model, n, c["seed"], v0=c.get("v0", 0.1), outside=c.get("outside", 0))
    rng = np.random.default_rng(c["seed"] + 1000)
    kprev = rng.normal(0.0, 0.5, n * s)
    knext = 777.0 + np.arange(n * s, dtype=np.float64)  # sentinel: shows entries the RHS leaves untouched
    files = {}
    for key, arr in (("state", state), ("kprev", kprev), ("knext", knext)):
        path = os.path.join(tmp, "%s_%s.bin" % (c["name"], key))
        arr.astype(np.float64).tofile(path)
        files[key] = path
    arrays = dict(state_in=state, kprev_in=kprev, knext_in=knext)
    if c.get("freqs"):
        f = rng.normal(0.0, 0.1, n)
        path = os.path.join(tmp, c["name"] + "_freqs.bin")
        f.tofile(path)
        files["freqs"] = path
        arrays["freqs"] = f
    if c.get("noise"):
        per = NORMALS[(c["mode"], model, c["stepper"])]
        normals = rng.normal(0.0, 1.0, n * per * c["nsteps"])
        path = os.path.join(tmp, c["name"] + "_noise.bin")
        normals.tofile(path)
        files["noise"] = path
        arrays["normals"] = normals
    out = os.path.join(tmp, c["name"])
    cfg = dict(model=model, flavor=c["flavor"], mode=c["mode"], variant=c.get("variant", 0),
               stepper=c.get("stepper", "rk4"), n=n, nsteps=c.get("nsteps", 1),
               higher_order=c.get("higher_order", 0), k_coef=c.get("k_coef", 0.0), dt=c["dt"], rho=c["rho"],
               out=out)
    for k in ("v0", "xi", "xi_r", "D_r", "xi_phi", "D_phi", "sigma", "alpha"):
        cfg[k] = c.get(k, 0.0)
    cfg.update(files)
    cfg_path = os.path.join(tmp, c["name"] + ".cfg")
    with open(cfg_path, "w") as f:
        for k, v in cfg.items():
            f.write("%s %s\n" % (k, repr(float(v)) if isinstance(v, (float, np.floating)) else v))
    subprocess.run([REF_BIN, cfg_path], check=True)

    def rd(suffix, dtype):
        p = "%s_%s.bin" % (out, suffix)
        return np.fromfile(p, dtype=dtype) if os.path.exists(p) else None

    if c["mode"] == "rhs":
        arrays["knext_out"] = rd("knext", np.float64)
    else:
        arrays["state_out"] = rd("state", np.float64)
    for key, suffix, dtype in (("pll", "pll", np.int32), ("cells", "cells", np.int32), ("verlet", "verlet", np.int32),
                               ("caf", "caf", np.float64)):
        v = rd(suffix, dtype)
        if v is not None and v.size:
            arrays[key] = v
    meta = {}
    with open(out + "_meta.txt") as f:
        for line in f:
            k, v = line.split()
            meta[k] = float(v)
    params = {k: (float(v) if isinstance(v, (float, np.floating)) else v) for k, v in c.items()}
    arrays["params"] = np.array(json.dumps(params))
    arrays["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, c["name"] + ".npz"), **arrays)
    return meta


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("SPSS_REFERENCE"),
                    help="reference source tree (default: $SPSS_REFERENCE)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give the reference source tree with --ref or SPSS_REFERENCE")
    subprocess.run(["make", "-s", "-C", ORACLE, "ref", "REF=" + args.ref], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        for c in CASES:
            meta = run_case(c, tmp)
            print("%-34s %s" % (c["name"], meta))
    return 0


if __name__ == "__main__":
    sys.exit(main())
