"""The CPU restatement (oracle/spss_oracle.c) against fixtures produced by the
reference's own sources compiled unmodified (tests/golden/make_golden.py).

Both sides are FP64 built with -ffp-contract=off and keep the reference's
summation order, so floating-point outputs must agree bit for bit; integer
outputs (cell ids, per-cell member lists, Verlet lists) must be identical.
"""
import glob
import json
import os

import numpy as np
import pytest

from oracle import binding as ob

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))
PER = {(1, "se"): 1, (1, "srk"): 2, (2, "se"): 3, (2, "srk"): 6}


def load_fixture(path):
    z = np.load(path)
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    d["meta"] = json.loads(str(d["meta"]))
    return d


def make_system(p, **kw):
    return ob.System(p["model"], p["n"], p["rho"], v0=p.get("v0", 0.0), xi=p.get("xi", 0.0), xi_r=p.get("xi_r", 0.0),
                     D_r=p.get("D_r", 0.0), xi_phi=p.get("xi_phi", 0.0), D_phi=p.get("D_phi", 0.0),
                     sigma=p.get("sigma", 0.0), alpha=p.get("alpha", 0.0),
                     flavor=1 if p["flavor"] == "ptr" else 0, **kw)


def csr_from_flat(flat, rows):
    return flat[: rows + 1], flat[rows + 1:]


def test_fixtures_present():
    assert len(FIXTURES) >= 30


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_oracle_matches_reference(path):
    f = load_fixture(path)
    p = f["params"]
    sysm = make_system(p)
    if p.get("higher_order"):
        sysm.set_higher_order(True)
    if "freqs" in f:
        sysm.set_natural_frequencies(f["freqs"])
    variant = p.get("variant", 0)
    if p["mode"] == "rhs":
        k_next = f["knext_in"].copy()
        sysm.evaluate(variant, f["state_in"], f["kprev_in"], k_next, p["k_coef"], p["dt"])
        np.testing.assert_array_equal(k_next, f["knext_out"])
        if "caf" in f and p.get("higher_order"):
            np.testing.assert_array_equal(sysm.complementary_force(), f["caf"])
    else:
        state = f["state_in"].copy()
        stepper = {"rk4": ob.RK4, "rk4_direct": ob.RK4, "se": ob.SE, "srk": ob.SRK}[p["stepper"]]
        per = PER.get((p["model"], p["stepper"]), 0)
        n, t = p["n"], 0.0
        for k in range(p["nsteps"]):
            t += p["dt"]
            normals = f["normals"][k * n * per:(k + 1) * n * per] if per else None
            sysm.step(stepper, variant, state, t, p["dt"], normals)
        np.testing.assert_array_equal(state, f["state_out"])
        assert sysm.accumulated_displacement == f["meta"]["accumulated_displacement"]
        assert sysm.should_update_lists == int(f["meta"]["should_update_lists"])

    builds_cells = variant in (ob.LINKED_LIST, ob.LINKED_LIST_VERLET) or (
        variant == 0 and p["rho"] <= 0.25)
    if builds_cells and "pll" in f:
        np.testing.assert_array_equal(sysm.pre_linked_list(), f["pll"])
        off, mem = sysm.cells()
        ref_off, ref_mem = csr_from_flat(f["cells"], off.size - 1)
        np.testing.assert_array_equal(off, ref_off)
        np.testing.assert_array_equal(mem, ref_mem)
    uses_verlet = variant in (ob.VERLET, ob.LINKED_LIST_VERLET) or (
        variant == 0 and p["model"] == 1 and p["rho"] <= 0.5 and p["rho"] < np.sqrt(0.5))
    if uses_verlet and "verlet" in f:
        off, ent = sysm.verlet()
        ref_off, ref_ent = csr_from_flat(f["verlet"], p["n"])
        np.testing.assert_array_equal(off, ref_off)
        np.testing.assert_array_equal(ent, ref_ent)


def test_isolated_particles_keep_stale_component():
    """RK4 k buffers persist: an isolated particle's k[..+3] keeps the previous step's value
    (ParticleSystemFirstOrder.cpp:223-226 with RungeKutta4Stepper.cpp:36-48)."""
    f = load_fixture(os.path.join(GOLDEN, "fo_rk4_sparse_serial.npz"))
    p = f["params"]
    sysm = make_system(p)
    state = f["state_in"].copy()
    sysm.step(ob.RK4, 0, state, p["dt"], p["dt"])
    # at least one isolated particle exists in this fixture
    k = np.full(state.size, 123.0)
    sysm.evaluate(0, state, np.zeros_like(state), k, 0.0, p["dt"])
    assert np.any(k[3::4] == 123.0)


def test_parallel_oracle_is_bitwise_serial():
    f = load_fixture(os.path.join(GOLDEN, "so_se_linkedlist_serial.npz"))
    p = f["params"]
    out = []
    for threads in (1, 4):
        ob.set_threads(threads)
        sysm = make_system(p)
        state = f["state_in"].copy()
        n = p["n"]
        for k in range(p["nsteps"]):
            sysm.step(ob.SE, 0, state, (k + 1) * p["dt"], p["dt"], f["normals"][k * n * 3:(k + 1) * n * 3])
        out.append(state)
    ob.set_threads(1)
    np.testing.assert_array_equal(out[0], out[1])
