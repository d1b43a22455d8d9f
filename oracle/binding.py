"""ctypes binding of ``libspss_oracle.so`` (the FP64 CPU restatement).

Test infrastructure: see ``oracle/spss_oracle.h``.  ``build()`` compiles the
library with ``make`` in this directory if it is missing.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_BIN = os.path.join(HERE, "_ref", "spss_ref")

DISPATCH, ALL_PAIRS, LINKED_LIST, VERLET, LINKED_LIST_VERLET, GLOBAL_FIELD = range(6)
RK4, SE, SRK = 0, 1, 2


class Params(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int),
        ("flavor", ctypes.c_int),
        ("n", ctypes.c_int),
        ("v0", ctypes.c_double),
        ("xi", ctypes.c_double),
        ("xi_r", ctypes.c_double),
        ("D_r", ctypes.c_double),
        ("xi_phi", ctypes.c_double),
        ("D_phi", ctypes.c_double),
        ("sigma", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("r_max", ctypes.c_double),
        ("nc_verlet", ctypes.c_int),
    ]


def build(ref=False):
    """Compile the restatement (and, with ``ref=True``, the reference itself)."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


_libs = {}


def load(bench=False):
    name = "libspss_oracle_bench.so" if bench else "libspss_oracle.so"
    if name in _libs:
        return _libs[name]
    path = os.path.join(BUILD, name)
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    d, i, vp = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    dp = P(ctypes.c_double)
    ip = P(ctypes.c_int)
    sig = {
        "spo_create": (vp, [P(Params)]),
        "spo_destroy": (None, [vp]),
        "spo_set_threads": (None, [i]),
        "spo_get_threads": (i, []),
        "spo_set_higher_order": (None, [vp, i]),
        "spo_set_natural_frequencies": (None, [vp, dp]),
        "spo_evaluate": (i, [vp, i, dp, dp, dp, d, d]),
        "spo_get_complementary_force": (None, [vp, dp]),
        "spo_calculate_max_displacement": (None, [vp, dp]),
        "spo_accumulated_displacement": (d, [vp]),
        "spo_should_update_lists": (i, [vp]),
        "spo_set_should_update_lists": (None, [vp, i]),
        "spo_uses_verlet_list": (i, [vp]),
        "spo_num_cells_per_side": (i, [vp, i]),
        "spo_get_pre_linked_list": (None, [vp, ip]),
        "spo_get_cells": (ctypes.c_long, [vp, ip, ip]),
        "spo_get_verlet": (ctypes.c_long, [vp, ip, ip]),
        "spo_stepper_create": (vp, [i, i]),
        "spo_stepper_destroy": (None, [vp]),
        "spo_rk4_step": (i, [vp, vp, i, dp, d, d]),
        "spo_se_step": (i, [vp, vp, i, dp, d, d, dp]),
        "spo_srk_step": (i, [vp, vp, i, dp, d, d, dp]),
        "spo_normals_per_particle": (i, [i, i]),
        "spo_apply_pbc": (None, [i, i, dp]),
        "spo_order_parameters": (None, [i, i, dp, dp]),
        "spo_philox_normals": (None, [ctypes.c_ulonglong, ctypes.c_ulonglong, i, ctypes.c_long, dp]),
    }
    for fn, (res, args) in sig.items():
        f = getattr(lib, fn)
        f.restype = res
        f.argtypes = args
    _libs[name] = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class System:
    """One reference particle system (first or second order) on the CPU."""

    def __init__(self, model, n, rho, v0=0.0, xi=0.0, xi_r=0.0, D_r=0.0, xi_phi=0.0, D_phi=0.0, sigma=0.0,
                 alpha=0.0, r_max=0.0, nc_verlet=0, flavor=1, bench=False):
        self.lib = load(bench)
        self.model, self.n = model, n
        self.s = 4 if model == 1 else 6
        self.params = Params(model, flavor, n, v0, xi, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha, r_max, nc_verlet)
        self.h = self.lib.spo_create(ctypes.byref(self.params))
        if not self.h:
            raise ValueError("invalid oracle parameters")
        self.st = self.lib.spo_stepper_create(n, self.s)

    def close(self):
        if self.h:
            self.lib.spo_destroy(self.h)
            self.lib.spo_stepper_destroy(self.st)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_higher_order(self, on):
        self.lib.spo_set_higher_order(self.h, int(on))

    def set_natural_frequencies(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        self.lib.spo_set_natural_frequencies(self.h, _dp(f))

    def evaluate(self, variant, state, k_prev, k_next, k_coef, dt):
        """EvaluateRhs semantics: ``k_next`` is updated in place (and returned)."""
        state = np.ascontiguousarray(state, dtype=np.float64)
        k_prev = np.ascontiguousarray(k_prev, dtype=np.float64)
        assert k_next.dtype == np.float64 and k_next.flags.c_contiguous
        rc = self.lib.spo_evaluate(self.h, variant, _dp(state), _dp(k_prev), _dp(k_next), k_coef, dt)
        if rc:
            raise ValueError("bad variant")
        return k_next

    def complementary_force(self):
        out = np.zeros(self.n)
        self.lib.spo_get_complementary_force(self.h, _dp(out))
        return out

    def calculate_max_displacement(self, td):
        td = np.ascontiguousarray(td, dtype=np.float64)
        self.lib.spo_calculate_max_displacement(self.h, _dp(td))

    @property
    def accumulated_displacement(self):
        return self.lib.spo_accumulated_displacement(self.h)

    @property
    def should_update_lists(self):
        return self.lib.spo_should_update_lists(self.h)

    @should_update_lists.setter
    def should_update_lists(self, v):
        self.lib.spo_set_should_update_lists(self.h, int(v))

    @property
    def uses_verlet_list(self):
        return self.lib.spo_uses_verlet_list(self.h)

    def pre_linked_list(self):
        out = np.zeros(self.n, dtype=np.int32)
        self.lib.spo_get_pre_linked_list(self.h, _ip(out))
        return out

    def cells(self):
        ncell = self.lib.spo_get_cells(self.h, None, None)
        off = np.zeros(ncell + 1, dtype=np.int32)
        mem = np.zeros(self.n, dtype=np.int32)
        self.lib.spo_get_cells(self.h, _ip(off), _ip(mem))
        return off, mem

    def verlet(self):
        total = self.lib.spo_get_verlet(self.h, None, None)
        off = np.zeros(self.n + 1, dtype=np.int32)
        ent = np.zeros(max(total, 1), dtype=np.int32)
        self.lib.spo_get_verlet(self.h, _ip(off), _ip(ent))
        return off, ent[:total]

    def step(self, stepper, variant, state, t, dt, normals=None):
        """One stepper step in place on ``state`` (float64, reference AoS)."""
        assert state.dtype == np.float64 and state.flags.c_contiguous
        if stepper == RK4:
            rc = self.lib.spo_rk4_step(self.h, self.st, variant, _dp(state), t, dt)
        else:
            normals = np.ascontiguousarray(normals, dtype=np.float64)
            need = self.n * self.lib.spo_normals_per_particle(self.model, stepper)
            if normals.size < need:
                raise ValueError("need %d normals" % need)
            fn = self.lib.spo_se_step if stepper == SE else self.lib.spo_srk_step
            rc = fn(self.h, self.st, variant, _dp(state), t, dt, _dp(normals))
        if rc:
            raise ValueError("bad variant")
        return state


def normals_per_particle(model, stepper):
    return load().spo_normals_per_particle(model, stepper)


def order_parameters(model, state):
    state = np.ascontiguousarray(state, dtype=np.float64)
    s = 4 if model == 1 else 6
    out = np.zeros(4)
    load().spo_order_parameters(model, state.size // s, _dp(state), _dp(out))
    return out


def apply_pbc(model, state):
    s = 4 if model == 1 else 6
    load().spo_apply_pbc(state.size // s, s, _dp(state))
    return state


def set_threads(n, bench=False):
    load(bench).spo_set_threads(int(n))


def philox_normals(seed, step, stream, count, bench=False):
    out = np.zeros(count)
    load(bench).spo_philox_normals(seed, step, stream, count, _dp(out))
    return out
