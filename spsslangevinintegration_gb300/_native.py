"""ctypes binding of libspss_gpu.so (the C ABI declared in include/spss_gpu.h).

The library is built in-tree (``spsslangevinintegration_gb300/_build``); there
is no CPU fallback: ``lib()`` raises if the library is missing or cannot load.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libspss_gpu.so")

OK = 0
ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_NOT_SUPPORTED, ERR_NONFINITE, ERR_SIZE = -1, -2, -3, -4, -5, -6

VARIANT_DISPATCH, ALL_PAIRS, LINKED_LIST, VERLET, LINKED_LIST_VERLET, GLOBAL_FIELD = range(6)
PRECISION_F64, PRECISION_F32 = 0, 1
FRAME_RAW, FRAME_WRAPPED = 0, 1
RK4, STOCHASTIC_EULER, STOCHASTIC_RUNGE_KUTTA = 0, 1, 2


class Params(ctypes.Structure):
    """spss_params (include/spss_gpu.h)."""
    _fields_ = [
        ("model", ctypes.c_int),
        ("flavor", ctypes.c_int),
        ("n", ctypes.c_int),
        ("variant", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("nc_verlet", ctypes.c_int),
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
        ("seed", ctypes.c_ulonglong),
        ("replica", ctypes.c_uint),
    ]


class SpssError(RuntimeError):
    def __init__(self, code, what=""):
        msg = lib().spss_error_string(code).decode(errors="replace")
        super().__init__("%s failed (%d): %s" % (what, code, msg))
        self.code = code


_lib = None

# name -> (restype, argtypes); every exported symbol of the C ABI
P = ctypes.POINTER
_d, _i, _l, _vp = ctypes.c_double, ctypes.c_int, ctypes.c_long, ctypes.c_void_p
_dp, _ip, _fp = P(ctypes.c_double), P(ctypes.c_int), P(ctypes.c_float)
_ull = ctypes.c_ulonglong
SIGNATURES = {
    "spss_version": (_i, []),
    "spss_error_string": (ctypes.c_char_p, [_i]),
    "spss_create": (_i, [P(Params), P(_vp)]),
    "spss_destroy": (_i, [_vp]),
    "spss_set_state": (_i, [_vp, _dp, _l]),
    "spss_get_state": (_i, [_vp, _dp, _l]),
    "spss_evaluate_rhs": (_i, [_vp, _i, _dp, _dp, _dp, _d, _d]),
    "spss_set_higher_order": (_i, [_vp, _i]),
    "spss_get_complementary_force": (_i, [_vp, _dp, _l]),
    "spss_set_natural_frequencies": (_i, [_vp, _dp, _l]),
    "spss_calculate_max_displacement": (_i, [_vp, _dp, _l]),
    "spss_get_verlet_state": (_i, [_vp, _dp, _ip, _ip]),
    "spss_set_should_update_lists": (_i, [_vp, _i]),
    "spss_get_rebuild_count": (_i, [_vp, ctypes.POINTER(ctypes.c_ulonglong)]),
    "spss_get_pre_linked_list": (_i, [_vp, _ip, _l]),
    "spss_get_cells": (_i, [_vp, _ip, _l, _ip, _l, _ip]),
    "spss_get_verlet_lists": (_i, [_vp, _ip, _l, _ip, _l, P(_l)]),
    "spss_step": (_i, [_vp, _i, _d, _d]),
    "spss_steps": (_i, [_vp, _i, _d, _d, _i]),
    "spss_step_host": (_i, [_vp, _i, _dp, _l, _d, _d]),
    "spss_get_step_counter": (_i, [_vp, P(_ull)]),
    "spss_set_step_counter": (_i, [_vp, _ull]),
    "spss_noise": (_i, [_vp, _i, _ull, _dp, _l]),
    "spss_apply_pbc": (_i, [_vp]),
    "spss_order_parameters": (_i, [_vp, _dp]),
    "spss_average_accumulate": (_i, [_vp]),
    "spss_average_get": (_i, [_vp, _dp, _l, _ip]),
    "spss_synchronize": (_i, [_vp]),
    "spss_kernel_launches": (_i, [_vp, P(_ull)]),
    "spss_set_stream": (_i, [_vp, _vp]),
    "spss_set_timing": (_i, [_vp, _i]),
    "spss_get_timing": (_i, [_vp, _dp, P(_ull)]),
    # device pointers in, device pointer out, caller's stream
    "spss_order_parameters_noalloc": (_i, [_i, _vp, _l, _vp, _vp]),
    "spss_batch_create": (_i, [P(Params), _i, P(_vp)]),
    "spss_batch_size": (_i, [_vp, _ip, P(_l)]),
    "spss_batch_order_parameters": (_i, [_vp, _dp, _l]),
    "spss_batch_run": (_i, [_vp, _i, _d, _d, _l, _l, _l]),
    "spss_batch_stats": (_i, [_vp, _dp, _l]),
    "spss_batch_reset_stats": (_i, [_vp]),
    "spss_set_tiling": (_i, [_vp, _i, _i]),
    "spss_get_tiling": (_i, [_vp, _ip, _ip]),
    "spss_set_device_rebuild": (_i, [_vp, _i]),
    "spss_autotune": (_i, [_vp, _i, _d, _i, _dp]),
    "spss_frame_async": (_i, [_vp, _i, _fp, _l]),
    "spss_integrate_dopri5": (_i, [_vp, _d, _d, _d, _d, _d, _vp, _vp, P(_l)]),
    "spss_pinned_alloc": (_i, [ctypes.c_size_t, P(_vp)]),
    "spss_pinned_free": (_i, [_vp]),
    # learned surrogate (include/spss_surrogate.h)
    "spss_mlp_create": (_i, [_ull, P(_vp)]),
    "spss_mlp_destroy": (_i, [_vp]),
    "spss_mlp_set_params": (_i, [_vp, _fp, _l]),
    "spss_mlp_get_params": (_i, [_vp, _fp, _l]),
    "spss_mlp_forward": (_i, [_vp, _fp, _l, _fp]),
    "spss_mlp_gradient": (_i, [_vp, _fp, _fp, _fp, _l, _fp, _dp]),
    "spss_mlp_set_data": (_i, [_vp, _fp, _fp, _l]),
    "spss_mlp_train": (_i, [_vp, _i, _i, ctypes.c_float, _fp, _ull, _fp]),
    "spss_mlp_kernel_launches": (_i, [_vp, P(_ull)]),
}

MLP_INPUTS, MLP_HIDDEN, MLP_OUTPUTS, MLP_PARAMS = 5, 128, 4, 34308

STATS_PER_SYSTEM = 5

# spss_observer_fn: int (*)(const double *state, long len, double t, void *user)
OBSERVER_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_long, ctypes.c_double,
                               ctypes.c_void_p)


def lib(path=None):
    """Load libspss_gpu.so (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libspss_gpu.so is not built (%s); run spsslangevinintegration_gb300.build" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc, what):
    if rc != OK:
        raise SpssError(rc, what)


def dptr(a):
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)


def fptr(a):
    return a.ctypes.data_as(_fp)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)
