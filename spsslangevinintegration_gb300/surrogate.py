"""Learned surrogate of the stationary order parameters (include/spss_surrogate.h).

``Network`` is the handle on the GPU network (tcgen05 kernels in
csrc/surrogate.cu).  ``Surrogate`` adds the feature and target transforms:
inputs are the physical point (sigma, D, density, m, v0), targets the
time-averaged phase and velocity order parameters and their variances as
``spss_batch_stats`` reports them.  ``active_sweep`` maps a (sigma, D) grid:
the network predicts every point, points whose predicted fluctuation is large
(near a transition) or whose prediction lies in the ambiguous middle are
re-simulated with the plain batched simulation, which stays the judge.
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
