"""Python handle on one spss_ctx (include/spss_gpu.h): thin, allocation-free
wrappers that pass numpy arrays to the C ABI and raise on any error code."""
import ctypes

import numpy as np

from . import _native as N


def make_params(model, n, rho, precision=N.PRECISION_F64, variant=N.VARIANT_DISPATCH, flavor=1, v0=0.0, xi=0.0,
                xi_r=0.0, D_r=0.0, xi_phi=0.0, D_phi=0.0, sigma=0.0, alpha=0.0, r_max=0.0, nc_verlet=0, seed=0,
                replica=0):
    """spss_params of one system (reference parameter names, unit box)."""
    return N.Params(int(model), flavor, int(n), variant, precision, nc_verlet, v0, xi, xi_r, D_r, xi_phi, D_phi, sigma,
                    rho, alpha, r_max, seed, replica)


class _PinnedAllocation:
    """Owner of one spss_pinned_alloc block; freed when the last reference
    (a PinnedArray or any numpy view of its memory) goes away."""

    def __init__(self, nbytes):
        ptr = ctypes.c_void_p()
        N.check(N.lib().spss_pinned_alloc(int(nbytes), ctypes.byref(ptr)), "spss_pinned_alloc")
        self.ptr = ptr

    def free(self):
        if self.ptr:
            N.lib().spss_pinned_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedArray:
    """A page-locked, device-mapped host array (spss_pinned_alloc).  Passed to
    Context.step_host, the upload and download kernels read and write it over
    the host link directly (no registration, no staging copy); the observers'
    frame buffers are of this kind too.  The memory lives as long as the
    PinnedArray or any numpy view of `array` does (the views hold the
    allocation); `free()` releases it at once, after which existing views
    must not be used."""

    def __init__(self, count, dtype=np.float64):
        dtype = np.dtype(dtype)
        nbytes = int(count) * dtype.itemsize
        self._alloc = _PinnedAllocation(nbytes)
        raw = (ctypes.c_char * nbytes).from_address(self._alloc.ptr.value)
        raw._owner = self._alloc  # numpy views keep `raw`, and `raw` keeps the allocation
        self.array = np.frombuffer(raw, dtype=dtype, count=int(count))

    @property
    def ptr(self):
        return self._alloc.ptr

    def free(self):
        if getattr(self, "_alloc", None) is not None:
            self.array = None
            self._alloc.free()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()


class Context:
    """One particle system on the GPU: state, interaction routine, steppers."""

    def __init__(self, model, n, rho, **kw):
        self.L = N.lib()
        self.model, self.n = int(model), int(n)
        self.s = 4 if self.model == 1 else 6
        self.nsys = 1
        self.first = np.array([0, self.n])
        self.params = make_params(model, n, rho, **kw)
        h = ctypes.c_void_p()
        N.check(self.L.spss_create(ctypes.byref(self.params), ctypes.byref(h)), "spss_create")
        self.h = h

    # -- lifetime
    def close(self):
        if getattr(self, "h", None):
            self.L.spss_destroy(self.h)
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
    def length(self):
        return self.n * self.s

    # -- state
    def set_state(self, state):
        state = N.f64(state)
        N.check(self.L.spss_set_state(self.h, N.dptr(state), state.size), "spss_set_state")

    def get_state(self):
        out = np.empty(self.length)
        N.check(self.L.spss_get_state(self.h, N.dptr(out), out.size), "spss_get_state")
        return out

    # -- right-hand side
    def evaluate_rhs(self, variant, state, k_prev, k_next, k_coef, dt):
        """EvaluateRhs semantics: returns k_next updated (input array untouched)."""
        state, k_prev = N.f64(state), N.f64(k_prev)
        out = np.array(k_next, dtype=np.float64, copy=True)
        N.check(self.L.spss_evaluate_rhs(self.h, variant, N.dptr(state), N.dptr(k_prev), N.dptr(out), k_coef, dt),
                "spss_evaluate_rhs")
        return out

    def set_higher_order(self, on):
        N.check(self.L.spss_set_higher_order(self.h, int(bool(on))), "spss_set_higher_order")

    def complementary_force(self):
        out = np.empty(self.n)
        N.check(self.L.spss_get_complementary_force(self.h, N.dptr(out), out.size), "spss_get_complementary_force")
        return out

    def set_natural_frequencies(self, f):
        f = N.f64(f)
        N.check(self.L.spss_set_natural_frequencies(self.h, N.dptr(f), f.size), "spss_set_natural_frequencies")

    # -- Verlet bookkeeping
    def calculate_max_displacement(self, td):
        td = N.f64(td)
        N.check(self.L.spss_calculate_max_displacement(self.h, N.dptr(td), td.size), "calculate_max_displacement")

    def verlet_state(self):
        acc = ctypes.c_double()
        flag = ctypes.c_int()
        uses = ctypes.c_int()
        N.check(self.L.spss_get_verlet_state(self.h, ctypes.byref(acc), ctypes.byref(flag), ctypes.byref(uses)),
                "spss_get_verlet_state")
        return acc.value, flag.value, uses.value

    def set_should_update_lists(self, flag):
        N.check(self.L.spss_set_should_update_lists(self.h, int(flag)), "spss_set_should_update_lists")

    @property
    def rebuild_count(self):
        """List builds performed so far (spss_get_rebuild_count)."""
        c = ctypes.c_ulonglong()
        N.check(self.L.spss_get_rebuild_count(self.h, ctypes.byref(c)), "spss_get_rebuild_count")
        return c.value

    # -- lists
    def pre_linked_list(self):
        out = np.empty(self.n, dtype=np.int32)
        N.check(self.L.spss_get_pre_linked_list(self.h, N.iptr(out), out.size), "spss_get_pre_linked_list")
        return out

    def cells(self):
        nc = ctypes.c_int()
        N.check(self.L.spss_get_cells(self.h, None, 0, None, 0, ctypes.byref(nc)), "spss_get_cells")
        off = np.empty(nc.value + 1, dtype=np.int32)
        mem = np.empty(self.n, dtype=np.int32)
        N.check(self.L.spss_get_cells(self.h, N.iptr(off), off.size, N.iptr(mem), mem.size, ctypes.byref(nc)),
                "spss_get_cells")
        return off, mem

    def verlet_lists(self):
        total = ctypes.c_long()
        N.check(self.L.spss_get_verlet_lists(self.h, None, 0, None, 0, ctypes.byref(total)), "spss_get_verlet_lists")
        off = np.empty(self.n + 1, dtype=np.int32)
        ent = np.empty(max(total.value, 1), dtype=np.int32)
        N.check(self.L.spss_get_verlet_lists(self.h, N.iptr(off), off.size, N.iptr(ent), ent.size,
                                             ctypes.byref(total)), "spss_get_verlet_lists")
        return off, ent[: total.value]

    # -- steppers
    def step(self, stepper, t, dt):
        N.check(self.L.spss_step(self.h, stepper, t, dt), "spss_step")

    def steps(self, stepper, t0, dt, nsteps):
        N.check(self.L.spss_steps(self.h, stepper, t0, dt, int(nsteps)), "spss_steps")

    def step_host(self, stepper, state, t, dt):
        """Drop-in DoStep on a host float64 array (updated in place)."""
        assert state.dtype == np.float64 and state.flags.c_contiguous
        N.check(self.L.spss_step_host(self.h, stepper, N.dptr(state), state.size, t, dt), "spss_step_host")
        return state

    @property
    def step_counter(self):
        c = ctypes.c_ulonglong()
        N.check(self.L.spss_get_step_counter(self.h, ctypes.byref(c)), "spss_get_step_counter")
        return c.value

    @step_counter.setter
    def step_counter(self, v):
        N.check(self.L.spss_set_step_counter(self.h, int(v)), "spss_set_step_counter")

    def noise(self, stepper, step):
        per = {N.RK4: 0, N.STOCHASTIC_EULER: 1 if self.model == 1 else 3,
               N.STOCHASTIC_RUNGE_KUTTA: 2 if self.model == 1 else 6}[stepper]
        out = np.empty(self.n * per)
        if per:
            N.check(self.L.spss_noise(self.h, stepper, int(step), N.dptr(out), out.size), "spss_noise")
        return out

    def apply_pbc(self):
        N.check(self.L.spss_apply_pbc(self.h), "spss_apply_pbc")

    # -- observers
    def order_parameters(self):
        out = np.empty(4)
        N.check(self.L.spss_order_parameters(self.h, N.dptr(out)), "spss_order_parameters")
        return out

    def average_accumulate(self):
        N.check(self.L.spss_average_accumulate(self.h), "spss_average_accumulate")

    def average(self):
        out = np.empty(self.length)
        cnt = ctypes.c_int()
        N.check(self.L.spss_average_get(self.h, N.dptr(out), out.size, ctypes.byref(cnt)), "spss_average_get")
        return out, cnt.value

    def synchronize(self):
        N.check(self.L.spss_synchronize(self.h), "spss_synchronize")

    def set_stream(self, stream_handle):
        """Issue work on a caller's cudaStream_t (an int handle; 0/None: own stream)."""
        N.check(self.L.spss_set_stream(self.h, ctypes.c_void_p(stream_handle or None)), "spss_set_stream")

    def set_timing(self, on):
        N.check(self.L.spss_set_timing(self.h, int(bool(on))), "spss_set_timing")

    def timing(self):
        ms = ctypes.c_double()
        cnt = ctypes.c_ulonglong()
        N.check(self.L.spss_get_timing(self.h, ctypes.byref(ms), ctypes.byref(cnt)), "spss_get_timing")
        return ms.value, cnt.value

    @property
    def kernel_launches(self):
        c = ctypes.c_ulonglong()
        N.check(self.L.spss_kernel_launches(self.h, ctypes.byref(c)), "spss_kernel_launches")
        return c.value

    # -- adaptive integration (FP64 contexts)
    def integrate_dopri5(self, t0, t1, dt_out, eps_abs=1e-6, eps_rel=1e-6, observer=None):
        """Dormand-Prince 5(4) with dense output from t0 to t1 (the reference's
        odeint path); `observer(state, t)` is called at t0, t0 + dt_out, ...
        with a copy of the host state and may return True to stop.  Returns
        the number of accepted steps."""
        def cb(ptr, n, t, user):
            if observer is None:
                return 0
            return 1 if observer(np.ctypeslib.as_array(ptr, shape=(n,)).copy(), t) else 0

        fn = N.OBSERVER_FN(cb)
        steps = ctypes.c_long()
        N.check(self.L.spss_integrate_dopri5(self.h, t0, t1, dt_out, eps_abs, eps_rel,
                                             ctypes.cast(fn, ctypes.c_void_p), None, ctypes.byref(steps)),
                "spss_integrate_dopri5")
        return steps.value

    # -- tiling of the pair-and-update kernel (F32 contexts)
    def set_tiling(self, tile_cells, persistent=False):
        N.check(self.L.spss_set_tiling(self.h, int(tile_cells), int(bool(persistent))), "spss_set_tiling")

    def tiling(self):
        tc, pers = ctypes.c_int(), ctypes.c_int()
        N.check(self.L.spss_get_tiling(self.h, ctypes.byref(tc), ctypes.byref(pers)), "spss_get_tiling")
        return tc.value, bool(pers.value)

    def set_device_rebuild(self, enabled):
        """Graph-driven steps rebuild lists through a device-launched graph (True, default) or
        under a conditional graph node (False); results are identical."""
        N.check(self.L.spss_set_device_rebuild(self.h, int(bool(enabled))), "spss_set_device_rebuild")

    def autotune(self, stepper, dt, steps=5):
        """Fastest tiling over trial steps; the state is restored.  Returns ms per step."""
        ms = ctypes.c_double()
        N.check(self.L.spss_autotune(self.h, stepper, dt, int(steps), ctypes.byref(ms)), "spss_autotune")
        return ms.value

    # -- per-system order parameters and their time averages (F32 contexts)
    def system_order_parameters(self):
        out = np.empty((self.nsys, 4))
        N.check(self.L.spss_batch_order_parameters(self.h, N.dptr(out), out.size), "spss_batch_order_parameters")
        return out

    def run(self, stepper, t0, dt, nsteps, sample_every=0, sample_from=0):
        N.check(self.L.spss_batch_run(self.h, stepper, t0, dt, int(nsteps), int(sample_every), int(sample_from)),
                "spss_batch_run")

    def stats(self):
        """(nsys, 5): mean and variance of the phase order, mean and variance of
        the velocity-direction order, number of samples."""
        out = np.empty((self.nsys, N.STATS_PER_SYSTEM))
        N.check(self.L.spss_batch_stats(self.h, N.dptr(out), out.size), "spss_batch_stats")
        return out

    def reset_stats(self):
        N.check(self.L.spss_batch_reset_stats(self.h), "spss_batch_reset_stats")


class Batch(Context):
    """Independent systems stepped together (spss_batch_create); every
    element of `systems` is a dict of make_params keywords.  State arrays are
    the systems' AoS arrays concatenated in order (`first` holds the
    particle offsets)."""

    def __init__(self, systems):
        self.L = N.lib()
        plist = [make_params(**kw) for kw in systems]
        arr = (N.Params * len(plist))(*plist)
        self.model = int(plist[0].model)
        self.s = 4 if self.model == 1 else 6
        self.n = int(sum(p.n for p in plist))
        self.params = plist[0]
        self.systems = plist
        h = ctypes.c_void_p()
        N.check(self.L.spss_batch_create(arr, len(plist), ctypes.byref(h)), "spss_batch_create")
        self.h = h
        ns = ctypes.c_int()
        N.check(self.L.spss_batch_size(self.h, ctypes.byref(ns), None), "spss_batch_size")
        self.nsys = ns.value
        first = (ctypes.c_long * (self.nsys + 1))()
        N.check(self.L.spss_batch_size(self.h, ctypes.byref(ns), first), "spss_batch_size")
        self.first = np.array(first[:], dtype=np.int64)

    def system_rows(self, state, r):
        """The AoS rows of system r in a concatenated state array."""
        return state[self.s * self.first[r]: self.s * self.first[r + 1]]
