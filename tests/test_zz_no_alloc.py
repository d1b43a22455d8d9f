"""spss_order_parameters_noalloc: the order-parameter reduction for callers
that must not allocate device memory (for instance a host application whose
own allocator owns the GPU's memory), with its scratch in a fixed array
inside the library.

Called through the C ABI on device buffers the test owns, twice in a row,
and compared with the existing entry point spss_order_parameters within the
FP64 path's tolerance (1e-12 relative); also captured into a CUDA graph after
one warm call (the use the header's "first call before any stream capture"
rule is for) and replayed on two different states.  This file sorts last so
that a run stopping at the first failure has run every other test first."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(model, n, seed):
    rng = np.random.default_rng(seed)
    s = 4 if model == 1 else 6
    x = np.zeros((n, s))
    x[:, 0], x[:, 1] = rng.random(n), rng.random(n)
    phi = rng.normal(0.3, 0.8, n)  # partly aligned phases: |R| well away from 0
    x[:, s - 2] = phi
    if model == 2:
        x[:, 2], x[:, 3] = np.cos(phi) * rng.random(n), np.sin(phi) * rng.random(n)
    return x.reshape(-1)


@pytest.mark.parametrize("model,n", [(2, 300000), (1, 5000), (2, 1)])
def test_noalloc_matches_existing_entry_point_on_two_calls(model, n):
    import torch

    from spsslangevinintegration_gb300 import Context, _native as N

    L = N.lib()
    x = _state(model, n, seed=n)
    with Context(model, n, 0.01) as ctx:
        ctx.set_state(x)
        ref = ctx.order_parameters()
    d_state = torch.from_numpy(x).to("cuda")
    d_out = torch.empty(4, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        d_out.fill_(float("nan"))
        rc = L.spss_order_parameters_noalloc(model, ctypes.c_void_p(d_state.data_ptr()), n,
                                             ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream))
        assert rc == N.OK, L.spss_error_string(rc)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)


def test_noalloc_call_captured_in_a_graph_replays_on_new_state():
    """One warm call looks up the scratch's device address; the next call is
    captured into a graph on torch's capture stream, and each replay reduces
    whatever state the buffer then holds."""
    import torch

    from spsslangevinintegration_gb300 import Context, _native as N

    L = N.lib()
    model, n = 2, 200000
    xs = [_state(model, n, seed=s) for s in (11, 12)]
    refs = []
    for x in xs:
        with Context(model, n, 0.01) as ctx:
            ctx.set_state(x)
            refs.append(ctx.order_parameters())
    d_state = torch.from_numpy(xs[1]).to("cuda")
    d_out = torch.empty(4, dtype=torch.float64, device="cuda")
    sp, op = ctypes.c_void_p(d_state.data_ptr()), ctypes.c_void_p(d_out.data_ptr())
    rc = L.spss_order_parameters_noalloc(model, sp, n, op, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.OK, L.spss_error_string(rc)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = L.spss_order_parameters_noalloc(model, sp, n, op, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.OK, L.spss_error_string(rc)
    for x, ref in zip(xs, refs):
        d_state.copy_(torch.from_numpy(x))
        d_out.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_allclose(d_out.cpu().numpy(), ref, rtol=1e-12, atol=1e-12)


def test_noalloc_rejects_sizes_beyond_the_limit():
    import torch

    from spsslangevinintegration_gb300 import _native as N

    L = N.lib()
    d = torch.zeros(6, dtype=torch.float64, device="cuda")
    ptr = ctypes.c_void_p(d.data_ptr())
    assert L.spss_order_parameters_noalloc(2, ptr, (1 << 30) + 1, ptr, None) == N.ERR_SIZE
    assert L.spss_order_parameters_noalloc(2, ptr, 0, ptr, None) == N.ERR_SIZE
    assert L.spss_order_parameters_noalloc(3, ptr, 1, ptr, None) == N.ERR_INVALID_ARGUMENT
