"""Every kernel launched with the programmatic-dependent-launch attribute
(launch_chained in csrc/) must begin with pdl_enter(), the wait for the
kernel before it in the stream: without it the kernel could read its
predecessor's outputs (cell offsets, slot order, parity) before they are
written.  Checked on the sources, so it runs without a GPU."""
import os
import re

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "spsslangevinintegration_gb300",
                    "csrc")


def _sources():
    out = {}
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".cu", ".cuh")):
            with open(os.path.join(CSRC, name)) as f:
                out[name] = f.read()
    return out


def _chained_kernels(src):
    """Kernel names passed to launch_chained (template arguments stripped)."""
    names = set()
    # call sites only: the helper's own definition starts with "bool chained"
    for m in re.finditer(r"launch_chained\(\s*(?!bool\b)[^,]+,\s*([A-Za-z_][A-Za-z0-9_]*)", src):
        names.add(m.group(1))
    return names


def _first_statement(src, kernel):
    """First statement of each __global__ definition of `kernel`, skipping
    __shared__ declarations."""
    firsts = []
    for m in re.finditer(r"__global__[^;{]*?\b%s\s*\(" % re.escape(kernel), src):
        body = src.index("{", m.end())
        stmts = [s.strip() for s in src[body + 1:body + 4000].split(";")]
        for s in stmts:
            s = re.sub(r"//[^\n]*", "", s).strip()
            if s and not s.startswith("__shared__"):
                firsts.append(s)
                break
    return firsts


def test_every_chained_kernel_begins_with_its_wait():
    srcs = _sources()
    allsrc = "\n".join(srcs.values())
    kernels = set()
    for s in srcs.values():
        kernels |= _chained_kernels(s)
    assert {"fast_tile_kernel", "fast_permute_kernel", "bin_scatter_kernel", "scan_tile_kernel"} <= kernels
    for k in sorted(kernels):
        firsts = _first_statement(allsrc, k)
        assert firsts, "no __global__ definition found for %s" % k
        for s in firsts:
            assert s.startswith("pdl_enter()"), "%s begins with %r, not pdl_enter()" % (k, s[:60])


def test_pdl_enter_waits_on_the_predecessor():
    with open(os.path.join(CSRC, "spss_internal.cuh")) as f:
        src = f.read()
    m = re.search(r"void pdl_enter\(\)\s*\{(.*?)\}", src, re.S)
    assert m and "griddepcontrol.wait" in m.group(1)
