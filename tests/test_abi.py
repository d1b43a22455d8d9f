"""The C ABI library loads without a GPU and exports every entry point that
include/spss_gpu.h declares; the Python binding covers all of them."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(spss_\w+)\s*\(", text, flags=re.M))
    return names


def built_library():
    from spsslangevinintegration_gb300 import build

    return build.build_library()


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("spss_create", "spss_destroy", "spss_evaluate_rhs", "spss_step", "spss_noise",
                 "spss_order_parameters"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(built_library())
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    from spsslangevinintegration_gb300 import _native

    assert declared_symbols() <= set(_native.SIGNATURES), declared_symbols() - set(_native.SIGNATURES)


def test_error_strings_without_gpu():
    from spsslangevinintegration_gb300 import _native

    L = _native.lib(built_library())
    assert L.spss_error_string(0) == b"ok"
    assert b"invalid" in L.spss_error_string(-1)
    # argument checks run before any CUDA call
    assert L.spss_create(None, None) == _native.ERR_INVALID_ARGUMENT
    assert L.spss_step(None, 0, 0.0, 0.01) == _native.ERR_INVALID_ARGUMENT


def test_batch_argument_checks_without_gpu():
    """spss_batch_create validates the system table before any CUDA call."""
    from spsslangevinintegration_gb300 import _native, make_params

    L = _native.lib(built_library())
    h = ctypes.c_void_p()
    a = make_params(2, 1000, 0.05, precision=_native.PRECISION_F32, variant=_native.LINKED_LIST, seed=1)
    b = make_params(1, 500, 0.05, precision=_native.PRECISION_F32, variant=_native.LINKED_LIST, seed=1)
    arr = (_native.Params * 2)(a, b)
    assert L.spss_batch_create(arr, 2, ctypes.byref(h)) == _native.ERR_INVALID_ARGUMENT  # models differ
    c = make_params(2, 1000, 0.05, precision=_native.PRECISION_F32, variant=_native.LINKED_LIST, seed=2)
    arr = (_native.Params * 2)(a, c)
    assert L.spss_batch_create(arr, 2, ctypes.byref(h)) == _native.ERR_INVALID_ARGUMENT  # seeds differ
    d = make_params(2, 1000, 0.05, precision=_native.PRECISION_F64, variant=_native.LINKED_LIST, seed=1)
    arr = (_native.Params * 1)(d)
    assert L.spss_batch_create(arr, 1, ctypes.byref(h)) == _native.ERR_NOT_SUPPORTED  # batches run in F32
    assert L.spss_batch_create(arr, 0, ctypes.byref(h)) == _native.ERR_INVALID_ARGUMENT
    assert L.spss_batch_run(None, 1, 0.0, 0.005, 10, 1, 0) == _native.ERR_INVALID_ARGUMENT
    assert L.spss_set_tiling(None, 32, 0) == _native.ERR_INVALID_ARGUMENT
    assert L.spss_autotune(None, 1, 0.005, 2, None) == _native.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("program", ["dropin_example.cpp", "engine_loops.cpp"])
def test_cpp_dropin_programs_compile_and_link(tmp_path, program):
    """The reference-named C++ classes (include/spss/spss.hpp) and the programs
    that drive them as the reference's engines do compile warning-free and
    link against the library without a GPU (running them needs one)."""
    import subprocess

    lib = built_library()
    exe = str(tmp_path / program.replace(".cpp", ""))
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", program), "-o", exe, "-pthread",
                    "-L" + os.path.dirname(lib), "-lspss_gpu", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    assert os.path.getsize(exe) > 0


def test_no_cpu_fallback_without_a_gpu():
    """Without a GPU the library refuses to create a context (a CUDA error
    code, raised as SpssError) instead of computing on the CPU."""
    import pytest

    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from spsslangevinintegration_gb300 import LINKED_LIST, PRECISION_F32, Context, SpssError

    built_library()
    with pytest.raises(SpssError):
        Context(2, 1000, 0.05, precision=PRECISION_F32, variant=LINKED_LIST)
