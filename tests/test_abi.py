"""The C ABI library loads without a GPU and exports every entry point that
include/spss_gpu.h declares; the Python binding covers all of them."""
import ctypes
import os
import re

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
