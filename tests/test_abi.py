"""The C-ABI library builds, loads and exports every declared entry point
(no compute call: this runs without a GPU)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"\b(dgtm_[a-zA-Z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    names = declared_symbols()
    assert names, "no declarations found"
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header(pkg, built_lib):
    assert set(pkg.ABI_SYMBOLS) == declared_symbols()
    lib = pkg.load_library()
    assert lib.dgtm_version() >= 10000


def test_invalid_arguments_are_rejected_without_a_device(pkg, built_lib):
    lib = pkg.load_library()
    h = ctypes.c_void_p()
    # bad shapes fail before any CUDA call
    assert lib.dgtm_ctx_create(0, 3, 4, 2, None, 3, None, 2, 0, ctypes.byref(h)) == 1
    assert b"bad shape" in lib.dgtm_last_error_string()
    assert lib.dgtm_ctx_destroy(None) == 0
    assert lib.dgtm_estep(None, 1.0, 1, 1.0, None, None) == 1
