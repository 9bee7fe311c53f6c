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


def test_context_rejects_unknown_forms_before_any_device_call(pkg, built_lib):
    import numpy as np
    import pytest
    T, FI = np.zeros((8, 3)), np.zeros((4, 2))
    with pytest.raises(ValueError, match="precision"):
        pkg.Context(T, FI, "fp16")
    with pytest.raises(ValueError, match="solver"):
        pkg.Context(T, FI, "fp64", solver="qr")


def test_set_solver_is_kept_for_a_rebuilt_context(pkg, built_lib):
    """set_basis (the hierarchical expansion) re-creates the context with the
    solver last set, not the constructor's.  The library is replaced by a
    stub that records the calls: no device is needed."""
    import numpy as np

    class Stub:
        def __init__(self):
            self.calls = []

        def dgtm_set_solver(self, h, s):
            self.calls.append(("solver", s))
            return 0

        def dgtm_ctx_create(self, *args):
            self.calls.append(("create", args[2]))
            return 0

    c = object.__new__(pkg.Context)
    c._h, c.solver, c.precision = None, "cholesky", "fp64"
    c.N, c.D, c.M1 = 8, 3, 2
    stub = Stub()
    real = pkg.load_library
    try:
        pkg.load_library = lambda *a, **k: stub
        c.set_solver("svd")
        c.K = 16  # what set_basis does between close() and _create()
        c._create(np.zeros((8, 3)), np.zeros((16, 2)))
    finally:
        pkg.load_library = real
    assert c.solver == "svd"
    assert stub.calls == [("solver", pkg.SOLVE_SVD), ("create", 16), ("solver", pkg.SOLVE_SVD)]
