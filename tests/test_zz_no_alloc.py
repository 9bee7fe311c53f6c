"""The free-energy forward that allocates nothing (dgtm_fe_forward_noalloc).

It exists for callers that cannot allocate device memory at all -- code that
runs where cudaMalloc is forbidden or too costly, or whose device memory is
owned by another allocator.  Through the C ABI it must give the same F as
dgtm_fe_forward (which takes a caller workspace) and as the oracle, on two
calls in a row with different problems, allocate no device memory once its
first call on the device has run (that call may be the one that makes the
driver load the library's device code, array included), and refuse a
problem too large for its fixed scratch array with a clear error.  This file
is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def forward_with_workspace(lib, Y, T, beta, temp, stream):
    K, D = Y.shape
    N = T.shape[0]
    size = ctypes.c_size_t()
    assert lib.dgtm_fe_workspace_size(N, K, D, ctypes.byref(size)) == 0
    ws = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
    ptr = ws.data_ptr() + ((-ws.data_ptr()) % 256)
    F = torch.empty((), dtype=torch.float64, device="cuda")
    rc = lib.dgtm_fe_forward(Y.data_ptr(), T.data_ptr(), N, K, D, beta, temp, ptr, size.value,
                             stream, F.data_ptr())
    assert rc == 0, lib.dgtm_last_error_string()
    torch.cuda.synchronize()
    return F.item()


def forward_noalloc(lib, Y, T, beta, temp, stream, F):
    K, D = Y.shape
    N = T.shape[0]
    rc = lib.dgtm_fe_forward_noalloc(Y.data_ptr(), T.data_ptr(), N, K, D, beta, temp, stream,
                                     F.data_ptr())
    assert rc == 0, lib.dgtm_last_error_string()
    torch.cuda.synchronize()
    return F.item()


def problem(seed, N, K, D):
    rng = np.random.default_rng(seed)
    T = rng.random((N, D)).astype(np.float32)
    Y = T[rng.integers(0, N, K)] + 0.05 * rng.standard_normal((K, D)).astype(np.float32)
    return (torch.tensor(Y, device="cuda").contiguous(),
            torch.tensor(T, device="cuda").contiguous())


def oracle_F(orc, Y, T, beta, temp):
    """F = N nfree of the reference's DA quality (FP64, on the FP32 inputs)."""
    Yh = Y.double().cpu().numpy()
    Th = T.double().cpu().numpy()
    N, D = Th.shape
    K = Yh.shape[0]
    _, _, vgc2 = orc.resp(orc.dist(Yh, Th), beta, 1, temp)
    return N * orc.qual(N, K, D, beta, vgc2, 1, temp)


def test_noalloc_forward_matches_the_workspace_forward(pkg, orc):
    lib = pkg.load_library()
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row; the second, smaller problem reuses the array the
    # first one filled.  The first call on the device may load the library's
    # device code (and with it the array), so the second is the one whose
    # memory is watched: free device memory and torch's own counters.
    cases = [(11, 4096, 256, 16, 5.0, 1.7), (12, 1000, 100, 12, 9.0, 1.0)]
    for i, (seed, N, K, D, beta, temp) in enumerate(cases):
        Y, T = problem(seed, N, K, D)
        F_ref = forward_with_workspace(lib, Y, T, beta, temp, stream)
        F_out = torch.empty((), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        if i == 1:
            free_before = torch.cuda.mem_get_info()[0]
            alloc_before = torch.cuda.memory_allocated()
            reserved_before = torch.cuda.memory_reserved()
        F = forward_noalloc(lib, Y, T, beta, temp, stream, F_out)
        if i == 1:
            assert torch.cuda.memory_allocated() == alloc_before
            assert torch.cuda.memory_reserved() == reserved_before
            assert torch.cuda.mem_get_info()[0] == free_before
        assert np.isfinite(F)
        # the free-energy tests' tolerance on F
        assert F == pytest.approx(F_ref, rel=1e-5)
        assert F == pytest.approx(oracle_F(orc, Y, T, beta, temp), rel=1e-5)


def test_noalloc_forward_rejects_problems_beyond_its_scratch(pkg):
    lib = pkg.load_library()
    Y, T = problem(13, 64, 16, 8)
    F = torch.empty((), dtype=torch.float64, device="cuda")
    rc = lib.dgtm_fe_forward_noalloc(Y.data_ptr(), T.data_ptr(), 10_000_000, 16, 8, 1.0, 1.0,
                                     torch.cuda.current_stream().cuda_stream, F.data_ptr())
    assert rc == 1
    assert b"bytes of scratch" in lib.dgtm_last_error_string()
