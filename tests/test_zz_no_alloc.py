"""The allocation-free tridiagonal entry point (GPU required).

lesgo_gpu_tridag_array_noalloc exists for callers that cannot allocate
device memory; it runs the same solve as lesgo_gpu_tridag_array with its
scratch in a fixed array inside the library.  This file is collected last so
that a run stopping at the first failure has already run every other test;
it passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from test_gpu_tridag import gpu_solve, solved_entries, tridiag_case

pytestmark = pytest.mark.gpu

TOL = 1e-12          # the tolerance of the other GPU tridiagonal tests


def _noalloc_call(lib):
    def call(a, b, c, r, u, lh, ny, n):
        rc = lib.lesgo_gpu_tridag_array_noalloc(C.c_void_p(a), C.c_void_p(b), C.c_void_p(c), C.c_void_p(r),
                                               C.c_void_p(u), lh, ny, n, None)
        assert rc == 0, lib.lesgo_gpu_last_error(None).decode()
    return call


def test_noalloc_matches_allocating_entry_point_twice(built_lib):
    from lesgo_gb300 import _lib
    from lesgo_gb300.solver import LesgoGPU
    lib = _lib.load()
    g = LesgoGPU(nx=32, ny=32, Nz=16)
    # two calls in a row with different sizes and data: the shared scratch
    # keeps the first call's contents, which must not leak into the second
    for seed, (lh, ny, n) in ((11, (65, 128, 130)), (12, (33, 64, 40))):
        a, b, c, r = tridiag_case(lh=lh, ny=ny, n=n, seed=seed)
        ref = gpu_solve(g.tridag_array, a, b, c, r)
        out = gpu_solve(_noalloc_call(lib), a, b, c, r)
        m = solved_entries(out, ref)
        err = np.max(np.abs(out[m] - ref[m])) / np.max(np.abs(ref[m]))
        assert err <= TOL, err
        assert np.array_equal(out[~m], ref[~m])       # untouched entries identical (sentinel)


def test_noalloc_zero_pivot_then_good_call_on_callers_stream(built_lib):
    import torch
    from lesgo_gb300 import _lib
    from lesgo_gb300.solver import LesgoGPU
    lib = _lib.load()
    g = LesgoGPU(nx=32, ny=32, Nz=16)
    s = torch.cuda.Stream()

    def on_stream(a, b, c, r, u, lh, ny, n):
        return lib.lesgo_gpu_tridag_array_noalloc(C.c_void_p(a), C.c_void_p(b), C.c_void_p(c), C.c_void_p(r),
                                                  C.c_void_p(u), lh, ny, n, C.c_void_p(s.cuda_stream))

    # a zero pivot is reported as LESGO_ERR_NUMERIC ...
    a, b, c, r = tridiag_case(lh=5, ny=4, n=6, seed=3)
    b[0] = 0.0
    rcs = []
    gpu_solve(lambda *args: rcs.append(on_stream(*args)), a, b, c, r)
    assert rcs == [_lib.LESGO_ERR_NUMERIC]
    assert b"zero pivot" in lib.lesgo_gpu_last_error(None)
    # ... and the flag left set by that call does not fail the next good one
    a, b, c, r = tridiag_case(lh=33, ny=64, n=40, seed=4)
    ref = gpu_solve(g.tridag_array, a, b, c, r)
    rcs.clear()
    out = gpu_solve(lambda *args: rcs.append(on_stream(*args)), a, b, c, r)
    assert rcs == [_lib.LESGO_OK]
    m = solved_entries(out, ref)
    err = np.max(np.abs(out[m] - ref[m])) / np.max(np.abs(ref[m]))
    assert err <= TOL, err


def test_noalloc_rejects_sizes_beyond_its_scratch(built_lib):
    from lesgo_gb300 import _lib
    lib = _lib.load()
    rc = lib.lesgo_gpu_tridag_array_noalloc(C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), C.c_void_p(16),
                                           C.c_void_p(16), 129, 256, 194, None)
    assert rc == _lib.LESGO_ERR_ARG
    assert b"exceeds the fixed scratch" in lib.lesgo_gpu_last_error(None)


def test_noalloc_refuses_a_capturing_stream_and_keeps_the_capture(built_lib):
    """The call waits for its own result, so it cannot be captured: on a
    capturing stream it returns LESGO_ERR_ARG before queueing anything, and
    the caller's capture still ends and replays."""
    import torch
    from lesgo_gb300 import _lib
    lib = _lib.load()
    x = torch.zeros(4, device="cuda")
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        x.add_(1.0)
        rc = lib.lesgo_gpu_tridag_array_noalloc(C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), C.c_void_p(16),
                                               C.c_void_p(16), 5, 4, 6,
                                               C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.LESGO_ERR_ARG
    assert b"capturing" in lib.lesgo_gpu_last_error(None)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.all(x == 1.0)   # the captured add ran once, in the replay
