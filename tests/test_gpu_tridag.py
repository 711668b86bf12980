"""The stand-alone tridag_array entry point against the oracle's Thomas
solve (tridag_array.f90:166-246), through the C ABI on device buffers."""
import numpy as np
import pytest

from oracle.lesgo_oracle import tridag_array

pytestmark = pytest.mark.gpu

TOL = 1e-12


def tridiag_case(lh, ny, n, seed=0):
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.5, 1.0, (n, ny, lh))
    c = rng.uniform(0.5, 1.0, (n, ny, lh))
    b = -(a + c + rng.uniform(0.1, 2.0, (n, ny, lh)))
    r = rng.standard_normal((n, ny, lh)) + 1j * rng.standard_normal((n, ny, lh))
    return a, b, c, r


def oracle_solve(a, b, c, r):
    n, ny, lh = a.shape
    pad = lambda x: np.concatenate([np.zeros((1, ny, lh), dtype=x.dtype), x], axis=0)
    mask = np.ones((ny, lh), dtype=bool)
    mask[:, lh - 1] = False
    mask[ny // 2, :] = False
    mask[0, 0] = False
    return tridag_array(pad(a), pad(b), pad(c), pad(r), mask)[1:]


def gpu_solve(call, a, b, c, r, sentinel=7.0):
    import torch
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    da, db, dc = dev(a), dev(b), dev(c)
    dr = dev(r.view(np.float64).copy())
    du = torch.full_like(dr, sentinel)
    torch.cuda.synchronize()          # the library may launch on a stream of its own
    n, ny, lh = a.shape
    call(da.data_ptr(), db.data_ptr(), dc.data_ptr(), dr.data_ptr(), du.data_ptr(), lh, ny, n)
    torch.cuda.synchronize()
    return du.cpu().numpy().view(np.complex128)


def solved_entries(u_gpu, u_ref):
    n, ny, lh = u_ref.shape
    m = np.zeros(u_ref.shape, dtype=bool)
    m[0, :, :lh - 1] = True                      # level 1: every kx < nx/2
    cols = np.ones((ny, lh), dtype=bool)
    cols[:, lh - 1] = False
    cols[ny // 2, :] = False
    cols[0, 0] = False
    m[:, cols] = True
    return m


def test_tridag_array_matches_oracle(built_lib):
    from lesgo_gb300.solver import LesgoGPU
    g = LesgoGPU(nx=32, ny=32, Nz=16)
    a, b, c, r = tridiag_case(lh=33, ny=64, n=70)
    ref = oracle_solve(a, b, c, r)
    out = gpu_solve(g.tridag_array, a, b, c, r)
    m = solved_entries(out, ref)
    err = np.max(np.abs(out[m] - ref[m])) / np.max(np.abs(ref[m]))
    assert err < TOL, err
    assert np.all(out[:, :, 32] == 7.0 + 7.0j)      # the kx = nx/2 column is never written


def test_tridag_array_zero_pivot_status(built_lib):
    from lesgo_gb300.solver import LesgoError, LesgoGPU
    g = LesgoGPU(nx=32, ny=32, Nz=16)
    a, b, c, r = tridiag_case(lh=5, ny=4, n=6)
    b[0] = 0.0
    with pytest.raises(LesgoError) as ei:
        gpu_solve(g.tridag_array, a, b, c, r)
    assert ei.value.code == 5
