"""Transform semantics pinned against a second FFT library (GPU required).

The reference's x-y transforms are FFTW's unnormalised r2c / c2r
(fft.f90:114-121), an external library that is not available here.  The
oracle uses numpy's pocketfft and the library its own Stockham transforms;
this test checks both against cuFFT, called through torch.fft on the GPU
in FP64 (test side only), on the spectral operations of derivatives.f90:
filt_da (:166-211) and ddxy (:129-163), with the oddballs zeroed
(derivatives.f90:64-65).  Radix-2 and radix-3 grids; 1e-12 of each
output's maximum.
"""
import numpy as np
import pytest

from gpu_util import make_pair, oracle_field

pytestmark = pytest.mark.gpu

GRIDS = [(32, 32, 16), (48, 96, 12), (128, 64, 8)]


def _cufft_ops(x, Lx, Ly):
    """filtered field, d/dx, d/dy of x[..., ny, nx] through cuFFT (FP64)."""
    import torch
    nz, ny, nx = x.shape
    t = torch.tensor(x, dtype=torch.float64, device="cuda")
    F = torch.fft.rfft2(t) / (nx * ny)
    F[..., nx // 2] = 0
    F[..., ny // 2, :] = 0
    kx = torch.arange(nx // 2 + 1, dtype=torch.float64, device="cuda") * (2 * np.pi / Lx)
    m = torch.fft.fftfreq(ny, d=1.0 / ny, dtype=torch.float64, device="cuda")
    ky = m * (2 * np.pi / Ly)
    ky[ny // 2] = 0
    inv = lambda G: (torch.fft.irfft2(G, s=(ny, nx)) * (nx * ny)).cpu().numpy()
    return inv(F), inv(1j * kx[None, None, :] * F), inv(1j * ky[None, :, None] * F)


def _err(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("grid", GRIDS)
def test_library_and_oracle_transforms_match_cufft(built_lib, grid):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    nx, ny, Nz = grid
    Ly = 2.0 if ny != nx else np.pi
    p, o, g = make_pair(nx=nx, ny=ny, Nz=Nz, L_y=Ly)
    nz = p.nz
    for f in ("u", "v", "w"):
        src = g.get(f)
        ref_f, ref_dx, ref_dy = _cufft_ops(src[1:nz, :, :nx], p.L_x, Ly)
        # the library (its own transforms)
        g.filt_da(f, "d%sdx" % f, "d%sdy" % f)
        for name, ref in ((f, ref_f), ("d%sdx" % f, ref_dx), ("d%sdy" % f, ref_dy)):
            assert _err(g.get(name)[1:nz, :, :nx], ref) < 1e-12, (grid, name)
        g.set(f, src)
        g.ddxy(f, "d%sdx" % f, "d%sdy" % f)
        assert _err(g.get("d%sdx" % f)[1:nz, :, :nx], ref_dx) < 1e-12, (grid, f, "ddxy x")
        assert _err(g.get("d%sdy" % f)[1:nz, :, :nx], ref_dy) < 1e-12, (grid, f, "ddxy y")
        # the oracle (pocketfft) on the same input
        a = oracle_field(o, f).copy()
        a[1:nz, :, :nx] = src[1:nz, :, :nx]
        dx, dy = np.zeros_like(a), np.zeros_like(a)
        o.filt_da(a, dx, dy)
        assert _err(a[1:nz, :, :nx], ref_f) < 1e-12, (grid, f, "oracle filt")
        assert _err(dx[1:nz, :, :nx], ref_dx) < 1e-12, (grid, f, "oracle d/dx")
        assert _err(dy[1:nz, :, :nx], ref_dy) < 1e-12, (grid, f, "oracle d/dy")
    g.close()
