"""The identities behind the y pass's transform-free outputs, checked in
numpy FP64 against explicit transforms (CPU).

The y pass of each spectral stage takes one x-spectrum column (fixed kx,
physical y), transforms it along y, applies the stage's multiplier with the
ky Nyquist row zeroed (derivatives.f90:64-65) and transforms back, all
unnormalised (FFTW's r2c / c2r convention, fft.f90:114-121).  The library
skips those transforms where an identity gives the output directly:

- a multiplier that depends on kx alone (1 or i kx) commutes with the y
  transforms, and the round trip with the Nyquist row zeroed is, per
  column, ny x(y) - (-1)^y s with s = sum_l (-1)^l x(l);
- in an inverse-only pass, the i kx output is i kx times the plain
  output's inverse transform;
- the test filters (test_filtermodule.f90:38-123, spectral cut-off) vanish
  on every kx column past the cut-off circle, for every ky.
"""
import numpy as np
import pytest

from oracle.lesgo_oracle import Oracle, Params


def _round_trip(x, mult):
    """forward y DFT, multiplier with the Nyquist row zeroed, inverse y DFT
    (unnormalised), of complex columns x[y, c]."""
    ny = x.shape[0]
    X = np.fft.fft(x, axis=0)
    X[ny // 2, :] = 0
    return np.fft.ifft(mult[:, None] * X if mult.ndim == 1 else mult * X, axis=0) * ny


@pytest.mark.parametrize("ny", [16, 48, 96, 128])
def test_kx_only_multiplier_round_trip_is_a_nyquist_projection(ny):
    rng = np.random.default_rng(ny)
    x = rng.standard_normal((ny, 7)) + 1j * rng.standard_normal((ny, 7))
    sign = (-1.0) ** np.arange(ny)
    s = (sign[:, None] * x).sum(axis=0)
    direct = ny * x - sign[:, None] * s[None, :]
    ref = _round_trip(x, np.ones(ny))
    assert np.max(np.abs(direct - ref)) <= 1e-12 * np.max(np.abs(ref))
    # an i kx multiplier is constant on the column: the same identity times i kx
    kx = 3.0
    ref_kx = _round_trip(x, np.full(ny, 1j * kx))
    assert np.max(np.abs(1j * kx * direct - ref_kx)) <= 1e-12 * np.max(np.abs(ref_kx))


@pytest.mark.parametrize("ny", [32, 96])
def test_ikx_output_of_an_inverse_pass_is_ikx_times_the_plain_output(ny):
    rng = np.random.default_rng(7)
    X = rng.standard_normal((ny, 5)) + 1j * rng.standard_normal((ny, 5))   # y spectra (pressure solve output)
    X[ny // 2, :] = 0
    kx = np.array([0.0, 1.0, 2.0, 3.0, 4.0])
    plain = np.fft.ifft(X, axis=0) * ny
    ikx = np.fft.ifft(1j * kx[None, :] * X, axis=0) * ny
    assert np.max(np.abs(1j * kx[None, :] * plain - ikx)) <= 1e-12 * np.max(np.abs(ikx))


@pytest.mark.parametrize("grid", [(128, 128, 8), (48, 48, 8), (96, 96, 8), (64, 32, 8)])
def test_test_filters_vanish_past_their_cutoff_column(grid):
    nx, ny, Nz = grid
    o = Oracle(Params(nx=nx, ny=ny, Nz=Nz))
    for G in (o.G_test, o.G_test_test):
        nonzero = np.nonzero(np.any(G != 0.0, axis=0))[0]
        kmax = nonzero.max()
        # every column past kmax is zero for every ky, and the columns up to
        # it are not all zero: the y pass may write zeros (or nothing) there
        assert np.all(G[:, kmax + 1:] == 0.0)
        assert kmax < G.shape[1] - 1
    # the 4-delta filter's cut-off lies inside the 2-delta one's
    k1 = np.nonzero(np.any(o.G_test != 0.0, axis=0))[0].max()
    k2 = np.nonzero(np.any(o.G_test_test != 0.0, axis=0))[0].max()
    assert k2 < k1
