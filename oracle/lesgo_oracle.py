"""FP64 CPU restatement of LESGO's per-timestep LES step.  TEST INFRASTRUCTURE ONLY.

This module is the oracle that the CUDA path is checked against.  Only the test
suite, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / reference legs of
``bench.py`` may import it, and only as the checker or as the timed CPU
baseline -- never as part of the product path.

Parity status: UNPINNED.  The reference (lesgo-jhu/lesgo, Fortran 90 + FFTW3 +
MPI) ships no golden vectors or known-answer tests, and it cannot be built in
this environment (no Fortran compiler, MPI or FFTW; FFTW is an external
library).  The restatement follows the reference source line by line (each
function cites the file:line it restates) and is pinned only by the analytic
known-answer tests in ``tests/test_oracle_kat.py``.

Conventions
-----------
* Every 3-D field is a float64 array of shape ``(nz+1, ny, ld)`` in C order,
  which is byte-identical to the reference's Fortran ``(ld, ny, 0:nz)``
  column-major array: index ``[k, j, i]`` is Fortran ``(i+1, j+1, k)``.  The
  serial reference uses ``lbz = 1`` for most fields (level 0 is unused here)
  and ``0:nz`` for the pressure (param.f90:49-55, sim_param.f90:313-365).
* ``nz = Nz + 1`` internally; uv levels 1..nz-1 are physical, w level 1 is the
  wall and w level nz the lid (input_util.f90:196-201).
* The x-y transforms are FFTW's unnormalised r2c/c2r on the first ``nx``
  entries of each ``ld`` row; here ``numpy.fft.rfft2`` / ``irfft2``.  The pad
  columns ``ld-1:ld`` of a c2r result are set to zero (FFTW leaves them
  undefined; no valid entry ever reads them).
* ``SAFETYMODE`` BOGUS fills are reproduced where the reference writes them.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

BOGUS = -1234567890.0  # param.f90:93
PI = 3.1415926535897932384626433  # param.f90:94


# --------------------------------------------------------------------------
# Parameters (param.f90, input_util.f90:196-235, 403-409, 534-542)
# --------------------------------------------------------------------------
@dataclass
class Params:
    nx: int = 32
    ny: int = 32
    Nz: int = 32                      # total vertical points as read (nz_tot)
    L_x: float = 2.0 * PI
    L_y: float = PI
    L_z: float = 1.0
    z_i: float = 1000.0
    u_star: float = 0.45
    vonk: float = 0.4
    zo: float = 1.0e-4
    dt: float = 2.0e-4
    cs_count: int = 5
    dyn_init: int = 100
    lbc_mom: int = 2
    ubc_mom: int = 0
    sgs_model: int = 5
    ifilter: int = 1
    molec: bool = False
    nu_molec: float = 1.14e-5
    ubot: float = 0.0
    utop: float = 0.0
    use_mean_p_force: bool = True
    eval_mean_p_force: bool = True
    mean_p_force_x_in: float = 1.0
    mean_p_force_y_in: float = 0.0
    initu: bool = False
    turbines: Optional["TurbineFarm"] = None
    use_cfl_dt: bool = False
    cfl: float = float(np.float32(0.05))    # param.f90: a default-real literal

    def __post_init__(self):
        nproc = 1
        # input_util.f90:196-225
        self.nz = int(math.floor(self.Nz / nproc)) + 1
        self.nz_tot = (self.nz - 1) * nproc + 1
        self.nx2 = 3 * self.nx // 2
        self.ny2 = 3 * self.ny // 2
        self.lh = self.nx // 2 + 1
        self.ld = 2 * self.lh
        self.lh_big = self.nx2 // 2 + 1
        self.ld_big = 2 * self.lh_big
        self.dx = self.L_x / self.nx
        self.dy = self.L_y / self.ny
        self.dz = self.L_z / (self.nz_tot - 1)
        # input_util.f90:403-409 (fixed dt => AB2 constants)
        self.tadv1 = 1.5
        self.tadv2 = 1.0 - self.tadv1
        # input_util.f90:534-542
        mpx, mpy = self.mean_p_force_x_in, self.mean_p_force_y_in
        if self.use_mean_p_force and self.eval_mean_p_force:
            mpx = mpx / math.sqrt(mpx ** 2 + mpy ** 2) / self.L_z
            mpy = mpy / math.sqrt(mpx ** 2 + mpy ** 2) / self.L_z
        self.mean_p_force_x = mpx
        self.mean_p_force_y = mpy
        # sgs_param.f90:187-192
        self.delta = 1.0 * (self.dx * self.dy * self.dz) ** (1.0 / 3.0)
        self.nu = self.nu_molec / (self.u_star * self.z_i) if self.molec else 0.0
        # sgs_stag_util.f90:60-62 (fixed dt)
        self.lagran_dt = float(self.cs_count) * self.dt
        if self.use_cfl_dt:
            self.lagran_dt = 0.0                # sgs_param.f90:51, accumulated per step


# --------------------------------------------------------------------------
# Seeded initial condition (counter-based; identical in the CUDA generator)
# --------------------------------------------------------------------------
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_G = np.uint64(0x9E3779B97F4A7C15)


def _mix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        x = (x ^ (x >> np.uint64(30))) * _M1
        x = (x ^ (x >> np.uint64(27))) * _M2
        return x ^ (x >> np.uint64(31))


def uniform_pm1(seed: int, fld: int, i, j, k) -> np.ndarray:
    """U(-1,1) keyed by (seed, field, i, j, k), all zero-based.

    key = ((((seed*8 + field)*65536 + k)*65536 + j)*65536 + i) mod 2^64,
    x = splitmix64(key + golden); U = 2*(x >> 11)*2^-53 - 1 (exact in FP64).
    """
    i = np.asarray(i, dtype=np.uint64)
    j = np.asarray(j, dtype=np.uint64)
    k = np.asarray(k, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = np.uint64(seed) * np.uint64(8) + np.uint64(fld)
        key = key * np.uint64(65536) + k
        key = key * np.uint64(65536) + j
        key = key * np.uint64(65536) + i
        x = _mix64(key + _G)
    u01 = (x >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return 2.0 * u01 - 1.0


def initial_condition(p: Params, seed: int):
    """Half-channel IC: u = (1/0.4) ln(z/z0) (1 + 0.1 U), v, w = 0.1 U.

    Stands in for ic_les (initial.f90:550-598), whose /dev/urandom seeding
    (init_random_seed.f90:42-46) is not reproducible.  Boundary fix-ups follow
    initial.f90:600-623: w(1)=w(nz)=0, u(nz)=u(nz-1), v(nz)=v(nz-1).
    """
    nz, ny, nx, ld = p.nz, p.ny, p.nx, p.ld
    u = np.zeros((nz + 1, ny, ld))
    v = np.zeros((nz + 1, ny, ld))
    w = np.zeros((nz + 1, ny, ld))
    k, j, i = np.meshgrid(np.arange(1, nz), np.arange(ny), np.arange(nx), indexing="ij")
    zk = (np.arange(1, nz) - 0.5) * p.dz
    ubar = (1.0 / 0.4) * np.log(zk / p.zo)
    u[1:nz, :, :nx] = ubar[:, None, None] * (1.0 + 0.1 * uniform_pm1(seed, 0, i, j, k))
    v[1:nz, :, :nx] = 0.1 * uniform_pm1(seed, 1, i, j, k)
    w[1:nz, :, :nx] = 0.1 * uniform_pm1(seed, 2, i, j, k)
    w[1] = 0.0
    w[nz] = 0.0
    u[nz] = u[nz - 1]
    v[nz] = v[nz - 1]
    return u, v, w


# --------------------------------------------------------------------------
# Turbines (actuator disks): turbines.f90, turbine_indicator.f90
# --------------------------------------------------------------------------
@dataclass
class Turbine:
    xloc: float
    yloc: float
    height: float
    dia: float
    thk: float
    theta1: float = 0.0
    theta2: float = 0.0
    Ct_prime: float = 1.33


@dataclass
class TurbineFarm:
    turbines: List[Turbine]
    alpha1: float = 1.5
    alpha2: float = 1.5
    filter_cutoff: float = 1e-2
    adm_correction: bool = True
    T_avg_dim: float = -1.0
    u_d_T0: float = -1.0              # turbines.f90:404-407 (no u_d_T.dat)
    # control schedules (turbines.f90:500-515): 0 theta1, 1 theta2, 2 Ct' ->
    # rows (nt, 1 + nloc) of (dimensional time, one value per turbine)
    sched: dict = field(default_factory=dict)


def sched_interp(x, v, xq):
    """binary_search (functions.f90:811-860) + linear_interp_sa_nocheck
    (:712-735): v(1) below x(1), v(N) above x(N), else linear between the
    bracketing samples, u1 + (xq - x(i)) * (u2 - u1) / (x(i+1) - x(i))."""
    N = len(x)
    if xq < x[0]:
        low = 0
    elif xq > x[N - 1]:
        low = N
    else:
        low, high = 1, N
        while high - low > 1:
            mid = (low + high) // 2
            if x[mid - 1] > xq:
                high = mid
            elif x[mid - 1] < xq:
                low = mid
            else:
                low = mid
                break
    if low == 0:
        return float(v[0])
    if low == N:
        return float(v[N - 1])
    return float(v[low - 1] + (xq - x[low - 1]) * (v[low] - v[low - 1]) / (x[low] - x[low - 1]))


def _erf(x):
    v = np.vectorize(math.erf, otypes=[float])
    return v(x)


class IndicatorFunction:
    """Filtered disk indicator lookup (turbine_indicator.f90:43-169)."""

    def __init__(self, delta1, delta2, thk, dia, N=2048):
        self.ell = 0.5 * dia
        self.delta1 = delta1 / self.ell
        self.delta2 = delta2 / self.ell
        self.thk = thk / self.ell
        self.sqrt6overdelta1 = math.sqrt(6.0) / self.delta1
        L = 1 + 10 * self.delta2 / math.sqrt(12.0)
        d = 2 * L / N
        yz = -L + d * (np.arange(1, N + 1) - 0.5)
        # g(i,j), h(i,j): Fortran (i,j) -> here [j, i] (i fastest)
        Y, Z = yz[:, None], yz[None, :]      # Y = yz(i) along axis 0? keep (i, j)
        r2 = Y ** 2 + Z ** 2                  # array[i, j]
        g = 6.0 / (PI * self.delta2 ** 2) * np.exp(-6 * r2 / self.delta2 ** 2)
        h = np.where(np.sqrt(r2) < 1, 1.0 / PI, 0.0)
        # Fortran arrays are (i,j) column-major => C array [j, i]
        gC, hC = g.T.copy(), h.T.copy()
        ghat = np.fft.rfft2(gC)
        hhat = np.fft.rfft2(hC)
        fx = np.fft.irfft2(ghat * hhat * d ** 2, s=(N, N)) * (N * N)
        self.r = yz[: N // 2] + L
        # fx(1, 1:N/2) -> C [0:N/2, 0] (first i, j = 1..N/2)
        R2 = fx[: N // 2, 0] / N ** 2
        dr = self.r[1] - self.r[0]
        self.R2 = R2 / np.sum(2 * PI * self.r * R2 * dr)
        self.M = np.sum(2 * PI * self.r * self.R2 ** 2 * dr) * PI

    def val(self, r, x):
        rr = np.asarray(r) / self.ell
        xx = np.asarray(x) / self.ell
        R2 = _linear_interp(self.r, self.R2, rr)
        R1 = 0.5 / self.thk * (_erf(self.sqrt6overdelta1 * (xx + 0.5 * self.thk))
                               - _erf(self.sqrt6overdelta1 * (xx - 0.5 * self.thk)))
        return R1 * R2 / self.ell ** 3


def _linear_interp(x, v, xq):
    """functions.f90:712-735: clamp outside, linear inside."""
    xq = np.asarray(xq, dtype=float)
    i = np.searchsorted(x, xq, side="right")        # x[i-1] <= xq < x[i]
    out = np.empty_like(xq)
    lo = i == 0
    hi = i >= len(x)
    mid = ~(lo | hi)
    out[lo] = v[0]
    out[hi] = v[-1]
    im = i[mid] - 1
    out[mid] = v[im] + (xq[mid] - x[im]) * (v[im + 1] - v[im]) / (x[im + 1] - x[im])
    return out


# --------------------------------------------------------------------------
# The oracle solver
# --------------------------------------------------------------------------
FIELDS_3D = [
    "u", "v", "w", "dudx", "dudy", "dudz", "dvdx", "dvdy", "dvdz",
    "dwdx", "dwdy", "dwdz", "RHSx", "RHSy", "RHSz", "RHSx_f", "RHSy_f",
    "RHSz_f", "txx", "txy", "txz", "tyy", "tyz", "tzz", "divtx", "divty",
    "divtz", "pres", "dpdx", "dpdy", "dpdz", "fxa", "fya", "fza",
    "S11", "S12", "S13", "S22", "S23", "S33", "Nu_t", "Cs_opt2",
    "F_LM", "F_MM", "F_QN", "F_NN", "Beta", "Tn_all", "ee_now",
]


class Oracle:
    def __init__(self, p: Params):
        self.p = p
        nz, ny, ld = p.nz, p.ny, p.ld
        for name in FIELDS_3D:
            setattr(self, name, np.zeros((nz + 1, ny, ld)))
        self.ustar_lbc = np.zeros((ny, p.nx))
        self.jt = 0
        self.jt_total = 0
        self.time = 0.0
        self.time_dim = 0.0                  # total_time_dim (main.f90:150)
        self.F_LM_MM_init = False
        self.F_QN_NN_init = False
        self._init_wavenumber()
        self._test_filter_init()
        self._grid_build()
        self.farm = None
        if p.turbines is not None:
            self._turbines_init(p.turbines)

    # ---------------- set-up ------------------------------------------------
    def _init_wavenumber(self):
        """fft.f90:130-160 -> kx, ky, k2 as (ny, lh)."""
        p = self.p
        lh, ny = p.lh, p.ny
        kx = np.zeros((ny, lh))
        kx[:, : lh - 1] = np.arange(lh - 1, dtype=float)[None, :]
        ky = np.empty((ny, lh))
        ky[:, :] = (np.mod(np.arange(ny) + ny // 2, ny) - ny // 2).astype(float)[:, None]
        kx[:, lh - 1] = 0.0
        ky[:, lh - 1] = 0.0
        kx[ny // 2, :] = 0.0
        ky[ny // 2, :] = 0.0
        kx = 2.0 * PI / p.L_x * kx
        ky = 2.0 * PI / p.L_y * ky
        self.kx, self.ky = kx, ky
        self.k2 = kx * kx + ky * ky

    def _test_filter_init(self):
        """test_filtermodule.f90:38-123 (ifilter=1, spectral cutoff)."""
        p = self.p
        if p.ifilter != 1:
            raise NotImplementedError("only the spectral cut-off test filter")

        def make(alpha):
            G = np.full((p.ny, p.lh), 1.0 / (p.nx * p.ny))
            delta_test = alpha * math.sqrt(p.dx * p.dy)
            kc2 = (PI / delta_test) ** 2
            G[self.k2 >= kc2] = 0.0
            G[:, p.lh - 1] = 0.0
            G[p.ny // 2, :] = 0.0
            return G

        self.G_test = make(2.0)
        self.G_test_test = make(4.0)

    def _grid_build(self):
        """grid.f90:44-104."""
        p = self.p
        self.x = (np.arange(1, p.nx + 2) - 1) * p.dx          # x(1..nx+1)
        self.y = (np.arange(1, p.ny + 2) - 1) * p.dy
        k = np.arange(0, p.nz + 1)
        self.z = (k - 0.5) * p.dz                              # z(k), k=0..nz
        self.zw = self.z - p.dz / 2.0

    # ---------------- spectral helpers ------------------------------------------
    # ``workers`` > 1 routes the same transforms through scipy.fft's threaded
    # pocketfft (used only when the oracle is timed as the CPU baseline).
    workers: int = 1

    def _rfft2(self, a):
        if self.workers > 1:
            import scipy.fft as sf
            return sf.rfft2(a, axes=(-2, -1), workers=self.workers)
        return np.fft.rfft2(a, axes=(-2, -1))

    def _irfft2(self, A, s):
        if self.workers > 1:
            import scipy.fft as sf
            return sf.irfft2(A, s=s, axes=(-2, -1), workers=self.workers)
        return np.fft.irfft2(A, s=s, axes=(-2, -1))

    def r2c(self, f):
        return self._rfft2(f[..., : self.p.nx])

    def c2r(self, F):
        p = self.p
        out = np.zeros(F.shape[:-1] + (p.ld,))
        out[..., : p.nx] = self._irfft2(F, (p.ny, p.nx)) * (p.nx * p.ny)
        return out

    def r2c_big(self, f):
        return self._rfft2(f[..., : self.p.nx2])

    def c2r_big(self, F):
        p = self.p
        out = np.zeros(F.shape[:-1] + (p.ld_big,))
        out[..., : p.nx2] = self._irfft2(F, (p.ny2, p.nx2)) * (p.nx2 * p.ny2)
        return out

    def zero_oddballs(self, F):
        """f(ld-1:ld,:) = 0 ; f(:,ny/2+1) = 0 (derivatives.f90:64-65)."""
        F[..., :, self.p.lh - 1] = 0.0
        F[..., self.p.ny // 2, :] = 0.0
        return F

    @staticmethod
    def muli(F, k):
        """emul_complex.f90:154-208: a .MULI. k = a * (i k)."""
        return (-F.imag * k) + 1j * (F.real * k)

    def padd(self, F):
        """fft.f90:43-72: (ny, lh) -> (ny2, lh_big), oddballs dropped."""
        p = self.p
        B = np.zeros(F.shape[:-2] + (p.ny2, p.lh_big), dtype=complex)
        nyh, nxh = p.ny // 2, p.nx // 2
        B[..., :nyh, :nxh] = F[..., :nyh, :nxh]
        B[..., p.ny2 - nyh + 1:, :nxh] = F[..., nyh + 1:, :nxh]
        return B

    def unpadd(self, B):
        """fft.f90:75-99: (ny2, lh_big) -> (ny, lh), oddballs zeroed."""
        p = self.p
        F = np.zeros(B.shape[:-2] + (p.ny, p.lh), dtype=complex)
        nyh, nxh = p.ny // 2, p.nx // 2
        F[..., :nyh, :nxh] = B[..., :nyh, :nxh]
        F[..., nyh + 1:, :nxh] = B[..., p.ny2 - nyh + 1:, :nxh]
        return F

    # ---------------- derivatives (derivatives.f90) -----------------------------
    def filt_da(self, f, dfdx, dfdy):
        """derivatives.f90:166-211 over levels lbz..nz (=1..nz)."""
        p = self.p
        const = 1.0 / (p.nx * p.ny)
        F = self.zero_oddballs(self.r2c(const * f[1:]))
        dfdx[1:] = self.c2r(self.muli(F, self.kx))
        dfdy[1:] = self.c2r(self.muli(F, self.ky))
        f[1:] = self.c2r(F)

    def ddx(self, f, dfdx):
        """derivatives.f90:37-70."""
        p = self.p
        F = self.zero_oddballs(self.r2c((1.0 / (p.nx * p.ny)) * f[1:]))
        dfdx[1:] = self.c2r(self.muli(F, self.kx))

    def ddy(self, f, dfdy):
        """derivatives.f90:73-106."""
        p = self.p
        F = self.zero_oddballs(self.r2c((1.0 / (p.nx * p.ny)) * f[1:]))
        dfdy[1:] = self.c2r(self.muli(F, self.ky))

    def ddxy(self, f, dfdx, dfdy):
        """derivatives.f90:109-163."""
        p = self.p
        F = self.zero_oddballs(self.r2c((1.0 / (p.nx * p.ny)) * f[1:]))
        dfdy[1:] = self.c2r(self.muli(F, self.ky))
        dfdx[1:] = self.c2r(self.muli(F, self.kx))

    def ddz_uv(self, f, dfdz):
        """derivatives.f90:214-264: dfdz(2:nz) on w-nodes; 1 and nz BOGUS."""
        p = self.p
        nz, nx = p.nz, p.nx
        dfdz[2:nz + 1, :, :nx] = (1.0 / p.dz) * (f[2:nz + 1, :, :nx] - f[1:nz, :, :nx])
        dfdz[1] = BOGUS
        dfdz[nz] = BOGUS

    def ddz_w(self, f, dfdz):
        """derivatives.f90:267-311: dfdz(1:nz-1) on uv-nodes; nz BOGUS."""
        p = self.p
        nz, nx = p.nz, p.nx
        dfdz[1:nz, :, :nx] = (1.0 / p.dz) * (f[2:nz + 1, :, :nx] - f[1:nz, :, :nx])
        dfdz[nz] = BOGUS

    # ---------------- test filters (test_filtermodule.f90:126-169) --------------
    def test_filter(self, f):
        return self.c2r(self.r2c(f) * self.G_test)

    def test_test_filter(self, f):
        return self.c2r(self.r2c(f) * self.G_test_test)

    # ---------------- wall stress (wallstress.f90) --------------------------------
    def wallstress(self):
        p = self.p
        nx, nz = p.nx, p.nz
        u, v = self.u, self.v
        if p.lbc_mom == 0:                               # :107-117
            for a in (self.txz, self.tyz, self.dudz, self.dvdz):
                a[1] = 0.0
        elif p.lbc_mom == 1:                             # :131-148
            self.dudz[1, :, :nx] = (u[1, :, :nx] - p.ubot) / (0.5 * p.dz)
            self.dvdz[1, :, :nx] = v[1, :, :nx] / (0.5 * p.dz)
            c = -p.nu_molec / (p.z_i * p.u_star)
            self.txz[1, :, :nx] = c * self.dudz[1, :, :nx]
            self.tyz[1, :, :nx] = c * self.dvdz[1, :, :nx]
        elif p.lbc_mom == 2:                             # :171-219
            u1 = self.test_filter(u[1])
            v1 = self.test_filter(v[1])
            denom = math.log(0.5 * p.dz / p.zo)
            u_avg = np.sqrt(u1[:, :nx] ** 2 + v1[:, :nx] ** 2)
            ustar = u_avg * p.vonk / denom
            self.ustar_lbc = ustar
            const = -(ustar ** 2) / u_avg
            self.txz[1, :, :nx] = const * u1[:, :nx]
            self.tyz[1, :, :nx] = const * v1[:, :nx]
            dudz = ustar / (0.5 * p.dz * p.vonk) * u[1, :, :nx] / u_avg
            dvdz = ustar / (0.5 * p.dz * p.vonk) * v[1, :, :nx] / u_avg
            self.dudz[1, :, :nx] = np.where(u[1, :, :nx] == 0.0, 0.0, dudz)
            self.dvdz[1, :, :nx] = np.where(v[1, :, :nx] == 0.0, 0.0, dvdz)
        else:
            raise NotImplementedError("lbc_mom")
        if p.ubc_mom == 0:                               # :119-128
            for a in (self.txz, self.tyz, self.dudz, self.dvdz):
                a[nz] = 0.0
        elif p.ubc_mom == 1:                             # :151-168
            self.dudz[nz, :, :nx] = (p.utop - u[nz - 1, :, :nx]) / (0.5 * p.dz)
            self.dvdz[nz, :, :nx] = -v[nz - 1, :, :nx] / (0.5 * p.dz)
            c = -p.nu_molec / (p.z_i * p.u_star)
            self.txz[nz, :, :nx] = c * self.dudz[nz, :, :nx]
            self.tyz[nz, :, :nx] = c * self.dvdz[nz, :, :nx]
        elif p.ubc_mom == 2:                             # :222-255
            u1 = self.test_filter(u[nz - 1])
            v1 = self.test_filter(v[nz - 1])
            denom = math.log(0.5 * p.dz / p.zo)
            u_avg = np.sqrt(u1[:, :nx] ** 2 + v1[:, :nx] ** 2)
            ustar = u_avg * p.vonk / denom
            const = (ustar ** 2) / u_avg
            self.txz[nz, :, :nx] = const * u1[:, :nx]
            self.tyz[nz, :, :nx] = const * v1[:, :nx]
            dudz = -ustar / (0.5 * p.dz * p.vonk) * u[nz - 1, :, :nx] / u_avg
            dvdz = -ustar / (0.5 * p.dz * p.vonk) * v[nz - 1, :, :nx] / u_avg
            self.dudz[nz, :, :nx] = np.where(u[nz - 1, :, :nx] == 0.0, 0.0, dudz)
            self.dvdz[nz, :, :nx] = np.where(v[nz - 1, :, :nx] == 0.0, 0.0, dvdz)
        else:
            raise NotImplementedError("ubc_mom")

    # ---------------- SGS (sgs_stag_util.f90) -------------------------------------
    def calc_Sij(self):
        """sgs_stag_util.f90:467-634."""
        p = self.p
        nx, nz = p.nx, p.nz
        X = np.s_[:, :nx]
        dudx, dudy, dudz = self.dudx, self.dudy, self.dudz
        dvdx, dvdy, dvdz = self.dvdx, self.dvdy, self.dvdz
        dwdx, dwdy, dwdz = self.dwdx, self.dwdy, self.dwdz
        S11, S12, S13 = self.S11, self.S12, self.S13
        S22, S23, S33 = self.S22, self.S23, self.S33
        # bottom (coord == 0)
        if p.lbc_mom == 0:
            S11[1][X] = dudx[1][X]
            S12[1][X] = 0.5 * (dudy[1][X] + dvdx[1][X])
            S13[1][X] = 0.5 * (dudz[1][X] + dwdx[1][X])
            S22[1][X] = dvdy[1][X]
            S23[1][X] = 0.5 * (dvdz[1][X] + dwdy[1][X])
            S33[1][X] = 0.5 * (dwdz[1][X] + 0.0)
        else:
            S11[1][X] = dudx[1][X]
            S12[1][X] = 0.5 * (dudy[1][X] + dvdx[1][X])
            wx = 0.5 * (dwdx[1][X] + dwdx[2][X])
            S13[1][X] = 0.5 * (dudz[1][X] + wx)
            S22[1][X] = dvdy[1][X]
            wy = 0.5 * (dwdy[1][X] + dwdy[2][X])
            S23[1][X] = 0.5 * (dvdz[1][X] + wy)
            S33[1][X] = dwdz[1][X]
        # top (coord == nproc-1)
        if p.ubc_mom == 0:
            S11[nz][X] = dudx[nz - 1][X]
            S12[nz][X] = 0.5 * (dudy[nz - 1][X] + dvdx[nz - 1][X])
            S13[nz][X] = 0.5 * (dudz[nz][X] + dwdx[nz][X])
            S22[nz][X] = dvdy[nz - 1][X]
            S23[nz][X] = 0.5 * (dvdz[nz][X] + dwdy[nz][X])
            S33[nz][X] = 0.5 * (dwdz[nz - 1][X] + 0.0)
        else:
            S11[nz][X] = dudx[nz - 1][X]
            S12[nz][X] = 0.5 * (dudy[nz - 1][X] + dvdx[nz - 1][X])
            wx = 0.5 * (dwdx[nz - 1][X] + dwdx[nz][X])
            S13[nz][X] = 0.5 * (dudz[nz][X] + wx)
            S22[nz][X] = dvdy[nz - 1][X]
            wy = 0.5 * (dwdy[nz - 1][X] + dwdy[nz][X])
            S23[nz][X] = 0.5 * (dvdz[nz][X] + wy)
            S33[nz][X] = dwdz[nz - 1][X]
        # interior
        K = np.s_[2:nz, :, :nx]
        Km = np.s_[1:nz - 1, :, :nx]
        S11[K] = 0.5 * (dudx[K] + dudx[Km])
        uy = dudy[K] + dudy[Km]
        vx = dvdx[K] + dvdx[Km]
        S12[K] = 0.25 * (uy + vx)
        S13[K] = 0.5 * (dudz[K] + dwdx[K])
        S22[K] = 0.5 * (dvdy[K] + dvdy[Km])
        S23[K] = 0.5 * (dvdz[K] + dwdy[K])
        S33[K] = 0.5 * (dwdz[K] + dwdz[Km])

    def sgs_stag(self):
        """sgs_stag_util.f90:33-464 (dynamic-model branch, sgs=.true.)."""
        p = self.p
        nx, nz = p.nx, p.nz
        if p.sgs_model != 5:
            raise NotImplementedError("only the Lagrangian scale-dependent model (5)")
        self.calc_Sij()
        if p.use_cfl_dt and (self.jt >= p.dyn_init - p.cs_count + 1 or p.initu):
            p.lagran_dt += p.dt                                       # :72-83
        inilag = not p.initu
        if self.jt == 1 and inilag:                                   # :187-189
            self.Cs_opt2[:] = 0.03
        elif (self.jt >= p.dyn_init or p.initu) and (self.jt_total % p.cs_count == 0):
            self.lagrange_Sdep()                                      # :192-217
            if p.use_cfl_dt:
                p.lagran_dt = 0.0                                     # lagrange_Sdep.f90:430
        l2 = p.delta ** 2
        X = np.s_[1:nz + 1, :, :nx]
        S = np.sqrt(2.0 * (self.S11[X] ** 2 + self.S22[X] ** 2 + self.S33[X] ** 2
                           + 2.0 * (self.S12[X] ** 2 + self.S13[X] ** 2 + self.S23[X] ** 2)))
        self.Nu_t[X] = S * self.Cs_opt2[X] * l2                     # :226-235
        Nu, nu = self.Nu_t, p.nu
        S11, S12, S13, S22, S23, S33 = self.S11, self.S12, self.S13, self.S22, self.S23, self.S33
        txx, txy, txz, tyy, tyz, tzz = self.txx, self.txy, self.txz, self.tyy, self.tyz, self.tzz
        C = np.s_[:, :nx]
        # bottom level (:238-300)
        if p.lbc_mom == 0:
            const = 0.5 * (Nu[1][C] + Nu[2][C]) + nu
            txx[1][C] = -const * (S11[1][C] + S11[2][C])
            txy[1][C] = -const * (S12[1][C] + S12[2][C])
            tyy[1][C] = -const * (S22[1][C] + S22[2][C])
            tzz[1][C] = -const * (S33[1][C] + S33[2][C])
        else:
            const = -2.0 * (Nu[1][C] + nu)
            txx[1][C] = const * S11[1][C]
            txy[1][C] = const * S12[1][C]
            tyy[1][C] = const * S22[1][C]
            tzz[1][C] = const * S33[1][C]
        # top level (:304-385)
        m = nz - 1
        if p.ubc_mom == 0:
            const = 0.5 * (Nu[m][C] + Nu[nz][C]) + nu
            const2 = 2.0 * (Nu[m][C] + nu)
            txx[m][C] = -const * (S11[m][C] + S11[nz][C])
            txy[m][C] = -const * (S12[m][C] + S12[nz][C])
            tyy[m][C] = -const * (S22[m][C] + S22[nz][C])
            tzz[m][C] = -const * (S33[m][C] + S33[nz][C])
            txz[m][C] = -const2 * S13[m][C]
            tyz[m][C] = -const2 * S23[m][C]
        else:
            const = -2.0 * (Nu[nz][C] + nu)
            const2 = -2.0 * (Nu[m][C] + nu)
            txx[m][C] = const * S11[nz][C]
            txy[m][C] = const * S12[nz][C]
            tyy[m][C] = const * S22[nz][C]
            tzz[m][C] = const * S33[nz][C]
            txz[m][C] = const2 * S13[m][C]
            tyz[m][C] = const2 * S23[m][C]
        # interior 2..nz-2 (:392-428)
        const3 = -2.0 * nu * 0.5
        const4 = -2.0 * nu
        K = np.s_[2:nz - 1, :, :nx]
        Kp = np.s_[3:nz, :, :nx]
        const = -0.5 * (Nu[K] + Nu[Kp])
        const2 = -2.0 * Nu[K]
        txx[K] = (const + const3) * (S11[K] + S11[Kp])
        txy[K] = (const + const3) * (S12[K] + S12[Kp])
        tyy[K] = (const + const3) * (S22[K] + S22[Kp])
        tzz[K] = (const + const3) * (S33[K] + S33[Kp])
        txz[K] = (const2 + const4) * S13[K]
        tyz[K] = (const2 + const4) * S23[K]
        for a in (txx, txy, tyy, tzz):                                # :453-458
            a[nz] = BOGUS

    # ---------------- Lagrangian scale-dependent model ------------------------
    def _fmodulo(self, a, pp):
        """Fortran MODULO for reals: a - floor(a/p)*p."""
        return a - np.floor(a / pp) * pp

    def trilinear_interp_w(self, var, xq, yq, zq):
        """functions.f90:349-474 (+ cell_indx_w :188-265), vectorised.

        ``var`` is (nz+1, ny, ld); xq, yq, zq are arrays of query points.
        """
        p = self.p
        nx, ny, nz = p.nx, p.ny, p.nz
        thresh = 1.0e-9
        # 'i' (the reference's cell_indx_w wraps its argument in place)
        px = self._fmodulo(xq, p.L_x)
        ist = np.where(np.abs(px) / p.L_x < thresh, 1,
                       np.where(np.abs(px - p.L_x) / p.L_x < thresh, nx,
                                np.floor(px / p.dx).astype(np.int64) + 1))
        py = self._fmodulo(yq, p.L_y)
        jst = np.where(np.abs(py) / p.L_y < thresh, 1,
                       np.where(np.abs(py - p.L_y) / p.L_y < thresh, ny,
                                np.floor(py / p.dy).astype(np.int64) + 1))
        ist1 = np.where(ist + 1 > nx, 1, ist + 1)
        jst1 = np.where(jst + 1 > ny, 1, jst + 1)
        xdiff = px - self.x[ist - 1]
        ydiff = py - self.y[jst - 1]
        z, zw = self.z, self.zw
        kst = np.empty_like(ist)
        kst1 = np.empty_like(ist)
        zdiff = np.empty_like(xq)
        low = (p.lbc_mom > 0) & (zq < zw[2])
        high = (~low) & (p.ubc_mom > 0) & (zq > zw[nz - 1])
        mid = ~(low | high)
        below = low & (zq < z[1])
        lowin = low & ~(zq < z[1])
        kst[below] = 1
        kst1[below] = 1
        zdiff[below] = 0.0
        kst[lowin] = 1
        kst1[lowin] = 2
        zdiff[lowin] = 2.0 * (zq[lowin] - z[1])
        above = high & (zq > z[nz - 1])
        highin = high & ~(zq > z[nz - 1])
        kst[above] = nz
        kst1[above] = nz
        zdiff[above] = 0.0
        kst[highin] = nz - 1
        kst1[highin] = nz
        zdiff[highin] = 2.0 * (zq[highin] - zw[nz - 1])
        zm = zq[mid]
        km = np.where(np.abs(zm - zw[nz]) / p.L_z < thresh, nz - 1,
                      np.floor((zm - zw[1]) / p.dz).astype(np.int64) + 1)
        kst[mid] = km
        kst1[mid] = km + 1
        zdiff[mid] = zm - zw[km]
        i0, i1, j0, j1 = ist - 1, ist1 - 1, jst - 1, jst1 - 1

        def V(k, j, i):
            return var[k, j, i]

        u1 = V(kst, j0, i0) + xdiff * (V(kst, j0, i1) - V(kst, j0, i0)) / p.dx
        u2 = V(kst, j1, i0) + xdiff * (V(kst, j1, i1) - V(kst, j1, i0)) / p.dx
        u3 = V(kst1, j0, i0) + xdiff * (V(kst1, j0, i1) - V(kst1, j0, i0)) / p.dx
        u4 = V(kst1, j1, i0) + xdiff * (V(kst1, j1, i1) - V(kst1, j1, i0)) / p.dx
        u5 = u1 + ydiff * (u2 - u1) / p.dy
        u6 = u3 + ydiff * (u4 - u3) / p.dy
        return u5 + zdiff * (u6 - u5) / p.dz

    def interpolag_Sdep(self):
        """interpolag_Sdep.f90:21-270 (without the CFL print)."""
        p = self.p
        nx, ny, nz = p.nx, p.ny, p.nz
        ldt = p.lagran_dt
        u, v, w = self.u, self.v, self.w
        temps = [a.copy() for a in (self.F_LM, self.F_MM, self.F_QN, self.F_NN)]
        X = self.x[:nx][None, None, :]
        Y = self.y[:ny][None, :, None]
        shape = (nz, ny, nx)
        xq = np.empty(shape)
        yq = np.empty(shape)
        zq = np.empty(shape)
        # k = 1 (index 0 here)
        if p.lbc_mom == 0:
            xq[0] = X[0] - u[1, :, :nx] * ldt
            yq[0] = Y[0] - v[1, :, :nx] * ldt
            zq[0] = self.zw[1]
        else:
            xq[0] = X[0] - u[1, :, :nx] * ldt
            yq[0] = Y[0] - v[1, :, :nx] * ldt
            zq[0] = self.z[1] - 0.25 * w[2, :, :nx] * ldt
        # k = 2 .. nz-1
        K = np.s_[2:nz, :, :nx]
        Km = np.s_[1:nz - 1, :, :nx]
        xq[1:nz - 1] = X - 0.5 * (u[Km] + u[K]) * ldt
        yq[1:nz - 1] = Y - 0.5 * (v[Km] + v[K]) * ldt
        zq[1:nz - 1] = self.zw[2:nz][:, None, None] - w[K] * ldt
        # k = nz
        if p.ubc_mom == 0:
            xq[nz - 1] = X[0] - u[nz - 1, :, :nx] * ldt
            yq[nz - 1] = Y[0] - v[nz - 1, :, :nx] * ldt
            zq[nz - 1] = self.zw[nz]
        else:
            xq[nz - 1] = X[0] - u[nz - 1, :, :nx] * ldt
            yq[nz - 1] = Y[0] - v[nz - 1, :, :nx] * ldt
            zq[nz - 1] = self.z[nz - 1] - 0.25 * w[nz - 1, :, :nx] * ldt
        for dst, src in zip((self.F_LM, self.F_MM, self.F_QN, self.F_NN), temps):
            dst[1:nz + 1, :, :nx] = self.trilinear_interp_w(src, xq, yq, zq)

    def lagrange_Sdep(self):
        """lagrange_Sdep.f90:21-432 (PPDYN_TN off, inflow off), all planes at once."""
        p = self.p
        nz, ld = p.nz, p.ld
        zero = 1.0e-24
        opftdelta = 1.5 * p.delta
        powcoeff = -1.0 / 8.0
        const = 2.0 * (p.delta ** 2)
        tf1, tf2 = 2.0, 4.0
        tf1_2, tf2_2 = tf1 ** 2, tf2 ** 2
        self.interpolag_Sdep()
        u, v, w = self.u, self.v, self.w
        # u_bar, v_bar, w_bar on w-nodes (levels 1..nz -> index 0..nz-1)
        ub = np.empty((nz, p.ny, ld))
        vb = np.empty_like(ub)
        wb = np.empty_like(ub)
        ub[1:nz - 1] = 0.5 * (u[2:nz] + u[1:nz - 1])
        vb[1:nz - 1] = 0.5 * (v[2:nz] + v[1:nz - 1])
        wb[1:nz - 1] = w[2:nz]
        if p.lbc_mom == 0:
            ub[0], vb[0], wb[0] = u[1], v[1], 0.0
        else:
            ub[0], vb[0], wb[0] = u[1], v[1], 0.25 * w[2]
        if p.ubc_mom == 0:
            ub[nz - 1], vb[nz - 1], wb[nz - 1] = u[nz - 1], v[nz - 1], 0.0
        else:
            ub[nz - 1], vb[nz - 1], wb[nz - 1] = u[nz - 1], v[nz - 1], 0.25 * w[nz - 1]
        uh, vh, wh = ub.copy(), vb.copy(), wb.copy()
        L11, L12, L13 = ub * ub, ub * vb, ub * wb
        L23, L22, L33 = vb * wb, vb * vb, wb * wb
        Q11, Q12, Q13, Q22, Q23, Q33 = L11, L12, L13, L22, L23, L33
        tf, ttf = self.test_filter, self.test_test_filter
        ub, vb, wb = tf(ub), tf(vb), tf(wb)
        L11 = tf(L11) - ub * ub
        L12 = tf(L12) - ub * vb
        L13 = tf(L13) - ub * wb
        L22 = tf(L22) - vb * vb
        L23 = tf(L23) - vb * wb
        L33 = tf(L33) - wb * wb
        uh, vh, wh = ttf(uh), ttf(vh), ttf(wh)
        Q11 = ttf(Q11) - uh * uh
        Q12 = ttf(Q12) - uh * vh
        Q13 = ttf(Q13) - uh * wh
        Q22 = ttf(Q22) - vh * vh
        Q23 = ttf(Q23) - vh * wh
        Q33 = ttf(Q33) - wh * wh
        Z = np.s_[1:nz + 1]
        S11, S12, S13 = self.S11[Z], self.S12[Z], self.S13[Z]
        S22, S23, S33 = self.S22[Z], self.S23[Z], self.S33[Z]
        S = np.sqrt(2.0 * (S11 ** 2 + S22 ** 2 + S33 ** 2 + 2.0 * (S12 ** 2 + S13 ** 2 + S23 ** 2)))
        Sb = [tf(a) for a in (S11, S12, S13, S22, S23, S33)]
        Sh = [ttf(a) for a in (S11, S12, S13, S22, S23, S33)]
        S_bar = np.sqrt(2.0 * (Sb[0] ** 2 + Sb[3] ** 2 + Sb[5] ** 2 + 2.0 * (Sb[1] ** 2 + Sb[2] ** 2 + Sb[4] ** 2)))
        S_hat = np.sqrt(2.0 * (Sh[0] ** 2 + Sh[3] ** 2 + Sh[5] ** 2 + 2.0 * (Sh[1] ** 2 + Sh[2] ** 2 + Sh[4] ** 2)))
        SSb = [tf(S * a) for a in (S11, S12, S13, S22, S23, S33)]
        SSh = [ttf(S * a) for a in (S11, S12, S13, S22, S23, S33)]
        M = [const * (SSb[n] - tf1_2 * S_bar * Sb[n]) for n in range(6)]
        N = [const * (SSh[n] - tf2_2 * S_hat * Sh[n]) for n in range(6)]
        M11, M12, M13, M22, M23, M33 = M
        N11, N12, N13, N22, N23, N33 = N
        LM = L11 * M11 + L22 * M22 + L33 * M33 + 2.0 * (L12 * M12 + L13 * M13 + L23 * M23)
        MM = M11 ** 2 + M22 ** 2 + M33 ** 2 + 2.0 * (M12 ** 2 + M13 ** 2 + M23 ** 2)
        QN = Q11 * N11 + Q22 * N22 + Q33 * N33 + 2.0 * (Q12 * N12 + Q13 * N13 + Q23 * N23)
        NN = N11 ** 2 + N22 ** 2 + N33 ** 2 + 2.0 * (N12 ** 2 + N13 ** 2 + N23 ** 2)
        Cs = self.Cs_opt2[Z]
        self.ee_now[Z] = (L11 ** 2 + L22 ** 2 + L33 ** 2 + 2.0 * (L12 ** 2 + L13 ** 2 + L23 ** 2)
                          - 2.0 * LM * Cs + MM * Cs ** 2)
        inilag = not p.initu
        F_LM, F_MM, F_QN, F_NN = self.F_LM[Z], self.F_MM[Z], self.F_QN[Z], self.F_NN[Z]
        if inilag and (not self.F_LM_MM_init) and (self.jt == p.cs_count or self.jt == p.dyn_init):
            F_MM[:] = MM
            F_LM[:] = 0.03 * MM
            F_MM[:, :, ld - 2:] = 1.0
            F_LM[:, :, ld - 2:] = 1.0
            self.F_LM_MM_init = True
        Tn = np.maximum(F_LM * F_MM, zero)
        Tn = opftdelta * (Tn ** powcoeff)
        Tn = np.maximum(zero, Tn)
        dumfac = p.lagran_dt / Tn
        epsi = dumfac / (1.0 + dumfac)
        F_LM[:] = epsi * LM + (1.0 - epsi) * F_LM
        F_MM[:] = epsi * MM + (1.0 - epsi) * F_MM
        F_LM[:] = np.maximum(zero, F_LM)
        Cs2d = F_LM / (F_MM + zero)
        Cs2d[:, :, ld - 1] = zero
        Cs2d[:, :, ld - 2] = zero
        Cs2d = np.maximum(zero, Cs2d)
        if inilag and (not self.F_QN_NN_init) and (self.jt == p.cs_count or self.jt == p.dyn_init):
            F_NN[:] = NN
            F_QN[:] = 0.03 * NN
            F_NN[:, :, ld - 2:] = 1.0
            F_QN[:, :, ld - 2:] = 1.0
            self.F_QN_NN_init = True
        Tn = np.maximum(F_QN * F_NN, zero)
        Tn = opftdelta * (Tn ** powcoeff)
        Tn = np.maximum(zero, Tn)
        dumfac = p.lagran_dt / Tn
        epsi = dumfac / (1.0 + dumfac)
        F_QN[:] = epsi * QN + (1.0 - epsi) * F_QN
        F_NN[:] = epsi * NN + (1.0 - epsi) * F_NN
        F_QN[:] = np.maximum(zero, F_QN)
        Cs4d = F_QN / (F_NN + zero)
        Cs4d[:, :, ld - 1] = zero
        Cs4d[:, :, ld - 2] = zero
        Cs4d = np.maximum(zero, Cs4d)
        beta_exp = math.log(tf1) / (math.log(tf2) - math.log(tf1))
        Beta = (Cs4d / Cs2d) ** beta_exp
        if p.ubc_mom == 0:
            Beta[nz - 1] = 1.0
        if p.lbc_mom == 0:
            Beta[0] = 1.0
        self.Beta[Z] = Beta
        Betaclip = np.maximum(Beta, 1.0 / (tf1 * tf2))
        Csn = Cs2d / Betaclip
        Csn[:, :, ld - 1] = zero
        Csn[:, :, ld - 2] = zero
        self.Cs_opt2[Z] = np.maximum(zero, Csn)
        self.Tn_all[Z] = Tn

    # ---------------- stress divergence -----------------------------------------
    def divstress_uv(self):
        """divstress_uv.f90:21-85."""
        p = self.p
        nz, ld = p.nz, p.ld
        shp = self.u.shape
        dtxdx, dtydy, dtzdz = np.zeros(shp), np.zeros(shp), np.zeros(shp)
        dtxdx2, dtydy2, dtzdz2 = np.zeros(shp), np.zeros(shp), np.zeros(shp)
        self.ddx(self.txx, dtxdx)
        self.ddz_w(self.txz, dtzdz)
        self.ddy(self.tyy, dtydy2)
        self.ddz_w(self.tyz, dtzdz2)
        self.ddxy(self.txy, dtxdx2, dtydy)
        K = np.s_[1:nz]
        self.divtx[K] = dtxdx[K] + dtydy[K] + dtzdz[K]
        self.divtx[1:nz, :, ld - 2:] = 0.0
        self.divtx[nz] = BOGUS
        self.divty[K] = dtxdx2[K] + dtydy2[K] + dtzdz2[K]
        self.divty[1:nz, :, ld - 2:] = 0.0
        self.divty[nz] = BOGUS

    def divstress_w(self):
        """divstress_w.f90:21-116."""
        p = self.p
        nz, nx, ld = p.nz, p.nx, p.ld
        shp = self.u.shape
        dtxdx, dtydy, dtzdz = np.zeros(shp), np.zeros(shp), np.zeros(shp)
        self.ddx(self.txz, dtxdx)
        self.ddy(self.tyz, dtydy)
        self.ddz_uv(self.tzz, dtzdz)
        d = self.divtz
        C = np.s_[:, :nx]
        d[1][C] = dtxdx[1][C] + dtydy[1][C]
        d[nz][C] = dtxdx[nz][C] + dtydy[nz][C]
        d[2:nz, :, :nx] = dtxdx[2:nz, :, :nx] + dtydy[2:nz, :, :nx] + dtzdz[2:nz, :, :nx]
        d[1:nz, :, ld - 2:] = 0.0

    # ---------------- convective term (convec.f90:21-333) ------------------------
    def convec(self):
        p = self.p
        nz, nx = p.nz, p.nx
        const = 1.0 / (p.nx * p.ny)
        L = np.s_[1:nz + 1]
        ub = self.c2r_big(self.padd(self.r2c(const * self.u[L])))
        vb = self.c2r_big(self.padd(self.r2c(const * self.v[L])))
        wb = self.c2r_big(self.padd(self.r2c(const * self.w[L])))
        r1 = np.zeros((nz, p.ny, p.ld))
        r2 = np.zeros((nz, p.ny, p.ld))
        dwdy, dvdz, dudz, dwdx = self.dwdy, self.dvdz, self.dudz, self.dwdx
        # generic levels
        r1[:] = const * (dwdy[L] - dvdz[L])
        r2[:] = const * (dudz[L] - dwdx[L])
        # jz = 1 (coord == 0)
        if p.lbc_mom == 0:
            r1[0] = 0.0
            r2[0] = 0.0
        else:
            r1[0] = const * (0.5 * (dwdy[1] + dwdy[2]) - dvdz[1])
            r2[0] = const * (dudz[1] - 0.5 * (dwdx[1] + dwdx[2]))
        # jz = nz (coord == nproc-1): for ubc_mom == 0 the generic line wins
        if p.ubc_mom > 0:
            r1[nz - 1] = const * (0.5 * (dwdy[nz - 1] + dwdy[nz]) - dvdz[nz - 1])
            r2[nz - 1] = const * (dudz[nz - 1] - 0.5 * (dwdx[nz - 1] + dwdx[nz]))
        r3 = const * (self.dvdx[L] - self.dudy[L])
        o1 = self.c2r_big(self.padd(self.r2c(r1)))
        o2 = self.c2r_big(self.padd(self.r2c(r2)))
        o3 = self.c2r_big(self.padd(self.r2c(r3)))
        # big arrays indexed by level-1
        c = 1.0 / (p.nx2 * p.ny2)
        cc = np.zeros((nz, p.ny2, p.ld_big))
        # RHSx
        cc[0] = c * (vb[0] * (-o3[0]) + 0.5 * wb[1] * (o2[1]))
        cc[nz - 2] = c * (vb[nz - 2] * (-o3[nz - 2]) + 0.5 * wb[nz - 2] * (o2[nz - 2]))
        J = np.s_[1:nz - 2]
        Jp = np.s_[2:nz - 1]
        cc[J] = c * (vb[J] * (-o3[J]) + 0.5 * (wb[Jp] * (o2[Jp]) + wb[J] * (o2[J])))
        self.RHSx[1:nz] = self.c2r(self.unpadd(self.r2c_big(cc[0:nz - 1])))
        # RHSy
        cc[0] = c * (ub[0] * (o3[0]) + 0.5 * wb[1] * (-o1[1]))
        cc[nz - 2] = c * (ub[nz - 2] * (o3[nz - 2]) + 0.5 * wb[nz - 2] * (-o1[nz - 2]))
        cc[J] = c * (ub[J] * (o3[J]) + 0.5 * (wb[Jp] * (-o1[Jp]) + wb[J] * (-o1[J])))
        self.RHSy[1:nz] = self.c2r(self.unpadd(self.r2c_big(cc[0:nz - 1])))
        # RHSz
        cc[0] = 0.0
        cc[nz - 1] = 0.0
        J = np.s_[1:nz - 1]
        Jm = np.s_[0:nz - 2]
        cc[J] = c * 0.5 * ((ub[J] + ub[Jm]) * (-o2[J]) + (vb[J] + vb[Jm]) * (o1[J]))
        self.RHSz[1:nz + 1] = self.c2r(self.unpadd(self.r2c_big(cc)))
        self.RHSx[nz] = BOGUS
        self.RHSy[nz] = BOGUS

    # ---------------- pressure (press_stag_array.f90, tridag_array.f90) -------------
    def press_stag_array(self):
        p = self.p
        nx, ny, nz, lh = p.nx, p.ny, p.nz, p.lh
        const = 1.0 / (nx * ny)
        const2 = const / p.tadv1 / p.dt
        const3 = 1.0 / (p.dz ** 2)
        const4 = 1.0 / p.dz
        K = np.s_[1:nz]
        rH_x = np.zeros((nz + 1, ny, lh), dtype=complex)
        rH_y = np.zeros_like(rH_x)
        rH_z = np.zeros_like(rH_x)
        rH_x[K] = self.r2c(const2 * self.u[K])
        rH_y[K] = self.r2c(const2 * self.v[K])
        rH_z[K] = self.r2c(const2 * self.w[K])
        rH_z[nz] = self.r2c(const2 * self.w[nz])
        rbottomw = self.r2c(const * self.divtz[1])
        rtopw = self.r2c(const * self.divtz[nz])
        for a in (rH_x, rH_y, rH_z, rbottomw, rtopw):
            self.zero_oddballs(a)
        n = nz + 1
        a = np.zeros((n + 1, ny, lh))
        b = np.zeros((n + 1, ny, lh))
        c = np.zeros((n + 1, ny, lh))
        r = np.zeros((n + 1, ny, lh), dtype=complex)
        b[1] = -1.0
        c[1] = 1.0
        r[1] = -p.dz * rbottomw
        a[n] = -1.0
        b[n] = 1.0
        r[n] = -p.dz * rtopw
        kx, ky = self.kx, self.ky
        for jz in range(2, nz + 1):
            a[jz] = const3
            b[jz] = -(kx ** 2 + ky ** 2 + 2.0 * const3)
            c[jz] = const3
            aHx = self.muli(rH_x[jz - 1], kx)
            aHy = self.muli(rH_y[jz - 1], ky)
            r[jz] = aHx + aHy + (rH_z[jz] - rH_z[jz - 1]) * const4
        # tridag_array (serial), columns jx = 1..lh-1, skipping jy = ny/2+1 and (1,1)
        mask = np.ones((ny, lh), dtype=bool)
        mask[:, lh - 1] = False
        mask[ny // 2, :] = False
        mask[0, 0] = False
        P = tridag_array(a, b, c, r, mask)
        ph = P[1:]                                         # levels 0..nz
        # zero-wavenumber solution (:226-234)
        ph[0, 0, 0] = 0.0
        ph[1, 0, 0] = ph[0, 0, 0] - p.dz * rbottomw[0, 0]
        for jz in range(2, nz + 1):
            ph[jz, 0, 0] = ph[jz - 1, 0, 0] + rH_z[jz, 0, 0] * p.dz
        ph[:, :, lh - 1] = 0.0
        ph[:, ny // 2, :] = 0.0
        self.dpdx[K] = self.c2r(self.muli(ph[K], kx))
        self.dpdy[K] = self.c2r(self.muli(ph[K], ky))
        pr = self.c2r(ph)                                   # levels 0..nz
        self.pres[:] = pr
        self.dpdx[nz] = BOGUS
        self.dpdy[nz] = BOGUS
        self.dpdz[1:nz, :, :nx] = (pr[1:nz, :, :nx] - pr[0:nz - 1, :, :nx]) / p.dz
        self.dpdz[nz, :, :nx] = (pr[nz, :, :nx] - pr[nz - 1, :, :nx]) / p.dz

    # ---------------- turbines (turbines.f90:465-638, forcing.f90:79-117) --------------
    def _turbines_init(self, farm: TurbineFarm):
        """turbines.f90:123-462: indicator functions, then node lists and
        normalised indicator values."""
        p = self.p
        self.farm = farm
        self.turb_nodes = []
        dx, dy, dz = p.dx, p.dy, p.dz
        for t in farm.turbines:
            # `dx * 1.01`: the literal is default (single) precision
            t.thk = max(t.thk, dx * float(np.float32(1.01)))
        delta1 = farm.alpha1 * math.sqrt(dx ** 2 + dy ** 2 + dz ** 2)
        delta2 = farm.alpha2 * math.sqrt(dx ** 2 + dy ** 2 + dz ** 2)
        for t in farm.turbines:
            t.ind_f = IndicatorFunction(delta1, delta2, t.thk, t.dia)
            t.M = t.ind_f.M
            t.u_d_T = farm.u_d_T0
            t.u_d = 0.0
            t.f_n = 0.0
        self._turbines_nodes()

    def _turbines_nodes(self):
        """turbines_nodes (turbines.f90:275-462) for the current yaw and tilt."""
        p = self.p
        farm = self.farm
        dx, dy, dz = p.dx, p.dy, p.dz
        z_tot = (np.arange(1, p.nz_tot + 1) - 0.5) * dz
        x, y = self.x, self.y
        for t in farm.turbines:
            ind_f = t.ind_f
            search_rad = 0.5 * t.dia + 3 * max(farm.alpha1, farm.alpha2) * math.sqrt(dx ** 2 + dy ** 2 + dz ** 2)
            imax = min(int(search_rad / dx + 2), p.nx // 2)
            jmax = min(int(search_rad / dy + 2), p.ny // 2)
            kmax = int(search_rad / dz + 2)
            nh1 = -math.cos(PI * t.theta1 / 180.0) * math.cos(PI * t.theta2 / 180.0)
            nh2 = -math.sin(PI * t.theta1 / 180.0) * math.cos(PI * t.theta2 / 180.0)
            nh3 = math.sin(PI * t.theta2 / 180.0)
            t.nhat = (nh1, nh2, nh3)
            icp = int(round_half_away(t.xloc / dx))
            jcp = int(round_half_away(t.yloc / dy))
            kcp = int(round_half_away(t.height / dz + 0.5))
            t.icp, t.jcp, t.kcp = icp, jcp, kcp
            min_i, max_i = icp - imax + 1, icp + imax
            min_j, max_j = jcp - jmax + 1, jcp + jmax
            min_k, max_k = max(kcp - kmax, 1), min(kcp + kmax, p.nz_tot)
            filt_max = float(ind_f.val(np.array([0.0]), np.array([0.0]))[0])
            kk, jj, ii = np.meshgrid(np.arange(1, p.nz + 1), np.arange(min_j, max_j + 1),
                                     np.arange(min_i, max_i + 1), indexing="ij")
            i2 = np.where((ii < 1) | (ii > p.nx), np.mod(ii + p.nx - 1, p.nx) + 1, ii)
            j2 = np.where((jj < 1) | (jj > p.ny), np.mod(jj + p.ny - 1, p.ny) + 1, jj)
            rx = np.where(ii < 1, (x[i2 - 1] - p.L_x) - t.xloc,
                          np.where(ii > p.nx, (p.L_x + x[i2 - 1]) - t.xloc, x[i2 - 1] - t.xloc))
            ry = np.where(jj < 1, (y[j2 - 1] - p.L_y) - t.yloc,
                          np.where(jj > p.ny, (p.L_y + y[j2 - 1]) - t.yloc, y[j2 - 1] - t.yloc))
            kidx = np.minimum(kk, p.nz_tot) - 1
            rz = z_tot[kidx] - t.height
            r = np.sqrt(rx * rx + ry * ry + rz * rz)
            r_norm = np.abs(rx * nh1 + ry * nh2 + rz * nh3)
            r_disk = np.sqrt(r * r - r_norm * r_norm)
            filt = ind_f.val(r_disk.ravel(), r_norm.ravel()).reshape(r.shape)
            # k_start..k_end = 1..nz (serial); k > nz_tot has no z_tot entry
            sel = (filt > farm.filter_cutoff * filt_max) & (kk <= p.nz_tot)
            ind = filt[sel]
            sumA = np.sum(ind * dx * dy * dz)
            ind = ind / sumA
            t.ind = ind
            t.nodes = (i2[sel] - 1, j2[sel] - 1, kk[sel])     # zero-based i, j; level k

    def turbines_forcing(self):
        """forcing_applied + turbines_forcing (turbines.f90:465-638)."""
        p = self.p
        nz = p.nz
        self.fxa[:] = 0.0
        self.fya[:] = 0.0
        self.fza[:] = 0.0
        w_uv = np.zeros_like(self.w)
        w_uv[1:nz] = 0.5 * (self.w[2:nz + 1] + self.w[1:nz])
        w_uv[nz] = w_uv[nz - 1]
        farm = self.farm
        # time-varying controls (turbines.f90:504-515)
        nloc = len(farm.turbines)
        for s, t in enumerate(farm.turbines):
            for which, attr in ((0, "theta1"), (1, "theta2"), (2, "Ct_prime")):
                rows = farm.sched.get(which)
                if rows is not None and len(rows):
                    rows = np.asarray(rows, dtype=float).reshape(-1, 1 + nloc)
                    setattr(t, attr, sched_interp(rows[:, 0], rows[:, 1 + s], self.time_dim))
        if any(farm.sched.get(w) is not None and len(farm.sched.get(w)) for w in (0, 1)):
            self._turbines_nodes()
        dt_dim = p.dt * p.z_i / p.u_star
        if farm.T_avg_dim > 0.0:
            eps = (dt_dim / farm.T_avg_dim) / (1.0 + dt_dim / farm.T_avg_dim)
        else:
            eps = 1.0
        disk = []
        for t in farm.turbines:
            i, j, k = t.nodes
            s = np.sum(p.dx * p.dy * p.dz * t.ind * (t.nhat[0] * self.u[k, j, i] + t.nhat[1] * self.v[k, j, i]
                                                      + t.nhat[2] * w_uv[k, j, i]))
            disk.append(s)
        for t, dav in zip(farm.turbines, disk):
            t.u_d = dav
            if farm.adm_correction:
                t.u_d = t.u_d / (1 + 0.25 * (1 - t.M) * t.Ct_prime)
            t.u_d_T = (1.0 - eps) * t.u_d_T + eps * t.u_d
            t.f_n = -0.5 * t.Ct_prime * abs(t.u_d_T) * t.u_d_T * 0.25 * PI * t.dia ** 2
            i, j, k = t.nodes
            # assignment: overlapping disks overwrite in turbine order
            self.fxa[k, j, i] = t.f_n * t.nhat[0] * t.ind
            self.fya[k, j, i] = t.f_n * t.nhat[1] * t.ind
            self.fza[k, j, i] = t.f_n * t.nhat[2] * t.ind
        fz = self.fza.copy()
        self.fza[2:nz + 1] = 0.5 * (fz[1:nz] + fz[2:nz + 1])
        self.fza[1] = 0.0

    def turbine_power(self):
        """P = -f_n * u_d_T per turbine (turbines.f90:583-588)."""
        return np.array([-t.f_n * t.u_d_T for t in self.farm.turbines])

    # ---------------- projection (forcing.f90:149-244) ----------------------------
    def project(self):
        p = self.p
        nz, nx = p.nz, p.nx
        K = np.s_[1:nz, :, :nx]
        self.u[K] = self.u[K] + p.dt * (-p.tadv1 * self.dpdx[K])
        self.v[K] = self.v[K] + p.dt * (-p.tadv1 * self.dpdy[K])
        K2 = np.s_[2:nz, :, :nx]
        self.w[K2] = self.w[K2] + p.dt * (-p.tadv1 * self.dpdz[K2])
        if p.ubc_mom == 0:
            self.u[nz] = self.u[nz - 1]
            self.v[nz] = self.v[nz - 1]
        self.w[nz] = 0.0
        self.w[1] = 0.0

    # ---------------- diagnostics ------------------------------------------------
    def rmsdiv(self):
        """rmsdiv.f90:21-60."""
        p = self.p
        K = np.s_[1:p.nz, :, :p.nx]
        return float(np.sum(np.abs(self.dudx[K] + self.dvdy[K] + self.dwdz[K])) / (p.nx * p.ny * (p.nz - 1)))

    def energy(self):
        """io.f90:99-141."""
        p = self.p
        nz, nx = p.nz, p.nx
        tw = 0.5 * (self.w[1:nz, :, :nx] + self.w[2:nz + 1, :, :nx])
        ke = np.sum(self.u[1:nz, :, :nx] ** 2 + self.v[1:nz, :, :nx] ** 2 + tw ** 2)
        return float(ke * 0.5 / (nx * p.ny * (nz - 1)))

    def max_cfl(self):
        """cfl_util.f90:35-64."""
        p = self.p
        K = np.s_[1:p.nz, :, :p.nx]
        cu = np.max(np.abs(self.u[K])) / p.dx
        cv = np.max(np.abs(self.v[K])) / p.dy
        cw = np.max(np.abs(self.w[K])) / p.dz
        return float(p.dt * max(cu, cv, cw))

    def tau_wall_bot(self):
        """functions.f90:882-905."""
        p = self.p
        tx = np.sum(self.txz[1, :, :p.nx]) / (p.nx * p.ny)
        ty = np.sum(self.tyz[1, :, :p.nx]) / (p.nx * p.ny)
        return float(math.sqrt(tx ** 2 + ty ** 2))

    # ---------------- one time step (main.f90:130-344) ------------------------------
    def set_ic(self, seed: int):
        self.u, self.v, self.w = initial_condition(self.p, seed)

    def get_cfl_dt(self):
        """cfl_util.f90:70-111."""
        p = self.p
        K = np.s_[1:p.nz, :, :p.nx]
        iu = np.max(np.abs(self.u[K])) / p.dx
        iv = np.max(np.abs(self.v[K])) / p.dy
        iw = np.max(np.abs(self.w[K])) / p.dz
        m = iu
        if iv > m:
            m = iv
        if iw > m:
            m = iw
        return float(p.cfl / m)

    def begin_step(self):
        """main.f90:135-157."""
        p = self.p
        if p.use_cfl_dt:
            dt_f = p.dt
            p.dt = self.get_cfl_dt()
            p.tadv1 = 1.0 + 0.5 * p.dt / dt_f
            p.tadv2 = 1.0 - p.tadv1
        self.jt_total += 1
        self.jt += 1
        self.time += self.p.dt
        self.time_dim += self.p.dt * p.z_i / p.u_star
        self.RHSx_f[:] = self.RHSx
        self.RHSy_f[:] = self.RHSy
        self.RHSz_f[:] = self.RHSz

    def rhs_assemble(self):
        """main.f90:211-267 (coriolis, sponge, random forcing off)."""
        p = self.p
        nz = p.nz
        K = np.s_[1:nz]
        self.RHSx[K] = -self.RHSx[K] - self.divtx[K]
        self.RHSy[K] = -self.RHSy[K] - self.divty[K]
        self.RHSz[K] = -self.RHSz[K] - self.divtz[K]
        self.RHSz[nz] = -self.RHSz[nz] - self.divtz[nz]
        if p.use_mean_p_force:
            self.RHSx[K] = self.RHSx[K] + p.mean_p_force_x
            self.RHSy[K] = self.RHSy[K] + p.mean_p_force_y
        if self.farm is not None:
            self.RHSx[K] = self.RHSx[K] + self.fxa[K]
            self.RHSy[K] = self.RHSy[K] + self.fya[K]
            self.RHSz[K] = self.RHSz[K] + self.fza[K]

    def ab2(self):
        """main.f90:273-311: Euler first step, AB2 intermediate velocity."""
        p = self.p
        nz = p.nz
        K = np.s_[1:nz]
        if self.jt_total == 1 and not p.initu:
            self.RHSx_f[:] = self.RHSx
            self.RHSy_f[:] = self.RHSy
            self.RHSz_f[:] = self.RHSz
        t1, t2, dt = p.tadv1, p.tadv2, p.dt
        self.u[K] = self.u[K] + dt * (t1 * self.RHSx[K] + t2 * self.RHSx_f[K])
        self.v[K] = self.v[K] + dt * (t1 * self.RHSy[K] + t2 * self.RHSy_f[K])
        self.w[K] = self.w[K] + dt * (t1 * self.RHSz[K] + t2 * self.RHSz_f[K])
        self.w[nz] = self.w[nz] + dt * (t1 * self.RHSz[nz] + t2 * self.RHSz_f[nz])
        self.u[nz] = BOGUS
        self.v[nz] = BOGUS

    def rhs_sub_dp(self):
        """main.f90:321-326."""
        nz = self.p.nz
        K = np.s_[1:nz]
        self.RHSx[K] = self.RHSx[K] - self.dpdx[K]
        self.RHSy[K] = self.RHSy[K] - self.dpdy[K]
        self.RHSz[K] = self.RHSz[K] - self.dpdz[K]
        self.RHSz[nz] = self.RHSz[nz] - self.dpdz[nz]

    def stages(self):
        """The step as (name, callable, fields written) in main.f90 order.

        ``name`` is the matching entry point of the GPU library's host mirror.
        """
        st = [
            ("begin_step", self.begin_step, ["RHSx_f", "RHSy_f", "RHSz_f"]),
            ("filt_da:u", lambda: self.filt_da(self.u, self.dudx, self.dudy), ["u", "dudx", "dudy"]),
            ("filt_da:v", lambda: self.filt_da(self.v, self.dvdx, self.dvdy), ["v", "dvdx", "dvdy"]),
            ("filt_da:w", lambda: self.filt_da(self.w, self.dwdx, self.dwdy), ["w", "dwdx", "dwdy"]),
            ("ddz_uv:u", lambda: self.ddz_uv(self.u, self.dudz), ["dudz"]),
            ("ddz_uv:v", lambda: self.ddz_uv(self.v, self.dvdz), ["dvdz"]),
            ("ddz_w:w", lambda: self.ddz_w(self.w, self.dwdz), ["dwdz"]),
            ("wallstress", self.wallstress, ["txz", "tyz", "dudz", "dvdz"]),
            ("sgs_stag", self.sgs_stag, ["S11", "S12", "S13", "S22", "S23", "S33", "Cs_opt2",
                                         "txx", "txy", "txz", "tyy", "tyz", "tzz",
                                         "F_LM", "F_MM", "F_QN", "F_NN"]),
            ("divstress_uv", self.divstress_uv, ["divtx", "divty"]),
            ("divstress_w", self.divstress_w, ["divtz"]),
            ("convec", self.convec, ["RHSx", "RHSy", "RHSz"]),
        ]
        if self.farm is not None:
            st.append(("turbines_forcing", self.turbines_forcing, ["fxa", "fya", "fza"]))
        st += [
            ("rhs_assemble", self.rhs_assemble, ["RHSx", "RHSy", "RHSz"]),
            ("ab2", self.ab2, ["u", "v", "w"]),
            ("press_stag_array", self.press_stag_array, ["p", "dpdx", "dpdy", "dpdz"]),
            ("rhs_sub_dp", self.rhs_sub_dp, ["RHSx", "RHSy", "RHSz"]),
            ("project", self.project, ["u", "v", "w"]),
        ]
        return st

    def step(self):
        for _, fn, _ in self.stages():
            fn()


# ---------------------------------------------------------------------------
# Time-averaging statistics: time_average.f90:176-319 (compute), :616-629
# (Reynolds stresses) and the schedule of io.f90:557-580.  Serial layout:
# levels 1..nz (lbz = 1).  interp_to_w_grid leaves level 1 unset in a serial
# run; here it is 0 (the reference zeroes it itself whenever lbc_mom > 0).
# ---------------------------------------------------------------------------
TAVG_NAMES = ["u", "v", "w", "u_w", "v_w", "w_uv", "u2", "v2", "w2", "uv", "uw", "vw",
              "txx", "tyy", "tzz", "txy", "txz", "tyz", "p", "fx", "fy", "fz", "cs_opt2",
              "vortx", "vorty", "vortz"]
TAVG_RS_NAMES = ["up2", "vp2", "wp2", "upvp", "upwp", "vpwp"]


class TimeAverage:
    def __init__(self, o: "Oracle", nstart: int, nend: int, nskip: int):
        self.o = o
        self.nstart, self.nend, self.nskip = nstart, nend, nskip
        self.initialized = False
        self.dt = 0.0
        self.total_time = 0.0
        nz, ny, nx = o.p.nz, o.p.ny, o.p.nx
        self.acc = {n: np.zeros((nz + 1, ny, nx)) for n in TAVG_NAMES}

    def after_step(self):
        """io.f90:557-580."""
        jt = self.o.jt_total
        if self.nstart <= jt <= self.nend:
            self.dt += self.o.p.dt
            if (jt - self.nstart) % self.nskip == 0:
                if not self.initialized:
                    self.init()
                else:
                    self.compute()

    def init(self):
        """time_average.f90:63-173: zero sums, or the sums of tavg.out."""
        for a in self.acc.values():
            a[:] = 0.0
        self.total_time = 0.0
        if getattr(self, "loaded", None) is not None:
            total, sums = self.loaded
            for n, a in sums.items():
                self.acc[n][:] = a
            self.total_time = total
            self.loaded = None
        self.dt = 0.0
        self.initialized = True

    def sample(self):
        """The 26 sampled quantities at levels 1..nz (index 0 unused)."""
        o, p = self.o, self.o.p
        nx, nz = p.nx, p.nz
        g = lambda f: f[:, :, :nx]
        u, v, w, pr = g(o.u), g(o.v), g(o.w), g(o.pres)

        def to_uv(f):                      # functions.f90:51-105
            r = np.zeros_like(f)
            r[1:nz] = 0.5 * (f[2:nz + 1] + f[1:nz])
            r[nz] = r[nz - 1]
            return r

        def to_w(f):                       # functions.f90:108-185, level 1 left 0
            r = np.zeros_like(f)
            r[2:nz + 1] = 0.5 * (f[1:nz] + f[2:nz + 1])
            return r

        w_uv, u_w, v_w = to_uv(w), to_w(u), to_w(v)
        vortz = to_w(g(o.dvdx) - g(o.dudy))
        vortz[1] = 0.0
        if p.lbc_mom > 0:
            u_w[1] = 0.0
            v_w[1] = 0.0
        if p.ubc_mom > 0:
            u_w[nz] = 0.0
            v_w[nz] = 0.0
        pres = pr - 0.5 * (u ** 2 + w_uv ** 2 + v ** 2)
        if self.o.farm is not None:
            fx, fy, fz = g(o.fxa), g(o.fya), to_uv(g(o.fza))
        else:
            fx = fy = fz = np.zeros_like(u)
        vals = dict(u=u, v=v, w=w, u_w=u_w, v_w=v_w, w_uv=w_uv, u2=u * u, v2=v * v, w2=w * w,
                    uv=u * v, uw=u_w * w, vw=v_w * w, txx=g(o.txx), tyy=g(o.tyy), tzz=g(o.tzz),
                    txy=g(o.txy), txz=g(o.txz), tyz=g(o.tyz), p=pres, fx=fx, fy=fy, fz=fz,
                    cs_opt2=g(o.Cs_opt2), vortx=g(o.dwdy) - g(o.dvdz), vorty=g(o.dudz) - g(o.dwdx),
                    vortz=vortz)
        for k in vals:
            vals[k] = vals[k].copy()
            vals[k][0] = 0.0
        return vals

    def compute(self):
        vals = self.sample()
        for n in TAVG_NAMES:
            self.acc[n] += vals[n] * self.dt
        self.total_time += self.dt
        self.dt = 0.0

    def mean(self, name: str) -> np.ndarray:
        """Time average of a sampled quantity or a Reynolds stress, (nz+1, ny, nx)."""
        A = lambda n: self.acc[n] / self.total_time
        rs = {"up2": ("u2", "u", "u"), "vp2": ("v2", "v", "v"), "wp2": ("w2", "w", "w"),
              "upvp": ("uv", "u", "v"), "upwp": ("uw", "u_w", "w"), "vpwp": ("vw", "v_w", "w")}
        if name in rs:
            a, b, c = rs[name]
            return A(a) - A(b) * A(c)
        return A(name)


# ---------------------------------------------------------------------------
# Restart files: io.f90:1173-1267 (checkpoint), initial.f90:20-380 (restart,
# ic_interp), io.f90:60-96 (total_time.dat), time_average.f90:114-150 and
# :665-716 (tavg.out).  Fortran sequential unformatted records as gfortran
# frames them: 4-byte little-endian length before and after the payload; a
# payload above SUBMAX bytes is split into subrecords, the leading length
# negated when more follow, the trailing length negated when one precedes.
# ---------------------------------------------------------------------------
SUBMAX = 2147483639
VEL_FIELDS = ["u", "v", "w", "RHSx", "RHSy", "RHSz", "Cs_opt2", "F_LM", "F_MM", "F_QN", "F_NN"]
TAVG_FILE = [n for n in TAVG_NAMES if n != "p"]


def fortran_record_bytes(payload: bytes, submax: int = SUBMAX) -> bytes:
    out = bytearray()
    left, off, first = len(payload), 0, True
    while True:
        n = min(left, submax)
        more = left > n
        out += struct.pack("<i", -n if more else n)
        out += payload[off:off + n]
        out += struct.pack("<i", n if first else -n)
        off += n
        left -= n
        first = False
        if left <= 0:
            return bytes(out)


def fortran_records(data: bytes):
    """Split a file's bytes into record payloads."""
    recs, pos = [], 0
    while pos < len(data):
        buf, first = bytearray(), True
        while True:
            lead, = struct.unpack_from("<i", data, pos)
            n = abs(lead)
            buf += data[pos + 4:pos + 4 + n]
            trail, = struct.unpack_from("<i", data, pos + 4 + n)
            if abs(trail) != n or (trail < 0) == first:
                raise ValueError("bad record marker")
            pos += 8 + n
            first = False
            if lead >= 0:
                break
        recs.append(bytes(buf))
    return recs


def write_checkpoint(o: "Oracle", prefix: str, ta: Optional["TimeAverage"] = None, mpi_names: bool = False):
    p = o.p
    sfx = ".c0" if mpi_names else ""
    payload = b"".join(np.ascontiguousarray(oracle_state(o, n)[1:p.nz + 1]).tobytes() for n in VEL_FIELDS)
    with open(prefix + "vel.out" + sfx, "wb") as f:
        f.write(fortran_record_bytes(payload))
    with open(prefix + "grid.out", "wb") as f:
        f.write(fortran_record_bytes(struct.pack("<4i3d", 1, p.nx, p.ny, p.nz, p.L_x, p.L_y, p.L_z)))
    if ta is not None and ta.initialized:
        with open(prefix + "tavg.out" + sfx, "wb") as f:
            f.write(fortran_record_bytes(struct.pack("<d", ta.total_time)))
            for n in TAVG_FILE:
                f.write(fortran_record_bytes(np.ascontiguousarray(ta.acc[n][1:]).tobytes()))
    with open(prefix + "total_time.dat", "w") as f:
        f.write(" %d %.17E %.17E %.17E %.17E\n" % (o.jt_total, o.time, o.time_dim, p.dt,
                                                  p.cfl if p.use_cfl_dt else o.max_cfl()))


def oracle_state(o: "Oracle", name: str) -> np.ndarray:
    return o.pres if name == "p" else getattr(o, name)


def binary_search(arr, val) -> int:
    """functions.f90:811-860 (1-based interval index, 0 below, N above)."""
    n = len(arr)
    if val < arr[0]:
        return 0
    if val > arr[n - 1]:
        return n
    low, high = 1, n
    while high - low > 1:
        mid = (low + high) // 2
        if arr[mid - 1] > val:
            high = mid
        elif arr[mid - 1] < val:
            low = mid
        else:
            return mid
    return low


def ic_interp(p: Params, grid_f, uf, vf, wf):
    """initial.f90:242-380: u, v, w (levels 1..nz_f of the file grid, arrays
    (nz_f, ny_f, ld_f)) onto the grid of p, arrays (nz, ny, ld) at levels 1..nz."""
    nx_f, ny_f, nz_f, Lx_f, Ly_f, Lz_f = grid_f
    dx_f, dy_f, dz_f = Lx_f / nx_f, Ly_f / ny_f, Lz_f / (nz_f - 1)
    x_f = [i * Lx_f / nx_f for i in range(nx_f)]
    y_f = [j * Ly_f / ny_f for j in range(ny_f)]
    zw_r = [k * dz_f for k in range(nz_f)]
    z_r = [z + 0.5 * dz_f for z in zw_r]
    out = [np.zeros((p.nz, p.ny, p.ld)) for _ in range(3)]

    def F(a, i, j, k):
        return a[k - 1, j - 1, i - 1]

    for i in range(1, p.nx + 1):
        xg = (i - 1) * p.dx
        xx = xg - math.floor(xg / Lx_f) * Lx_f
        i1 = binary_search(x_f, xx)
        i2 = i1 % nx_f + 1
        bx = (xx - x_f[i1 - 1]) / dx_f
        ax = 1.0 - bx
        for j in range(1, p.ny + 1):
            yg = (j - 1) * p.dy
            yy = yg - math.floor(yg / Ly_f) * Ly_f
            j1 = binary_search(y_f, yy)
            j2 = j1 % ny_f + 1
            by = (yy - y_f[j1 - 1]) / dy_f
            ay = 1.0 - by

            def plane(a, kk):
                return (ax * ay * F(a, i1, j1, kk) + bx * ay * F(a, i2, j1, kk) + ax * by * F(a, i1, j2, kk)
                        + bx * by * F(a, i2, j2, kk))

            def vol(a, k1, az, bz):
                return (ax * ay * az * F(a, i1, j1, k1) + bx * ay * az * F(a, i2, j1, k1)
                        + ax * by * az * F(a, i1, j2, k1) + bx * by * az * F(a, i2, j2, k1)
                        + ax * ay * bz * F(a, i1, j1, k1 + 1) + bx * ay * bz * F(a, i2, j1, k1 + 1)
                        + ax * by * bz * F(a, i1, j2, k1 + 1) + bx * by * bz * F(a, i2, j2, k1 + 1))

            for k in range(1, p.nz + 1):
                z = (k - 0.5) * p.dz
                k1 = binary_search(z_r, z)
                for a, o in ((uf, out[0]), (vf, out[1])):
                    if k1 == nz_f:
                        o[k - 1, j - 1, i - 1] = plane(a, k1)
                    elif k1 == 0:
                        o[k - 1, j - 1, i - 1] = plane(a, 1)
                    else:
                        bz = (z - z_r[k1 - 1]) / dz_f
                        o[k - 1, j - 1, i - 1] = vol(a, k1, 1.0 - bz, bz)
                zw = (k - 1) * p.dz
                k1 = binary_search(zw_r, zw)
                if k1 == nz_f:
                    out[2][k - 1, j - 1, i - 1] = plane(wf, k1)
                elif k1 == 0:
                    out[2][k - 1, j - 1, i - 1] = plane(wf, 1)
                else:
                    bz = (zw - zw_r[k1 - 1]) / dz_f
                    out[2][k - 1, j - 1, i - 1] = vol(wf, k1, 1.0 - bz, bz)
    return out


def read_checkpoint(o: "Oracle", prefix: str, ta: Optional["TimeAverage"] = None) -> bool:
    """Restart o from the files under prefix (initial.f90:20-239, io.f90:60-96);
    True when the checkpoint was of this grid (initu)."""
    import os
    p = o.p
    nproc, nx_f, ny_f, nz_f, Lx_f, Ly_f, Lz_f = 1, p.nx, p.ny, p.nz, p.L_x, p.L_y, p.L_z
    if os.path.exists(prefix + "grid.out"):
        with open(prefix + "grid.out", "rb") as f:
            rec, = fortran_records(f.read())
        nproc, nx_f, ny_f, nz_f, Lx_f, Ly_f, Lz_f = struct.unpack("<4i3d", rec)
    exact = (nproc == 1 and nx_f == p.nx and ny_f == p.ny and nz_f == p.nz and Lx_f == p.L_x
             and Ly_f == p.L_y and Lz_f == p.L_z)
    shape = (p.nz, p.ny, p.ld)
    if exact:
        name = prefix + "vel.out"
        if not os.path.exists(name):
            name += ".c0"
        with open(name, "rb") as f:
            rec = fortran_records(f.read())[0]
        a = np.frombuffer(rec, dtype="<f8").reshape((11,) + shape)
        for n, arr in zip(VEL_FIELDS, a):
            oracle_state(o, n)[1:] = arr
    else:
        ld_f = 2 * (nx_f // 2 + 1)
        nzt = (nz_f - 1) * nproc + 1
        g = [np.zeros((nzt, ny_f, ld_f)) for _ in range(3)]
        for c in range(nproc):
            name = prefix + "vel.out" + (".c%d" % c if nproc > 1 else "")
            if nproc == 1 and not os.path.exists(name):
                name += ".c0"
            with open(name, "rb") as f:
                rec = fortran_records(f.read())[0]
            blk = np.frombuffer(rec[:3 * nz_f * ny_f * ld_f * 8], dtype="<f8").reshape(3, nz_f, ny_f, ld_f)
            for fi in range(3):
                g[fi][c * (nz_f - 1):c * (nz_f - 1) + nz_f] = blk[fi]
        u, v, w = ic_interp(p, (nx_f, ny_f, nzt, Lx_f, Ly_f, Lz_f), *g)
        for n in VEL_FIELDS:
            oracle_state(o, n)[1:] = 0.0
        o.u[1:], o.v[1:], o.w[1:] = u, v, w
    p.initu = exact
    if p.use_cfl_dt:
        p.lagran_dt = 0.0
    o.jt = 0
    o.F_LM_MM_init = o.F_QN_NN_init = False
    o.jt_total, o.time = 0, 0.0
    if os.path.exists(prefix + "total_time.dat"):
        with open(prefix + "total_time.dat") as f:
            vals = f.read().replace(",", " ").replace("D", "E").split()
        o.jt_total, o.time = int(vals[0]), float(vals[1])
        o.time_dim = float(vals[2])
        if p.use_cfl_dt:
            p.dt = float(vals[3])                     # io.f90:91-94
    tname = prefix + "tavg.out"
    if not os.path.exists(tname):
        tname += ".c0"
    if ta is not None and os.path.exists(tname):
        with open(tname, "rb") as f:
            recs = fortran_records(f.read())
        total, = struct.unpack("<d", recs[0])
        sums = {n: np.zeros((p.nz + 1, p.ny, p.nx)) for n in TAVG_FILE}
        for n, r in zip(TAVG_FILE, recs[1:]):
            sums[n][1:] = np.frombuffer(r, dtype="<f8").reshape(p.nz, p.ny, p.nx)
        ta.loaded = (total, sums)
        ta.initialized = False
        ta.dt = 0.0
    return exact


def tridag_array(a, b, c, r, mask):
    """tridag_array.f90:166-246 (serial Thomas algorithm) on all columns.

    a, b, c: real (n+1, ny, lh) with index 1..n used; r: complex, same shape.
    ``mask`` selects the columns the reference solves (it skips the ky
    Nyquist row and the kx = ky = 0 column in the sweeps); level 1 is set
    for every kx < nx/2 column as in the reference.  Returns u (index 1..n).
    """
    n = a.shape[0] - 1
    lh = a.shape[2]
    cols = np.s_[:, : lh - 1]
    u = np.zeros(r.shape, dtype=complex)
    if np.any(b[1][cols] == 0.0):
        raise ZeroDivisionError("tridag_array: rewrite eqs (b(1) = 0)")
    u[1][cols] = r[1][cols] / b[1][cols]
    bet = b[1].copy()
    gam = np.zeros(a.shape)
    for j in range(2, n + 1):
        g = np.where(mask, c[j - 1] / np.where(mask, bet, 1.0), 0.0)
        gam[j] = g
        bet = np.where(mask, b[j] - a[j] * g, bet)
        if np.any(mask & (bet == 0.0)):
            raise ZeroDivisionError("tridag_array failed (zero pivot)")
        u[j] = np.where(mask, (r[j] - a[j] * u[j - 1]) / np.where(mask, bet, 1.0), u[j])
    for j in range(n - 1, 0, -1):
        u[j] = np.where(mask, u[j] - gam[j + 1] * u[j + 1], u[j])
    return u


def round_half_away(x: float) -> float:
    """Fortran NINT: round half away from zero."""
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def compare_valid(p: Params, name: str, a: np.ndarray, b: np.ndarray) -> float:
    """Max |a-b| / max |b| over the entries the reference defines as valid."""
    nz, nx = p.nz, p.nx
    levels = {
        "u": (1, nz - 1), "v": (1, nz - 1), "w": (2, nz - 1),
        "p": (1, nz - 1), "dpdx": (1, nz - 1), "dpdy": (1, nz - 1),
        "txz": (1, nz - 1), "tyz": (1, nz - 1),
    }.get(name, (1, nz - 1))
    lo, hi = levels
    A = a[lo:hi + 1, :, :nx]
    B = b[lo:hi + 1, :, :nx]
    den = np.max(np.abs(B))
    return float(np.max(np.abs(A - B)) / (den if den > 0 else 1.0))
