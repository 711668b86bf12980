// Non-spectral kernels of the LES step: the fused z-column SGS sweep, the
// Lagrangian pathline interpolation, the batched Thomas solve, the pressure
// correction / projection, step glue, diagnostics and the seeded IC.
#pragma once
#include "stages.cuh"

namespace lesgo {

// ---------------------------------------------------------------------------
// Wall models (wallstress.f90:107-255), evaluated in FP64 in every form.
// Returns txz, tyz, dudz, dvdz at the wall level.
// ---------------------------------------------------------------------------
struct WallOut { double txz, tyz, dudz, dvdz; };

__device__ __forceinline__ WallOut wall_bottom(const KP& kp, double zo, double u1f, double v1f, double u1, double v1) {
  WallOut o{0.0, 0.0, 0.0, 0.0};
  if (kp.lbc == 1) {                      // ws_dns_lbc (:131-148)
    o.dudz = (u1 - kp.ubot) / (0.5 * kp.dz);
    o.dvdz = v1 / (0.5 * kp.dz);
    o.txz = -kp.nu_nd * o.dudz;
    o.tyz = -kp.nu_nd * o.dvdz;
  } else if (kp.lbc == 2) {               // ws_equilibrium_lbc (:171-219)
    const double denom = log(0.5 * kp.dz / zo);
    const double u_avg = sqrt(u1f * u1f + v1f * v1f);
    const double ustar = u_avg * kp.vonk / denom;
    const double c = -(ustar * ustar) / u_avg;
    o.txz = c * u1f;
    o.tyz = c * v1f;
    o.dudz = (u1 == 0.0) ? 0.0 : ustar / (0.5 * kp.dz * kp.vonk) * u1 / u_avg;
    o.dvdz = (v1 == 0.0) ? 0.0 : ustar / (0.5 * kp.dz * kp.vonk) * v1 / u_avg;
  }
  return o;
}

__device__ __forceinline__ WallOut wall_top(const KP& kp, double zo, double utf, double vtf, double ut, double vt) {
  WallOut o{0.0, 0.0, 0.0, 0.0};
  if (kp.ubc == 1) {                      // ws_dns_ubc (:151-168)
    o.dudz = (kp.utop - ut) / (0.5 * kp.dz);
    o.dvdz = -vt / (0.5 * kp.dz);
    o.txz = -kp.nu_nd * o.dudz;
    o.tyz = -kp.nu_nd * o.dvdz;
  } else if (kp.ubc == 2) {               // ws_equilibrium_ubc (:222-255)
    const double denom = log(0.5 * kp.dz / zo);
    const double u_avg = sqrt(utf * utf + vtf * vtf);
    const double ustar = u_avg * kp.vonk / denom;
    const double c = (ustar * ustar) / u_avg;
    o.txz = c * utf;
    o.tyz = c * vtf;
    o.dudz = (ut == 0.0) ? 0.0 : -ustar / (0.5 * kp.dz * kp.vonk) * ut / u_avg;
    o.dvdz = (vt == 0.0) ? 0.0 : -ustar / (0.5 * kp.dz * kp.vonk) * vt / u_avg;
  }
  return o;
}

// ---------------------------------------------------------------------------
// Fused z-column sweep: ddz_uv/ddz_w (derivatives.f90:214-311), the wall
// values, calc_Sij (sgs_stag_util.f90:467-634), |S|, Nu_t and the stresses
// (sgs_stag_util.f90:223-428).  One thread owns an (i,j) column over a
// chunk of levels [k0, k1) and recomputes the level above the chunk.
// FLAGS: COL_DDZ compute+store dudz/dvdz/dwdz and the wall values (else
//        they are read from their fields); COL_STORE_S store S_ij;
//        COL_TAU emit the stresses; COL_READ_S read S_ij instead of
//        computing them.
// ---------------------------------------------------------------------------
enum : int { COL_DDZ = 1, COL_STORE_S = 2, COL_TAU = 4, COL_READ_S = 8 };

template <typename R>
struct ColArgs {
  const R *u, *v, *w, *dudx, *dudy, *dvdx, *dvdy, *dwdx, *dwdy;
  R *dudz, *dvdz, *dwdz;
  R *S11, *S12, *S13, *S22, *S23, *S33;
  R *Cs, *txx, *txy, *txz, *tyy, *tyz, *tzz;
  const R *wb_u, *wb_v, *wt_u, *wt_v;   // test-filtered wall planes
  KP kp;
  double delta2;
  int chunk;
};

template <typename R>
struct Sij { R s11, s12, s13, s22, s23, s33; };

template <typename R, int FLAGS>
__global__ void __launch_bounds__(256) k_column(ColArgs<R> a) {
  const KP& kp = a.kp;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= kp.nx * kp.ny) return;
  const int j = col / kp.nx, i = col - j * kp.nx;
  const int nz = kp.nz;
  const int k0 = 1 + blockIdx.y * a.chunk;
  if (k0 > nz) return;
  const int k1 = min(nz + 1, k0 + a.chunk);
  const int inst = blockIdx.z;
  const long long P = kp.plane;
  const long long cw = inst * P + (long long)j * kp.ld + i;          // wall planes (ld, ny) per instance
  const long long c0 = inst * kp.istride + (long long)j * kp.ld + i;  // 3-D fields
  const double zo = kp.zo_i[inst];
  const bool cs_fill = (kp.iflags[inst] & IF_CSFILL) != 0;
  const R inv_dz = (R)kp.idz;
  const R h = (R)0.5;

  // wall values (needed at k = 1 and k = nz)
  WallOut wb{0, 0, 0, 0}, wt{0, 0, 0, 0};
  if (FLAGS & COL_DDZ) {
    if (k0 == 1) {
      double uf = 0, vf = 0;
      if (kp.lbc == 2) { uf = a.wb_u[cw]; vf = a.wb_v[cw]; }
      wb = wall_bottom(kp, zo, uf, vf, (double)a.u[P + c0], (double)a.v[P + c0]);
    }
    if (k1 >= nz) {
      double uf = 0, vf = 0;
      if (kp.ubc == 2) { uf = a.wt_u[cw]; vf = a.wt_v[cw]; }
      wt = wall_top(kp, zo, uf, vf, (double)a.u[(nz - 1) * P + c0], (double)a.v[(nz - 1) * P + c0]);
    }
  }
  auto uz_at = [&](int k) -> R {
    const long long q = k * P + c0;
    if (!(FLAGS & COL_DDZ)) return a.dudz[q];
    if (k == 1) return (R)wb.dudz;
    if (k == nz) return (R)wt.dudz;
    return inv_dz * (a.u[q] - a.u[q - P]);
  };
  auto vz_at = [&](int k) -> R {
    const long long q = k * P + c0;
    if (!(FLAGS & COL_DDZ)) return a.dvdz[q];
    if (k == 1) return (R)wb.dvdz;
    if (k == nz) return (R)wt.dvdz;
    return inv_dz * (a.v[q] - a.v[q - P]);
  };
  auto wz_at = [&](int k) -> R {
    const long long q = k * P + c0;
    if (k >= nz) return (R)0;
    if (!(FLAGS & COL_DDZ)) return a.dwdz[q];
    return inv_dz * (a.w[q + P] - a.w[q]);
  };

  // derivative window: values at level k-1 (p*) and k (c*)
  R pux = 0, puy = 0, pvx = 0, pvy = 0, pwx = 0, pwy = 0, pwz = 0;
  if (!(FLAGS & COL_READ_S) && k0 > 1) {
    const long long q = (k0 - 1) * P + c0;
    pux = a.dudx[q]; puy = a.dudy[q]; pvx = a.dvdx[q]; pvy = a.dvdy[q];
    pwx = a.dwdx[q]; pwy = a.dwdy[q]; pwz = wz_at(k0 - 1);
  }
  Sij<R> Sp{0, 0, 0, 0, 0, 0};
  R Np = 0;
  const int kend = min(k1, nz);
  for (int k = k0; k <= kend; ++k) {
    const long long q = k * P + c0;
    Sij<R> S;
    if (FLAGS & COL_READ_S) {
      S = Sij<R>{a.S11[q], a.S12[q], a.S13[q], a.S22[q], a.S23[q], a.S33[q]};
    } else {
      const R ux = a.dudx[q], uy = a.dudy[q], vx = a.dvdx[q], vy = a.dvdy[q];
      const R wx = a.dwdx[q], wy = a.dwdy[q];
      const R uz = uz_at(k), vz = vz_at(k), wz = wz_at(k);
      if (k == 1) {
        if (kp.lbc == 0) {
          S = Sij<R>{ux, h * (uy + vx), h * (uz + wx), vy, h * (vz + wy), h * (wz + (R)0)};
        } else {
          const R wx2 = h * (wx + a.dwdx[q + P]);
          const R wy2 = h * (wy + a.dwdy[q + P]);
          S = Sij<R>{ux, h * (uy + vx), h * (uz + wx2), vy, h * (vz + wy2), wz};
        }
      } else if (k == nz) {
        if (kp.ubc == 0) {
          S = Sij<R>{pux, h * (puy + pvx), h * (uz + wx), pvy, h * (vz + wy), h * (pwz + (R)0)};
        } else {
          const R wx2 = h * (pwx + wx), wy2 = h * (pwy + wy);
          S = Sij<R>{pux, h * (puy + pvx), h * (uz + wx2), pvy, h * (vz + wy2), pwz};
        }
      } else {
        const R uyy = uy + puy, vxx = vx + pvx;
        S = Sij<R>{h * (ux + pux), (R)0.25 * (uyy + vxx), h * (uz + wx), h * (vy + pvy), h * (vz + wy), h * (wz + pwz)};
      }
      if (k < k1) {
        if (FLAGS & COL_STORE_S) {
          a.S11[q] = S.s11; a.S12[q] = S.s12; a.S13[q] = S.s13;
          a.S22[q] = S.s22; a.S23[q] = S.s23; a.S33[q] = S.s33;
        }
        if (FLAGS & COL_DDZ) {
          a.dudz[q] = uz;
          a.dvdz[q] = vz;
          if (k <= nz - 1) a.dwdz[q] = wz;
          if (k == 1) { a.txz[q] = (R)wb.txz; a.tyz[q] = (R)wb.tyz; }
          if (k == nz) { a.txz[q] = (R)wt.txz; a.tyz[q] = (R)wt.tyz; }
        }
      }
      pux = ux; puy = uy; pvx = vx; pvy = vy; pwx = wx; pwy = wy; pwz = wz;
    }
    if (FLAGS & COL_TAU) {
      R cs;
      if (cs_fill) {
        cs = (R)0.03;
        if (k < k1) a.Cs[q] = cs;
      } else {
        cs = a.Cs[q];
      }
      const R Sm = sqrt((R)2 * (S.s11 * S.s11 + S.s22 * S.s22 + S.s33 * S.s33 +
                                (R)2 * (S.s12 * S.s12 + S.s13 * S.s13 + S.s23 * S.s23)));
      const R Nu = Sm * cs * (R)a.delta2;
      const int m = k - 1;   // emit the stresses of level m = k-1
      if (m >= k0 && m <= nz - 1) {
        const long long qm = q - P;
        const R nu = (R)kp.nu;
        if (m == nz - 1) {
          if (kp.ubc == 0) {
            const R c = h * (Np + Nu) + nu, c2 = (R)2 * (Np + nu);
            a.txx[qm] = -c * (Sp.s11 + S.s11); a.txy[qm] = -c * (Sp.s12 + S.s12);
            a.tyy[qm] = -c * (Sp.s22 + S.s22); a.tzz[qm] = -c * (Sp.s33 + S.s33);
            a.txz[qm] = -c2 * Sp.s13; a.tyz[qm] = -c2 * Sp.s23;
          } else {
            const R c = (R)-2 * (Nu + nu), c2 = (R)-2 * (Np + nu);
            a.txx[qm] = c * S.s11; a.txy[qm] = c * S.s12; a.tyy[qm] = c * S.s22; a.tzz[qm] = c * S.s33;
            a.txz[qm] = c2 * Sp.s13; a.tyz[qm] = c2 * Sp.s23;
          }
        } else if (m == 1) {
          if (kp.lbc == 0) {
            const R c = h * (Np + Nu) + nu;
            a.txx[qm] = -c * (Sp.s11 + S.s11); a.txy[qm] = -c * (Sp.s12 + S.s12);
            a.tyy[qm] = -c * (Sp.s22 + S.s22); a.tzz[qm] = -c * (Sp.s33 + S.s33);
          } else {
            const R c = (R)-2 * (Np + nu);
            a.txx[qm] = c * Sp.s11; a.txy[qm] = c * Sp.s12; a.tyy[qm] = c * Sp.s22; a.tzz[qm] = c * Sp.s33;
          }
        } else {
          const R c = -h * (Np + Nu), c2 = (R)-2 * Np, c3 = (R)-2 * nu * h, c4 = (R)-2 * nu;
          a.txx[qm] = (c + c3) * (Sp.s11 + S.s11); a.txy[qm] = (c + c3) * (Sp.s12 + S.s12);
          a.tyy[qm] = (c + c3) * (Sp.s22 + S.s22); a.tzz[qm] = (c + c3) * (Sp.s33 + S.s33);
          a.txz[qm] = (c2 + c4) * Sp.s13; a.tyz[qm] = (c2 + c4) * Sp.s23;
        }
      }
      Np = Nu;
    }
    Sp = S;
  }
}

// Flat thread index over (instance, level 1..nz, j, i < nx) -> field offset.
// Point index t (x fastest, then y, level 1..nz, instance) -> coordinates.
// Launches cover fewer than 2^31 points (checked when a handle is made), so
// the decomposition divides 32-bit values by multiply-high reciprocals.
struct PtIdx { int inst, k, j, i; long long q; };
__device__ __forceinline__ PtIdx pt_index(long long t, const KP& kp) {
  PtIdx r;
  const int ti = (int)t;
  const int a = kp.fnx.div(ti);
  r.i = ti - a * kp.nx;
  const int b = kp.fny.div(a);
  r.j = a - b * kp.ny;
  r.inst = kp.fnz.div(b);
  r.k = 1 + (b - r.inst * kp.nz);
  r.q = r.inst * kp.istride + (long long)r.k * kp.plane + (long long)r.j * kp.ld + r.i;
  return r;
}

// Plain staggered z-derivatives for the stand-alone entry points.
// uv: dfdz(k) = (f(k)-f(k-1))/dz, k = 2..nz; w: dfdz(k) = (f(k+1)-f(k))/dz, k = 1..nz-1.
template <typename R, bool UV>
__global__ void k_ddz(const R* __restrict__ f, R* __restrict__ dfdz, KP kp) {
  const long long n = (long long)kp.nx * kp.ny * kp.nz * kp.ninst;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const PtIdx x = pt_index(t, kp);
    const int k = x.k;
    const long long q = x.q;
    const R c = (R)kp.idz;
    if (UV) { if (k >= 2) dfdz[q] = c * (f[q] - f[q - kp.plane]); }
    else    { if (k <= kp.nz - 1) dfdz[q] = c * (f[q + kp.plane] - f[q]); }
  }
}

// Stand-alone wallstress (wallstress.f90:21-257) from filtered planes.
template <typename R>
__global__ void k_wall(const R* u, const R* v, const R* wb_u, const R* wb_v, const R* wt_u, const R* wt_v,
                       R* txz, R* tyz, R* dudz, R* dvdz, KP kp) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= kp.nx * kp.ny) return;
  const int j = col / kp.nx, i = col - j * kp.nx;
  const int inst = blockIdx.y;
  const long long P = kp.plane;
  const long long cw = inst * P + (long long)j * kp.ld + i;
  const long long c0 = inst * kp.istride + (long long)j * kp.ld + i;
  const int nz = kp.nz;
  const double zo = kp.zo_i[inst];
  WallOut b = wall_bottom(kp, zo, kp.lbc == 2 ? (double)wb_u[cw] : 0.0, kp.lbc == 2 ? (double)wb_v[cw] : 0.0,
                          (double)u[P + c0], (double)v[P + c0]);
  WallOut t = wall_top(kp, zo, kp.ubc == 2 ? (double)wt_u[cw] : 0.0, kp.ubc == 2 ? (double)wt_v[cw] : 0.0,
                       (double)u[(nz - 1) * P + c0], (double)v[(nz - 1) * P + c0]);
  txz[P + c0] = (R)b.txz; tyz[P + c0] = (R)b.tyz; dudz[P + c0] = (R)b.dudz; dvdz[P + c0] = (R)b.dvdz;
  const long long qt = nz * P + c0;
  txz[qt] = (R)t.txz; tyz[qt] = (R)t.tyz; dudz[qt] = (R)t.dudz; dvdz[qt] = (R)t.dvdz;
}

// ---------------------------------------------------------------------------
// interpolag_Sdep.f90:21-270 with trilinear_interp_w / cell_indx_w
// (functions.f90:188-265, 349-474): backward Lagrangian advection of the
// four running averages.  Positions are formed in FP64.
// ---------------------------------------------------------------------------
template <typename R>
struct InterpArgs {
  const R *u, *v, *w;
  const R *Fin[4];
  R* Fout[4];
  KP kp;
};

// The mixed form's departure point in grid units: a cell index plus a
// fraction from the displacement -u lagran_dt / dx (below one cell under
// the Lagrangian CFL), so FP32 keeps the weights to its own precision (an
// absolute coordinate in FP32 would lose them to cancellation).  The cell
// and weight rules are cell_indx_w's and trilinear_interp_w's
// (functions.f90:188-474) in those units: z(m) = m - 1/2, zw(m) = m - 1,
// the half cell at the wall and lid, periodic wrap in x and y.
template <typename R>
__device__ __forceinline__ void interp_fp32(const InterpArgs<R>& a, int i, int j, int k, long long q, long long ib,
                                            int inst) {
  const KP& kp = a.kp;
  const long long P = kp.plane;
  const int nz = kp.nz;
  const float ldt = (float)kp.sc[inst * SC_N + SC_LDT];
  const float cx = ldt * (float)kp.idx, cy = ldt * (float)kp.idy, cz = ldt * (float)kp.idz;
  float fx, fy, fz;
  int bz;   // z / dz = bz + fz
  if (k == 1) {
    fx = -(float)a.u[q] * cx;
    fy = -(float)a.v[q] * cy;
    bz = 0;
    fz = (kp.lbc == 0) ? 0.0f : 0.5f - 0.25f * (float)a.w[q + P] * cz;
  } else if (k == nz) {
    fx = -(float)a.u[q - P] * cx;
    fy = -(float)a.v[q - P] * cy;
    if (kp.ubc == 0) { bz = nz - 1; fz = 0.0f; }
    else { bz = nz - 2; fz = 0.5f - 0.25f * (float)a.w[q - P] * cz; }
  } else {
    fx = -0.5f * ((float)a.u[q - P] + (float)a.u[q]) * cx;
    fy = -0.5f * ((float)a.v[q - P] + (float)a.v[q]) * cy;
    bz = k - 1;
    fz = -(float)a.w[q] * cz;
  }
  const float flx = floorf(fx), fly = floorf(fy);
  int ist = i + (int)flx, jst = j + (int)fly;   // zero-based cells, one period at most away
  if (ist < 0) ist += kp.nx;
  else if (ist >= kp.nx) ist -= kp.nx;
  if (jst < 0) jst += kp.ny;
  else if (jst >= kp.ny) jst -= kp.ny;
  ist = min(max(ist, 0), kp.nx - 1);   // guards the memory access only
  jst = min(max(jst, 0), kp.ny - 1);
  const int ist1 = ist + 1 == kp.nx ? 0 : ist + 1;
  const int jst1 = jst + 1 == kp.ny ? 0 : jst + 1;
  const R wx = (R)(fx - flx), wy = (R)(fy - fly);
  int kst, kst1;
  float wz;
  const float zg = (float)bz + fz;   // only compared against the wall and lid cells
  if (kp.lbc > 0 && zg < 1.0f) {
    if (zg < 0.5f) { kst = 1; kst1 = 1; wz = 0.0f; }
    else { kst = 1; kst1 = 2; wz = 2.0f * (((float)bz - 0.5f) + fz); }
  } else if (kp.ubc > 0 && zg > (float)(nz - 2)) {
    if (zg > (float)nz - 1.5f) { kst = nz; kst1 = nz; wz = 0.0f; }
    else { kst = nz - 1; kst1 = nz; wz = 2.0f * ((float)(bz - (nz - 2)) + fz); }
  } else {
    const float flz = floorf(fz);
    kst = bz + (int)flz + 1;
    // the reference assumes a Lagrangian CFL below one, which keeps kst in
    // 1..nz-1; the clamp only guards the memory access
    kst = min(max(kst, 1), nz - 1);
    kst1 = kst + 1;
    wz = (float)(bz - (kst - 1)) + fz;
  }
  const long long b00 = ib + (long long)jst * kp.ld, b01 = ib + (long long)jst1 * kp.ld;
  const long long z0 = kst * P, z1 = kst1 * P;
  const R wzr = (R)wz;
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const R* V = a.Fin[f];
    const R v000 = V[z0 + b00 + ist], v001 = V[z0 + b00 + ist1];
    const R v010 = V[z0 + b01 + ist], v011 = V[z0 + b01 + ist1];
    const R v100 = V[z1 + b00 + ist], v101 = V[z1 + b00 + ist1];
    const R v110 = V[z1 + b01 + ist], v111 = V[z1 + b01 + ist1];
    const R u1 = v000 + wx * (v001 - v000);
    const R u2 = v010 + wx * (v011 - v010);
    const R u3 = v100 + wx * (v101 - v100);
    const R u4 = v110 + wx * (v111 - v110);
    const R u5 = u1 + wy * (u2 - u1);
    const R u6 = u3 + wy * (u4 - u3);
    a.Fout[f][q] = u5 + wzr * (u6 - u5);
  }
}

template <typename R>
__global__ void k_interp(InterpArgs<R> a) {
  const KP& kp = a.kp;
  const long long n = (long long)kp.nx * kp.ny * kp.nz * kp.ninst;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const PtIdx x_ = pt_index(t, kp);
  const int i = x_.i, j = x_.j, k = x_.k;
  const long long P = kp.plane;
  const long long q = x_.q;
  const long long ib = x_.inst * kp.istride;
  const int nz = kp.nz;
  if constexpr (std::is_same<R, float>::value) {
    interp_fp32(a, i, j, k, q, ib, x_.inst);
    return;
  }
  const double ldt = kp.sc[x_.inst * SC_N + SC_LDT], dz = kp.dz;
  const double x = i * kp.dx, y = j * kp.dy;
  auto zc = [&](int kk) { return (kk - 0.5) * dz; };          // grid%z
  auto zwc = [&](int kk) { return zc(kk) - dz / 2.0; };       // grid%zw
  double xq, yq, zq;
  if (k == 1) {
    xq = x - (double)a.u[q] * ldt;
    yq = y - (double)a.v[q] * ldt;
    zq = (kp.lbc == 0) ? zwc(1) : zc(1) - 0.25 * (double)a.w[q + P] * ldt;
  } else if (k == nz) {
    xq = x - (double)a.u[q - P] * ldt;
    yq = y - (double)a.v[q - P] * ldt;
    zq = (kp.ubc == 0) ? zwc(nz) : zc(nz - 1) - 0.25 * (double)a.w[q - P] * ldt;
  } else {
    xq = x - 0.5 * ((double)a.u[q - P] + (double)a.u[q]) * ldt;
    yq = y - 0.5 * ((double)a.v[q - P] + (double)a.v[q]) * ldt;
    zq = zwc(k) - (double)a.w[q] * ldt;
  }
  // cell_indx_w with reciprocal multiplies (FP64 division is a long DFMA
  // sequence on this part); the weights differ from the reference's
  // divisions by at most an ulp, and a cell flip at an exact face leaves the
  // linear interpolant unchanged
  const double thresh = 1.0e-9;
  const double idx = kp.idx, idy = kp.idy, idz = kp.idz;   // reciprocals made on the host
  double px = xq - floor(xq * kp.iLx) * kp.L_x;
  int ist = (fabs(px) < thresh * kp.L_x) ? 1 : (fabs(px - kp.L_x) < thresh * kp.L_x) ? kp.nx : (int)floor(px * idx) + 1;
  double py = yq - floor(yq * kp.iLy) * kp.L_y;
  int jst = (fabs(py) < thresh * kp.L_y) ? 1 : (fabs(py - kp.L_y) < thresh * kp.L_y) ? kp.ny : (int)floor(py * idy) + 1;
  ist = min(max(ist, 1), kp.nx);
  jst = min(max(jst, 1), kp.ny);
  const int ist1 = ist + 1 > kp.nx ? 1 : ist + 1;
  const int jst1 = jst + 1 > kp.ny ? 1 : jst + 1;
  const double xdiff = px - (ist - 1) * kp.dx;
  const double ydiff = py - (jst - 1) * kp.dy;
  int kst, kst1;
  double zdiff;
  if (kp.lbc > 0 && zq < zwc(2)) {
    if (zq < zc(1)) { kst = 1; kst1 = 1; zdiff = 0.0; }
    else { kst = 1; kst1 = 2; zdiff = 2.0 * (zq - zc(1)); }
  } else if (kp.ubc > 0 && zq > zwc(nz - 1)) {
    if (zq > zc(nz - 1)) { kst = nz; kst1 = nz; zdiff = 0.0; }
    else { kst = nz - 1; kst1 = nz; zdiff = 2.0 * (zq - zwc(nz - 1)); }
  } else {
    if (fabs(zq - zwc(nz)) < thresh * kp.L_z) kst = nz - 1;
    else kst = (int)floor((zq - zwc(1)) * idz) + 1;
    // the reference assumes a Lagrangian CFL below one, which keeps kst in
    // 1..nz-1; the clamp only guards the memory access
    kst = min(max(kst, 1), nz - 1);
    kst1 = kst + 1;
    zdiff = zq - zwc(kst);
  }
  const R wx = (R)(xdiff * idx), wy = (R)(ydiff * idy), wz = (R)(zdiff * idz);
  const long long b00 = ib + (long long)(jst - 1) * kp.ld, b01 = ib + (long long)(jst1 - 1) * kp.ld;
  const int i0 = ist - 1, i1 = ist1 - 1;
  const long long z0 = kst * P, z1 = kst1 * P;
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const R* V = a.Fin[f];
    const R v000 = V[z0 + b00 + i0], v001 = V[z0 + b00 + i1];
    const R v010 = V[z0 + b01 + i0], v011 = V[z0 + b01 + i1];
    const R v100 = V[z1 + b00 + i0], v101 = V[z1 + b00 + i1];
    const R v110 = V[z1 + b01 + i0], v111 = V[z1 + b01 + i1];
    const R u1 = v000 + wx * (v001 - v000);
    const R u2 = v010 + wx * (v011 - v010);
    const R u3 = v100 + wx * (v101 - v100);
    const R u4 = v110 + wx * (v111 - v110);
    const R u5 = u1 + wy * (u2 - u1);
    const R u6 = u3 + wy * (u4 - u3);
    a.Fout[f][q] = u5 + wz * (u6 - u5);
  }
}

// ---------------------------------------------------------------------------
// press_stag_array.f90:186-234 + tridag_array.f90:166-246: the z-tridiagonal
// pressure solve per (kx, ky) column in FP64, the kx = ky = 0 mode by
// vertical integration, Nyquist rows zeroed.  Spectra layout [level][jy][kx].
//
// The pivots of the Thomas elimination depend only on (kx, ky, dz), so
// ibet_j = 1/bet_j and gam_j are computed once per grid (host, FP64, the
// reference's recurrence) and a zero pivot is reported when the solver is
// created.  Each column's sweeps are split into SEG segments worked on by
// SEG threads: a first pass per segment composes the affine map from the
// segment's input value to its end value, shared memory chains the maps
// across segments, and a second pass re-sweeps every segment from its exact
// input in the reference's order: u_j = (r_j - a_j u_{j-1}) / bet_j forward,
// u_j = u_j - gam_{j+1} u_{j+1} backward.
// ---------------------------------------------------------------------------
// SEG segments per column, COLS columns per block (SEG * COLS threads).
// The host picks among this looped form, the register-held k_thomas_r and
// the sequential k_thomas_seq (below) by column count and unknowns.

struct ThomasArgs {
  const double2 *Hx, *Hy, *Hz;   // levels 1..nz at index level-1, [inst][nz][P]
  const double2 *Hb, *Ht;        // r2c of divtz(1), divtz(nz) (scaled), [inst][2][P]
  double2* phat;                 // levels 0..nz, [inst][nz+1][P]; holds r, then u
  const double *ibet, *gam;      // [n+1][P], index j = 1..n (shared by instances)
  const double *kxw, *kyw;
  double dz, idz, idz2;   // dz, 1/dz, 1/dz^2 (made on the host)
  int nz, ny, K, ninst;
};

__device__ __forceinline__ double2 thomas_rhs(const ThomasArgs& a, const double2* Hx, const double2* Hy,
                                              const double2* Hz, const double2* Hb, const double2* Ht, int j,
                                              long long P, int t, double kxv, double kyv) {
  const int nz = a.nz;
  if (j == 1) { const double2 h = Hb[t]; return make_double2(-a.dz * h.x, -a.dz * h.y); }
  if (j == nz + 1) { const double2 h = Ht[t]; return make_double2(-a.dz * h.x, -a.dz * h.y); }
  const double c4 = a.idz;
  const double2 hx = Hx[(j - 2) * P + t], hy = Hy[(j - 2) * P + t];
  const double2 hz = Hz[(j - 1) * P + t], hzp = Hz[(j - 2) * P + t];
  // i kx Hx(j-1) + i ky Hy(j-1) + (Hz(j) - Hz(j-1)) / dz
  return make_double2((-hx.y * kxv) + (-hy.y * kyv) + (hz.x - hzp.x) * c4,
                      (hx.x * kxv) + (hy.x * kyv) + (hz.y - hzp.y) * c4);
}

template <int SEG, int COLS>
__global__ void __launch_bounds__(SEG * COLS) k_thomas(ThomasArgs a) {
  __shared__ double2 s_x[SEG][COLS];   // segment end value / start value
  __shared__ double s_h[SEG][COLS];    // segment map slope
  const int lane = threadIdx.x % COLS, seg = threadIdx.x / COLS;
  const long long P = (long long)a.ny * a.K;
  const long long gcol = (long long)blockIdx.x * COLS + lane;
  const bool live = gcol < P * a.ninst;
  const int inst = live ? (int)(gcol / P) : 0;
  const int t = live ? (int)(gcol - inst * P) : 0;
  const int jy = t / a.K, kx = t - jy * a.K;
  const int nz = a.nz, n = nz + 1;
  const double2* Hx = a.Hx + (long long)inst * nz * P;
  const double2* Hy = a.Hy + (long long)inst * nz * P;
  const double2* Hz = a.Hz + (long long)inst * nz * P;
  const double2* Hb = a.Hb + (long long)inst * 2 * P;
  const double2* Ht = a.Ht + (long long)inst * 2 * P;
  double2* phat = a.phat + (long long)inst * (nz + 1) * P;   // u_j at phat[(j-1)*P]
  const bool nyq = jy == a.ny / 2;
  const bool mean = kx == 0 && jy == 0;
  const int L = (n + SEG - 1) / SEG;
  const int j0 = 1 + seg * L, j1 = min(n, j0 + L - 1);   // this thread's levels (may be empty)
  const double c3 = a.idz2;
  const double kxv = a.kxw[kx], kyv = a.kyw[jy];
  const bool solve = live && !nyq && !mean;

  // ---- forward: r_j into phat, and the segment's map x -> u_{j1} = ut + h x
  double2 ut = make_double2(0.0, 0.0);
  double h = 1.0;
  if (solve) {
    for (int j = j0; j <= j1; ++j) {
      const double2 r = thomas_rhs(a, Hx, Hy, Hz, Hb, Ht, j, P, t, kxv, kyv);
      phat[(j - 1) * P + t] = r;
      const double ib = a.ibet[(long long)j * P + t];
      const double aj = (j == 1) ? 0.0 : (j <= nz ? c3 : -1.0);
      ut = make_double2((r.x - aj * ut.x) * ib, (r.y - aj * ut.y) * ib);
      h = -aj * ib * h;
    }
  }
  s_x[seg][lane] = ut;
  s_h[seg][lane] = h;
  __syncthreads();
  double2 x = make_double2(0.0, 0.0);   // u_{j0-1}
  for (int s = 0; s < seg; ++s) {
    const double2 e = s_x[s][lane];
    const double hs = s_h[s][lane];
    x = make_double2(e.x + hs * x.x, e.y + hs * x.y);
  }
  __syncthreads();
  // ---- forward re-sweep from the exact input; the segment end is u_{j1}
  double2 up = x;
  if (solve) {
    for (int j = j0; j <= j1; ++j) {
      const double2 r = phat[(j - 1) * P + t];
      const double ib = a.ibet[(long long)j * P + t];
      const double aj = (j == 1) ? 0.0 : (j <= nz ? c3 : -1.0);
      up = make_double2((r.x - aj * up.x) * ib, (r.y - aj * up.y) * ib);
      phat[(j - 1) * P + t] = up;
    }
  }
  // ---- backward: v_j = u_j - gam_{j+1} v_{j+1}; map y = v_{j1+1} -> v_{j0} = vt + g y
  double2 vt = make_double2(0.0, 0.0);
  double g = 1.0;
  if (solve) {
    for (int j = j1; j >= j0; --j) {
      const double2 uj = phat[(j - 1) * P + t];
      const double gj = (j == n) ? 0.0 : a.gam[(long long)(j + 1) * P + t];
      vt = make_double2(uj.x - gj * vt.x, uj.y - gj * vt.y);
      g = -gj * g;
    }
  }
  s_x[seg][lane] = vt;
  s_h[seg][lane] = g;
  __syncthreads();
  double2 y = make_double2(0.0, 0.0);   // v_{j1+1}; the top segment has none
  for (int s = SEG - 1; s > seg; --s) {
    const double2 e = s_x[s][lane];
    const double gs = s_h[s][lane];
    y = make_double2(e.x + gs * y.x, e.y + gs * y.y);
  }
  if (solve) {
    double2 vn = y;
    for (int j = j1; j >= j0; --j) {
      double2 uj = phat[(j - 1) * P + t];
      if (j < n) {
        const double gj = a.gam[(long long)(j + 1) * P + t];
        uj = make_double2(uj.x - gj * vn.x, uj.y - gj * vn.y);
      }
      phat[(j - 1) * P + t] = uj;
      vn = uj;
    }
  }
  if (!live) return;
  if (nyq) {
    for (int j = j0; j <= j1; ++j) phat[(j - 1) * P + t] = make_double2(0.0, 0.0);
  } else if (mean && seg == 0) {
    // kx = ky = 0: p(0) = 0, p(1) = -dz rbottomw, p(jz) = p(jz-1) + Hz(jz) dz
    double2 p = make_double2(0.0, 0.0);
    phat[t] = p;
    const double2 hb = Hb[t];
    p = make_double2(p.x - a.dz * hb.x, p.y - a.dz * hb.y);
    phat[P + t] = p;
    for (int jz = 2; jz <= nz; ++jz) {
      const double2 hz = Hz[(jz - 1) * P + t];
      p = make_double2(p.x + hz.x * a.dz, p.y + hz.y * a.dz);
      phat[jz * P + t] = p;
    }
  }
}

// The same solve with each thread's segment (at most LMAX levels) held in
// registers: all of the segment's loads (right-hand side inputs, pivots)
// are issued before the recurrences run, and phat is written once.  The
// arithmetic is k_thomas's, operation for operation.
template <int SEG, int COLS, int LMAX>
__global__ void __launch_bounds__(SEG * COLS) k_thomas_r(ThomasArgs a) {
  __shared__ double2 s_x[SEG][COLS];
  __shared__ double s_h[SEG][COLS];
  const int lane = threadIdx.x % COLS, seg = threadIdx.x / COLS;
  const long long P = (long long)a.ny * a.K;
  const long long gcol = (long long)blockIdx.x * COLS + lane;
  const bool live = gcol < P * a.ninst;
  const int inst = live ? (int)(gcol / P) : 0;
  const int t = live ? (int)(gcol - inst * P) : 0;
  const int jy = t / a.K, kx = t - jy * a.K;
  const int nz = a.nz, n = nz + 1;
  const double2* Hx = a.Hx + (long long)inst * nz * P;
  const double2* Hy = a.Hy + (long long)inst * nz * P;
  const double2* Hz = a.Hz + (long long)inst * nz * P;
  const double2* Hb = a.Hb + (long long)inst * 2 * P;
  const double2* Ht = a.Ht + (long long)inst * 2 * P;
  double2* phat = a.phat + (long long)inst * (nz + 1) * P;
  const bool nyq = jy == a.ny / 2;
  const bool mean = kx == 0 && jy == 0;
  const int L = (n + SEG - 1) / SEG;
  const int j0 = 1 + seg * L, j1 = min(n, j0 + L - 1);
  const double c3 = a.idz2;
  const double kxv = a.kxw[kx], kyv = a.kyw[jy];
  const bool solve = live && !nyq && !mean;
  double2 rr[LMAX];
  double ib[LMAX], gm[LMAX];
#pragma unroll
  for (int m = 0; m < LMAX; ++m) {
    const int j = j0 + m;
    rr[m] = make_double2(0.0, 0.0);
    ib[m] = 0.0;
    gm[m] = 0.0;
    if (solve && j <= j1) {
      rr[m] = thomas_rhs(a, Hx, Hy, Hz, Hb, Ht, j, P, t, kxv, kyv);
      ib[m] = a.ibet[(long long)j * P + t];
      if (j < n) gm[m] = a.gam[(long long)(j + 1) * P + t];
    }
  }
  // forward map x -> u_{j1} = ut + h x
  double2 ut = make_double2(0.0, 0.0);
  double h = 1.0;
#pragma unroll
  for (int m = 0; m < LMAX; ++m) {
    const int j = j0 + m;
    if (solve && j <= j1) {
      const double aj = (j == 1) ? 0.0 : (j <= nz ? c3 : -1.0);
      ut = make_double2((rr[m].x - aj * ut.x) * ib[m], (rr[m].y - aj * ut.y) * ib[m]);
      h = -aj * ib[m] * h;
    }
  }
  s_x[seg][lane] = ut;
  s_h[seg][lane] = h;
  __syncthreads();
  double2 x = make_double2(0.0, 0.0);
  for (int s = 0; s < seg; ++s) {
    const double2 e = s_x[s][lane];
    const double hs = s_h[s][lane];
    x = make_double2(e.x + hs * x.x, e.y + hs * x.y);
  }
  __syncthreads();
  // forward re-sweep from the exact input: rr becomes u
  double2 up = x;
#pragma unroll
  for (int m = 0; m < LMAX; ++m) {
    const int j = j0 + m;
    if (solve && j <= j1) {
      const double aj = (j == 1) ? 0.0 : (j <= nz ? c3 : -1.0);
      up = make_double2((rr[m].x - aj * up.x) * ib[m], (rr[m].y - aj * up.y) * ib[m]);
      rr[m] = up;
    }
  }
  // backward map y = v_{j1+1} -> v_{j0} = vt + g y
  double2 vt = make_double2(0.0, 0.0);
  double g = 1.0;
#pragma unroll
  for (int m = LMAX - 1; m >= 0; --m) {
    const int j = j0 + m;
    if (solve && j <= j1) {
      const double gj = gm[m];   // 0 at j = n
      vt = make_double2(rr[m].x - gj * vt.x, rr[m].y - gj * vt.y);
      g = -gj * g;
    }
  }
  s_x[seg][lane] = vt;
  s_h[seg][lane] = g;
  __syncthreads();
  double2 y = make_double2(0.0, 0.0);
  for (int s = SEG - 1; s > seg; --s) {
    const double2 e = s_x[s][lane];
    const double gs = s_h[s][lane];
    y = make_double2(e.x + gs * y.x, e.y + gs * y.y);
  }
  if (solve) {
    double2 vn = y;
#pragma unroll
    for (int m = LMAX - 1; m >= 0; --m) {
      const int j = j0 + m;
      if (j <= j1) {
        double2 uj = rr[m];
        if (j < n) uj = make_double2(uj.x - gm[m] * vn.x, uj.y - gm[m] * vn.y);
        phat[(j - 1) * P + t] = uj;
        vn = uj;
      }
    }
  }
  if (!live) return;
  if (nyq) {
    for (int j = j0; j <= j1; ++j) phat[(j - 1) * P + t] = make_double2(0.0, 0.0);
  } else if (mean && seg == 0) {
    double2 p = make_double2(0.0, 0.0);
    phat[t] = p;
    const double2 hb = Hb[t];
    p = make_double2(p.x - a.dz * hb.x, p.y - a.dz * hb.y);
    phat[P + t] = p;
    for (int jz = 2; jz <= nz; ++jz) {
      const double2 hz = Hz[(jz - 1) * P + t];
      p = make_double2(p.x + hz.x * a.dz, p.y + hz.y * a.dz);
      phat[jz * P + t] = p;
    }
  }
}

// The sequential form: one thread per column sweeps all n levels in the
// reference's order (forward u_j = (r_j - a_j u_{j-1}) / bet_j, then
// u_j -= gam_{j+1} u_{j+1}), with half the FP64 work of the segmented form
// (no segment maps).  Chunks of C levels are double-buffered in registers:
// the next chunk's loads are in flight while the current one is swept.
template <int C>
__device__ __forceinline__ void thomas_fwd_load(const ThomasArgs& a, const double2* Hx, const double2* Hy,
                                                const double2* Hz, const double2* Hb, const double2* Ht,
                                                long long P, int t, double kxv, double kyv, int j0, int n,
                                                double2* rr, double* ib) {
#pragma unroll
  for (int m = 0; m < C; ++m) {
    const int j = j0 + m;
    if (j <= n) {
      rr[m] = thomas_rhs(a, Hx, Hy, Hz, Hb, Ht, j, P, t, kxv, kyv);
      ib[m] = a.ibet[(long long)j * P + t];
    }
  }
}

template <int C>
__device__ __forceinline__ void thomas_fwd_sweep(double2* phat, long long P, int t, int j0, int n, int nz,
                                                 double c3, const double2* rr, const double* ib, double2& up) {
#pragma unroll
  for (int m = 0; m < C; ++m) {
    const int j = j0 + m;
    if (j <= n) {
      const double aj = (j == 1) ? 0.0 : (j <= nz ? c3 : -1.0);
      up = make_double2((rr[m].x - aj * up.x) * ib[m], (rr[m].y - aj * up.y) * ib[m]);
      phat[(j - 1) * P + t] = up;
    }
  }
}

template <int C>
__device__ __forceinline__ void thomas_bwd_load(const ThomasArgs& a, const double2* phat, long long P, int t, int j1,
                                                double2* uu, double* gg) {
#pragma unroll
  for (int m = 0; m < C; ++m) {
    const int j = j1 - m;
    if (j >= 1) {
      uu[m] = phat[(j - 1) * P + t];
      gg[m] = a.gam[(long long)(j + 1) * P + t];
    }
  }
}

template <int C>
__device__ __forceinline__ void thomas_bwd_sweep(double2* phat, long long P, int t, int j1, const double2* uu,
                                                 const double* gg, double2& vn) {
#pragma unroll
  for (int m = 0; m < C; ++m) {
    const int j = j1 - m;
    if (j >= 1) {
      vn = make_double2(uu[m].x - gg[m] * vn.x, uu[m].y - gg[m] * vn.y);
      phat[(j - 1) * P + t] = vn;
    }
  }
}

template <int C>
__global__ void __launch_bounds__(128) k_thomas_seq(ThomasArgs a) {
  const long long P = (long long)a.ny * a.K;
  const long long gcol = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gcol >= P * a.ninst) return;
  const int inst = (int)(gcol / P);
  const int t = (int)(gcol - inst * P);
  const int jy = t / a.K, kx = t - jy * a.K;
  const int nz = a.nz, n = nz + 1;
  const double2* Hx = a.Hx + (long long)inst * nz * P;
  const double2* Hy = a.Hy + (long long)inst * nz * P;
  const double2* Hz = a.Hz + (long long)inst * nz * P;
  const double2* Hb = a.Hb + (long long)inst * 2 * P;
  const double2* Ht = a.Ht + (long long)inst * 2 * P;
  double2* phat = a.phat + (long long)inst * (nz + 1) * P;
  if (jy == a.ny / 2) {
    for (int j = 1; j <= n; ++j) phat[(j - 1) * P + t] = make_double2(0.0, 0.0);
    return;
  }
  if (kx == 0 && jy == 0) {
    double2 p = make_double2(0.0, 0.0);
    phat[t] = p;
    const double2 hb = Hb[t];
    p = make_double2(p.x - a.dz * hb.x, p.y - a.dz * hb.y);
    phat[P + t] = p;
    for (int jz = 2; jz <= nz; ++jz) {
      const double2 hz = Hz[(jz - 1) * P + t];
      p = make_double2(p.x + hz.x * a.dz, p.y + hz.y * a.dz);
      phat[jz * P + t] = p;
    }
    return;
  }
  const double c3 = a.idz2;
  const double kxv = a.kxw[kx], kyv = a.kyw[jy];
  double2 rA[C], rB[C];
  double iA[C], iB[C];
  double2 up = make_double2(0.0, 0.0);
  thomas_fwd_load<C>(a, Hx, Hy, Hz, Hb, Ht, P, t, kxv, kyv, 1, n, rA, iA);
  for (int j0 = 1; j0 <= n; j0 += 2 * C) {
    thomas_fwd_load<C>(a, Hx, Hy, Hz, Hb, Ht, P, t, kxv, kyv, j0 + C, n, rB, iB);
    thomas_fwd_sweep<C>(phat, P, t, j0, n, nz, c3, rA, iA, up);
    thomas_fwd_load<C>(a, Hx, Hy, Hz, Hb, Ht, P, t, kxv, kyv, j0 + 2 * C, n, rA, iA);
    thomas_fwd_sweep<C>(phat, P, t, j0 + C, n, nz, c3, rB, iB, up);
  }
  // u_n stays; levels n-1 .. 1
  double2 vn = up;
  double2 uA[C], uB[C];
  double gA[C], gB[C];
  thomas_bwd_load<C>(a, phat, P, t, n - 1, uA, gA);
  for (int j1 = n - 1; j1 >= 1; j1 -= 2 * C) {
    thomas_bwd_load<C>(a, phat, P, t, j1 - C, uB, gB);
    thomas_bwd_sweep<C>(phat, P, t, j1, uA, gA, vn);
    thomas_bwd_load<C>(a, phat, P, t, j1 - 2 * C, uA, gA);
    thomas_bwd_sweep<C>(phat, P, t, j1 - C, uB, gB, vn);
  }
}

// press_stag_array.f90:284-288 dpdz + main.f90:321-326 + forcing.f90:184-243
// (FUSED: RHSz -= dpdz, project w, boundary conditions) or just dpdz.
template <typename R, bool FUSED>
__global__ void k_wproj(const R* __restrict__ p, R* dpdz, R* RHSz, R* u, R* v, R* w, KP kp) {
  const long long n = (long long)kp.nx * kp.ny * kp.nz * kp.ninst;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const PtIdx x = pt_index(t, kp);
  const int k = x.k;
  const long long P = kp.plane;
  const long long q = x.q;
  // (p(k) - p(k-1)) / dz as a multiply by 1/dz: within an ulp of the
  // division, which is a long instruction sequence in FP64 on this part
  const R d = (p[q] - p[q - P]) * (R)kp.idz;
  if (!FUSED) { dpdz[q] = d; return; }
  RHSz[q] = RHSz[q] - d;
  const int nz = kp.nz;
  const double* c = kp.sc + x.inst * SC_N;
  if (k >= 2 && k <= nz - 1) w[q] = w[q] + (R)c[SC_DT] * (-(R)c[SC_T1] * d);
  if (k == 1) w[q] = (R)0;
  if (k == nz) {
    w[q] = (R)0;
    if (kp.ubc == 0) { u[q] = u[q - P]; v[q] = v[q - P]; }
  }
}

// forcing.f90:149-244 stand-alone projection (two kernels: update, then BCs).
template <typename R>
__global__ void k_project(const R* dpdx, const R* dpdy, const R* dpdz, R* u, R* v, R* w, KP kp) {
  const long long n = (long long)kp.nx * kp.ny * kp.nz * kp.ninst;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const PtIdx x = pt_index(t, kp);
  const int k = x.k;
  const long long q = x.q;
  const double* c = kp.sc + x.inst * SC_N;
  const R dt = (R)c[SC_DT], t1 = (R)c[SC_T1];
  if (k <= kp.nz - 1) {
    u[q] = u[q] + dt * (-t1 * dpdx[q]);
    v[q] = v[q] + dt * (-t1 * dpdy[q]);
  }
  if (k >= 2 && k <= kp.nz - 1) w[q] = w[q] + dt * (-t1 * dpdz[q]);
}

template <typename R>
__global__ void k_project_bc(R* u, R* v, R* w, KP kp) {
  const long long pl = kp.plane;
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gt >= pl * kp.ninst) return;
  const long long t = (gt / pl) * kp.istride + gt % pl;
  const int nz = kp.nz;
  if (kp.ubc == 0) { u[nz * pl + t] = u[(nz - 1) * pl + t]; v[nz * pl + t] = v[(nz - 1) * pl + t]; }
  w[nz * pl + t] = (R)0;
  w[pl + t] = (R)0;
}

// main.f90 step glue for the stand-alone entry points (whole planes, like
// the reference's array syntax).
template <typename R>
__global__ void k_rhs_assemble(R* RHSx, R* RHSy, R* RHSz, const R* divtx, const R* divty, const R* divtz,
                               const R* fxa, const R* fya, const R* fza, KP kp) {
  const long long pl = kp.plane;
  const long long n = pl * kp.nz;
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gt >= n * kp.ninst) return;
  const long long t = gt % n;
  const long long q = (gt / n) * kp.istride + pl + t;   // levels 1..nz
  const int k = 1 + (int)(t / pl);
  if (k <= kp.nz - 1) {
    R x = -RHSx[q] - divtx[q], y = -RHSy[q] - divty[q], z = -RHSz[q] - divtz[q];
    if (kp.use_mpf) { x = x + (R)kp.mpfx; y = y + (R)kp.mpfy; }
    if (kp.turbines) { x = x + fxa[q]; y = y + fya[q]; z = z + fza[q]; }
    RHSx[q] = x; RHSy[q] = y; RHSz[q] = z;
  } else {
    RHSz[q] = -RHSz[q] - divtz[q];
  }
}

template <typename R>
__global__ void k_ab2(R* u, R* v, R* w, const R* RHSx, const R* RHSy, const R* RHSz,
                      const R* fx, const R* fy, const R* fz, KP kp) {
  const long long pl = kp.plane;
  const long long n = pl * kp.nz;
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gt >= n * kp.ninst) return;
  const long long t = gt % n;
  const long long q = (gt / n) * kp.istride + pl + t;
  const int k = 1 + (int)(t / pl);
  const double* c = kp.sc + (gt / n) * SC_N;
  const R dt = (R)c[SC_DT], t1 = (R)c[SC_T1], t2 = (R)c[SC_T2];
  if (k <= kp.nz - 1) {
    u[q] = u[q] + dt * (t1 * RHSx[q] + t2 * fx[q]);
    v[q] = v[q] + dt * (t1 * RHSy[q] + t2 * fy[q]);
  }
  w[q] = w[q] + dt * (t1 * RHSz[q] + t2 * fz[q]);
}

template <typename R>
__global__ void k_rhs_sub_dp(R* RHSx, R* RHSy, R* RHSz, const R* dpdx, const R* dpdy, const R* dpdz, KP kp) {
  const long long pl = kp.plane;
  const long long n = pl * kp.nz;
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gt >= n * kp.ninst) return;
  const long long t = gt % n;
  const long long q = (gt / n) * kp.istride + pl + t;
  const int k = 1 + (int)(t / pl);
  if (k <= kp.nz - 1) { RHSx[q] = RHSx[q] - dpdx[q]; RHSy[q] = RHSy[q] - dpdy[q]; }
  RHSz[q] = RHSz[q] - dpdz[q];
}

template <typename R>
__global__ void k_fill(R* p, long long n, R val) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) p[t] = val;
}

template <typename A, typename B>
__global__ void k_convert(const A* __restrict__ src, B* __restrict__ dst, long long n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) dst[t] = (B)src[t];
}

// ---------------------------------------------------------------------------
// Seeded IC: counter-based splitmix64 hash of (seed, field, i, j, k).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double hash_pm1(uint64_t seed, uint64_t fld, uint64_t i, uint64_t j, uint64_t k) {
  uint64_t key = seed * 8ull + fld;
  key = key * 65536ull + k;
  key = key * 65536ull + j;
  key = key * 65536ull + i;
  uint64_t x = key + 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x = x ^ (x >> 31);
  const double u01 = (double)(x >> 11) * (1.0 / 9007199254740992.0);
  return 2.0 * u01 - 1.0;
}

// Writes instance `inst` (all levels) with its own seed and roughness.
template <typename R>
__global__ void k_ic(R* u, R* v, R* w, KP kp, uint64_t seed, int inst) {
  const long long pl = kp.plane;
  const long long n = pl * (kp.nz + 1);
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t0 >= n) return;
  const long long t = inst * kp.istride + t0;
  const int k = (int)(t0 / pl);
  const long long rr = t0 - (long long)k * pl;
  const int j = (int)(rr / kp.ld), i = (int)(rr - (long long)j * kp.ld);
  const int nz = kp.nz;
  double uu = 0, vv = 0, ww = 0;
  const int kk = (k == nz) ? nz - 1 : k;   // u(nz) = u(nz-1), v(nz) = v(nz-1)
  if (i < kp.nx && kk >= 1 && kk <= nz - 1) {
    const double zk = (kk - 0.5) * kp.dz;
    const double ubar = (1.0 / 0.4) * log(zk / kp.zo_i[inst]);
    uu = ubar * (1.0 + 0.1 * hash_pm1(seed, 0, i, j, kk));
    vv = 0.1 * hash_pm1(seed, 1, i, j, kk);
    if (k >= 2 && k <= nz - 1) ww = 0.1 * hash_pm1(seed, 2, i, j, k);
  }
  u[t] = (R)uu; v[t] = (R)vv; w[t] = (R)ww;
}

// ---------------------------------------------------------------------------
// Diagnostics: per-block partial sums / maxima, then one reduction block.
// slots: 0 sum|div|, 1 sum ke, 2 max|u|, 3 max|v|, 4 max|w|, 5 sum txz(1), 6 sum tyz(1)
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_diag(const R* dudx, const R* dvdy, const R* dwdz, const R* u, const R* v,
                                              const R* w, const R* txz, const R* tyz, KP kp, double* partial, int inst) {
  __shared__ double sh[7][256];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  const long long n = (long long)kp.nx * kp.ny * (kp.nz - 1);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = t % kp.nx;
    const long long r = t / kp.nx;
    const int j = r % kp.ny;
    const int k = 1 + (int)(r / kp.ny);
    const long long q = inst * kp.istride + k * kp.plane + (long long)j * kp.ld + i;
    acc[0] += fabs((double)dudx[q] + (double)dvdy[q] + (double)dwdz[q]);
    const double tw = 0.5 * ((double)w[q] + (double)w[q + kp.plane]);
    acc[1] += (double)u[q] * u[q] + (double)v[q] * v[q] + tw * tw;
    acc[2] = fmax(acc[2], fabs((double)u[q]));
    acc[3] = fmax(acc[3], fabs((double)v[q]));
    acc[4] = fmax(acc[4], fabs((double)w[q]));
    if (k == 1) { acc[5] += (double)txz[q]; acc[6] += (double)tyz[q]; }
  }
  for (int s = 0; s < 7; ++s) sh[s][threadIdx.x] = acc[s];
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      for (int s = 0; s < 7; ++s) {
        if (s >= 2 && s <= 4) sh[s][threadIdx.x] = fmax(sh[s][threadIdx.x], sh[s][threadIdx.x + st]);
        else sh[s][threadIdx.x] += sh[s][threadIdx.x + st];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < 7) partial[blockIdx.x * 7 + threadIdx.x] = sh[threadIdx.x][0];
}

static __global__ void k_diag_final(const double* partial, int nblocks, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int b = 0; b < nblocks; ++b)
    for (int s = 0; s < 7; ++s) {
      const double x = partial[b * 7 + s];
      if (s >= 2 && s <= 4) acc[s] = fmax(acc[s], x); else acc[s] += x;
    }
  for (int s = 0; s < 7; ++s) out[s] = acc[s];
}

// The same reduction into one row of an instance's diagnostics log, with the
// host-side formulas of lesgo_gpu_diag applied on the device (rmsdiv.f90,
// io.f90:99-141, cfl_util.f90:35-64, functions.f90:882-905): jt_total,
// total_time, rmsdiv, ke, cfl, tau_wall_bot.
static __global__ void k_diag_log_final(const double* partial, int nblocks, const double* sc_row, double* row,
                                 double jt_total, double npts, double nxy, double dx, double dy, double dz) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int b = 0; b < nblocks; ++b)
    for (int s = 0; s < 7; ++s) {
      const double x = partial[b * 7 + s];
      if (s >= 2 && s <= 4) acc[s] = fmax(acc[s], x); else acc[s] += x;
    }
  row[0] = jt_total;
  row[1] = sc_row[SC_TIME];
  row[2] = acc[0] / npts;
  row[3] = acc[1] * 0.5 / npts;
  row[4] = sc_row[SC_DT] * fmax(fmax(acc[2] / dx, acc[3] / dy), acc[4] / dz);
  row[5] = sqrt((acc[5] / nxy) * (acc[5] / nxy) + (acc[6] / nxy) * (acc[6] / nxy));
}

// ---------------------------------------------------------------------------
// Actuator disks (turbines.f90:465-638).  Node lists are static; the
// reduction is one block per turbine, the scatter writes each node once with
// the value of the last turbine that claims it (the reference assigns in
// turbine order, turbines.f90:601-616).
// ---------------------------------------------------------------------------
struct TurbDev {
  int nturb;
  const int* node_off;      // [nturb+1] into node arrays
  const long long* node_q;  // flat index (level, jy, i) of each node
  const double* node_ind;   // indicator value
  const int* win_turb;      // scatter list: turbine owning node (last writer)
  const long long* win_q;
  const double* win_ind;
  int nwin;
  const double* nhat;       // [nturb*3]
  const double* ctp;        // Ct'
  const double* corr;       // 1 + 0.25 (1-M) Ct' or 1
  double* u_d;              // state
  double* u_d_T;
  double* f_n;
  double* disk;             // scratch per turbine
  const int* tinst;         // instance of each turbine
  const double* sc;         // step constants (disk-velocity filter weight)
  double dvol;
  const double* dia;
};

template <typename R>
__global__ void __launch_bounds__(256) k_turb_disk(TurbDev td, const R* u, const R* v, const R* w, long long plane, int nz,
                                                   long long istride) {
  __shared__ double sh[256];
  const int s = blockIdx.x;
  double acc = 0.0;
  const double n0 = td.nhat[3 * s], n1 = td.nhat[3 * s + 1], n2 = td.nhat[3 * s + 2];
  for (int l = td.node_off[s] + threadIdx.x; l < td.node_off[s + 1]; l += blockDim.x) {
    const long long q = td.node_q[l];
    // interp_to_uv_grid (functions.f90:87-105): level nz repeats level nz-1
    const long long qq = ((q % istride) / plane >= nz) ? q - plane : q;
    const double wuv = 0.5 * ((double)w[qq + plane] + (double)w[qq]);
    acc += td.dvol * td.node_ind[l] * (n0 * (double)u[q] + n1 * (double)v[q] + n2 * wuv);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double ud = sh[0];
    ud = ud / td.corr[s];
    const double eps = td.sc[td.tinst[s] * SC_N + SC_EPS];
    const double udT = (1.0 - eps) * td.u_d_T[s] + eps * ud;
    td.u_d[s] = ud;
    td.u_d_T[s] = udT;
    // turbines.f90:583: -0.5*Ct'*abs(u_d_T)*u_d_T*0.25*pi*dia**2
    td.f_n[s] = -0.5 * td.ctp[s] * fabs(udT) * udT * 0.25 * 3.14159265358979323846 * (td.dia[s] * td.dia[s]);
  }
}

template <typename R>
__global__ void k_turb_scatter(TurbDev td, R* fxa, R* fya, R* fza) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= td.nwin) return;
  const int s = td.win_turb[l];
  const double fn = td.f_n[s], ind = td.win_ind[l];
  const long long q = td.win_q[l];
  fxa[q] = (R)(fn * td.nhat[3 * s] * ind);
  fya[q] = (R)(fn * td.nhat[3 * s + 1] * ind);
  fza[q] = (R)(fn * td.nhat[3 * s + 2] * ind);
}

// ---------------------------------------------------------------------------
// Time-varying turbine controls (turbines.f90:500-515): yaw theta1, tilt
// theta2 and Ct' interpolated at total_time_dim; with a yaw or tilt schedule
// the nodes of every disk are re-selected from its search box each step
// (turbines_nodes, turbines.f90:337-462).
// ---------------------------------------------------------------------------
struct TurbDyn {
  int nturb, dyn_nodes, adm;
  const int* s_nt;          // [3][nturb] schedule rows (0: none)
  const int* s_off;         // [3][nturb] offset into s_t / s_v
  const double* s_t;        // dimensional times
  const double* s_v;        // values
  const double* M;          // indicator M of each turbine (ADM correction)
  double* nhat;             // [nturb*3]     (read by the disk and scatter kernels)
  double* theta;            // [2][nturb]    current yaw, tilt (degrees)
  double* ctp;              // [nturb]       current Ct'
  double* corr;             // [nturb]       1 + 0.25 (1 - M) Ct', or 1
  const int* tinst;
  const double* sc;
  // box nodes
  const int* dyn_list;      // turbines whose nodes are their search box
  int ndyn;
  const int* node_off;      // [nturb+1]
  const double* box_r;      // [node][3] offset (rx, ry, rz) from the disk centre
  double* node_ind;         // normalised indicator of each box node (0: not selected)
  const int* node_turb;     // turbine of each box node
  const int* tab_off;       // radial table of each turbine (tab_n entries)
  const double* tab_r;
  const double* tab_R2;
  int tab_n;
  const double* ipar;       // [nturb][4] ell, thk / ell, sqrt(6) / (delta1 / ell), filt_max
  double cutoff, dx, dy, dz;
  const long long* win_q;   // window points (union of the boxes)
  const int* win_coff;      // [nwin+1] candidates of each point, in turbine order
  const int* win_cand;      // box-node indices
  int nwin;
};

// binary_search (functions.f90:811-860) and linear_interp_sa_nocheck
// (:712-735): v(1) below x(1), v(N) above x(N), else
// u1 + (xq - x(i)) * (u2 - u1) / (x(i+1) - x(i)).
__device__ __forceinline__ double sched_interp(const double* x, const double* v, int N, double xq) {
  int low;
  if (xq < x[0]) {
    low = 0;
  } else if (xq > x[N - 1]) {
    low = N;
  } else {
    low = 1;
    int high = N;   // one-based, as the reference
    while (high - low > 1) {
      const int mid = (low + high) / 2;
      if (x[mid - 1] > xq) high = mid;
      else if (x[mid - 1] < xq) low = mid;
      else { low = mid; break; }
    }
  }
  if (low == 0) return v[0];
  if (low == N) return v[N - 1];
  return v[low - 1] + (xq - x[low - 1]) * (v[low] - v[low - 1]) / (x[low] - x[low - 1]);
}

// One thread per turbine.
static __global__ void k_turb_controls(TurbDyn a) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.nturb) return;
  const int n = a.nturb;
  const double t = a.sc[a.tinst[s] * SC_N + SC_TDIM];
  bool turned = false;
  for (int w = 0; w < 2; ++w) {
    const int nt = a.s_nt[w * n + s];
    if (nt > 0) {
      a.theta[w * n + s] = sched_interp(a.s_t + a.s_off[w * n + s], a.s_v + a.s_off[w * n + s], nt, t);
      turned = true;
    }
  }
  if (turned) {   // turbines.f90:343-345
    const double pi = 3.14159265358979323846;
    const double t1 = pi * a.theta[s] / 180., t2 = pi * a.theta[n + s] / 180.;
    a.nhat[3 * s] = -cos(t1) * cos(t2);
    a.nhat[3 * s + 1] = -sin(t1) * cos(t2);
    a.nhat[3 * s + 2] = sin(t2);
  }
  const int nc = a.s_nt[2 * n + s];
  if (nc > 0) {
    const double c = sched_interp(a.s_t + a.s_off[2 * n + s], a.s_v + a.s_off[2 * n + s], nc, t);
    a.ctp[s] = c;
    a.corr[s] = a.adm ? (1 + 0.25 * (1 - a.M[s]) * c) : 1.0;   // turbines.f90:579-582
  }
}

// The indicator value (turbine_indicator.f90:43-64): the axial window
// R1 = (erf(s (x/ell + thk/2)) - erf(s (x/ell - thk/2))) / (2 thk) times the
// radial table interpolated at r/ell (clamped outside it), over ell^3.
__device__ __forceinline__ double turb_ind_val(const double* r, const double* R2, int N, double ell, double thk,
                                               double s6d1, double rd, double x) {
  const double rr = rd / ell, xx = x / ell;
  int lo = 0, hi = N;   // first index with r[i] > rr
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (r[mid] <= rr) lo = mid + 1;
    else hi = mid;
  }
  double R;
  if (lo == 0) R = R2[0];
  else if (lo >= N) R = R2[N - 1];
  else R = R2[lo - 1] + (rr - r[lo - 1]) * (R2[lo] - R2[lo - 1]) / (r[lo] - r[lo - 1]);
  const double R1 = 0.5 / thk * (erf(s6d1 * (xx + 0.5 * thk)) - erf(s6d1 * (xx - 0.5 * thk)));
  return R1 * R / (ell * ell * ell);
}

// One block per box-node turbine: select its nodes (filt > filter_cutoff * filt_max)
// and normalise them to integrate to one (turbines.f90:388-437).  The
// geometry is rounded operation by operation as the reference evaluates it
// (no fused multiply-adds: r*r - r_norm*r_norm is exactly zero on the axis).
static __global__ void __launch_bounds__(256) k_turb_nodes(TurbDyn a) {
  __shared__ double sh[256];
  const int s = a.dyn_list[blockIdx.x];
  const double n0 = a.nhat[3 * s], n1 = a.nhat[3 * s + 1], n2 = a.nhat[3 * s + 2];
  const double* tr = a.tab_r + a.tab_off[s];
  const double* tR = a.tab_R2 + a.tab_off[s];
  const double ell = a.ipar[4 * s], thk = a.ipar[4 * s + 1], s6d1 = a.ipar[4 * s + 2];
  const double thr = a.cutoff * a.ipar[4 * s + 3];
  double acc = 0.0;
  for (int l = a.node_off[s] + threadIdx.x; l < a.node_off[s + 1]; l += blockDim.x) {
    const double rx = a.box_r[3 * l], ry = a.box_r[3 * l + 1], rz = a.box_r[3 * l + 2];
    const double r = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)));
    const double rn = fabs(__dadd_rn(__dadd_rn(__dmul_rn(rx, n0), __dmul_rn(ry, n1)), __dmul_rn(rz, n2)));
    const double rd = sqrt(__dsub_rn(__dmul_rn(r, r), __dmul_rn(rn, rn)));
    const double filt = turb_ind_val(tr, tR, a.tab_n, ell, thk, s6d1, rd, rn);
    double v = 0.0;
    if (filt > thr) {
      v = filt;
      acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(__dmul_rn(filt, a.dx), a.dy), a.dz));
    }
    a.node_ind[l] = v;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  const double sumA = sh[0];
  for (int l = a.node_off[s] + threadIdx.x; l < a.node_off[s + 1]; l += blockDim.x) {
    const double v = a.node_ind[l];
    if (v != 0.0) a.node_ind[l] = v / sumA;
  }
}

// Window point p takes the force of the last turbine (in order) that
// selected it this step, or zero.
template <typename R>
__global__ void k_turb_scatter_dyn(TurbDyn a, const double* f_n, R* fxa, R* fya, R* fza) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.nwin) return;
  int owner = -1;
  double ind = 0.0;
  for (int c = a.win_coff[p]; c < a.win_coff[p + 1]; ++c) {
    const int l = a.win_cand[c];
    const double v = a.node_ind[l];
    if (v != 0.0) { owner = a.node_turb[l]; ind = v; }
  }
  const long long q = a.win_q[p];
  if (owner < 0) {
    fxa[q] = (R)0; fya[q] = (R)0; fza[q] = (R)0;
    return;
  }
  const double fn = f_n[owner];
  fxa[q] = (R)(fn * a.nhat[3 * owner] * ind);
  fya[q] = (R)(fn * a.nhat[3 * owner + 1] * ind);
  fza[q] = (R)(fn * a.nhat[3 * owner + 2] * ind);
}

// fza onto the w grid (functions.f90:131-185): fzw(k) = (fza(k-1)+fza(k))/2,
// k >= 2, fzw(1) = 0, over the turbine footprint columns.
template <typename R>
__global__ void k_turb_fzw(const R* fza, R* fzw, const long long* cols, int ncols, KP kp) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)ncols * kp.nz) return;
  const int c = t % ncols;
  const int k = 1 + (int)(t / ncols);
  const long long q = k * kp.plane + cols[c];
  fzw[q] = (k == 1) ? (R)0 : (R)0.5 * (fza[q - kp.plane] + fza[q]);
}

}  // namespace lesgo

namespace lesgo {

// tridag_array.f90:166-246 on caller arrays in the reference layout:
// a, b, c real (lh, ny, n); r, u interleaved complex (2*lh, ny, n).  One
// thread per (kx, ky) column: u(1) = r(1)/b(1) for every kx < nx/2, then
// the Thomas sweeps skip the ky Nyquist row and the kx = ky = 0 column.
// `gam` is scratch of lh*ny*n doubles; a zero pivot sets *err.
static __global__ void __launch_bounds__(128) k_tridag(const double* __restrict__ a, const double* __restrict__ b,
                                                const double* __restrict__ c, const double2* __restrict__ r,
                                                double2* __restrict__ u, double* __restrict__ gam,
                                                int lh, int ny, int n, int* err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ncol = (lh - 1) * ny;
  if (t >= ncol) return;
  const int jy = t / (lh - 1), jx = t - jy * (lh - 1);
  const long long col = (long long)jy * lh + jx;
  const long long L = (long long)lh * ny;     // stride between levels
  double bet = b[col];
  if (bet == 0.0) { atomicExch(err, 1); return; }
  double2 up = make_double2(r[col].x / bet, r[col].y / bet);
  u[col] = up;
  if (jy == ny / 2 || (jx == 0 && jy == 0)) return;
  for (int j = 1; j < n; ++j) {
    const long long q = j * L + col;
    const double g = c[q - L] / bet;
    gam[q] = g;
    bet = b[q] - a[q] * g;
    if (bet == 0.0) { atomicExch(err, 1); return; }
    const double2 rr = r[q];
    up = make_double2((rr.x - a[q] * up.x) / bet, (rr.y - a[q] * up.y) / bet);
    u[q] = up;
  }
  double2 un = up;
  for (int j = n - 2; j >= 0; --j) {
    const long long q = j * L + col;
    const double g = gam[q + L];
    double2 uj = u[q];
    uj = make_double2(uj.x - g * un.x, uj.y - g * un.y);
    u[q] = uj;
    un = uj;
  }
}

}  // namespace lesgo

namespace lesgo {

// ---------------------------------------------------------------------------
// Time-averaging statistics (time_average.f90:176-319): 26 FP64 accumulators
// per instance, each sample weighted by the time since the previous sample.
// ---------------------------------------------------------------------------
enum : int {
  TA_U = 0, TA_V, TA_W, TA_U_W, TA_V_W, TA_W_UV, TA_U2, TA_V2, TA_W2, TA_UV, TA_UW, TA_VW,
  TA_TXX, TA_TYY, TA_TZZ, TA_TXY, TA_TXZ, TA_TYZ, TA_P, TA_FX, TA_FY, TA_FZ, TA_CS, TA_VORTX, TA_VORTY,
  TA_VORTZ, TA_N
};

template <typename R>
struct TavgArgs {
  const R *u, *v, *w, *p, *txx, *tyy, *tzz, *txy, *txz, *tyz, *fxa, *fya, *fza, *cs;
  const R *dudy, *dudz, *dvdx, *dvdz, *dwdx, *dwdy;
  double* acc;            // [TA_N][inst][nz+1][ny][ld]
  long long acc_stride;   // elements between quantities
  const double* wgt;      // per-instance sample weight (0: no sample)
  KP kp;
};

template <typename R>
__global__ void k_tavg(TavgArgs<R> a) {
  const KP& kp = a.kp;
  const long long n = (long long)kp.nx * kp.ny * kp.nz * kp.ninst;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const PtIdx x = pt_index(t, kp);
  const double wt = a.wgt[x.inst];
  if (wt == 0.0) return;
  const int k = x.k, nz = kp.nz;
  const long long q = x.q, P = kp.plane;
  const double u = a.u[q], v = a.v[q], w = a.w[q];
  // interp_to_uv_grid (functions.f90:51-105): level nz repeats nz-1
  const long long qu = (k == nz) ? q - P : q;
  const double w_uv = 0.5 * ((double)a.w[qu + P] + (double)a.w[qu]);
  // interp_to_w_grid (functions.f90:108-185); zero at a wall (time_average.f90:227-232)
  double u_w = 0.0, v_w = 0.0, vortz = 0.0;
  if (k >= 2) {
    u_w = 0.5 * ((double)a.u[q - P] + (double)a.u[q]);
    v_w = 0.5 * ((double)a.v[q - P] + (double)a.v[q]);
    vortz = 0.5 * (((double)a.dvdx[q - P] - (double)a.dudy[q - P]) + ((double)a.dvdx[q] - (double)a.dudy[q]));
  }
  if (k == nz && kp.ubc > 0) { u_w = 0.0; v_w = 0.0; }
  if (k == 1 && kp.lbc > 0) { u_w = 0.0; v_w = 0.0; }
  const double pres = (double)a.p[q] - 0.5 * (u * u + w_uv * w_uv + v * v);
  double fz_uv = 0.0;
  if (kp.turbines) fz_uv = 0.5 * ((double)a.fza[qu + P] + (double)a.fza[qu]);
  const double vals[TA_N] = {
      u, v, w, u_w, v_w, w_uv, u * u, v * v, w * w, u * v, u_w * w, v_w * w,
      (double)a.txx[q], (double)a.tyy[q], (double)a.tzz[q], (double)a.txy[q], (double)a.txz[q], (double)a.tyz[q],
      pres, kp.turbines ? (double)a.fxa[q] : 0.0, kp.turbines ? (double)a.fya[q] : 0.0, fz_uv, (double)a.cs[q],
      (double)a.dwdy[q] - (double)a.dvdz[q], (double)a.dudz[q] - (double)a.dwdx[q], vortz};
#pragma unroll
  for (int f = 0; f < TA_N; ++f) a.acc[f * a.acc_stride + q] += vals[f] * wt;
}

// The time average of quantity `which` (accumulator / total time), or a
// Reynolds stress (time_average.f90:616-629): 26 u'u', 27 v'v', 28 w'w',
// 29 u'v', 30 u'w' (w grid), 31 v'w' (w grid).  One instance, levels 0..nz.
static __global__ void k_tavg_get(const double* acc, long long acc_stride, long long ib, int which, double inv_t,
                           double* out, long long n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  auto A = [&](int f) { return acc[f * acc_stride + ib + t] * inv_t; };
  double r;
  switch (which) {
    case TA_N + 0: r = A(TA_U2) - A(TA_U) * A(TA_U); break;
    case TA_N + 1: r = A(TA_V2) - A(TA_V) * A(TA_V); break;
    case TA_N + 2: r = A(TA_W2) - A(TA_W) * A(TA_W); break;
    case TA_N + 3: r = A(TA_UV) - A(TA_U) * A(TA_V); break;
    case TA_N + 4: r = A(TA_UW) - A(TA_U_W) * A(TA_W); break;
    case TA_N + 5: r = A(TA_VW) - A(TA_V_W) * A(TA_W); break;
    default: r = A(which);
  }
  out[t] = r;
}

// Plane mean over x < nx of a (ld, ny, levels) double array: one block per level.
static __global__ void k_plane_mean(const double* f, int nx, int ny, int ld, double* out) {
  __shared__ double sh[256];
  const long long base = (long long)blockIdx.x * ny * ld;
  double s = 0.0;
  for (int t = threadIdx.x; t < nx * ny; t += blockDim.x) {
    const int j = t / nx, i = t - j * nx;
    s += f[base + (long long)j * ld + i];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0] / ((double)nx * ny);
}

}  // namespace lesgo

namespace lesgo {

// ---------------------------------------------------------------------------
// Time step on the device.  k_cfl_max: per instance the maxima of |u|, |v|,
// |w| over x < nx and levels 1..nz-1 (cfl_util.f90:70-111), folded into
// mx[inst][3] as the bit patterns of non-negative doubles (ordered like the
// values).  Grid (blocks, instances).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_cfl_max(const R* u, const R* v, const R* w, KP kp,
                                                 unsigned long long* mx) {
  __shared__ double sh[3][256];
  const int inst = blockIdx.y;
  const long long m = (long long)kp.nx * kp.ny * (kp.nz - 1);
  const long long base = inst * kp.istride + kp.plane;
  double au = 0.0, av = 0.0, aw = 0.0;
  for (long long t = blockIdx.x * 256LL + threadIdx.x; t < m; t += (long long)gridDim.x * 256) {
    const int ti = (int)t;
    const int r = kp.fnx.div(ti);
    const int i = ti - r * kp.nx;
    const int k = kp.fny.div(r);     // 0 .. nz-2 (level k + 1)
    const int j = r - k * kp.ny;
    const long long q = base + k * kp.plane + (long long)j * kp.ld + i;
    au = fmax(au, fabs((double)u[q]));
    av = fmax(av, fabs((double)v[q]));
    aw = fmax(aw, fabs((double)w[q]));
  }
  sh[0][threadIdx.x] = au; sh[1][threadIdx.x] = av; sh[2][threadIdx.x] = aw;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] = fmax(sh[c][threadIdx.x], sh[c][threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x < 3)
    atomicMax(&mx[inst * 3 + threadIdx.x], (unsigned long long)__double_as_longlong(sh[threadIdx.x][0]));
}

// Start of a step, one thread per instance: with cfl_mode, dt from the maxima
// (cfl_util.f90:70-111) and the AB2 weights for a varying step (main.f90:
// 135-144), the pressure-RHS scale, the disk filter weight, lagran_dt
// (sgs_stag_util.f90:72-83, reset lagrange_Sdep.f90:430); always total_time
// and the pending time-average weight (io.f90:559-562).
struct StepBeginArgs {
  double* sc;
  const int* iflags;
  unsigned long long* mx;
  int ninst, cfl_mode;
  double cfl, dx, dy, dz, c1, z_i, u_star, T_avg_dim;
};

static __global__ void k_step_begin(StepBeginArgs a) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= a.ninst) return;
  double* c = a.sc + inst * SC_N;
  const int f = a.iflags[inst];
  if (a.cfl_mode) {
    const double iu = __longlong_as_double((long long)a.mx[inst * 3 + 0]) / a.dx;
    const double iv = __longlong_as_double((long long)a.mx[inst * 3 + 1]) / a.dy;
    const double iw = __longlong_as_double((long long)a.mx[inst * 3 + 2]) / a.dz;
    a.mx[inst * 3 + 0] = 0ULL; a.mx[inst * 3 + 1] = 0ULL; a.mx[inst * 3 + 2] = 0ULL;
    double m = iu;
    if (iv > m) m = iv;
    if (iw > m) m = iw;
    const double dt_f = c[SC_DT];
    const double dt = a.cfl / m;
    c[SC_DTF] = dt_f;
    c[SC_DT] = dt;
    c[SC_T1] = 1.0 + 0.5 * dt / dt_f;
    c[SC_T2] = 1.0 - c[SC_T1];
    c[SC_PS] = a.c1 / c[SC_T1] / dt;
    if (a.T_avg_dim > 0) {
      const double dt_dim = dt * a.z_i / a.u_star;
      c[SC_EPS] = (dt_dim / a.T_avg_dim) / (1. + dt_dim / a.T_avg_dim);
    }
    if (f & IF_LAGRESET) c[SC_LDT] = 0.0;
    if (f & IF_LAGACC) c[SC_LDT] = c[SC_LDT] + dt;
  }
  c[SC_TIME] = c[SC_TIME] + c[SC_DT];
  c[SC_TDIM] = c[SC_TDIM] + c[SC_DT] * a.z_i / a.u_star;   // total_time_dim + dt_dim
  if (f & IF_TAACC) c[SC_TAW] = c[SC_TAW] + c[SC_DT];
}

// Time-averaging bookkeeping after a step, one thread per instance: act 1
// starts fresh sums (tavg%init), 2 starts from sums read from tavg.out, 3
// takes a sample weighted by the pending time (tavg%compute); w receives the
// sample weight (0: none).
static __global__ void k_tavg_prep(double* sc, const int* act, double* w, int ninst) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= ninst) return;
  double* c = sc + inst * SC_N;
  const int a = act[inst];
  double wt = 0.0;
  if (a == 1) { c[SC_TAW] = 0.0; c[SC_TAT] = 0.0; }
  else if (a == 2) { c[SC_TAW] = 0.0; }
  else if (a == 3) { wt = c[SC_TAW]; c[SC_TAT] = c[SC_TAT] + wt; c[SC_TAW] = 0.0; }
  w[inst] = wt;
}

}  // namespace lesgo
