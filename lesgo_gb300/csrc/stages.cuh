// Stage functors (row loaders, spectral operators, row epilogues) and the
// non-spectral kernels of the LES step.  Each functor cites the reference
// lines whose arithmetic it restates.
#pragma once
#include "fft_core.cuh"

namespace lesgo {

// Run-time constants shared by the kernels (param.f90, input_util.f90:196-235).
struct KP {
  int nx, ny, nz, ld, lh, nx2, ny2, ld_big, K;  // K = nx/2 kept x modes
  long long plane, plane_big;                   // elements per (ld,ny) / (ld_big,ny2) plane
  double dx, dy, dz, L_x, L_y, L_z;
  double vonk, zo, nu, delta;
  double mpfx, mpfy, nu_nd, ubot, utop;
  int lbc, ubc, use_mpf, turbines;
  int ninst;                 // instances (slots) stacked in every field
  long long istride;         // elements between instances of a field: (nz+1)*plane
  long long istride_big;     // same on the 3/2 grid
  const double* zo_i;        // per-instance roughness length
  const int* iflags;         // per-instance step flags (IF_*)
  const double* sc;          // per-instance step constants [inst][SC_N] (SC_*)
  FastDiv fnx, fny, fnz;     // by nx, ny, nz (point-index decomposition)
  double idx, idy, idz, iLx, iLy;   // 1/dx, 1/dy, 1/dz, 1/L_x, 1/L_y
};

// Per-instance step constants, resident on the device so that a time step
// chosen on the device (cfl_util.f90:70-111) reaches every kernel of a
// replayed step: dt, the AB2 weights tadv1/tadv2 (main.f90:135-144),
// lagran_dt (sgs_stag_util.f90:72-83), the pressure-RHS scale
// 1/(nx ny tadv1 dt) (press_stag_array.f90:52), the disk-velocity filter
// weight of the turbines (turbines.f90:520-530), total_time, the
// time-averaging weight pending and its sum (time_average.f90), and
// total_time_dim (the sum of dt z_i / u_star, main.f90:139-150).
enum : int {
  SC_DT = 0, SC_T1, SC_T2, SC_LDT, SC_PS, SC_EPS, SC_TIME, SC_TAW, SC_TAT, SC_DTF, SC_TDIM, SC_N = 16
};

// Per-instance step flags: Euler first step (main.f90:273-280), Cs_opt2 =
// 0.03 (sgs_stag_util.f90:187-189), dynamic update due this step
// (:192-217), F_LM/F_MM and F_QN/F_NN initialisation (lagrange_Sdep.f90:266-276, 326-336).
enum : int { IF_EULER = 1, IF_CSFILL = 2, IF_LAG = 4, IF_INITLM = 8, IF_INITQN = 16 };
// Flags read only by the step-begin kernel: the step counts toward the
// pending time-average weight (io.f90:559-562); lagran_dt accumulates dt
// (sgs_stag_util.f90:74-79); lagran_dt restarts from zero after the previous
// step's dynamic update (lagrange_Sdep.f90:430).
enum : int { IF_TAACC = 32, IF_LAGACC = 64, IF_LAGRESET = 128 };
// Flags that change which kernels a step launches (such steps are not replayed).
constexpr int IF_SPECIAL = IF_EULER | IF_CSFILL | IF_INITLM | IF_INITQN;

// Launch level index li -> (instance, level within the instance).
struct InstMap {
  int nli = 1;          // levels per instance in this launch
  long long istr = 0;   // field elements between instances
  FastDiv fd;
  InstMap() = default;
  __host__ InstMap(int n, long long s) : nli(n), istr(s), fd((unsigned)n) {}
  __device__ __forceinline__ int inst(int li) const { return fd.div(li); }
};

// ---------------------------------------------------------------------------
// Xf row loaders
// ---------------------------------------------------------------------------
// NF fields scaled by one constant, at levels lev0 + li*levstride.
// With `isc` set, the scale is the instance's step constant isc[inst][isc_idx].
template <typename R, int NF>
struct SrcFields {
  using C = cplx<R>;   // the fields' complex pair type
  const R* p[NF];
  R scale;
  int lev0, levstride, ld;
  long long plane;
  InstMap im;
  const double* isc = nullptr;
  int isc_idx = 0;
  __device__ __forceinline__ void load2(int n, int jy, int li, cplx<R>* v) const {
    const int inst = im.inst(li), lv = li - inst * im.nli;
    const long long off = inst * im.istr + (long long)(lev0 + lv * levstride) * plane + (long long)jy * ld + 2 * n;
    const R scale = isc ? (R)isc[inst * SC_N + isc_idx] : this->scale;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      cplx<R> a = *reinterpret_cast<const cplx<R>*>(p[f] + off);
      v[f] = mkc(a.x * scale, a.y * scale);
    }
  }
};

// convec.f90:71-168: u, v, w and the vorticity components (with the wall
// and lid special cases), all scaled by 1/(nx*ny), levels 1..nz.  With
// VORT_ONLY the three vorticity components alone (the fused step takes the
// velocity spectra from filt_da's forward pass).
template <typename R, bool VORT_ONLY = false>
struct SrcVort {
  using C = cplx<R>;   // the fields' complex pair type
  const R *u, *v, *w, *dudy, *dudz, *dvdx, *dvdz, *dwdx, *dwdy;
  R c;
  int ld, nz, lbc, ubc;
  long long plane;
  InstMap im;
  __device__ __forceinline__ void load2(int n, int jy, int li, cplx<R>* out) const {
    const int inst = im.inst(li);
    const int k = li - inst * im.nli + 1;
    const long long o = inst * im.istr + (long long)k * plane + (long long)jy * ld + 2 * n;
    const long long om = o - plane, op = o + plane;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const long long q = o + e;
      R vals[6];
      if (!VORT_ONLY) {
        vals[0] = c * u[q];
        vals[1] = c * v[q];
        vals[2] = c * w[q];
      }
      R r1, r2;
      if (k == 1) {
        if (lbc == 0) {
          r1 = (R)0; r2 = (R)0;
        } else {
          r1 = c * ((R)0.5 * (dwdy[q] + dwdy[op + e]) - dvdz[q]);
          r2 = c * (dudz[q] - (R)0.5 * (dwdx[q] + dwdx[op + e]));
        }
      } else if (k == nz && ubc > 0) {
        r1 = c * ((R)0.5 * (dwdy[om + e] + dwdy[q]) - dvdz[om + e]);
        r2 = c * (dudz[om + e] - (R)0.5 * (dwdx[om + e] + dwdx[q]));
      } else {
        r1 = c * (dwdy[q] - dvdz[q]);
        r2 = c * (dudz[q] - dwdx[q]);
      }
      vals[3] = r1;
      vals[4] = r2;
      vals[5] = c * (dvdx[q] - dudy[q]);
      constexpr int f0 = VORT_ONLY ? 3 : 0;
#pragma unroll
      for (int f = f0; f < 6; ++f) {
        if (e == 0) out[f - f0].x = vals[f]; else out[f - f0].y = vals[f];
      }
    }
  }
};

// convec.f90:170-305: the three dealiased products on the 3/2 grid with
// the normalisation 1/(nx2*ny2), levels 1..nz.
template <typename R>
struct SrcConvProd {
  using C = cplx<R>;   // the fields' complex pair type
  const R *ub, *vb, *wb, *o1, *o2, *o3;
  R c;
  int ld, nz;
  long long plane;
  InstMap im;
  __device__ __forceinline__ void load2(int n, int jy, int li, cplx<R>* out) const {
    const int inst = im.inst(li);
    const int k = li - inst * im.nli + 1;
    const long long o = inst * im.istr + (long long)k * plane + (long long)jy * ld + 2 * n;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const long long q = o + e, qp = q + plane, qm = q - plane;
      const R h = (R)0.5;
      R cx, cy, cz;
      if (k == 1) {
        cx = c * (vb[q] * (-o3[q]) + h * wb[qp] * (o2[qp]));
        cy = c * (ub[q] * (o3[q]) + h * wb[qp] * (-o1[qp]));
      } else if (k == nz - 1) {
        cx = c * (vb[q] * (-o3[q]) + h * wb[q] * (o2[q]));
        cy = c * (ub[q] * (o3[q]) + h * wb[q] * (-o1[q]));
      } else if (k < nz - 1) {
        cx = c * (vb[q] * (-o3[q]) + h * (wb[qp] * (o2[qp]) + wb[q] * (o2[q])));
        cy = c * (ub[q] * (o3[q]) + h * (wb[qp] * (-o1[qp]) + wb[q] * (-o1[q])));
      } else {
        cx = (R)0; cy = (R)0;
      }
      if (k == 1 || k == nz) cz = (R)0;
      else cz = c * h * ((ub[q] + ub[qm]) * (-o2[q]) + (vb[q] + vb[qm]) * (o1[q]));
      if (e == 0) { out[0].x = cx; out[1].x = cy; out[2].x = cz; }
      else        { out[0].y = cx; out[1].y = cy; out[2].y = cz; }
    }
  }
};

// lagrange_Sdep.f90:88-205: the 21 quantities test-filtered at 2 Delta and
// 4 Delta: u_bar, v_bar, w_bar, the six products u_i u_j, S_ij and |S| S_ij,
// levels 1..nz (w-nodes; uv-node at the wall).
template <typename R>
struct SrcLagrange {
  using C = cplx<R>;   // the fields' complex pair type
  const R *u, *v, *w, *S11, *S12, *S13, *S22, *S23, *S33;
  int ld, nz, lbc, ubc;
  long long plane;
  InstMap im;
  __device__ __forceinline__ void load2(int n, int jy, int li, cplx<R>* out) const {
    const int inst = im.inst(li);
    const int k = li - inst * im.nli + 1;
    const long long o = inst * im.istr + (long long)k * plane + (long long)jy * ld + 2 * n;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const long long q = o + e;
      R ub, vb, wb;
      if (k == 1) {
        ub = u[q]; vb = v[q];
        wb = (lbc == 0) ? (R)0 : (R)0.25 * w[q + plane];
      } else if (k == nz) {
        ub = u[q - plane]; vb = v[q - plane];
        wb = (ubc == 0) ? (R)0 : (R)0.25 * w[q - plane];
      } else {
        ub = (R)0.5 * (u[q] + u[q - plane]);
        vb = (R)0.5 * (v[q] + v[q - plane]);
        wb = w[q];
      }
      const R s11 = S11[q], s12 = S12[q], s13 = S13[q], s22 = S22[q], s23 = S23[q], s33 = S33[q];
      const R S = sqrt((R)2 * (s11 * s11 + s22 * s22 + s33 * s33 + (R)2 * (s12 * s12 + s13 * s13 + s23 * s23)));
      R vals[21] = {ub, vb, wb, ub * ub, ub * vb, ub * wb, vb * vb, vb * wb, wb * wb,
                    s11, s12, s13, s22, s23, s33,
                    S * s11, S * s12, S * s13, S * s22, S * s23, S * s33};
#pragma unroll
      for (int f = 0; f < 21; ++f) {
        if (e == 0) out[f].x = vals[f]; else out[f].y = vals[f];
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Y spectral operator: out_o(ky) = sum_i mul(o,i)(kx,ky) * F_i(ky), with the
// 3/2-rule row maps of padd/unpadd (fft.f90:43-99).
// ---------------------------------------------------------------------------
enum : int { MUL_ZERO = 0, MUL_ONE = 1, MUL_IKX = 2, MUL_IKY = 3, MUL_G1 = 4, MUL_G2 = 5 };
enum : int { ROW_SAME = 0, ROW_PAD = 1, ROW_UNPAD = 2 };

// R is the transforms' arithmetic type (the multiplier tables are held in it).
template <typename R, int NIN, int NOUT, typename InT, typename OutT>
struct YOpLin {
  const InT* in;
  long long in_fs;       // elements between input fields (group g, input i -> g*NIN+i)
  int in_lev0, in_levstride, in_rows;
  int nli, in_inst_levels;   // launch levels per instance; input planes per instance
  FastDiv fnli;
  OutT* out;
  long long out_fs;
  int out_rows;
  int K, lh, ny_small, ny_big, rowmode;
  int mul[NOUT][NIN];
  const R *kxw, *kyw, *G1, *G2;
  // per output, set by the host (k_ypass): the first kx from which it is
  // zero (test-filter terms only), whether its operator depends on kx alone,
  // and (inverse-only passes) the output it is i kx times (-1: none) with an
  // input whose multiplier in it is MUL_IKX
  int zero_from[NOUT];
  bool store_zero = true;   // write the zero tiles (false: the consumer never reads those modes)
  bool sc_out[NOUT];
  int from[NOUT], from_in[NOUT];

  // row 0, column 0 of input i of group g at launch level li (rows K apart)
  __device__ __forceinline__ const InT* in_plane(int g, int i, int li) const {
    const int inst = fnli.div(li), lv = li - inst * nli;
    const long long plane_idx = (long long)inst * in_inst_levels + in_lev0 + lv * in_levstride;
    return in + (long long)(g * NIN + i) * in_fs + plane_idx * in_rows * K;
  }
  __device__ __forceinline__ OutT* out_plane(int g, int o, int li) const {
    return out + (long long)(g * NOUT + o) * out_fs + (long long)li * out_rows * K;
  }
  __device__ __forceinline__ int rowmap(int ko) const {
    const int hs = ny_small / 2;
    if (rowmode == ROW_SAME) return ko == hs ? -1 : ko;
    if (rowmode == ROW_PAD) {
      if (ko < hs) return ko;
      if (ko > ny_big - hs) return ko - ny_big + ny_small;
      return -1;
    }
    // ROW_UNPAD (big rows -> small rows)
    if (ko < hs) return ko;
    if (ko == hs) return -1;
    return ko + ny_big - ny_small;
  }
  // a plain copy of input i into output o (no multiply)
  __device__ __forceinline__ bool is_one(int o, int i) const { return mul[o][i] == MUL_ONE; }
  __device__ __forceinline__ bool is_zero(int o, int i) const { return mul[o][i] == MUL_ZERO; }
  __device__ __forceinline__ bool same_rows() const { return rowmode == ROW_SAME; }

  __device__ __forceinline__ bool coef(int g, int o, int i, int kx, int kin, cplx<R>& cf) const {
    switch (mul[o][i]) {
      case MUL_ONE: cf = mkc(FftConst<R>::one(), FftConst<R>::zero()); return true;
      case MUL_IKX: cf = mkc(FftConst<R>::zero(), kxw[kx]); return true;
      case MUL_IKY: cf = mkc(FftConst<R>::zero(), kyw[kin]); return true;
      case MUL_G1: cf = mkc(G1[kin * lh + kx], FftConst<R>::zero()); return true;
      case MUL_G2: cf = mkc(G2[kin * lh + kx], FftConst<R>::zero()); return true;
      default: return false;
    }
  }
};

// ---------------------------------------------------------------------------
// Xi row epilogues
// ---------------------------------------------------------------------------
template <typename R, int NF>
struct DstFields {
  using Real = R;     // the fields' storage type
  R* p[NF];
  int lev0, levstride, ld;
  long long plane;
  InstMap im;
  __device__ __forceinline__ void store(int jy, int li, int i, const R* vals) const {
    const int inst = im.inst(li), lv = li - inst * im.nli;
    const long long off = inst * im.istr + (long long)(lev0 + lv * levstride) * plane + (long long)jy * ld + i;
#pragma unroll
    for (int f = 0; f < NF; ++f) p[f][off] = vals[f];
  }
};

// divstress_uv.f90:38-82 and divstress_w.f90:38-113: horizontal part from
// the spectral pass plus the staggered z-derivative, levels 1..nz.
// WHICH: 1 = divtx, divty (NF=2); 2 = divtz (NF=1); 3 = all (NF=3).
template <typename R, int WHICH>
struct DstDiv {
  using Real = R;     // the fields' storage type
  R *divtx, *divty, *divtz;
  const R *txz, *tyz, *tzz;
  R inv_dz;
  int ld, nz;
  long long plane;
  InstMap im;
  __device__ __forceinline__ void store(int jy, int li, int i, const R* vals) const {
    const int inst = im.inst(li);
    const int k = li - inst * im.nli + 1;
    const long long q = inst * im.istr + (long long)k * plane + (long long)jy * ld + i;
    int f = 0;
    if (WHICH & 1) {
      if (k <= nz - 1) {
        divtx[q] = vals[0] + inv_dz * (txz[q + plane] - txz[q]);
        divty[q] = vals[1] + inv_dz * (tyz[q + plane] - tyz[q]);
      }
      f = 2;
    }
    if (WHICH & 2) {
      R d = vals[f];
      if (k >= 2 && k <= nz - 1) d = d + inv_dz * (tzz[q] - tzz[q - plane]);
      divtz[q] = d;
    }
  }
};

// convec.f90:207-317 output (RHS = convective term) or, FUSED, the step
// glue of main.f90:155-157, 211-296: RHS_f <- RHS, RHS = -conv - divt
// (+ mean_p_force) (+ f_a), Euler first step, AB2 intermediate velocity.
template <typename R, bool FUSED>
struct DstConvec {
  using Real = R;     // the fields' storage type
  R *RHSx, *RHSy, *RHSz, *RHSxf, *RHSyf, *RHSzf, *u, *v, *w;
  const R *divtx, *divty, *divtz, *fxa, *fya, *fza;
  const double* sc;   // step constants
  double mpfx, mpfy;
  int ld, nz, use_mpf, turbines;
  const int* iflags;
  long long plane;
  InstMap im;
  __device__ __forceinline__ void store(int jy, int li, int i, const R* vals) const {
    const int inst = im.inst(li);
    const int k = li - inst * im.nli + 1;
    const long long q = inst * im.istr + (long long)k * plane + (long long)jy * ld + i;
    if (!FUSED) {
      if (k <= nz - 1) { RHSx[q] = vals[0]; RHSy[q] = vals[1]; }
      RHSz[q] = vals[2];
      return;
    }
    const double* c = sc + inst * SC_N;
    const R dtr = (R)c[SC_DT], t1r = (R)c[SC_T1], t2r = (R)c[SC_T2];
    const bool euler = (iflags[inst] & IF_EULER) != 0;
    const bool in = k <= nz - 1;
    const R zero = (R)0;
    // every load first (the arrays may alias as far as the compiler knows,
    // so loads after a store could not be moved ahead of it)
    const R dx = in ? divtx[q] : zero, dy = in ? divty[q] : zero, dz = divtz[q];
    const R ax = (turbines && in) ? fxa[q] : zero, ay = (turbines && in) ? fya[q] : zero;
    const R az = (turbines && in) ? fza[q] : zero;
    const R ox = in ? RHSx[q] : zero, oy = in ? RHSy[q] : zero, oz = RHSz[q];
    const R u0 = in ? u[q] : zero, v0 = in ? v[q] : zero, w0 = w[q];
    if (in) {
      R nxr = -vals[0] - dx;
      R nyr = -vals[1] - dy;
      if (use_mpf) { nxr = nxr + (R)mpfx; nyr = nyr + (R)mpfy; }
      if (turbines) { nxr = nxr + ax; nyr = nyr + ay; }
      const R fx = euler ? nxr : ox;
      const R fy = euler ? nyr : oy;
      RHSxf[q] = fx; RHSyf[q] = fy;
      RHSx[q] = nxr; RHSy[q] = nyr;
      u[q] = u0 + dtr * (t1r * nxr + t2r * fx);
      v[q] = v0 + dtr * (t1r * nyr + t2r * fy);
    }
    R nzr = -vals[2] - dz;
    if (turbines && in) nzr = nzr + az;
    const R fz = euler ? nzr : oz;
    RHSzf[q] = fz;
    RHSz[q] = nzr;
    w[q] = w0 + dtr * (t1r * nzr + t2r * fz);
  }
};

// press_stag_array.f90:254-273 output for levels 1..nz-1 (p, dpdx, dpdy), or,
// FUSED, main.f90:321-326 and forcing.f90:165-183: RHS -= grad_h p and the
// projection of u and v.
template <typename R, bool FUSED>
struct DstPress {
  using Real = R;     // the fields' storage type
  R *p, *dpdx, *dpdy, *RHSx, *RHSy, *u, *v;
  const double* sc;   // step constants
  int ld;
  long long plane;
  InstMap im;
  __device__ __forceinline__ void store(int jy, int li, int i, const R* vals) const {
    const int inst = im.inst(li);
    const int k = li - inst * im.nli + 1;
    const long long q = inst * im.istr + (long long)k * plane + (long long)jy * ld + i;
    p[q] = vals[0];
    if (!FUSED) {
      dpdx[q] = vals[1];
      dpdy[q] = vals[2];
      return;
    }
    const double* c = sc + inst * SC_N;
    const R dtr = (R)c[SC_DT], t1r = (R)c[SC_T1];
    const R rx = RHSx[q], ry = RHSy[q], u0 = u[q], v0 = v[q];   // loads first
    RHSx[q] = rx - vals[1];
    RHSy[q] = ry - vals[2];
    u[q] = u0 + dtr * (-t1r * vals[1]);
    v[q] = v0 + dtr * (-t1r * vals[2]);
  }
};

// x^(-1/8) for x > 0 (the Lagrangian time scale, lagrange_Sdep.f90's
// Tn**(-1/8)): two square roots and a reciprocal square root, within a few
// ulps of pow and far cheaper than pow in FP64, where these three powers
// per point had bound the whole Lagrangian epilogue.
__device__ __forceinline__ double inv_root8(double x) { return rsqrt(sqrt(sqrt(x))); }
__device__ __forceinline__ float inv_root8(float x) { return rsqrtf(sqrtf(sqrtf(x))); }

// lagrange_Sdep.f90:110-404 pointwise part: Leonard terms L, Q, model
// tensors M, N, their contractions, the Lagrangian relaxation of F_LM,
// F_MM, F_QN, F_NN, beta and Cs^2.  vals[2q] = quantity q at 2 Delta,
// vals[2q+1] = at 4 Delta (q as in SrcLagrange).
template <typename R>
struct DstLagrange {
  using Real = R;     // the fields' storage type
  const R *FLMi, *FMMi, *FQNi, *FNNi;  // interpolated running averages
  R *FLM, *FMM, *FQN, *FNN, *Cs, *Beta, *Tn_all, *ee_now;
  double cst, opftdelta, beta_exp;
  int beta_exp_one;   // beta_exp == 1 exactly (the reference's tf1 = 2, tf2 = 4): pow(x, 1) = x
  const double* sc;   // step constants (lagran_dt)
  int ld, nz, lbc, ubc;
  const int* iflags;
  long long plane;
  InstMap im;
  __device__ __forceinline__ void store(int jy, int li, int i, const R* vals) const {
    const int inst = im.inst(li);
    const int fl = iflags[inst];
    if (!(fl & IF_LAG)) return;          // instance not due for the dynamic update
    const bool init_lm = (fl & IF_INITLM) != 0, init_qn = (fl & IF_INITQN) != 0;
    const int k = li - inst * im.nli + 1;
    const long long q = inst * im.istr + (long long)k * plane + (long long)jy * ld + i;
    const R zero = (R)1.0e-24;
    const R tf1 = (R)2, tf2 = (R)4, tf1_2 = tf1 * tf1, tf2_2 = tf2 * tf2;
    auto A = [&](int qq) { return vals[2 * qq]; };
    auto B = [&](int qq) { return vals[2 * qq + 1]; };
    const R ub = A(0), vb = A(1), wb = A(2);
    const R uh = B(0), vh = B(1), wh = B(2);
    const R L11 = A(3) - ub * ub, L12 = A(4) - ub * vb, L13 = A(5) - ub * wb;
    const R L22 = A(6) - vb * vb, L23 = A(7) - vb * wb, L33 = A(8) - wb * wb;
    const R Q11 = B(3) - uh * uh, Q12 = B(4) - uh * vh, Q13 = B(5) - uh * wh;
    const R Q22 = B(6) - vh * vh, Q23 = B(7) - vh * wh, Q33 = B(8) - wh * wh;
    const R Sb11 = A(9), Sb12 = A(10), Sb13 = A(11), Sb22 = A(12), Sb23 = A(13), Sb33 = A(14);
    const R Sh11 = B(9), Sh12 = B(10), Sh13 = B(11), Sh22 = B(12), Sh23 = B(13), Sh33 = B(14);
    const R S_bar = sqrt((R)2 * (Sb11 * Sb11 + Sb22 * Sb22 + Sb33 * Sb33 + (R)2 * (Sb12 * Sb12 + Sb13 * Sb13 + Sb23 * Sb23)));
    const R S_hat = sqrt((R)2 * (Sh11 * Sh11 + Sh22 * Sh22 + Sh33 * Sh33 + (R)2 * (Sh12 * Sh12 + Sh13 * Sh13 + Sh23 * Sh23)));
    const R M11 = (R)cst * (A(15) - tf1_2 * S_bar * Sb11), M12 = (R)cst * (A(16) - tf1_2 * S_bar * Sb12);
    const R M13 = (R)cst * (A(17) - tf1_2 * S_bar * Sb13), M22 = (R)cst * (A(18) - tf1_2 * S_bar * Sb22);
    const R M23 = (R)cst * (A(19) - tf1_2 * S_bar * Sb23), M33 = (R)cst * (A(20) - tf1_2 * S_bar * Sb33);
    const R N11 = (R)cst * (B(15) - tf2_2 * S_hat * Sh11), N12 = (R)cst * (B(16) - tf2_2 * S_hat * Sh12);
    const R N13 = (R)cst * (B(17) - tf2_2 * S_hat * Sh13), N22 = (R)cst * (B(18) - tf2_2 * S_hat * Sh22);
    const R N23 = (R)cst * (B(19) - tf2_2 * S_hat * Sh23), N33 = (R)cst * (B(20) - tf2_2 * S_hat * Sh33);
    const R LM = L11 * M11 + L22 * M22 + L33 * M33 + (R)2 * (L12 * M12 + L13 * M13 + L23 * M23);
    const R MM = M11 * M11 + M22 * M22 + M33 * M33 + (R)2 * (M12 * M12 + M13 * M13 + M23 * M23);
    const R QN = Q11 * N11 + Q22 * N22 + Q33 * N33 + (R)2 * (Q12 * N12 + Q13 * N13 + Q23 * N23);
    const R NN = N11 * N11 + N22 * N22 + N33 * N33 + (R)2 * (N12 * N12 + N13 * N13 + N23 * N23);
    const R cs = (R)Cs[q];
    ee_now[q] = (R)(L11 * L11 + L22 * L22 + L33 * L33 + (R)2 * (L12 * L12 + L13 * L13 + L23 * L23)
                    - (R)2 * LM * cs + MM * cs * cs);
    R fLM = FLMi[q], fMM = FMMi[q], fQN = FQNi[q], fNN = FNNi[q];
    if (init_lm) { fMM = MM; fLM = (R)0.03 * MM; }
    R Tn = max(fLM * fMM, zero);
    Tn = (R)opftdelta * inv_root8(Tn);
    Tn = max(zero, Tn);
    const R ldt = (R)sc[inst * SC_N + SC_LDT];
    R dumfac = ldt / Tn;
    R epsi = dumfac / ((R)1 + dumfac);
    fLM = epsi * LM + ((R)1 - epsi) * fLM;
    fMM = epsi * MM + ((R)1 - epsi) * fMM;
    fLM = max(zero, fLM);
    R cs2d = fLM / (fMM + zero);
    cs2d = max(zero, cs2d);
    if (init_qn) { fNN = NN; fQN = (R)0.03 * NN; }
    Tn = max(fQN * fNN, zero);
    Tn = (R)opftdelta * inv_root8(Tn);
    Tn = max(zero, Tn);
    dumfac = ldt / Tn;
    epsi = dumfac / ((R)1 + dumfac);
    fQN = epsi * QN + ((R)1 - epsi) * fQN;
    fNN = epsi * NN + ((R)1 - epsi) * fNN;
    fQN = max(zero, fQN);
    R cs4d = fQN / (fNN + zero);
    cs4d = max(zero, cs4d);
    R beta = beta_exp_one ? cs4d / cs2d : pow(cs4d / cs2d, (R)beta_exp);
    if (k == nz && ubc == 0) beta = (R)1;
    if (k == 1 && lbc == 0) beta = (R)1;
    const R betaclip = max(beta, (R)1 / (tf1 * tf2));
    const R csn = max(zero, cs2d / betaclip);
    FLM[q] = (R)fLM; FMM[q] = (R)fMM; FQN[q] = (R)fQN; FNN[q] = (R)fNN;
    Cs[q] = csn;
    Beta[q] = beta;
    Tn_all[q] = Tn;
  }
};

}  // namespace lesgo
