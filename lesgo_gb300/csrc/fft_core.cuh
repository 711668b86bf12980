// Shared-memory Stockham FFT core and the three batched plane-transform passes
// used by every spectral stage of the LES step.
//
// A horizontal (x-y) transform of a stack of planes is split into
//   Xf : real-to-complex along x (one row of nx reals per line), keeping the
//        modes kx < nx/2 (the kx = nx/2 "oddball" is always zeroed by the
//        reference, derivatives.f90:64, fft.f90:57-97),
//   Y  : complex transforms along y for each kept kx column, with the
//        stage's spectral multipliers (i kx, i ky, test-filter kernels,
//        3/2-rule padding/truncation) applied between the forward and the
//        inverse transform,
//   Xi : complex-to-real along x, fused with the stage's epilogue.
// Intermediates live in HBM as complex arrays [line][jy][kx] with kx
// fastest, so Xf/Xi rows and Y column tiles are both coalesced.
//
// Transforms follow FFTW's unnormalised r2c/c2r definitions (the reference's
// fft.f90:114-121); normalisation constants are applied by the callers
// exactly where the reference applies them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "df64.cuh"

namespace lesgo {

// Arithmetic types of the transforms: float (the mixed form), double (the
// plain FP64 form) and df64 (FP64 storage with double-word transforms).
// cplx<A> is the complex type held in shared memory and in the spectral
// buffers.
struct dfc {
  df64 x, y;
};

template <typename R> struct CplxOf;
template <> struct CplxOf<double> { using T = double2; };
template <> struct CplxOf<float> { using T = float2; };
template <> struct CplxOf<df64> { using T = dfc; };
template <typename R> using cplx = typename CplxOf<R>::T;

__host__ __device__ __forceinline__ double2 mkc(double a, double b) { return make_double2(a, b); }
__host__ __device__ __forceinline__ float2 mkc(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ dfc mkc(df64 a, df64 b) { return dfc{a, b}; }

// Constants of the butterflies in each arithmetic (the double-word ones
// split exactly: hi = the FP32 rounding, lo = the FP32 rounding of the rest).
template <typename R> struct FftConst;
template <> struct FftConst<float> {
  __device__ static float sin60() { return 0.86602540378443864676f; }
  __device__ static float rsqrt2() { return 0.70710678118654752440f; }
  __device__ static float half() { return 0.5f; }
  __device__ static float zero() { return 0.f; }
  __device__ static float one() { return 1.f; }
};
template <> struct FftConst<double> {
  __device__ static double sin60() { return 0.86602540378443864676372317075294; }
  __device__ static double rsqrt2() { return 0.70710678118654752440084436210485; }
  __device__ static double half() { return 0.5; }
  __device__ static double zero() { return 0.0; }
  __device__ static double one() { return 1.0; }
};
template <> struct FftConst<df64> {
  __device__ static df64 sin60() { return df64{__int_as_float(0x3f5db3d7), __int_as_float(0x328584cb)}; }
  __device__ static df64 rsqrt2() { return df64{__int_as_float(0x3f3504f3), __int_as_float(0x324fe77a)}; }
  __device__ static df64 half() { return df64{0.5f, 0.f}; }
  __device__ static df64 zero() { return df64{0.f, 0.f}; }
  __device__ static df64 one() { return df64{1.f, 0.f}; }
};
template <typename R> __device__ __forceinline__ R rmul_half(R a) { return FftConst<R>::half() * a; }
template <> __device__ __forceinline__ df64 rmul_half<df64>(df64 a) { return df64{0.5f * a.hi, 0.5f * a.lo}; }
template <typename T2> __device__ __forceinline__ T2 czero() {
  using R = decltype(T2{}.x);
  return mkc(FftConst<R>::zero(), FftConst<R>::zero());
}

// Conversions between the storage and arithmetic types.
template <typename D> struct Cvt;
template <> struct Cvt<float> {
  __device__ static float from(float a) { return a; }
  __device__ static float from(double a) { return (float)a; }
  __device__ static float from(df64 a) { return a.hi + a.lo; }
};
template <> struct Cvt<double> {
  __device__ static double from(float a) { return (double)a; }
  __device__ static double from(double a) { return a; }
  __device__ static double from(df64 a) { return df_to(a); }
};
template <> struct Cvt<df64> {
  __device__ static df64 from(float a) { return df64{a, 0.f}; }
  __device__ static df64 from(double a) { return df_from(a); }
  __device__ static df64 from(df64 a) { return a; }
};
template <typename D, typename S> __device__ __forceinline__ D cvt(S a) { return Cvt<D>::from(a); }
template <typename D2, typename S2> __device__ __forceinline__ D2 cvt2(S2 a) {
  using D = decltype(D2{}.x);
  return mkc(cvt<D>(a.x), cvt<D>(a.y));
}

// Read-only loads of table entries.
__device__ __forceinline__ float2 ldt(const float2* p) { return __ldg(p); }
__device__ __forceinline__ double2 ldt(const double2* p) { return __ldg(p); }
__device__ __forceinline__ dfc ldt(const dfc* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return dfc{df64{v.x, v.y}, df64{v.z, v.w}};
}

template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { return mkc(a.x + b.x, a.y + b.y); }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { return mkc(a.x - b.x, a.y - b.y); }
template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  return mkc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// FP32 complex adds as Blackwell's packed FP32x2 instructions (one issue
// slot for both components; each component rounds as __fadd_rn / __fmaf_rn):
// the transforms are bound by instruction issue
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) { return __fadd2_rn(a, b); }
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);   // a - b, exact product by -1
}
// a + conj(b) and a - conj(b) (the real-transform split steps)
template <typename T2> __device__ __forceinline__ T2 cadd_conj(T2 a, T2 b) { return mkc(a.x + b.x, a.y - b.y); }
template <typename T2> __device__ __forceinline__ T2 csub_conj(T2 a, T2 b) { return mkc(a.x - b.x, a.y + b.y); }
template <> __device__ __forceinline__ float2 cadd_conj<float2>(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(1.f, -1.f), a);
}
template <> __device__ __forceinline__ float2 csub_conj<float2>(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, 1.f), a);
}
template <typename T2> __device__ __forceinline__ T2 cmulconj(T2 a, T2 b) {  // a * conj(b)
  return mkc(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T2> __device__ __forceinline__ T2 cconj(T2 a) { return mkc(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <typename T2> __device__ __forceinline__ T2 mul_mi(T2 a) { return mkc(a.y, -a.x); }
template <typename T2> __device__ __forceinline__ T2 mul_pi(T2 a) { return mkc(-a.y, a.x); }

constexpr int kMaxStages = 12;

// Unsigned division by a run-time constant d >= 1 for dividends below 2^31,
// with one multiply-high and a shift: l = ceil(log2 d), p = 31 + l,
// m = ceil(2^p / d), q = umulhi(n, m) >> (l - 1) (Granlund and Montgomery's
// round-up reciprocal; the error m*d - 2^p < d keeps the quotient exact for
// n < 2^31).  Integer division would otherwise be a long instruction
// sequence inside every butterfly and every element copy.
struct FastDiv {
  unsigned d = 1, m = 0, sh = 0;
  FastDiv() = default;
  __host__ explicit FastDiv(unsigned dv) : d(dv) {
    if (dv <= 1) { d = 1; return; }
    unsigned l = 0;
    while ((1u << l) < dv) ++l;
    m = (unsigned)(((1ull << (31 + l)) + dv - 1) / dv);
    sh = l - 1;
  }
  __device__ __forceinline__ int div(int n) const {
    return d == 1 ? n : (int)(__umulhi((unsigned)n, m) >> sh);
  }
  // the same for a divisor known to be >= 2 (no test for d = 1)
  __device__ __forceinline__ int div2(int n) const { return (int)(__umulhi((unsigned)n, m) >> sh); }
};

// Plan for one complex FFT length n = prod(radix[]).
template <typename R>
struct FftPlan {
  int n;
  int nf;
  int radix[kMaxStages];
  int nbs[kMaxStages];        // butterflies per line in stage s (n / radix[s])
  int nss[kMaxStages];        // sub-transform length Ns entering stage s
  FastDiv fnb[kMaxStages], fns[kMaxStages];
  const cplx<R>* tw;   // tw[t] = exp(-2 pi i t / n), t = 0..n-1
  // stage twiddles: stage s, butterfly jm, input r (1..radix-1) at
  // stw[two[s] + jm * (radix - 1) + r - 1] = tw[r * jm * n / (Ns * radix)]
  const cplx<R>* stw;
  int two[kMaxStages];
  const cplx<R>* rtw;  // rtw[k] = exp(-2 pi i k / (2n)), k = 0..n (real-transform packing)
};

// Radix-R butterfly on registers (DFT_R, sign by INV).
template <typename T2, bool INV>
__device__ __forceinline__ void bfly2(T2& a0, T2& a1) {
  T2 t = a0;
  a0 = cadd(t, a1);
  a1 = csub(t, a1);
}

template <typename T2, bool INV>
__device__ __forceinline__ void bfly4(T2& a0, T2& a1, T2& a2, T2& a3) {
  T2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
  T2 t2 = cadd(a1, a3), d = csub(a1, a3);
  T2 t3 = INV ? mul_pi(d) : mul_mi(d);
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

// a - b/2 and s*a (the radix-3 butterfly)
template <typename T2> __device__ __forceinline__ T2 csub_half(T2 a, T2 b) {
  return mkc(a.x - rmul_half(b.x), a.y - rmul_half(b.y));
}
template <> __device__ __forceinline__ float2 csub_half<float2>(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-0.5f, -0.5f), a);
}
template <typename T2, typename R> __device__ __forceinline__ T2 cscale(T2 a, R s) { return mkc(s * a.x, s * a.y); }
template <> __device__ __forceinline__ float2 cscale<float2, float>(float2 a, float s) {
  return __fmul2_rn(a, make_float2(s, s));
}

template <typename T2, bool INV>
__device__ __forceinline__ void bfly3(T2& a0, T2& a1, T2& a2) {
  using R = decltype(a0.x);
  const R s = FftConst<R>::sin60();  // sin(2 pi / 3)
  T2 t1 = cadd(a1, a2);
  T2 t2 = csub_half(a0, t1);
  T2 d = csub(a1, a2);
  T2 t3 = cscale(d, s);
  a0 = cadd(a0, t1);
  // forward: y1 = t2 - i t3, y2 = t2 + i t3
  T2 it3 = mul_pi(t3);
  if (INV) {
    a1 = cadd(t2, it3);
    a2 = csub(t2, it3);
  } else {
    a1 = csub(t2, it3);
    a2 = cadd(t2, it3);
  }
}

template <typename T2, bool INV>
__device__ __forceinline__ void bfly8(T2* v) {
  using R = decltype(v[0].x);
  const R h = FftConst<R>::rsqrt2();
  // two radix-4 on even/odd, then combine with W8 twiddles
  T2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  T2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  bfly4<T2, INV>(e0, e1, e2, e3);
  bfly4<T2, INV>(o0, o1, o2, o3);
  // o_k *= W8^k (forward: exp(-2 pi i k/8))
  T2 w1 = INV ? mkc(h * (o1.x - o1.y), h * (o1.x + o1.y)) : mkc(h * (o1.x + o1.y), h * (o1.y - o1.x));
  T2 w2 = INV ? mul_pi(o2) : mul_mi(o2);
  T2 w3 = INV ? mkc(-h * (o3.x + o3.y), h * (o3.x - o3.y)) : mkc(h * (o3.y - o3.x), -h * (o3.x + o3.y));
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, w1);
  v[5] = csub(e1, w1);
  v[2] = cadd(e2, w2);
  v[6] = csub(e2, w2);
  v[3] = cadd(e3, w3);
  v[7] = csub(e3, w3);
}

template <typename T2, bool INV>
__device__ __forceinline__ T2 twid(const T2* tw, int idx, T2 a) {
  T2 w = ldt(tw + idx);
  return INV ? cmulconj(a, w) : cmul(a, w);
}

// Radix-RR butterfly on registers.
template <typename T2, bool INV, int RR>
__device__ __forceinline__ void bfly(T2* v) {
  if constexpr (RR == 8) bfly8<T2, INV>(v);
  else if constexpr (RR == 4) bfly4<T2, INV>(v[0], v[1], v[2], v[3]);
  else if constexpr (RR == 3) bfly3<T2, INV>(v[0], v[1], v[2]);
  else bfly2<T2, INV>(v[0], v[1]);
}

// One Stockham stage of radix RR over `total` butterflies.  Butterfly t is
// (line or column, j); `at(t, j)` gives the offset of its first input and
// `out(t, j)` the offset of output 0 of a butterfly with q = j / Ns, jm = j
// % Ns: inputs at src + r * sr, outputs at dst + r * sd (r < RR).  FIRST
// marks the first stage (Ns = 1: no twiddles, q = j).  The twiddles of
// butterfly jm are the RR - 1 consecutive entries at `twp` (the stage
// table); jm = 0 multiplies by 1 exactly, which keeps the warp on one path.
template <typename T2, bool INV, int RR, bool FIRST>
__device__ __forceinline__ void stage_bfly(const T2* src, T2* dst, int sr, int sd, const T2* twp) {
  T2 v[RR];
#pragma unroll
  for (int r = 0; r < RR; ++r) v[r] = src[r * sr];
  if (!FIRST) {
#pragma unroll
    for (int r = 1; r < RR; ++r) v[r] = twid<T2, INV>(twp, r - 1, v[r]);
  }
  bfly<T2, INV, RR>(v);
#pragma unroll
  for (int r = 0; r < RR; ++r) dst[r * sd] = v[r];
}

template <typename T2, bool INV, int RR, bool FIRST>
__device__ __forceinline__ void lines_stage(const T2* a, T2* b, int nl, int ls, int nb, int Ns,
                                            const FastDiv fnl, const FastDiv fns, const T2* stw) {
  // the line index runs fastest across threads: with an odd line stride
  // the stage's loads and stores fall in distinct banks
  const int total = nl * nb;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int j = fnl.div(t);
    const int l = t - j * nl;
    const int q = FIRST ? j : fns.div2(j);   // after the first stage Ns >= 2
    const int jm = j - q * Ns;
    stage_bfly<T2, INV, RR, FIRST>(a + l * ls + j, b + l * ls + q * Ns * RR + jm, nb, Ns, stw + jm * (RR - 1));
  }
}

// Double-word plans use radix 4, 3 and 2 only: their butterflies are long,
// and leaving radix 8 out of them keeps the kernels' code (and its compile
// time) small at the same arithmetic per point.
template <typename T2> constexpr bool kRadix8 = !std::is_same<T2, dfc>::value;

template <typename T2, bool INV, bool FIRST>
__device__ __forceinline__ void lines_stage_r(int Rr, const T2* a, T2* b, int nl, int ls, int nb, int Ns,
                                              const FastDiv fnl, const FastDiv fns, const T2* stw) {
  switch (Rr) {
    case 8:
      if constexpr (kRadix8<T2>) lines_stage<T2, INV, 8, FIRST>(a, b, nl, ls, nb, Ns, fnl, fns, stw);
      break;
    case 4: lines_stage<T2, INV, 4, FIRST>(a, b, nl, ls, nb, Ns, fnl, fns, stw); break;
    case 3: lines_stage<T2, INV, 3, FIRST>(a, b, nl, ls, nb, Ns, fnl, fns, stw); break;
    default: lines_stage<T2, INV, 2, FIRST>(a, b, nl, ls, nb, Ns, fnl, fns, stw); break;
  }
}

// Stockham autosort FFT of `nl` lines of length p.n held in shared memory
// (line l at a + l*ls).  `b` is scratch of the same shape.  Returns the
// buffer that holds the result.  All threads of the block must call it.
//
// The stage's sizes and divisors are read from the plan once per stage and
// passed by value (registers): the plan lives in the kernel's parameter
// block, and a reference into it with the run-time stage index would be
// re-read through the constant path inside the butterfly loop.
template <typename R, bool INV>
__device__ cplx<R>* fft_lines(cplx<R>* a, cplx<R>* b, int nl, int ls, const FastDiv fnl, const FftPlan<R>& p) {
  for (int s = 0; s < p.nf; ++s) {
    const int nb = p.nbs[s], Ns = p.nss[s];
    if (s == 0)
      lines_stage_r<cplx<R>, INV, true>(p.radix[s], a, b, nl, ls, nb, Ns, fnl, p.fns[s], p.stw);
    else
      lines_stage_r<cplx<R>, INV, false>(p.radix[s], a, b, nl, ls, nb, Ns, fnl, p.fns[s], p.stw + p.two[s]);
    __syncthreads();
    cplx<R>* tmp = a; a = b; b = tmp;
  }
  return a;
}

// ---------------------------------------------------------------------------
// Pass descriptors
// ---------------------------------------------------------------------------
struct XfGeom {
  int M;        // real row length (nx or nx2)
  int K;        // modes kept (nx/2)
  int nrows;    // rows per field in this launch (= ny_rows * nlev)
  int nyrows;   // rows per level (ny or ny2)
  int rpc;      // rows per CTA
  int ls;       // smem line stride (complex)
  long long out_field_stride;  // complex elements between fields in the output
  FastDiv fH, fK, fnyrows, frpc, fnl;   // by M/2, K, nyrows, rpc, NF * rpc
};

// Xf: r2c along x for NF fields at once.  Src::load2(n, jy, li, v[NF])
// supplies the real pairs (x[2n], x[2n+1]) of every field at row (jy, li)
// in the fields' storage type (Src::C), converted to the arithmetic type R.
// Output: out[f][li][jy][kx] for kx < K.
template <typename R, int NF, class Src>
__global__ void __launch_bounds__(256) k_xfwd(XfGeom g, FftPlan<R> plan, Src src, cplx<R>* __restrict__ out) {
  using T2 = cplx<R>;
  using SC = typename Src::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* A = reinterpret_cast<T2*>(smem_raw);
  const int nl = NF * g.rpc;
  T2* B = A + nl * g.ls;
  const int H = g.M / 2;
  const int row0 = blockIdx.x * g.rpc;
  #pragma unroll 4
  for (int t = threadIdx.x; t < g.rpc * H; t += blockDim.x) {
    const int r = g.fH.div(t), nn = t - r * H;
    const int row = row0 + r;
    SC v[NF];
    if (row < g.nrows) {
      const int li = g.fnyrows.div(row);
      const int jy = row - li * g.nyrows;
      src.load2(nn, jy, li, v);
    } else {
#pragma unroll
      for (int f = 0; f < NF; ++f) v[f] = czero<SC>();
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) A[(f * g.rpc + r) * g.ls + nn] = cvt2<T2>(v[f]);
  }
  __syncthreads();
  T2* Z = fft_lines<R, false>(A, B, nl, g.ls, g.fnl, plan);
  #pragma unroll 4
  for (int t = threadIdx.x; t < nl * g.K; t += blockDim.x) {
    const int l = g.fK.div(t), kk = t - l * g.K;
    const int f = g.frpc.div(l), r = l - f * g.rpc;
    const int row = row0 + r;
    if (row >= g.nrows) continue;
    T2 zk = Z[l * g.ls + kk];
    T2 zm = Z[l * g.ls + (kk == 0 ? 0 : H - kk)];
    T2 a = cadd_conj(zk, zm);   // Zk + conj(Zm)
    T2 b = csub_conj(zk, zm);   // Zk - conj(Zm)
    T2 w = ldt(plan.rtw + kk);
    // X = a/2 - (i/2) w b
    R wbx = w.x * b.x - w.y * b.y, wby = w.x * b.y + w.y * b.x;
    out[(long long)f * g.out_field_stride + (long long)row * g.K + kk] = mkc(rmul_half(a.x + wby), rmul_half(a.y - wbx));
  }
}

struct XiGeom {
  int M;        // real output row length (nx or nx2)
  int K;        // modes present in the input (nx/2); K..M/2 are zero
  int nrows;    // rows in this launch (ny_rows * nlev)
  int nyrows;
  int rpc;
  int ls;
  long long in_field_stride;
  FastDiv fH, fM, fnyrows, frpc, fnl;   // by M/2, M, nyrows, rpc, NF * rpc
  int kz0, kz1;   // modes kx >= kz0 (even fields) / kz1 (odd fields) are zero and not read (K: none)
};

// Xi: c2r along x for NF fields at once, then Dst::store(jy, li, i, vals)
// receives the NF reconstructed reals at x index i of row (jy, li), in the
// fields' storage type (Dst::Real).
template <typename R, int NF, class Dst>
__global__ void __launch_bounds__(256) k_xinv(XiGeom g, FftPlan<R> plan, const cplx<R>* __restrict__ in, Dst dst) {
  using T2 = cplx<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* A = reinterpret_cast<T2*>(smem_raw);
  const int H = g.M / 2;
  const int nl = NF * g.rpc;
  T2* B = A + nl * g.ls;
  const int row0 = blockIdx.x * g.rpc;
  // build Z[k] = (X[k] + conj X[H-k]) + i W^-k (X[k] - conj X[H-k])
  #pragma unroll 4
  for (int t = threadIdx.x; t < nl * H; t += blockDim.x) {
    const int l = g.fH.div(t), k = t - l * H;
    const int f = g.frpc.div(l), r = l - f * g.rpc;
    const int row = row0 + r;
    T2 z = czero<T2>();
    if (row < g.nrows) {
      const T2* src = in + (long long)f * g.in_field_stride + (long long)row * g.K;
      const int kzf = (f & 1) ? g.kz1 : g.kz0;   // a select: no indexing into the parameter block
      T2 xk = k < kzf ? src[k] : czero<T2>();
      const int km = H - k;   // k = 0 -> Nyquist (zero)
      T2 xm = (k > 0 && km < kzf) ? src[km] : czero<T2>();
      T2 a = cadd_conj(xk, xm);
      T2 b = csub_conj(xk, xm);
      T2 w = ldt(plan.rtw + k);
      R cx = w.x * b.x + w.y * b.y, cy = w.x * b.y - w.y * b.x;  // conj(w) * b
      z = mkc(a.x - cy, a.y + cx);
    }
    A[l * g.ls + k] = z;
  }
  __syncthreads();
  T2* Z = fft_lines<R, true>(A, B, nl, g.ls, g.fnl, plan);
  const R* Zr = reinterpret_cast<const R*>(Z);
  #pragma unroll 4
  for (int t = threadIdx.x; t < g.rpc * g.M; t += blockDim.x) {
    const int r = g.fM.div(t), i = t - r * g.M;
    const int row = row0 + r;
    if (row >= g.nrows) continue;
    const int li = g.fnyrows.div(row);
    const int jy = row - li * g.nyrows;
    typename Dst::Real vals[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) vals[f] = cvt<typename Dst::Real>(Zr[2 * ((f * g.rpc + r) * g.ls) + i]);
    dst.store(jy, li, i, vals);
  }
}

struct YGeom {
  int ny_in, ny_out;
  int K;         // columns (kx < K)
  int nlev;      // lines of planes in this launch
  int tk;        // columns per CTA
  int ls_in, ls_out;
  long long in_lev_stride;   // complex elements between planes of the input
  long long out_lev_stride;
  int tk_log2;               // tk is a power of two
  FastDiv fny_in, fny_out;
  FastDiv fwin;              // by NIN * tk (the width of the input tile)
  FastDiv ftk;               // by tk (the width of an output tile)
};

template <typename T2, bool INV, int RR, bool FIRST>
__device__ __forceinline__ void cols_stage(const T2* a, T2* b, int width, const FastDiv fw, int nb, int Ns,
                                           const FastDiv fns, const T2* stw) {
  const int total = nb * width;
  const int sr = nb * width, sd = Ns * width;   // strides between a butterfly's inputs / outputs
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int j = fw.div(t);
    const int l = t - j * width;
    const int q = FIRST ? j : fns.div2(j);   // after the first stage Ns >= 2
    const int jm = j - q * Ns;
    stage_bfly<T2, INV, RR, FIRST>(a + j * width + l, b + (q * Ns * RR + jm) * width + l, sr, sd,
                                   stw + jm * (RR - 1));
  }
}

template <typename T2, bool INV, bool FIRST>
__device__ __forceinline__ void cols_stage_r(int Rr, const T2* a, T2* b, int width, const FastDiv fw, int nb, int Ns,
                                             const FastDiv fns, const T2* stw) {
  switch (Rr) {
    case 8:
      if constexpr (kRadix8<T2>) cols_stage<T2, INV, 8, FIRST>(a, b, width, fw, nb, Ns, fns, stw);
      break;
    case 4: cols_stage<T2, INV, 4, FIRST>(a, b, width, fw, nb, Ns, fns, stw); break;
    case 3: cols_stage<T2, INV, 3, FIRST>(a, b, width, fw, nb, Ns, fns, stw); break;
    default: cols_stage<T2, INV, 2, FIRST>(a, b, width, fw, nb, Ns, fns, stw); break;
  }
}

// Stockham FFT along y of the columns of a row-major tile: element y of
// column l at a[y * width + l].  Threads run over (butterfly, column) with
// the column fastest, so a warp touches consecutive addresses at every step
// (no bank conflicts); the butterflies are those of fft_lines.
template <typename R, bool INV>
__device__ cplx<R>* fft_cols(cplx<R>* a, cplx<R>* b, int width, const FastDiv fw, const FftPlan<R>& p) {
  for (int s = 0; s < p.nf; ++s) {
    const int nb = p.nbs[s], Ns = p.nss[s];
    if (s == 0)
      cols_stage_r<cplx<R>, INV, true>(p.radix[s], a, b, width, fw, nb, Ns, p.fns[s], p.stw);
    else
      cols_stage_r<cplx<R>, INV, false>(p.radix[s], a, b, width, fw, nb, Ns, p.fns[s], p.stw + p.two[s]);
    __syncthreads();
    cplx<R>* tmp = a; a = b; b = tmp;
  }
  return a;
}

// Y pass.  NIN input spectra (after Xf) are loaded per column tile and, if
// FWD, transformed along y.  Each of NOUT outputs is a combination
// sum_i coef(o, i, kx, ky) * F_i(ky), mapped to ny_out rows (3/2 padding or
// truncation), inverse transformed if INV, and stored.  Op supplies
// pointers, coefficients and the row map.  Tiles are row-major: input i,
// row y, column c at S[y * NIN * tk + i * tk + c]; outputs W[y * tk + c].
//
// SC compiles in the transform-free path of kx-only outputs (the host picks
// the instance with it only for passes that have such an output, so that
// the other passes keep their register count).
template <typename R, int NIN, int NOUT, bool FWD, bool INV, bool SC, class Op>
__global__ void __launch_bounds__(256) k_ypass(YGeom g, FftPlan<R> pin, FftPlan<R> pout, Op op) {
  using T2 = cplx<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // S: the NIN*tk input columns (ny_in rows).  X: scratch of
  // max(NIN*tk*ny_in, 2*tk*ny_out) elements; W0/W1 (tk columns of ny_out
  // rows each) alias its front.
  const int win = NIN * g.tk;
  T2* S = reinterpret_cast<T2*>(smem_raw);
  T2* X = S + win * g.ny_in;
  T2* W0 = X;
  T2* W1 = X + g.tk * g.ny_out;
  const int kx0 = blockIdx.x * g.tk;
  const int li = blockIdx.y;
  const int grp = blockIdx.z;
  const int tkv = min(g.tk, g.K - kx0);
  // every thread keeps one column c and steps over rows r0, r0 + rstep, ...
  const int c = threadIdx.x & (g.tk - 1);
  const int r0 = threadIdx.x >> g.tk_log2;
  const int rstep = blockDim.x >> g.tk_log2;
  const bool live = c < tkv;
  const int kx = kx0 + c;
  // the forward transform's stages alternate between the tile and the
  // scratch: load into the buffer from which they end in S
  T2* L = (FWD && (pin.nf & 1)) ? X : S;
#pragma unroll
  for (int i = 0; i < NIN; ++i) {
    const auto* src = op.in_plane(grp, i, li) + kx;
    T2* s = L + i * g.tk + c;
#pragma unroll 4
    for (int jy = r0; jy < g.ny_in; jy += rstep) {
      T2 v = czero<T2>();
      if (live) v = cvt2<T2>(src[(long long)jy * g.K]);
      s[jy * win] = v;
    }
  }
  __syncthreads();
  // What each output needs on this tile (the same in every thread): 0 the
  // transforms, 1 none (its operator depends on kx alone), 2 the inverse
  // result of another output times i kx, 3 nothing (zero on this tile).
  // (Only the instances that can meet kinds 1-3 compile their paths: kx-only
  // outputs with SC, zero tiles in the one-input forward-inverse passes (the
  // test filters), derived outputs in the inverse-only passes.)
  constexpr bool kZero = FWD && INV && NIN == 1;
  constexpr bool kDerive = !FWD && INV;
  constexpr bool kPlain = !SC && !kZero && !kDerive;   // every output takes the transforms
  // two bits per output in a register (an array indexed in the output loop
  // would live in local memory)
  static_assert(NOUT <= 16, "two bits per output in 32");
  unsigned kinds = 0;
  auto kind = [&](int o) { return (int)((kinds >> (2 * o)) & 3u); };
  bool need_fwd = kPlain, any_sc = false;
  if constexpr (!kPlain) {
#pragma unroll
    for (int o = 0; o < NOUT; ++o) {
      int k = 0;
      if constexpr (kDerive) if (op.from[o] >= 0) k = 2;
      if constexpr (kZero) if (kx0 >= op.zero_from[o]) k = 3;
      if constexpr (SC) if (k == 0 && op.sc_out[o]) k = 1;
      kinds |= (unsigned)k << (2 * o);
      need_fwd |= k == 0;
      any_sc |= k == 1;
    }
  }
  if constexpr (SC) if (any_sc) {
    // A forward and inverse y transform with the y Nyquist row zeroed
    // between them is, per column, ny x(y) - (-1)^y s with
    // s = sum_l (-1)^l x(l) (the Nyquist component removed); a kx-only
    // operator then multiplies every row alike.  Partial sums of s over
    // each thread's rows go to the buffer the forward transform has not
    // loaded into.
    T2* F = (L == S) ? X : S;
    const int nr = min(rstep, g.ny_in);
    if (r0 < nr) {
#pragma unroll
      for (int i = 0; i < NIN; ++i) {
        T2 acc = czero<T2>();
        for (int jy = r0; jy < g.ny_in; jy += rstep) {
          const T2 v = L[jy * win + i * g.tk + c];
          acc = (jy & 1) ? csub(acc, v) : cadd(acc, v);
        }
        F[r0 * win + i * g.tk + c] = acc;
      }
    }
    __syncthreads();
    T2 sn[NIN];
#pragma unroll
    for (int i = 0; i < NIN; ++i) {
      T2 acc = czero<T2>();
      for (int r = 0; r < nr; ++r) acc = cadd(acc, F[r * win + i * g.tk + c]);
      sn[i] = acc;
    }
    const R nyr = cvt<R>((double)g.ny_in);
    for (int o = 0; o < NOUT; ++o) {
      if (kind(o) != 1) continue;
      auto* dst = op.out_plane(grp, o, li) + kx;
      using OutT = typename std::remove_pointer<decltype(dst)>::type;
#pragma unroll 2
      for (int jy = r0; jy < g.ny_out; jy += rstep) {
        T2 acc = czero<T2>();
#pragma unroll
        for (int i = 0; i < NIN; ++i) {
          const T2 v = L[jy * win + i * g.tk + c];
          const T2 sv = mkc(v.x * nyr, v.y * nyr);
          const T2 t = (jy & 1) ? cadd(sv, sn[i]) : csub(sv, sn[i]);
          T2 cf;
          if (op.is_one(o, i)) acc = cadd(acc, t);
          else if (op.coef(grp, o, i, kx, 0, cf)) acc = cadd(acc, cmul(t, cf));
        }
        if (live) dst[(long long)jy * g.K] = cvt2<OutT>(acc);
      }
    }
    __syncthreads();   // F is the forward transform's scratch
  }
  if (FWD && need_fwd) fft_cols<R, false>(L, L == S ? X : S, win, g.fwin, pin);   // ends in S
  for (int o = 0; o < NOUT; ++o) {
    if constexpr (!kPlain) if (kind(o) == 1 || kind(o) == 2) continue;
    if constexpr (kZero) if (kind(o) == 3) {
      if (live && op.store_zero) {
        auto* dst = op.out_plane(grp, o, li) + kx;
        using OutT = typename std::remove_pointer<decltype(dst)>::type;
        const OutT z{};
        for (int ky = r0; ky < g.ny_out; ky += rstep) dst[(long long)ky * g.K] = z;
      }
      continue;
    }
#pragma unroll 2
    for (int ky = r0; ky < g.ny_out; ky += rstep) {
      T2 acc = czero<T2>();
      const int kin = op.rowmap(ky);
      if (live && kin >= 0) {
#pragma unroll
        for (int i = 0; i < NIN; ++i) {
          if (NIN > 1 && op.is_zero(o, i)) continue;   // inputs this output does not use
          T2 cf;
          const T2 v = S[kin * win + i * g.tk + c];
          if (op.is_one(o, i)) acc = cadd(acc, v);
          else if (op.coef(grp, o, i, kx, kin, cf)) acc = cadd(acc, cmul(v, cf));
        }
      }
      W0[ky * g.tk + c] = acc;
    }
    __syncthreads();
    T2* res = W0;
    if (INV) res = fft_cols<R, true>(W0, W1, g.tk, g.ftk, pout);
    if (live) {
      auto* dst = op.out_plane(grp, o, li) + kx;
      using OutT = typename std::remove_pointer<decltype(dst)>::type;
#pragma unroll 4
      for (int ky = r0; ky < g.ny_out; ky += rstep) {
        dst[(long long)ky * g.K] = cvt2<OutT>(res[ky * g.tk + c]);
      }
      // outputs that are i kx times this one (inverse passes: the transform
      // is linear and kx is constant on a column)
      if constexpr (kDerive) for (int o2 = o + 1; o2 < NOUT; ++o2) {
        if (kind(o2) != 2 || op.from[o2] != o) continue;
        T2 cf;
        op.coef(grp, o2, op.from_in[o2], kx, 0, cf);
        auto* d2 = op.out_plane(grp, o2, li) + kx;
#pragma unroll 4
        for (int ky = r0; ky < g.ny_out; ky += rstep)
          d2[(long long)ky * g.K] = cvt2<OutT>(cmul(res[ky * g.tk + c], cf));
      }
    }
    __syncthreads();
  }
}

}  // namespace lesgo
