// Double-float ("double-word") arithmetic: a value held as the unevaluated
// sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2, about 48
// significand bits.  GB300 executes FP64 at 1/64 of its FP32 rate, so the
// double-word form's transforms run their butterflies in this arithmetic on
// the FP32 pipe and keep FP64 for storage and for every pointwise stage.
//
// The building blocks are the published error-free transformations and
// double-word algorithms:
//   * TwoSum (Knuth, TAOCP vol. 2) and FastTwoSum (Dekker 1971): s + e = a + b
//     exactly;
//   * TwoProd with a fused multiply-add (p = a b, e = fma(a, b, -p)):
//     p + e = a b exactly;
//   * double-word + double-word: the "sloppy" sum (TwoSum of the high parts,
//     the low parts added, one renormalisation), whose error is bounded by
//     a small multiple of 2^-48 (|x| + |y|): the norm-wise bound an FFT's
//     error analysis uses (Joldes, Muller and Popescu, "Tight and rigorous
//     error bounds for basic building blocks of double-word arithmetic",
//     ACM TOMS 44(2), 2017, algorithms 5 and 11);
//   * double-word x double-word with an FMA (the same paper's DWTimesDW).
// Every operation is written out with intrinsics that round to nearest and
// are never contracted, so the compiler cannot fuse or reorder the steps
// that make the transformations exact.
#pragma once
#include <cuda_runtime.h>

namespace lesgo {

struct df64 {
  float hi, lo;
};

// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// the same for |a| >= |b| (or a = 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ df64 operator+(df64 x, df64 y) {
  float sh, sl;
  two_sum(x.hi, y.hi, sh, sl);
  sl = __fadd_rn(sl, __fadd_rn(x.lo, y.lo));
  df64 z;
  fast_two_sum(sh, sl, z.hi, z.lo);
  return z;
}
__device__ __forceinline__ df64 operator-(df64 x) { return df64{-x.hi, -x.lo}; }
__device__ __forceinline__ df64 operator-(df64 x, df64 y) { return x + (-y); }

__device__ __forceinline__ df64 operator*(df64 x, df64 y) {
  const float ch = __fmul_rn(x.hi, y.hi);
  const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
  const float tl = __fmul_rn(x.hi, y.lo);
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl);
  const float cl3 = __fadd_rn(cl1, cl2);
  df64 z;
  fast_two_sum(ch, cl3, z.hi, z.lo);
  return z;
}

// FP64 <-> double-word: the high part is the FP64 value rounded to FP32, the
// low part the rounded remainder (exact in FP64).  Values here stay far from
// FP32's range limits (velocities, their products and transforms of them).
__device__ __forceinline__ df64 df_from(double d) {
  const float h = __double2float_rn(d);
  return df64{h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double df_to(df64 x) { return (double)x.hi + (double)x.lo; }

}  // namespace lesgo
