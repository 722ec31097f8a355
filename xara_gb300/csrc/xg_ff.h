// xg_ff.h -- float-float arithmetic on the single-precision pipes.
//
// GB300's FP64 pipe retires a small fraction of the single-precision
// pipes' operations; where a long sum of products only has to be as
// accurate as FP64's own rounding allows (an SpMV, a tangent's sum over
// integration points), the products and sums run here on pairs of floats.
// A double v is kept as hi + lo, hi = v rounded to single precision and
// lo = (v - hi) rounded: 48 of its 53 bits.  A product of two such pairs is
// hi_a hi_x exactly (the rounding error of the single-precision product
// recovered by an FMA: Dekker's TwoProduct, 1971, with a fused
// multiply-add) plus the cross terms hi_a lo_x + lo_a hi_x in single
// precision (lo_a lo_x, below 2^-48 of the product, is dropped); sums add
// the high parts exactly (Knuth's TwoSum, TAOCP vol. 2, 4.2.2) and collect
// every error in the low part.  Each product is good to about 2^-46 of its
// magnitude.  __fmul_rn / __fadd_rn keep the compiler from fusing a product
// into the following addition, which would break the error-free
// transformations.
#pragma once

#include <cuda_runtime.h>

namespace xg {

__device__ __forceinline__ float2 split2(double v) {
  const float hi = __double2float_rn(v);
  return make_float2(hi, __double2float_rn(v - (double)hi));
}

// (sh, sl) += a * x
__device__ __forceinline__ void ff_madd(float2 a, float2 x, float &sh, float &sl) {
  const float p = __fmul_rn(a.x, x.x);
  float e = __fmaf_rn(a.x, x.x, -p);
  e = __fmaf_rn(a.x, x.y, e);
  e = __fmaf_rn(a.y, x.x, e);
  const float t = __fadd_rn(sh, p);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// Whether a value can enter a float-float product: zero, or 2^-50 <= |v|
// < 2^50.  A product of two such values lies in [2^-100, 2^100], its
// rounding error and cross terms (2^-24 and 2^-48 of it) stay normal
// single-precision numbers, and a sum of up to 2^20 of them stays finite.
__device__ __forceinline__ bool ff_range(double v) {
  const double a = fabs(v);
  return a == 0.0 || (a >= 0x1p-50 && a < 0x1p50);
}

// The pair as a double.
__device__ __forceinline__ double ff_value(float sh, float sl) { return (double)sh + (double)sl; }

}  // namespace xg
