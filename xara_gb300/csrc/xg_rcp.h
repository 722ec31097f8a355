// xg_rcp.h -- the reciprocal on the pivot chains of the LDL' kernels.
#pragma once

#include <cuda_runtime.h>

namespace xg {

// 1/d with a short dependency chain: d's leading 24 bits re-encoded as a
// single-precision number by integer arithmetic (the exponent rebiased from
// 1023 to 127, no conversion instruction), the single-precision hardware
// reciprocal of that, re-encoded as a double, then one step of the
// cubically convergent reciprocal iteration in FP64,
// x1 = x0 (1 + e + e^2) with e = 1 - d x0 (the order-3 member of
// Householder's family for f(x) = 1/x - d: A. S. Householder, The Numerical
// Treatment of a Single Nonlinear Equation, McGraw-Hill 1970; the
// truncated series of 1/(1 - e)).  The relative error of x1 is e^3 plus
// the rounding of the two FMAs, so the seed's ~22 correct bits become more
// than double precision.  Outside 2^-100 .. 2^100 in magnitude the
// correctly rounded reciprocal is used.  The stored reciprocal pivots of
// the factorisations are the correctly rounded ones; this one only scales
// the columns during elimination.  xg_chain_reciprocal_check evaluates it
// beside __drcp_rn for the error-bound test.
__device__ __forceinline__ double chain_reciprocal(double d) {
  const int hi = __double2hiint(d), lo = __double2loint(d);
  const int ahi = hi & 0x7fffffff;
  if (ahi < ((1023 - 100) << 20) || ahi >= ((1023 + 100) << 20)) return __drcp_rn(d);
  const unsigned fb = ((unsigned)hi & 0x80000000u) |
                      ((unsigned)(ahi - (896 << 20)) << 3) | ((unsigned)lo >> 29);
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__uint_as_float(fb)));
  const unsigned rb = __float_as_uint(r);
  const int rhi = (int)((rb & 0x80000000u) | (((rb & 0x7fffffffu) >> 3) + (896u << 20)));
  const int rlo = (int)(rb << 29);
  const double x = __hiloint2double(rhi, rlo);
  const double e = fma(-d, x, 1.0);
  return fma(x, fma(e, e, e), x);
}

}  // namespace xg
