// Correctly rounded FP64 quotients a / b for divisors whose reciprocal is
// known, in multiplies and fused multiply-adds instead of a division.
//
// GB300's FP64 pipe runs at a small fraction of its FP32 rate, and a kernel
// that keeps the reference's divisions (to reproduce its doubles bit for bit)
// spends most of that pipe on them.  When y = RN(1/b) is at hand (computed
// once by an IEEE division, on the host for a constant divisor), RN(a/b)
// follows from Markstein's theorem (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990; stated as "Markstein's theorem" in Muller et al., Handbook of
// Floating-Point Arithmetic): if q is within one ulp of a/b and y is within
// half an ulp of 1/b, the remainder r = a - b q is exact under an FMA and
// RN(q + r y) = RN(a/b), barring underflow and overflow.  q0 = RN(a y) is only
// within two ulps, so one correction step first brings it within one ulp
// (q1 = RN(q0 + RN(a - b q0) y) errs by at most half an ulp plus 2^-51 ulp),
// and a second step, the theorem's, rounds correctly:
//     q0 = a y,  q1 = fma(fma(-b, q0, a), y, q0),  q2 = fma(fma(-b, q1, a), y, q1).
// Five FP64 operations.  The range guards keep every quantity normal: b and
// q0 within 2^-60..2^60 and 2^-900..2^900 in magnitude (exponent fields read
// with integer operations, off the FP64 pipe); anything else (zero, tiny or
// huge quotients, infinities, NaN) takes the plain division.  The kernels that
// use this are compared bit for bit with the oracle's divisions.
#pragma once

#include <cuda_runtime.h>

namespace gbmg {

__device__ __forceinline__ int fdiv_exp(double x) {
  return (__double2hiint(x) >> 20) & 0x7ff;
}

// y = RN(1/b), |b| in 2^-60..2^60 (checked by the caller)
__device__ __forceinline__ double div_known(double a, double b, double y) {
  const double q0 = __dmul_rn(a, y);
  const int e = fdiv_exp(q0);
  if (e < 1023 - 900 || e > 1023 + 900) return __ddiv_rn(a, b);
  const double q1 = __fma_rn(__fma_rn(-b, q0, a), y, q0);
  return __fma_rn(__fma_rn(-b, q1, a), y, q1);
}

// as div_known, with the range of b checked here (a divisor computed in the kernel)
__device__ __forceinline__ double div_known_checked(double a, double b, double y) {
  const int eb = fdiv_exp(b);
  if (eb < 1023 - 60 || eb > 1023 + 60) return __ddiv_rn(a, b);
  return div_known(a, b, y);
}

// the range condition on a constant divisor, for the host
inline bool fdiv_divisor_ok(double b) {
  const double m = b < 0 ? -b : b;
  return m >= 0x1p-60 && m <= 0x1p60;
}

}  // namespace gbmg
