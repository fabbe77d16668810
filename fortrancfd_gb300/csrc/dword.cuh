// Double-word ("float-float") arithmetic on the FP32 pipes.
//
// A value is hi + lo with two floats, |lo| <= ulp(hi)/2: about 48 significant
// bits.  GB300 runs FP32 at 57x its FP64 rate (68.6 vs 1.20 TFLOP/s measured),
// so the FP64-accuracy parts of the mixed-precision solve (residual of the
// FP64 operator, p += e) use these instead of native doubles.  The error-free
// transformations are the textbook ones: TwoSum (Knuth, TAOCP vol. 2,
// 4.2.2), Fast2Sum (Dekker 1971), and TwoProd with a fused multiply-add
// (error term fma(a, b, -ab)).  Sums use the "sloppy" double-word addition,
// whose absolute error is at most about 2u^2(|a| + |b|) (u = 2^-24); that is
// all the residual needs, because its accuracy is measured against the size
// of the flux terms, not of their sum.
#pragma once

#include <cuda_runtime.h>

namespace gbmg {

struct dw {
  float hi, lo;
};

__device__ __forceinline__ dw two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return dw{s, e};
}

__device__ __forceinline__ dw fast_two_sum(float a, float b) {  // needs |a| >= |b| or a == 0
  const float s = a + b;
  return dw{s, b - (s - a)};
}

__device__ __forceinline__ dw dw_add(dw a, dw b) {
  dw s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ dw dw_neg(dw a) { return dw{-a.hi, -a.lo}; }

__device__ __forceinline__ dw dw_sub(dw a, dw b) { return dw_add(a, dw_neg(b)); }

__device__ __forceinline__ dw dw_add_f(dw a, float b) {
  dw s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ dw dw_mul(dw a, dw b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ float dw_to_float(dw a) { return a.hi + a.lo; }

__device__ __forceinline__ dw dw_from_double(double x) {
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - (double)hi);
  return dw{hi, lo};
}

__device__ __forceinline__ double dw_to_double(dw a) { return (double)a.hi + (double)a.lo; }

// Accumulator of sum_f c_f (p_nb - p_c) with cascaded summation: the high
// parts are added error-free with TwoSum, everything of order u|term| goes
// into one float.  Absolute error O(u^2 sum |c_f (p_nb - p_c)|), the bound the
// residual needs; about 19 FP32 operations per term instead of ~30 with the
// normalised double-word operations.
struct flux_acc {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add_term(dw c, dw nb, dw pc) {
    // d = nb - pc: TwoSum of the high parts plus the low parts, unnormalised
    const dw s = two_sum(nb.hi, -pc.hi);
    const float dlo = s.lo + (nb.lo - pc.lo);
    // t = c * d: TwoProd of the high parts plus the cross terms
    const float th = c.hi * s.hi;
    float tl = fmaf(c.hi, s.hi, -th);
    tl = fmaf(c.hi, dlo, tl);
    tl = fmaf(c.lo, s.hi, tl);
    // acc += t
    const dw a = two_sum(hi, th);
    hi = a.hi;
    lo += a.lo + tl;
  }
  __device__ __forceinline__ dw value() const { return fast_two_sum(hi, lo); }
};

__device__ __forceinline__ dw dw_load(const float2* p) {
  const float2 v = *p;
  return dw{v.x, v.y};
}

__device__ __forceinline__ dw dw_ldg(const float2* p) {
  const float2 v = __ldg(p);
  return dw{v.x, v.y};
}

__device__ __forceinline__ void dw_store(float2* p, dw a) { *p = make_float2(a.hi, a.lo); }

}  // namespace gbmg
