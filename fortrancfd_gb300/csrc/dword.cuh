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

// The conversion-instruction paths of the two integer conversions below, for
// their rare inputs, as calls: an inlined fallback would be if-converted and
// its FP64-pipe instructions issued for every element.
static __device__ __noinline__ dw dw_from_double_rare(double x) { return dw_from_double(x); }
static __device__ __noinline__ double float_to_double_rare(float f) { return (double)f; }

// float(r) rounded to nearest even, for |r| <= 2^28, without a conversion
// instruction (GB300 runs those on its FP64 pipe): r = a 2^14 + c with
// |a| <= 2^14 and 0 <= c < 2^14; each part is exact as a float by the
// 1.5 * 2^23 bit-pattern offset, and a 2^14 + c is rounded once by the
// fused multiply-add.
__device__ __forceinline__ float int29_to_float(int r) {
  const int a = r >> 14;
  const int c = r & 0x3fff;
  const float fa = __int_as_float(0x4B400000 + a) - 12582912.0f;
  const float fc = __int_as_float(0x4B400000 + c) - 12582912.0f;
  return __fmaf_rn(fa, 16384.0f, fc);
}

// The same conversions with integer operations in place of the FP64
// conversion instructions, which GB300 runs at its FP64 rate (1/57 of FP32):
// results are bit-identical to dw_from_double / dw_to_double.
//
// dw_from_double_int: hi is x rounded to nearest-even at 24 bits, built from
// x's exponent and top significand bits; the remainder x - hi is the exact
// integer r = m - (top << 29) times 2^(e - 1075), and lo is r rounded to a
// float (an exact int -> float rounding, then an exact power-of-two
// scaling).  Inputs below 2^-74 (where lo could be subnormal) or near float
// overflow take the FP64 path; zeros give (+-0, +0) as dw_from_double does.
__device__ __forceinline__ dw dw_from_double_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned s = (unsigned)(b >> 63);
  if ((b << 1) == 0ull) return dw{__uint_as_float(s << 31), 0.f};
  const int e = (int)((b >> 52) & 0x7ffull);
  const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
  long long top = (long long)(m >> 29);
  const long long rb = (long long)(m & ((1ull << 29) - 1));
  top += (rb > (1ll << 28) || (rb == (1ll << 28) && (top & 1))) ? 1 : 0;
  const int carry = top == (1ll << 24) ? 1 : 0;
  const int fe = e - 896 + carry;
  if (e < 949 || fe > 254) return dw_from_double_rare(x);
  const unsigned hb =
      (s << 31) | ((unsigned)fe << 23) | ((unsigned)(carry ? (top >> 1) : top) & 0x7fffffu);
  const int r = (int)((long long)m - (top << 29));
  float lo = 0.f;
  if (r != 0) {
    lo = __int_as_float(__float_as_int(int29_to_float(r)) + (e - 1075) * (1 << 23));
    if (s) lo = -lo;
  }
  return dw{__uint_as_float(hb), lo};
}

// float -> double, exactly, by moving the exponent and significand bits
// (zeros included); subnormals, infinities and NaNs use the conversion.
__device__ __forceinline__ double float_to_double_int(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
  if ((u << 1) == 0u) return __longlong_as_double((long long)sgn);
  if (e == 0u || e == 255u) return float_to_double_rare(f);
  return __longlong_as_double((long long)(sgn | ((unsigned long long)(e + 896u) << 52) |
                                          ((unsigned long long)(u & 0x7fffffu) << 29)));
}

__device__ __forceinline__ double dw_to_double_int(dw a) {
  return float_to_double_int(a.hi) + float_to_double_int(a.lo);
}

// One flux term t = c (nb - pc), unnormalised (th + tl).  Every operation is
// sign-symmetric, so flux_term(c, pc, nb) is exactly -flux_term(c, nb, pc):
// a face's term can be computed once and used, negated, by its other cell.
__device__ __forceinline__ dw flux_term(dw c, dw nb, dw pc) {
  // d = nb - pc: TwoSum of the high parts plus the low parts, unnormalised
  const dw s = two_sum(nb.hi, -pc.hi);
  const float dlo = s.lo + (nb.lo - pc.lo);
  // t = c * d: TwoProd of the high parts plus the cross terms
  const float th = c.hi * s.hi;
  float tl = fmaf(c.hi, s.hi, -th);
  tl = fmaf(c.hi, dlo, tl);
  tl = fmaf(c.lo, s.hi, tl);
  return dw{th, tl};
}

// The residual b - sum_f t_f with cascaded summation started from b: the high
// parts are subtracted error-free with TwoSum, everything of order u|term|
// goes into one float.  Absolute error O(u^2 (|b| + sum |t_f|)), the bound
// the residual needs; the residual is needed only as a float (hi + lo), so
// no normalisation and no double-word subtraction follow.
struct residual_acc {
  float hi, lo;
  __device__ __forceinline__ explicit residual_acc(dw b) : hi(b.hi), lo(b.lo) {}
  // acc -= t
  __device__ __forceinline__ void sub(dw t) {
    const dw a = two_sum(hi, -t.hi);
    hi = a.hi;
    lo += a.lo - t.lo;
  }
  __device__ __forceinline__ float value_f() const { return hi + lo; }
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
