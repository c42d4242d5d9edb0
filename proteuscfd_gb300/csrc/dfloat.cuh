// Double-float ("df") arithmetic: an unevaluated sum hi + lo of two FP32
// numbers, carrying about 48 significant bits.  GB300 issues 2 FP64 FMAs per
// SM per clock against 128 FP32 FMAs, so the FP64-bound residual kernels are
// written once, templated on the scalar type, and instantiated either with
// double (the reference precision) or with dfl, which runs the same algebra
// on the FP32 pipes.
//
// The error-free transformations are the standard ones (Dekker 1971;
// Knuth TAOCP vol. 2 sec. 4.2.2): TwoSum, FastTwoSum, and TwoProd through a
// fused multiply-add.  Addition keeps the hi parts exact and rounds the lo
// sum, so its absolute error is about 2^-48 of the operands, the same order
// as the FP64 rounding of the inputs themselves.  All primitives use the
// explicit round-to-nearest intrinsics, which the compiler never contracts
// or reassociates.
#pragma once

#include <cuda_runtime.h>

namespace pcfd {

// the FP64 overloads stay visible next to the dfl ones below
using ::fabs;
using ::isnan;
using ::sqrt;

struct __align__(8) dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl mkdf(float h, float l) {
  dfl r;
  r.hi = h;
  r.lo = l;
  return r;
}

// exact split of a double into hi + lo (the low 5 bits of the 53-bit
// significand are rounded away)
__device__ __forceinline__ dfl to_df(double x) {
  float h = __double2float_rn(x);
  return mkdf(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double to_dbl(dfl a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ dfl fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return mkdf(s, e);
}
__device__ __forceinline__ dfl two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return mkdf(s, e);
}

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  dfl s = two_sum(a.hi, b.hi);
  float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ dfl operator-(dfl a) { return mkdf(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  // q1 from the FP32 reciprocal, then one correction from the residual
  // a - q1 b, whose leading part is exact: about 2^-47 relative error
  float r = __frcp_rn(b.hi);
  float q1 = __fmul_rn(a.hi, r);
  float p = __fmul_rn(q1, b.hi);
  float pe = __fmaf_rn(q1, b.hi, -p);
  pe = __fmaf_rn(q1, b.lo, pe);
  dfl d = two_sum(a.hi, -p);
  float rr = __fadd_rn(d.hi, __fadd_rn(__fsub_rn(d.lo, pe), a.lo));
  return fast_two_sum(q1, __fmul_rn(rr, r));
}
// 2a and a/2, exact (both parts scale by a power of two); the same values
// as a multiplication by the constant, without its error terms
__device__ __forceinline__ dfl twice(dfl a) { return mkdf(2.0f * a.hi, 2.0f * a.lo); }
__device__ __forceinline__ double twice(double a) { return 2.0 * a; }
__device__ __forceinline__ dfl halve(dfl a) { return mkdf(0.5f * a.hi, 0.5f * a.lo); }
__device__ __forceinline__ double halve(double a) { return 0.5 * a; }
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl& operator*=(dfl& a, dfl b) { return a = a * b; }
__device__ __forceinline__ bool operator<(dfl a, dfl b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dfl a, dfl b) { return b < a; }
__device__ __forceinline__ bool operator<=(dfl a, dfl b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dfl a, dfl b) { return !(a < b); }
__device__ __forceinline__ bool operator==(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }

// hardware reciprocal approximation (PTX rcp.approx, at most 1 ulp off)
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// s = sqrt(hi) in FP32, then one Newton correction (a - s^2) / (2 s) whose
// residual a - s^2 is formed exactly; the correction is about 2^-24 of the
// result, so an FP32 approximation of 1 / (2 s) is enough for it
__device__ __forceinline__ dfl sqrt(dfl a) {
  if (!(a.hi > 0.0f)) return mkdf(__fsqrt_rn(a.hi), 0.0f);
  float s = __fsqrt_rn(a.hi);
  float p = __fmul_rn(s, s);
  float pe = __fmaf_rn(s, s, -p);
  dfl d = two_sum(a.hi, -p);
  float r = __fadd_rn(__fsub_rn(d.lo, pe), a.lo);
  r = __fadd_rn(d.hi, r);
  return fast_two_sum(s, __fmul_rn(r, __fmul_rn(0.5f, rcp_approx(s))));
}
__device__ __forceinline__ dfl fabs(dfl a) { return (a.hi < 0.0f) ? -a : a; }
__device__ __forceinline__ bool isnan(dfl a) { return ::isnan(a.hi) || ::isnan(a.lo); }

// ---- scalar traits -------------------------------------------------------
template <class S>
struct Sc;
template <>
struct Sc<double> {
  static __device__ __forceinline__ double c(double x) { return x; }
  static __device__ __forceinline__ double from(double x) { return x; }
  static __device__ __forceinline__ double to(double x) { return x; }
};
template <>
struct Sc<float> {
  static __device__ __forceinline__ float c(double x) { return (float)x; }
  static __device__ __forceinline__ float from(double x) { return (float)x; }
  static __device__ __forceinline__ double to(float x) { return (double)x; }
};
template <>
struct Sc<dfl> {
  // for literal arguments the casts fold at compile time
  static __device__ __forceinline__ dfl c(double x) {
    float h = (float)x;
    return mkdf(h, (float)(x - (double)h));
  }
  static __device__ __forceinline__ dfl from(double x) { return to_df(x); }
  static __device__ __forceinline__ double to(dfl x) { return to_dbl(x); }
};

}  // namespace pcfd
