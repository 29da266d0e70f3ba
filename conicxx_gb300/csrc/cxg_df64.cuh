// Double-float ("df64") arithmetic for the high-precision fallback factor of the mixed-precision
// path.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2, about 48
// significant bits. Everything runs on the FP32 pipe, which on GB300 has 64x the FP64 rate per
// SM, so a df64 LDL' costs about a quarter of an FP64 one while keeping the residual of an FP64
// factor to within a small factor. The FP64 iterative refinement on top is unchanged.
//
// Building blocks (published error-free transformations; every float operation is an explicitly
// rounded intrinsic so that the compiler cannot contract a product into a following sum, which
// would break the error terms):
//  - TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s + e = a + b exactly, for any a, b.
//  - Fast2Sum (Dekker 1971): the same when |a| >= |b|; used to renormalise (hi, lo).
//  - TwoProduct with FMA: p + e = a * b exactly, e = fma(a, b, -p).
// Addition and multiplication follow the usual double-word algorithms (one TwoSum or TwoProduct
// of the high parts, the low-order terms added in float, one renormalisation). Division is one
// step of long division: q1 = a.hi / b.hi, then q2 from the df64 remainder a - q1 b.
#pragma once

#include <cuda_runtime.h>

namespace cxg {

struct df64 {
  float hi, lo;
  df64() = default;
  __device__ __forceinline__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ explicit df64(double d) {
    hi = __double2float_rn(d);
    lo = __double2float_rn(d - (double)hi);
  }
  __device__ __forceinline__ explicit df64(int v) : df64((double)v) {}
  __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ void dfTwoSum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bv = __fsub_rn(s, a);
  const float av = __fsub_rn(s, bv);
  e = __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
}

__device__ __forceinline__ void dfFastTwoSum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  float s, e, h, l;
  dfTwoSum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  dfFastTwoSum(s, e, h, l);
  return df64(h, l);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float h, l;
  dfFastTwoSum(p, e, h, l);
  return df64(h, l);
}

__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df64 r = a - df64(q1, 0.0f) * b;
  const float q2 = __fdiv_rn(r.hi, b.hi);
  float h, l;
  dfFastTwoSum(q1, q2, h, l);
  return df64(h, l);
}

// c + a * b with one renormalisation: the exact product of the high parts (TwoProduct), the
// cross terms folded into its error, then one TwoSum with c.hi (15 float operations instead of
// the 18 of a separate multiply and add).
__device__ __forceinline__ df64 dfMad(df64 c, df64 a, df64 b) {
  const float ph = __fmul_rn(a.hi, b.hi);
  float pl = __fmaf_rn(a.hi, b.hi, -ph);
  pl = __fmaf_rn(a.hi, b.lo, pl);
  pl = __fmaf_rn(a.lo, b.hi, pl);
  float s, e, h, l;
  dfTwoSum(c.hi, ph, s, e);
  e = __fadd_rn(e, __fadd_rn(c.lo, pl));
  dfFastTwoSum(s, e, h, l);
  return df64(h, l);
}

// Accumulation form of dfMad for long sums (tile products): the exact TwoSum of the high parts
// is kept, the low-order terms are added in float without renormalising (12 float operations);
// dfNorm renormalises once at the end. The low part only ever holds rounding terms of the high
// part's sums, so it stays small relative to it.
__device__ __forceinline__ df64 dfMadLoose(df64 c, df64 a, df64 b) {
  const float ph = __fmul_rn(a.hi, b.hi);
  float pl = __fmaf_rn(a.hi, b.hi, -ph);
  pl = __fmaf_rn(a.hi, b.lo, pl);
  pl = __fmaf_rn(a.lo, b.hi, pl);
  float s, e;
  dfTwoSum(c.hi, ph, s, e);
  return df64(s, __fadd_rn(c.lo, __fadd_rn(e, pl)));
}
__device__ __forceinline__ df64 dfNorm(df64 c) {
  float h, l;
  dfFastTwoSum(c.hi, c.lo, h, l);
  return df64(h, l);
}

__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }
__device__ __forceinline__ df64& operator/=(df64& a, df64 b) { return a = a / b; }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

}  // namespace cxg
