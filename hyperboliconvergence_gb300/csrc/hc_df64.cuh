// hc_df64.cuh -- double-float arithmetic: a value is the unevaluated sum
// hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2, giving a ~48-bit
// significand (relative rounding ~2^-47) computed entirely on the FP32 pipes.
//
// Algorithms: error-free transformations of Knuth (TwoSum, TAOCP vol. 2,
// 4.2.2) and Dekker ("A floating-point technique for extending the available
// precision", Numer. Math. 18, 1971; Fast2Sum), products through the fused
// multiply-add (the residual a*b - fl(a*b) is one FMA), division by two
// remainder corrections of an FP32 quotient estimate and square root by one
// Newton correction of the FP32 root (Karp & Markstein, "High-precision division
// and square root", ACM TOMS 23(4), 1997).  The exponent range is FP32's.
//
// Written for __host__ and __device__ so the same code is testable on a CPU.
// The type and its functions live in hc::dd and are found by argument-dependent
// lookup, so code in namespace hc keeps calling the global sqrt/fabs/fmax for
// double and float.
#pragma once

#include <cfloat>
#include <cmath>
#include <cuda_runtime.h>

namespace hc {
namespace dd {

struct df64 {
  float hi, lo;
  __host__ __device__ constexpr df64() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  // split of a double: hi = rn(x), lo = rn(x - hi); exact for |x| in FP32 range
  __host__ __device__ constexpr df64(double x) : hi(float(x)), lo(float(x - double(float(x)))) {}
  __host__ __device__ constexpr df64(int x) : df64(double(x)) {}
  __host__ __device__ double to_double() const { return double(hi) + double(lo); }
};

__host__ __device__ __forceinline__ float df_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

// s + e == a + b exactly (Knuth)
__host__ __device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return df64(s, e);
}
// s + e == a + b exactly when |a| >= |b| (Dekker)
__host__ __device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  const float s = a + b;
  const float e = b - (s - a);
  return df64(s, e);
}

// One TwoSum on the high parts, the low parts added in FP32: the error is bounded
// by ~2^-47 (|a| + |b|), relative to the operands rather than to the sum (the
// form with a second TwoSum on the low parts is relative to the sum but costs
// twice the instructions; no quantity of the stage needs more than
// operand-relative accuracy in a difference).
__host__ __device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__host__ __device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__host__ __device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = df_fma(a.hi, b.hi, -p);
  e = df_fma(a.hi, b.lo, e);
  e = df_fma(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ df64 mul_f(df64 a, float b) {
  const float p = a.hi * b;
  float e = df_fma(a.hi, b, -p);
  e = df_fma(a.lo, b, e);
  return fast_two_sum(p, e);
}
// FP32 reciprocal estimate of b.hi from the approximate-reciprocal instruction
__host__ __device__ __forceinline__ float approx_rcp(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;
#endif
}
// Quotient estimate q1 = a.hi / b.hi from the reciprocal estimate, then two
// corrections by the remainders a - b q (Karp & Markstein): each multiplies the
// relative error by that of the estimate (~2^-22), ending near 2^-47.
__host__ __device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  // the approximate reciprocal flushes subnormal inputs and results: take it of
  // b.hi scaled by a power of two into range, then undo the scaling (exact)
  const float bh = fabsf(b.hi);
  const float sc = bh > 0x1p125f ? 0x1p-64f : (bh < 0x1p-125f ? 0x1p64f : 1.0f);
  const float rb = approx_rcp(b.hi * sc) * sc;
  const float q1 = a.hi * rb;
  const df64 r = a - mul_f(b, q1);
  const float q2 = r.hi * rb;
  const df64 q = fast_two_sum(q1, q2);
  const df64 r2 = a - b * q;
  return fast_two_sum(q.hi, q.lo + r2.hi * rb);
}
__host__ __device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__host__ __device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }
__host__ __device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }

__host__ __device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__host__ __device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__host__ __device__ __forceinline__ bool operator<=(df64 a, df64 b) { return !(b < a); }
__host__ __device__ __forceinline__ bool operator>=(df64 a, df64 b) { return !(a < b); }
__host__ __device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }

__host__ __device__ __forceinline__ df64 fabs(df64 a) { return a.hi < 0.f ? -a : a; }
__host__ __device__ __forceinline__ df64 fmax(df64 a, df64 b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ df64 fmin(df64 a, df64 b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ df64 sqrt(df64 a) {
  if (!(a.hi > 0.f)) return df64(a.hi == 0.f ? 0.f : NAN, 0.f);
  const float s = sqrtf(a.hi);
  const float p = s * s;
  const float pe = df_fma(s, s, -p);
  const float e = ((a.hi - p) - pe + a.lo) * (0.5f / s);
  return fast_two_sum(s, e);
}
__host__ __device__ __forceinline__ bool isfinite(df64 a) { return ::isfinite(a.hi); }

}  // namespace dd
using dd::df64;
}  // namespace hc
