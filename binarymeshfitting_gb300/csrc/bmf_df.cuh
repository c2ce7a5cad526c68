// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats with |lo| <= ulp(hi) / 2, about 48 significant bits.  The QEF adjoint
// uses it in place of FP64, whose rate on this GPU is a small fraction of the
// FP32 rate.  Algorithms: Dekker / Knuth error-free transformations (TwoSum,
// FastTwoSum, the product error from one fused multiply-add), as in D. H.
// Bailey's double-double and Hida-Li-Bailey's QD library papers; division and
// square root refine the float quotient / root with the exact residual.
//
// Must be compiled with FMA available (the error-free product uses fmaf); the
// sums use plain adds, which contraction never touches.
#pragma once

#include <cuda_runtime.h>

namespace bmf {
// DF and its functions live in their own namespace: sqrt / fabs of a DF are
// found by argument-dependent lookup, and do not hide the float / double
// ones for code in namespace bmf.
namespace dfl {

struct DF {
  float hi, lo;
  DF() = default;
  __host__ __device__ constexpr DF(float h, float l) : hi(h), lo(l) {}
  __device__ DF(float v) : hi(v), lo(0.0f) {}  // NOLINT: implicit, like a double from a float
  __device__ DF(int v) {  // exact for every 32-bit int
    hi = (float)v;
    lo = (float)(v - (int)hi);
  }
  __device__ DF(double v) {  // constants
    hi = (float)v;
    lo = (float)(v - (double)hi);
  }
  __device__ explicit operator float() const { return hi + lo; }
};

__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return DF(s, b - (s - a));
}
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return DF(s, (a - (s - bb)) + (b - bb));
}

__device__ __forceinline__ DF operator+(DF a, DF b) {
  DF s = df_two_sum(a.hi, b.hi);
  const DF t = df_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = df_fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ DF operator-(DF a) { return DF(-a.hi, -a.lo); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__device__ __forceinline__ DF operator*(DF a, DF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
// Division and square root are out of line: inlined at every use they made
// the adjoint kernel too large for the instruction cache.
// The three partial quotients use the fast float reciprocal: each only has to
// be within a few ulps, the residuals carry the rest.
static __device__ __noinline__ DF operator/(DF a, DF b) {
  const float ib = __frcp_rn(b.hi);
  const float q1 = a.hi * ib;
  const DF r = a - b * DF(q1, 0.0f);
  const float q2 = r.hi * ib;
  const DF r2 = r - b * DF(q2, 0.0f);
  const float q3 = r2.hi * ib;
  return df_fast_two_sum(q1, q2) + DF(q3, 0.0f);
}
__device__ __forceinline__ DF& operator+=(DF& a, DF b) { return a = a + b; }
__device__ __forceinline__ DF& operator-=(DF& a, DF b) { return a = a - b; }
__device__ __forceinline__ DF& operator*=(DF& a, DF b) { return a = a * b; }
__device__ __forceinline__ DF& operator/=(DF& a, DF b) { return a = a / b; }

__device__ __forceinline__ bool operator<(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(DF a, DF b) { return b < a; }
__device__ __forceinline__ bool operator<=(DF a, DF b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(DF a, DF b) { return !(a < b); }
__device__ __forceinline__ bool operator==(DF a, DF b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(DF a, DF b) { return !(a == b); }

__device__ __forceinline__ DF fabs(DF a) { return a.hi < 0.0f ? -a : a; }
static __device__ __noinline__ DF sqrt(DF a) {
  if (a.hi <= 0.0f) return DF(0.0f, 0.0f);
  const float s = sqrtf(a.hi);
  const DF r = a - DF(s, 0.0f) * DF(s, 0.0f);  // exact residual of the float root
  return df_fast_two_sum(s, r.hi / (2.0f * s));
}

}  // namespace dfl
using dfl::DF;
}  // namespace bmf
