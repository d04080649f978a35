// df32: a real stored as an unevaluated sum hi + lo of two FP32 numbers ("double-float",
// |lo| <= ulp(hi)/2), with every operation built from FP32 instructions.  About 48 significant
// bits: unit roundoff u^2 = 2^-48 ~ 3.6e-15 per operation.  On GB300 the FP32 pipes issue
// roughly 60x more operations per second than FP64, so a df32 operation (7 to 20 FP32
// instructions) costs several times less than a native FP64 one.
//
// Algorithms (published error-free transformations, written here from their definitions):
//   two_sum        Knuth, TAOCP vol. 2: s = fl(a+b) and the exact error e, a + b = s + e
//   fast_two_sum   Dekker 1971: the same when |a| >= |b| (3 operations)
//   two_prod       with one fused multiply-add: p = fl(ab), e = fma(a, b, -p), ab = p + e
//   add            Joldes, Muller, Popescu, ACM TOMS 44(2), 2017, "accurate DW + DW"
//                  (relative error <= 3u^2 + 13u^3)
//   mul            the same paper, "DW x DW" with FMA, low-order product dropped (<= 5u^2)
//   div            one float quotient, its remainder in double-word, a second float quotient
//   sqrt           one Newton correction of the float square root (Karp and Markstein 1997)
// The device compiler does not reassociate FP32 additions, so the error-free transformations
// hold as written; the products inside them are explicit fmaf calls.
#pragma once
#include <cmath>
#include <cuda_runtime.h>

namespace dgadv {

// The overloads below sit beside, not in place of, the float and double functions.
using ::fabs;
using ::fmax;
using ::fmin;
using ::sqrt;
using ::__shfl_xor_sync;

struct df32 {
  float hi, lo;
  df32() = default;
  __host__ __device__ constexpr df32(float h, float l) : hi(h), lo(l) {}
  // explicit only: a float, double or int never turns into a df32 without being asked to
  __host__ __device__ constexpr explicit df32(float x) : hi(x), lo(0.0f) {}
  __host__ __device__ constexpr explicit df32(int x) : hi((float)x), lo(0.0f) {}
  // nearest pair: hi = fl32(x), lo = fl32(x - hi) (x - hi is exact in FP64)
  __host__ __device__ explicit df32(double x) : hi((float)x), lo(0.0f) {
    if (x - x == 0.0) lo = (float)(x - (double)hi);   // finite x only
  }
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

namespace df {

__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__host__ __device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  e = b - (s - a);
}
__host__ __device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = a * b;
  e = fmaf(a, b, -p);
}

}  // namespace df

__host__ __device__ __forceinline__ df32 operator-(const df32 &a) { return df32(-a.hi, -a.lo); }

__host__ __device__ __forceinline__ df32 operator+(const df32 &a, const df32 &b) {
  float sh, sl, th, tl, vh, vl, zh, zl;
  df::two_sum(a.hi, b.hi, sh, sl);
  df::two_sum(a.lo, b.lo, th, tl);
  df::fast_two_sum(sh, sl + th, vh, vl);
  df::fast_two_sum(vh, tl + vl, zh, zl);
  return df32(zh, zl);
}
__host__ __device__ __forceinline__ df32 operator-(const df32 &a, const df32 &b) { return a + (-b); }

__host__ __device__ __forceinline__ df32 operator*(const df32 &a, const df32 &b) {
  float ch, cl, zh, zl;
  df::two_prod(a.hi, b.hi, ch, cl);
  const float cross = fmaf(a.lo, b.hi, a.hi * b.lo);
  df::fast_two_sum(ch, cl + cross, zh, zl);
  return df32(zh, zl);
}

__host__ __device__ __forceinline__ df32 operator/(const df32 &a, const df32 &b) {
  const float q1 = a.hi / b.hi;
  if (!(q1 - q1 == 0.0f)) return df32(q1, 0.0f);          // inf / nan / division by zero
  // remainder a - q1 * b in double-word
  float ph, pl;
  df::two_prod(q1, b.hi, ph, pl);
  pl = fmaf(q1, b.lo, pl);
  const df32 r = a - df32(ph, pl);
  const float q2 = r.hi / b.hi;
  float zh, zl;
  df::fast_two_sum(q1, q2, zh, zl);
  return df32(zh, zl);
}

__host__ __device__ __forceinline__ df32 &operator+=(df32 &a, const df32 &b) { return a = a + b; }
__host__ __device__ __forceinline__ df32 &operator-=(df32 &a, const df32 &b) { return a = a - b; }
__host__ __device__ __forceinline__ df32 &operator*=(df32 &a, const df32 &b) { return a = a * b; }

// Ordering of normalised pairs: by hi, then by lo.
__host__ __device__ __forceinline__ bool operator<(const df32 &a, const df32 &b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__host__ __device__ __forceinline__ bool operator>(const df32 &a, const df32 &b) { return b < a; }
__host__ __device__ __forceinline__ bool operator<=(const df32 &a, const df32 &b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}
__host__ __device__ __forceinline__ bool operator>=(const df32 &a, const df32 &b) { return b <= a; }
__host__ __device__ __forceinline__ bool operator==(const df32 &a, const df32 &b) {
  return a.hi == b.hi && a.lo == b.lo;
}
__host__ __device__ __forceinline__ bool operator!=(const df32 &a, const df32 &b) { return !(a == b); }

__host__ __device__ __forceinline__ df32 fabs(const df32 &a) { return (a.hi < 0.0f) ? -a : a; }
__host__ __device__ __forceinline__ bool isnan_(const df32 &a) { return a.hi != a.hi; }
// NaN-ignoring minimum / maximum like fmin / fmax (and Matlab's min / max)
__host__ __device__ __forceinline__ df32 fmin(const df32 &a, const df32 &b) {
  if (isnan_(a)) return b;
  if (isnan_(b)) return a;
  return (b < a) ? b : a;
}
__host__ __device__ __forceinline__ df32 fmax(const df32 &a, const df32 &b) {
  if (isnan_(a)) return b;
  if (isnan_(b)) return a;
  return (a < b) ? b : a;
}
__host__ __device__ __forceinline__ df32 sqrt(const df32 &a) {
  if (!(a.hi > 0.0f)) return df32(sqrtf(a.hi), 0.0f);     // 0, negative or nan
  const float s = sqrtf(a.hi);
  float p, pe;
  df::two_prod(s, s, p, pe);
  const float r = ((a.hi - p) - pe) + a.lo;                // a - s^2, to first order
  float zh, zl;
  df::fast_two_sum(s, r / (2.0f * s), zh, zl);
  return df32(zh, zl);
}

__device__ __forceinline__ df32 __shfl_xor_sync(unsigned mask, const df32 &v, int lane) {
  return df32(::__shfl_xor_sync(mask, v.hi, lane), ::__shfl_xor_sync(mask, v.lo, lane));
}

}  // namespace dgadv
