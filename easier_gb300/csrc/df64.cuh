// Double-float ("df64") arithmetic: a value is an unevaluated sum hi + lo
// of two FP32 numbers with |lo| <= ulp(hi)/2, giving ~48 bits of
// significand on the FP32 pipes.  GB300 runs FP32 FMA at 59x its FP64 rate,
// so FP64-class vector arithmetic is cheaper this way.
//
// Building blocks (published error-free transformations):
//   two_sum        Knuth, TAOCP vol. 2, 4.2.2 (exact a + b = s + e)
//   quick_two_sum  Dekker 1971 (|a| >= |b|)
//   two_prod       exact a * b = p + e with one FMA (Ogita, Rump, Oishi 2005)
//   add / mul      the double-double add and mul of Hida, Li and Bailey,
//                  "Algorithms for quad-double precision floating point
//                  arithmetic" (2001), on FP32 pairs.
// Every operation uses explicit round-to-nearest intrinsics so the compiler
// cannot contract or reassociate the transformations.
#pragma once

#include <cstdint>

namespace df64 {

struct alignas(8) df {
  float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df{s, e};
}

__device__ __forceinline__ df quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return df{s, e};
}

__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  return df{p, e};
}

__device__ __forceinline__ df add(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return quick_two_sum(s.hi, e);
}

__device__ __forceinline__ df mul(df a, df b) {
  const df p = two_prod(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.lo, p.lo);
  e = __fmaf_rn(a.lo, b.hi, e);
  return quick_two_sum(p.hi, e);
}

__device__ __forceinline__ df fma(df a, df b, df c) { return add(mul(a, b), c); }

__device__ __forceinline__ df neg(df a) { return df{-a.hi, -a.lo}; }

__device__ __forceinline__ df from_double(double v) {
  const float hi = __double2float_rn(v);
  const float lo = __double2float_rn(v - (double)hi);
  return df{hi, lo};
}

__device__ __forceinline__ double to_double(df a) { return (double)a.hi + (double)a.lo; }

}  // namespace df64
