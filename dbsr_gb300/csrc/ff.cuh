// ff.cuh -- float-float arithmetic for the gather-sums of the split form.
//
// A value v is carried as two FP32 numbers (hi, lo) with hi = fl32(v) and
// lo = fl32(v - hi): 48 significant bits.  A gather-sum S = sum_e c_e K_e
// (25-60 terms here) is accumulated as
//   p  = hi(c) hi(K)                     rounded product
//   pe = fma(hi(c), hi(K), -p)           its exact rounding error (TwoProd)
//   x  = hi(c) lo(K) + lo(c) hi(K) + pe  the small terms, in FP32
//   (s_hi, e) = TwoSum(s_hi, p)          exact (Knuth, six additions)
//   s_lo += e + x
// so every product is exact to about 2^-48 of itself and the sum to about
// (terms) x 2^-48 of sum |c_e K_e| -- far inside the 1e-10 per-block bound of
// the split form, at FP32 instruction rates (GB300's FP64 pipe runs about
// 2 operations per clock per SM).  The compiler may contract a*b+c into
// FMA; the TwoSum contains no product, so contraction leaves it exact.
#pragma once
#include <cuda_runtime.h>

namespace ffa {

__device__ __forceinline__ float2 split(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}

__device__ __forceinline__ void mac(float2 c, float2 k, float &sh, float &sl) {
  const float p = c.x * k.x;
  const float pe = fmaf(c.x, k.x, -p);
  const float x = fmaf(c.x, k.y, fmaf(c.y, k.x, pe));
  const float s = sh + p;
  const float bp = s - sh;
  const float e = (sh - (s - bp)) + (p - bp);
  sh = s;
  sl = sl + (e + x);
}

// (sh, sl) += v for a float-float v (TwoSum of the high parts)
__device__ __forceinline__ void add(float2 v, float &sh, float &sl) {
  const float s = sh + v.x;
  const float bp = s - sh;
  const float e = (sh - (s - bp)) + (v.x - bp);
  sh = s;
  sl = sl + (e + v.y);
}

__device__ __forceinline__ double value(float sh, float sl) { return (double)sh + (double)sl; }

// (hi, lo) renormalised so that lo is below half an ulp of hi (Fast2Sum)
__device__ __forceinline__ float2 norm(float sh, float sl) {
  const float s = sh + sl;
  return make_float2(s, sl - (s - sh));
}

}  // namespace ffa
