// k_df64.cuh -- double-float ("df64") arithmetic for the FP64 wavefront
// sweeps.
//
// GB300 issues an FP64 FMA for a warp about every 64 cycles per SM
// sub-partition, so a dependency chain of FP64 FMAs advances at that pace no
// matter how few lanes are active.  The FP32 pipe is 64 times wider.  A value
// here is an unevaluated sum hi + lo of two floats (Dekker's double-length
// arithmetic): products are split exactly with an FMA (p = a*b rounded,
// e = fma(a, b, -p)) and sums exactly with Knuth's TwoSum, which keeps about
// 48 significant bits -- relative error about 2^-47 per operation, against
// 2^-53 for FP64 -- with the chain of a step on the FP32 pipe.
//
// The pairs are not renormalised after each operation: |lo| stays within a
// few ulps of hi, which is all the next product needs.  Explicit _rn
// intrinsics keep the compiler from contracting the error terms.
//
// Conversions to and from FP64 use integer instructions where they sit on a
// hot path (no FP64 instruction per element): a double is split by bit
// manipulation, a float is widened by rebuilding its exponent field.  Values
// whose magnitude lies outside [2^-100, 2^100] do not keep their accuracy
// (the float exponent range); the factor tiles are checked against that
// range before the df64 sweeps are used.
#pragma once
#include <cuda_runtime.h>

namespace gb {

struct __align__(8) DF {
  float hi, lo;
};

__device__ __forceinline__ DF df_zero() { return DF{0.0f, 0.0f}; }

// c - a*b
__device__ __forceinline__ DF df_fms(DF a, DF b, DF c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // a.hi*b.hi = p + e exactly
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  // s + t = c.hi - p exactly (TwoSum)
  const float s = __fsub_rn(c.hi, p);
  const float bb = __fsub_rn(s, c.hi);
  float t = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(-p, bb));
  t = __fadd_rn(t, __fsub_rn(c.lo, e));
  return DF{s, t};
}

// a*b
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return DF{p, e};
}

__device__ __forceinline__ DF df_shfl_up(DF v, int d) {
  return DF{__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d)};
}

// double -> df64 by bit manipulation: hi keeps the top 24 significant bits
// (truncated), lo the next 29 rounded to float.  Zero, denormal doubles and
// magnitudes below 2^-126 give zero; magnitudes from 2^128 give +-inf; NaN
// stays NaN.
__device__ __forceinline__ DF df_from_double(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned h = (unsigned)(u >> 32), l = (unsigned)u;
  const unsigned sign = h & 0x80000000u;
  const int e = (int)((h >> 20) & 0x7ffu);
  const int ef = e - 1023 + 127;
  if (e == 0x7ff)  // inf keeps its sign; any NaN becomes a quiet NaN
    return DF{__uint_as_float(sign | (((h & 0xfffffu) | l) ? 0x7fc00000u : 0x7f800000u)), 0.0f};
  if (ef <= 0) return DF{__uint_as_float(sign), 0.0f};
  if (ef >= 255) return DF{__uint_as_float(sign | 0x7f800000u), 0.0f};
  const unsigned mh = ((h & 0xfffffu) << 3) | (l >> 29);
  const float hi = __uint_as_float(sign | ((unsigned)ef << 23) | mh);
  // lo = (l & (2^29 - 1)) * 2^(e - 1075), scaled in two steps so that the
  // intermediate stays a normal float
  const unsigned rem = l & 0x1fffffffu;
  float lo = 0.0f;
  const int s1 = e - 1075 + 64 + 127;  // biased exponent of 2^(e - 1075 + 64)
  if (rem != 0u && s1 > 0) {
    lo = __fmul_rn(__uint2float_rn(rem), __uint_as_float((unsigned)s1 << 23));
    lo = __fmul_rn(lo, 5.421010862427522e-20f);  // 2^-64
    lo = __uint_as_float(__float_as_uint(lo) | sign);
  }
  return DF{hi, lo};
}

// float -> double bits, exact for normal floats and zero (denormal floats
// give zero), with integer instructions only
__device__ __forceinline__ double df_widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u) return __longlong_as_double((long long)sign);
  if (e == 0xffu)
    return __longlong_as_double((long long)(sign | 0x7ff0000000000000ULL |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
  const unsigned long long bits =
      sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// df64 -> double: the two widened halves added once in FP64
__device__ __forceinline__ double df_to_double(DF v) {
  return __dadd_rn(df_widen(v.hi), df_widen(v.lo));
}

// double -> df64 with FP64 instructions (exact split of the leading 48 bits;
// used once per factorisation on the factor tiles)
__device__ __forceinline__ DF df_from_double_fp64(double x) {
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - (double)hi);
  return DF{hi, lo};
}

}  // namespace gb
