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
// A double is split into a pair by bit manipulation (no FP64 instruction);
// a pair goes back to FP64 as its two floats widened by rebuilding their
// exponent fields and added once in FP64 (measured faster, in the sweeps,
// than an all-integer conversion, which costs the chain's warp more issue
// slots than the one FP64 add does).  Values
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

// double -> df64 by bit manipulation, without branches or conversion
// instructions: hi keeps the top 24 significant bits (truncated); lo the next
// 23 of the remaining 29, built as the difference of two floats that share
// hi's scale (2^(E-23) * 1.m - 2^(E-23), exact by Sterbenz), so the error is
// below 2^-47 relative.  Magnitudes below 2^-126 give zero (lo is zero below
// 2^-103); from 2^128 +-inf; NaN stays NaN.
__device__ __forceinline__ DF df_from_double(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned h = (unsigned)(u >> 32), l = (unsigned)u;
  const unsigned sign = h & 0x80000000u;
  const int e = (int)((h >> 20) & 0x7ffu);
  const int ef = e - 1023 + 127;
  const unsigned mh = ((h & 0xfffffu) << 3) | (l >> 29);
  unsigned hb = sign | ((unsigned)ef << 23) | mh;
  const unsigned base = (unsigned)(ef - 23) << 23;
  float lo = __fsub_rn(__uint_as_float(base | ((l & 0x1fffffffu) >> 6)), __uint_as_float(base));
  lo = (ef > 23 && ef < 255) ? lo : 0.0f;
  const bool nan = (e == 0x7ff) && (((h & 0xfffffu) | l) != 0u);
  hb = (ef <= 0) ? sign : hb;
  hb = (ef >= 255) ? (sign | (nan ? 0x7fc00000u : 0x7f800000u)) : hb;
  return DF{__uint_as_float(hb), __uint_as_float(__float_as_uint(lo) | sign)};
}

// float -> double bits, exact for normal floats and zero (denormal floats
// give zero), with integer instructions and selects only
__device__ __forceinline__ double df_widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long man = (unsigned long long)(u & 0x7fffffu) << 29;
  unsigned long long bits = sign | ((unsigned long long)(e + 896u) << 52) | man;
  bits = (e == 0u) ? sign : bits;
  bits = (e == 0xffu) ? (sign | 0x7ff0000000000000ULL | man) : bits;
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
