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

// df64 -> double in integer instructions, within one unit in the last place
// of the correctly rounded sum: hi's significand as a 53-bit integer plus
// or minus lo's, aligned to it (lo's bits below double precision are cut),
// renormalised by at most one place.  Pairs whose lo is not at least four
// times smaller than hi, and zero, denormal or non-finite hi, take the FP64
// add (rare in a sweep, whose pairs come from TwoSum).
__device__ __forceinline__ double df_to_double_int(DF v) {
  const unsigned uh = __float_as_uint(v.hi), ul = __float_as_uint(v.lo);
  const int eh = (int)((uh >> 23) & 0xffu), el = (int)((ul >> 23) & 0xffu);
  const int d = eh - el;
  if (eh == 0 || eh == 0xff || (el != 0 && d < 2)) return df_to_double(v);
  unsigned long long s = (unsigned long long)((uh & 0x7fffffu) | 0x800000u) << 29;
  if (el != 0) {
    const unsigned ml = (ul & 0x7fffffu) | 0x800000u;
    const unsigned long long lm = (d <= 29) ? ((unsigned long long)ml << (29 - d))
                                            : ((d < 61) ? (unsigned long long)(ml >> (d - 29)) : 0ULL);
    s = ((uh ^ ul) >> 31) ? s - lm : s + lm;
  }
  unsigned long long e = (unsigned long long)(eh + 896);
  if (s >> 53) {
    s >>= 1;
    e += 1;
  } else if (!(s >> 52)) {
    s <<= 1;
    e -= 1;
  }
  return __longlong_as_double(
      (long long)(((unsigned long long)(uh & 0x80000000u) << 32) | (e << 52) | (s & 0xfffffffffffffULL)));
}

// double -> df64 with FP64 instructions (exact split of the leading 48 bits;
// used once per factorisation on the factor tiles)
__device__ __forceinline__ DF df_from_double_fp64(double x) {
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - (double)hi);
  return DF{hi, lo};
}

}  // namespace gb
