// k_llword.cuh -- result words tagged with the epoch of the launch that
// wrote them, for kernels whose CTAs hand values to one another without
// fences or progress counters (the wavefront and level sweeps).
#pragma once
#include <cuda_runtime.h>

#include "k_df64.cuh"

namespace gb {

// Every spin-wait is bounded by the SM's cycle counter: 4e9 cycles, about
// 2 s at the GB300's 2.07 GHz maximum (longer at lower clocks, never
// unbounded).  The cycle counter is read in a few cycles; the global timer,
// read on every turn of a wait loop, delayed each wait's exit by far more
// than the hand-off it waited for.
constexpr unsigned long long kWaitCycles = 4000000000ULL;

__device__ __forceinline__ unsigned long long wclock() { return (unsigned long long)clock64(); }

// One result element with its sweep epoch.  The epoch travels in the same
// naturally aligned 8-byte access as the data it guards (FP64: both halves
// carry it), so a consumer that reads the current epoch holds the value:
// no fence and no progress counter stand between producer and consumer.
template <typename T>
struct LLWord;
template <>
struct alignas(16) LLWord<double> { unsigned long long v[2]; };
template <>
struct alignas(8) LLWord<float> { unsigned long long v; };
// df64: hi and lo each with the epoch in the upper half of its 8 bytes
template <>
struct alignas(16) LLWord<DF> { unsigned long long v[2]; };

// The stores carry no compiler memory clobber: nothing the writing thread
// does afterwards depends on their order, and shared-memory loads of the
// next steps may then be issued ahead of them.
__device__ __forceinline__ void ll_put(LLWord<double> *p, double x, unsigned ep) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long f = (unsigned long long)ep << 32;
  asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(p), "l"((b & 0xffffffffULL) | f),
               "l"((b >> 32) | f));
}
__device__ __forceinline__ void ll_put(LLWord<float> *p, float x, unsigned ep) {
  const unsigned long long v = (unsigned long long)__float_as_uint(x) | ((unsigned long long)ep << 32);
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v));
}
__device__ __forceinline__ void ll_put(LLWord<DF> *p, DF x, unsigned ep) {
  const unsigned long long f = (unsigned long long)ep << 32;
  asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(p),
               "l"((unsigned long long)__float_as_uint(x.hi) | f),
               "l"((unsigned long long)__float_as_uint(x.lo) | f));
}
__device__ __forceinline__ bool ll_get(const LLWord<DF> *p, unsigned ep, DF &x) {
  unsigned long long a, b;
  asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
  x = DF{__uint_as_float((unsigned)a), __uint_as_float((unsigned)b)};
  return (unsigned)(a >> 32) == ep && (unsigned)(b >> 32) == ep;
}
__device__ __forceinline__ bool ll_get(const LLWord<double> *p, unsigned ep, double &x) {
  unsigned long long a, b;
  asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
  x = __longlong_as_double((long long)((a & 0xffffffffULL) | (b << 32)));
  return (unsigned)(a >> 32) == ep && (unsigned)(b >> 32) == ep;
}
__device__ __forceinline__ bool ll_get(const LLWord<float> *p, unsigned ep, float &x) {
  unsigned long long a;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(a) : "l"(p) : "memory");
  x = __uint_as_float((unsigned)a);
  return (unsigned)(a >> 32) == ep;
}
// The value of a word known to be complete (read by a later kernel, or
// staged in shared memory after its kernel ended).
__device__ __forceinline__ double ll_val(const LLWord<double> &w) {
  return __longlong_as_double((long long)((w.v[0] & 0xffffffffULL) | (w.v[1] << 32)));
}
__device__ __forceinline__ float ll_val(const LLWord<float> &w) { return __uint_as_float((unsigned)w.v); }
__device__ __forceinline__ DF ll_val(const LLWord<DF> &w) {
  return DF{__uint_as_float((unsigned)w.v[0]), __uint_as_float((unsigned)w.v[1])};
}

// A word loaded ahead of its use: the load is issued now and its epoch is
// checked later, so that several chunks' loads are in flight at once.
struct LLRaw {
  unsigned long long a, b;
};
__device__ __forceinline__ void ll_issue(const LLWord<double> *p, LLRaw &r) {
  asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(r.a), "=l"(r.b) : "l"(p) : "memory");
}
__device__ __forceinline__ void ll_issue(const LLWord<DF> *p, LLRaw &r) {
  asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(r.a), "=l"(r.b) : "l"(p) : "memory");
}
__device__ __forceinline__ void ll_issue(const LLWord<float> *p, LLRaw &r) {
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(r.a) : "l"(p) : "memory");
  r.b = r.a;
}
template <typename T>
__device__ __forceinline__ bool ll_ready(const LLRaw &r, unsigned ep) {
  return (unsigned)(r.a >> 32) == ep && (unsigned)(r.b >> 32) == ep;
}
__device__ __forceinline__ void ll_take(const LLRaw &r, double &x) {
  x = __longlong_as_double((long long)((r.a & 0xffffffffULL) | (r.b << 32)));
}
__device__ __forceinline__ void ll_take(const LLRaw &r, float &x) { x = __uint_as_float((unsigned)r.a); }
__device__ __forceinline__ void ll_take(const LLRaw &r, DF &x) {
  x = DF{__uint_as_float((unsigned)r.a), __uint_as_float((unsigned)r.b)};
}

}  // namespace gb
