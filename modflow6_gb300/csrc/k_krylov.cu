// k_krylov.cu -- fused vector updates, deterministic reductions and the
// device-side control logic of the IMS Krylov accelerators.
//
// PCG: ims_base_cg (src/Solution/LinearMethods/ImsLinearBase.f90:30-240).
// BiCGSTAB: ims_base_bcgs (:249-549).  Convergence: ims_base_testcnvg
// (:1101-1146) and is_close (src/Utilities/MathUtil.f90:45-86).
//
// Each reduction kernel writes one partial per block; a single-block control
// kernel sums the partials in a fixed order (so results are reproducible run
// to run), then runs the scalar logic of the reference on the device: beta,
// alpha, omega with the +SIGN(DPREC, denominator) guard, the closure test,
// the stagnation exits and the NORTH residual schedule.  It sets Ctl::done,
// which every kernel of the loop checks first, and the WHILE condition of the
// CUDA graph, so the whole inner loop runs without a host round trip.
#include "gbims_internal.cuh"
#include "k_krylov.cuh"
#include <cfloat>

namespace gb {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ MaxLoc warp_maxloc(MaxLoc m) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    MaxLoc b;
    b.val = __shfl_xor_sync(0xffffffffu, m.val, o);
    b.idx = __shfl_xor_sync(0xffffffffu, m.idx, o);
    maxloc_merge(m, b);
  }
  return m;
}

// Sum NV values over the block; thread 0 gets the results (fixed order).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double sh[NV][kRedBlock / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = warp_sum(v[k]);
    if (lane == 0) sh[k][wid] = s;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = (lane < (int)(blockDim.x >> 5)) ? sh[k][lane] : 0.0;
      v[k] = warp_sum(s);
    }
  }
  __syncthreads();
}

template <int NM>
__device__ __forceinline__ void block_maxloc(MaxLoc (&m)[NM]) {
  __shared__ double shv[NM][kRedBlock / 32];
  __shared__ long long shi[NM][kRedBlock / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NM; ++k) {
    MaxLoc r = warp_maxloc(m[k]);
    if (lane == 0) {
      shv[k][wid] = r.val;
      shi[k][wid] = r.idx;
    }
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NM; ++k) {
      MaxLoc r;
      r.val = 0.0;
      r.idx = -1;
      if (lane < (int)(blockDim.x >> 5)) {
        r.val = shv[k][lane];
        r.idx = shi[k][lane];
      }
      m[k] = warp_maxloc(r);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(float v) { return (double)v; }

// 1 if v is Inf or NaN, tested on the exponent bits with integer
// instructions: on GB300 every FP64 instruction (a compare included) goes
// through the narrow FP64 pipe, which bounds the vector updates otherwise.
__device__ __forceinline__ unsigned nonfinite(double v) {
  return ((unsigned)__double2hiint(v) & 0x7ff00000u) == 0x7ff00000u;
}
__device__ __forceinline__ unsigned nonfinite(float v) {
  return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u;
}

// Sums of FP32 products with FP64-like accuracy and no FP64 instruction per
// element (on GB300 those run on a narrow pipe): each product is split
// exactly into p + e (p = x*y rounded, e = fma(x, y, -p)), and the p are
// added with Neumaier's compensated summation, their rounding errors and
// the e collected in c.  The pair enters the FP64 reductions as
// (double)s + (double)c.  Explicit _rn operations keep the compiler from
// contracting the splitting steps.
struct CSum {
  float s, c;
};
__device__ __forceinline__ void csum_add(CSum &a, float p) {
  const float t = __fadd_rn(a.s, p);
  const float bp = __fsub_rn(t, a.s);
  a.c = __fadd_rn(a.c, __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(p, bp)));
  a.s = t;
}
__device__ __forceinline__ void csum_prod(CSum &a, float x, float y) {
  const float p = __fmul_rn(x, y);
  const float e = __fmaf_rn(x, y, -p);
  csum_add(a, p);
  a.c = __fadd_rn(a.c, e);
}
__device__ __forceinline__ double csum_value(const CSum &a) { return (double)a.s + (double)a.c; }

// ---------------------------------------------------------------------------
// dot products: partial[b] (and partial[G+b])
// ---------------------------------------------------------------------------
template <typename TA, typename TB>
__global__ void __launch_bounds__(kRedBlock) k_dot(int n, const TA *__restrict__ a,
                                                    const TB *__restrict__ b,
                                                    double *__restrict__ part,
                                                    const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  double v[1] = {0.0};
  // four rows per trip, loads first: the same summation order as one row
  // per trip, with four times the loads in flight
  constexpr int R = 4;
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + (R - 1) * stride < n; i += R * stride) {
    double ar[R], br[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      ar[r] = to_d(a[i + r * stride]);
      br[r] = to_d(b[i + r * stride]);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) v[0] = fma(ar[r], br[r], v[0]);
  }
  for (; i < n; i += stride) v[0] = fma(to_d(a[i]), to_d(b[i]), v[0]);
  block_sum<1>(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// The mixed form's FP32 dot products, summed as above.
__global__ void __launch_bounds__(kRedBlock) k_dot32c(int n, const float *__restrict__ a,
                                                       const float *__restrict__ b,
                                                       double *__restrict__ part,
                                                       const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  CSum acc{0.f, 0.f};
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {
    const float a0 = a[i], b0 = b[i], a1 = a[i + stride], b1 = b[i + stride];
    csum_prod(acc, a0, b0);
    csum_prod(acc, a1, b1);
  }
  if (i < n) csum_prod(acc, a[i], b[i]);
  double v[1] = {csum_value(acc)};
  block_sum<1>(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void __launch_bounds__(kRedBlock) k_dot_tq_tt32c(int n, const float *__restrict__ t,
                                                             const float *__restrict__ q,
                                                             double *__restrict__ part,
                                                             const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  CSum tq{0.f, 0.f}, tt{0.f, 0.f};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float ti = t[i];
    csum_prod(tq, ti, q[i]);
    csum_prod(tt, ti, ti);
  }
  double v[2] = {csum_value(tq), csum_value(tt)};
  block_sum<2>(v);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = v[0];
    part[gridDim.x + blockIdx.x] = v[1];
  }
}

// t.q and t.t in one pass (BiCGSTAB omega)
template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_dot_tq_tt(int n, const T *__restrict__ t,
                                                          const T *__restrict__ q,
                                                          double *__restrict__ part,
                                                          const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double ti = to_d(t[i]);
    v[0] = fma(ti, to_d(q[i]), v[0]);
    v[1] = fma(ti, ti, v[1]);
  }
  block_sum<2>(v);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = v[0];
    part[gridDim.x + blockIdx.x] = v[1];
  }
}

// sum of squares (L2NORM0)
template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_sumsq(int n, const T *__restrict__ a,
                                                      double *__restrict__ part) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double ai = to_d(a[i]);
    v[0] = fma(ai, ai, v[0]);
  }
  block_sum<1>(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

// ---------------------------------------------------------------------------
// partial-sum finalisation inside the single-block control kernels
// ---------------------------------------------------------------------------
__device__ double ctl_reduce_sum(const double *part, int G) {
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < G; i += blockDim.x) v[0] += part[i];
  block_sum<1>(v);
  return v[0];  // valid in thread 0
}

__device__ MaxLoc ctl_reduce_maxloc(const double *pv, const double *pi, int G) {
  MaxLoc m[1];
  m[0].val = 0.0;
  m[0].idx = -1;
  for (int i = threadIdx.x; i < G; i += blockDim.x) {
    MaxLoc b;
    b.val = pv[i];
    b.idx = (long long)pi[i];
    maxloc_merge(m[0], b);
  }
  block_maxloc<1>(m);
  return m[0];
}

__device__ __forceinline__ bool d_is_close(double a, double b) {
  if (a == b) return true;
  double tol = 100.0 * DBL_EPSILON * fmax(fabs(a), fabs(b));
  if (tol < 0.0) tol = 0.0;
  return fabs(a - b) <= tol;
}

__device__ __forceinline__ void d_testcnvg(int icnvgopt, int &icnvg, int iiter, double dvmax,
                                           double rmax, double rmax0, double epfact,
                                           double dvclose, double rclose) {
  if (icnvgopt == 0) {
    if (fabs(dvmax) <= dvclose && fabs(rmax) <= rclose) icnvg = 1;
  } else if (icnvgopt == 1) {
    if (fabs(dvmax) <= dvclose && fabs(rmax) <= rclose) icnvg = (iiter == 1) ? 1 : -1;
  } else if (icnvgopt == 2) {
    if (fabs(dvmax) <= dvclose || rmax <= rclose) icnvg = 1;
    else if (rmax <= rmax0 * epfact) icnvg = -1;
  } else if (icnvgopt == 3) {
    if (fabs(dvmax) <= dvclose) icnvg = 1;
    else if (rmax <= rmax0 * rclose) icnvg = -1;
  } else if (icnvgopt == 4) {
    if (fabs(dvmax) <= dvclose && rmax <= rclose) icnvg = 1;
    else if (rmax <= rmax0 * epfact) icnvg = -1;
  }
}

__device__ __forceinline__ double sign_dprec(double den) { return copysign(DBL_EPSILON, den); }

// Sets the WHILE condition of the graph.  Independently of the IMS exit logic,
// the loop is cut after 2*itmax + 16 bodies, so no input can keep the device
// looping.
__device__ __forceinline__ void set_loop(Ctl *ctl, unsigned long long cond, int use_cond) {
  ctl->bodies += 1;
  if (ctl->bodies > 2 * ctl->itmax + 16 && !ctl->done) {
    ctl->done = 1;
    ctl->guard_tripped = 1;
  }
  if (use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, ctl->done ? 0u : 1u);
}

// ---------------------------------------------------------------------------
// PCG
// ---------------------------------------------------------------------------
__device__ void ctl_cg_rho(Ctl *ctl, const double *part, int G) {
  if (ctl->done) return;
  double s = ctl_reduce_sum(part, G);
  if (threadIdx.x == 0) {
    ctl->rho = s;
    ctl->beta = ctl->first ? 0.0 : s / ctl->rho0;
  }
}
__global__ void k_ctl_cg_rho(Ctl *ctl, const double *part, int G) {
  ctl_cg_rho(ctl, part, G);
}

__device__ void ctl_alpha(Ctl *ctl, const double *part, int G) {
  if (ctl->done) return;
  double s = ctl_reduce_sum(part, G);
  if (threadIdx.x == 0) {
    double den = s + sign_dprec(s);
    ctl->alpha = ctl->rho / den;
  }
}
__global__ void k_ctl_alpha(Ctl *ctl, const double *part, int G) {
  ctl_alpha(ctl, part, G);
}


__global__ void __launch_bounds__(256) k_cg_pupdate64(int n, const double *__restrict__ z,
                                                      double *__restrict__ p,
                                                      const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  p[i] = ctl->first ? z[i] : fma(ctl->beta, p[i], z[i]);
}


__global__ void __launch_bounds__(256) k_cg_pupdate32(int n, const float *__restrict__ z,
                                                      float *__restrict__ p,
                                                      const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  p[i] = ctl->first ? z[i] : fmaf((float)ctl->beta, p[i], z[i]);
}

// x += alpha*p ; d -= alpha*q ; max|alpha p|, max|d|, sum d^2 (FP64 path).
// partial slots: [0]=l2, [1]=dx val, [2]=dx idx, [3]=r val, [4]=r idx, [5]=nonfinite
// The sum of squares is taken only when the closure test reads it (L2 =
// true: RCLOSE options L2NORM_RCLOSE and RELATIVE_RCLOSE, ICNVGOPT 2-4); with
// the infinity-norm tests the reference computes it but never reads it
// inside the loop, and on GB300 it is a quarter of the kernel's FP64 work.
template <bool L2>
__global__ void __launch_bounds__(kRedBlock) k_cg_update64(int n, double *__restrict__ x,
                                                            double *__restrict__ d,
                                                            const double *__restrict__ p,
                                                            const double *__restrict__ q,
                                                            double *__restrict__ part,
                                                            const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  const double alpha = ctl->alpha;
  double v[2] = {0.0, 0.0};
  unsigned nf = 0;
  MaxLoc m[2];
  m[0].val = 0.0; m[0].idx = -1; m[1].val = 0.0; m[1].idx = -1;
  auto row = [&](int i, double pi, double xi, double qi, double dI) {
    double tv = alpha * pi;
    x[i] = xi + tv;
    if (absgt(tv, m[0].val)) { m[0].val = tv; m[0].idx = i; }
    double di = fma(-alpha, qi, dI);
    d[i] = di;
    if (absgt(di, m[1].val)) { m[1].val = di; m[1].idx = i; }
    if (L2) v[0] = fma(di, di, v[0]);
    nf |= nonfinite(di) | nonfinite(tv);
  };
  // four rows per trip, their 16 loads issued before any row is used (the
  // same order of rows per thread as one row per trip, so the same sums and
  // maxima): the loads of a trip cover the latency of the FP64 work of the
  // trip before
  constexpr int R = 4;
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + (R - 1) * stride < n; i += R * stride) {
    double pr[R], xr[R], qr[R], dr[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int j = i + r * stride;
      pr[r] = __ldcs(p + j);
      xr[r] = __ldcs(x + j);
      qr[r] = __ldcs(q + j);
      dr[r] = __ldcs(d + j);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) row(i + r * stride, pr[r], xr[r], qr[r], dr[r]);
  }
  for (; i < n; i += stride) row(i, p[i], x[i], q[i], d[i]);
  v[1] = (double)nf;
  block_sum<2>(v);
  block_maxloc<2>(m);
  if (threadIdx.x == 0) {
    int G = gridDim.x, b = blockIdx.x;
    part[b] = v[0];
    part[G + b] = m[0].val; part[2 * G + b] = (double)m[0].idx;
    part[3 * G + b] = m[1].val; part[4 * G + b] = (double)m[1].idx;
    part[5 * G + b] = v[1];
  }
}


// Mixed inner update: the step alpha*p in FP32, added to the FP64 heads;
// d32 -= alpha*q32; the maxima on FP32 magnitudes (integer compares of the
// bit patterns) and the L2 sum compensated in FP32, so that the only FP64
// instructions per row are the conversion of the step and the head update.
__global__ void __launch_bounds__(kRedBlock) k_cg_update_mixed(int n, double *__restrict__ x,
                                                                float *__restrict__ d,
                                                                const float *__restrict__ p,
                                                                const float *__restrict__ q,
                                                                double *__restrict__ part,
                                                                const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  const float alphaf = (float)ctl->alpha;
  CSum l2{0.f, 0.f};
  unsigned nf = 0;
  unsigned bdx = 0, brr = 0;  // largest magnitudes so far (bit patterns)
  float vdx = 0.f, vrr = 0.f;
  int idx_dx = -1, idx_rr = -1;
  auto row = [&](int i, float pi, double xi, float qi, float dI) {
    const float tv = __fmul_rn(alphaf, pi);
    x[i] = xi + (double)tv;
    const unsigned at = __float_as_uint(tv) & 0x7fffffffu;
    if (at > bdx) { bdx = at; vdx = tv; idx_dx = i; }
    const float di = __fmaf_rn(-alphaf, qi, dI);
    d[i] = di;
    const unsigned ad = __float_as_uint(di) & 0x7fffffffu;
    if (ad > brr) { brr = ad; vrr = di; idx_rr = i; }
    csum_prod(l2, di, di);
    nf |= nonfinite(di) | nonfinite(tv);
  };
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {
    const int j = i + stride;
    const float p0 = p[i], q0 = q[i], d0 = d[i];
    const double x0 = x[i];
    const float p1 = p[j], q1 = q[j], d1 = d[j];
    const double x1 = x[j];
    row(i, p0, x0, q0, d0);
    row(j, p1, x1, q1, d1);
  }
  if (i < n) row(i, p[i], x[i], q[i], d[i]);
  double v[2] = {csum_value(l2), (double)nf};
  MaxLoc m[2];
  m[0].val = (double)vdx; m[0].idx = idx_dx;
  m[1].val = (double)vrr; m[1].idx = idx_rr;
  block_sum<2>(v);
  block_maxloc<2>(m);
  if (threadIdx.x == 0) {
    int G = gridDim.x, b = blockIdx.x;
    part[b] = v[0];
    part[G + b] = m[0].val; part[2 * G + b] = (double)m[0].idx;
    part[3 * G + b] = m[1].val; part[4 * G + b] = (double)m[1].idx;
    part[5 * G + b] = v[1];
  }
}

// Finalise an update reduction into ctl (deltax, rmax, l2norm, nonfinite).
__device__ void ctl_finish_update(Ctl *ctl, const double *part, int G) {
  double l2 = ctl_reduce_sum(part, G);
  MaxLoc dx = ctl_reduce_maxloc(part + G, part + 2 * G, G);
  MaxLoc rm = ctl_reduce_maxloc(part + 3 * G, part + 4 * G, G);
  double nf = ctl_reduce_sum(part + 5 * G, G);
  if (threadIdx.x == 0) {
    ctl->l2norm = sqrt(l2);
    ctl->deltax = dx.val;
    ctl->xloc = dx.idx;
    ctl->rmax = rm.val;
    ctl->rloc = rm.idx;
    if (nf != 0.0) ctl->nonfinite = 1;
  }
}

// Per-model maxima of one iteration for the inner records, when the solution
// has more than one model (CONVNMOD > 1; ImsLinearBase.f90:141-182 for PCG,
// :431-480 for BiCGSTAB): for each model's rows, the largest head change
// (the step the update kernel added: PCG alpha*p, BiCGSTAB alpha*phat +
// omega*qhat, times DSCALE when scaled) and the largest residual (divided by
// DSCALE when scaled), signed, with its row.  The step is recomputed with the
// update kernel's own expression, so the values are the ones the update
// compared.  Partial slots per model im: [4im] dx value, [4im+1] its row,
// [4im+2] r value, [4im+3] its row (G blocks each).
template <bool BCGS>
__global__ void __launch_bounds__(kRedBlock) k_rec_models(int nm, const int *__restrict__ modstart,
                                                          const double *__restrict__ p,
                                                          const double *__restrict__ q,
                                                          const double *__restrict__ d,
                                                          const double *__restrict__ dscale,
                                                          double *__restrict__ part,
                                                          const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  const double alpha = ctl->alpha, omega = ctl->omega;
  const int G = gridDim.x, b = blockIdx.x;
  for (int im = 0; im < nm; ++im) {
    MaxLoc m[2];
    m[0].val = 0.0; m[0].idx = -1; m[1].val = 0.0; m[1].idx = -1;
    const int r0 = modstart[im], r1 = modstart[im + 1];
    for (int i = r0 + b * blockDim.x + threadIdx.x; i < r1; i += G * blockDim.x) {
      double tv;
      if (BCGS) tv = fma(alpha, p[i], omega * q[i]);
      else tv = alpha * p[i];
      double rv = d[i];
      if (BCGS && dscale) {
        tv = tv * dscale[i];
        rv = rv / dscale[i];
      }
      if (absgt(tv, m[0].val)) { m[0].val = tv; m[0].idx = i; }
      if (absgt(rv, m[1].val)) { m[1].val = rv; m[1].idx = i; }
    }
    block_maxloc<2>(m);
    if (threadIdx.x == 0) {
      part[(4 * im) * G + b] = m[0].val;
      part[(4 * im + 1) * G + b] = (double)m[0].idx;
      part[(4 * im + 2) * G + b] = m[1].val;
      part[(4 * im + 3) * G + b] = (double)m[1].idx;
    }
  }
}

// Writes this iteration's record (called by every thread of the control
// block after ctl_finish_update, before the iteration count advances):
// ITINNER, the CACCEL values (alpha; BiCGSTAB also omega) and per model
// dvmax, locdv, rmax, locr.  With one model these are the update's own
// maxima.  The reference resets the per-model locations every PCG iteration
// but not every BiCGSTAB iteration (ImsLinearBase.f90:141-146 against
// :432-435), so a BiCGSTAB model whose maxima stay zero keeps its last rows.
__device__ void ctl_record(Ctl *ctl, bool bcgs) {
  const int nm = ctl->rec_nmod, G = ctl->rec_G;
  const int row = ctl->iter - 1;
  const bool keep = row >= 0 && row < ctl->rec_cap;
  double *r = ctl->rec + (size_t)(keep ? row : 0) * (3 + 4 * nm);
  for (int im = 0; im < nm; ++im) {
    MaxLoc dx, rm;
    if (nm == 1) {
      dx.val = ctl->deltax; dx.idx = ctl->xloc;
      rm.val = ctl->rmax; rm.idx = ctl->rloc;
    } else {
      const double *pp = ctl->rec_part;
      dx = ctl_reduce_maxloc(pp + (4 * im) * G, pp + (4 * im + 1) * G, G);
      rm = ctl_reduce_maxloc(pp + (4 * im + 2) * G, pp + (4 * im + 3) * G, G);
    }
    if (threadIdx.x == 0) {
      long long ldv = dx.idx, lr = rm.idx;
      if (bcgs) {
        if (ldv < 0) ldv = ctl->rec_loc[2 * im];
        if (lr < 0) lr = ctl->rec_loc[2 * im + 1];
      }
      ctl->rec_loc[2 * im] = ldv;
      ctl->rec_loc[2 * im + 1] = lr;
      if (keep) {
        r[3 + 4 * im] = dx.val;
        r[4 + 4 * im] = (double)ldv;
        r[5 + 4 * im] = rm.val;
        r[6 + 4 * im] = (double)lr;
      }
    }
  }
  if (threadIdx.x == 0 && keep) {
    r[0] = (double)ctl->iter;
    r[1] = ctl->alpha;
    r[2] = bcgs ? ctl->omega : 0.0;
    ctl->rec_count = row + 1;
  }
}

// End of a PCG iteration: closure test and loop control (ImsLinearBase.f90:196-236).
__device__ void ctl_cg_cnvg(Ctl *ctl, const double *part, int G, unsigned long long cond,
                              int use_cond) {
  if (ctl->done) {
    if (threadIdx.x == 0) set_loop(ctl, cond, use_cond);
    return;
  }
  ctl_finish_update(ctl, part, G);
  if (ctl->rec) ctl_record(ctl, false);
  if (threadIdx.x != 0) return;
  double rcnvg = (ctl->icnvgopt == 2 || ctl->icnvgopt == 3 || ctl->icnvgopt == 4) ? ctl->l2norm
                                                                                : ctl->rmax;
  int icnvg = ctl->icnvg;
  d_testcnvg(ctl->icnvgopt, icnvg, ctl->iter, ctl->deltax, rcnvg, ctl->l2norm0, ctl->epfact,
             ctl->dvclose, ctl->rclose);
  if (rcnvg == 0.0) icnvg = 1;
  ctl->icnvg = icnvg;
  ctl->north_due = 0;
  if (ctl->nonfinite) {
    ctl->done = 1;
  } else if (icnvg != 0) {
    ctl->done = 1;
    ctl->exit_reason = (rcnvg == 0.0) ? kExitExact : kExitClosure;
  } else if (d_is_close(ctl->rho, ctl->rho0)) {
    ctl->done = 1;
    ctl->exit_reason = kExitStagnation;
  } else {
    if (ctl->north > 0 && ((ctl->iter + 1) % ctl->north) == 0) ctl->north_due = 1;
    if (ctl->rho == 0.0) {
      ctl->done = 1;
      ctl->exit_reason = kExitZeroRho;
    } else {
      ctl->rho0 = ctl->rho;
      if (ctl->iter >= ctl->itmax) {
        ctl->done = 1;
        ctl->exit_reason = kExitItmax;
      } else {
        ctl->iter += 1;
        ctl->first = 0;
      }
    }
  }
  if (ctl->done && ctl->icnvg < 0) ctl->icnvg = 0;
  set_loop(ctl, cond, use_cond);
}
__global__ void k_ctl_cg_cnvg(Ctl *ctl, const double *part, int G, unsigned long long cond,
                              int use_cond) {
  ctl_cg_cnvg(ctl, part, G, cond, use_cond);
}

// ---------------------------------------------------------------------------
// BiCGSTAB
// ---------------------------------------------------------------------------
__device__ void ctl_bcgs_rho(Ctl *ctl, const double *part, int G) {
  if (ctl->done) return;
  double s = ctl_reduce_sum(part, G);
  if (threadIdx.x == 0) {
    ctl->rho = s;
    if (!ctl->first) ctl->beta = (s / ctl->rho0) * (ctl->alpha0 / ctl->omega0);
  }
}
__global__ void k_ctl_bcgs_rho(Ctl *ctl, const double *part, int G) {
  ctl_bcgs_rho(ctl, part, G);
}

template <typename T>
__global__ void __launch_bounds__(256) k_bcgs_p(int n, const T *__restrict__ d, T *__restrict__ p,
                                                const T *__restrict__ v,
                                                const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (ctl->first) {
    p[i] = d[i];
  } else {
    T beta = (T)ctl->beta, om = (T)ctl->omega0;
    T inner = fma(-om, v[i], p[i]);
    p[i] = fma(beta, inner, d[i]);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_bcgs_q(int n, const T *__restrict__ d, const T *__restrict__ v,
                                                T *__restrict__ q, const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  q[i] = fma(-(T)ctl->alpha, v[i], d[i]);
}

__device__ void ctl_omega(Ctl *ctl, const double *part, int G) {
  if (ctl->done) return;
  double num = ctl_reduce_sum(part, G);
  double den = ctl_reduce_sum(part + G, G);
  if (threadIdx.x == 0) {
    den = den + sign_dprec(den);
    ctl->omega = num / den;
  }
}
__global__ void k_ctl_omega(Ctl *ctl, const double *part, int G) {
  ctl_omega(ctl, part, G);
}

// x += alpha*phat + omega*qhat ; d = q - omega*t (ImsLinearBase.f90:428-480).
// L2 as in k_cg_update64.
template <typename T, bool L2>
__global__ void __launch_bounds__(kRedBlock) k_bcgs_update(int n, double *__restrict__ x,
                                                            T *__restrict__ d,
                                                            const T *__restrict__ phat,
                                                            const T *__restrict__ qhat,
                                                            const T *__restrict__ q,
                                                            const T *__restrict__ t,
                                                            const double *__restrict__ dscale,
                                                            double *__restrict__ part,
                                                            const Ctl *__restrict__ ctl) {
  if (ctl->done) return;
  const double alpha = ctl->alpha, omega = ctl->omega;
  const T omegat = (T)omega;
  double v[2] = {0.0, 0.0};
  unsigned nf = 0;
  MaxLoc m[2];
  m[0].val = 0.0; m[0].idx = -1; m[1].val = 0.0; m[1].idx = -1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double tv = fma(alpha, to_d(phat[i]), omega * to_d(qhat[i]));
    x[i] = x[i] + tv;
    if (dscale) tv = tv * dscale[i];
    if (absgt(tv, m[0].val)) { m[0].val = tv; m[0].idx = i; }
    T di = fma(-omegat, t[i], q[i]);
    d[i] = di;
    double rv = to_d(di);
    if (dscale) rv = rv / dscale[i];
    if (absgt(rv, m[1].val)) { m[1].val = rv; m[1].idx = i; }
    if (L2) v[0] = fma(rv, rv, v[0]);
    nf |= nonfinite(rv) | nonfinite(tv);
  }
  v[1] = (double)nf;
  block_sum<2>(v);
  block_maxloc<2>(m);
  if (threadIdx.x == 0) {
    int G = gridDim.x, b = blockIdx.x;
    part[b] = v[0];
    part[G + b] = m[0].val; part[2 * G + b] = (double)m[0].idx;
    part[3 * G + b] = m[1].val; part[4 * G + b] = (double)m[1].idx;
    part[5 * G + b] = v[1];
  }
}

// End of a BiCGSTAB iteration (ImsLinearBase.f90:498-545).
__device__ void ctl_bcgs_cnvg(Ctl *ctl, const double *part, int G, unsigned long long cond,
                                int use_cond) {
  if (ctl->done) {
    if (threadIdx.x == 0) set_loop(ctl, cond, use_cond);
    return;
  }
  ctl_finish_update(ctl, part, G);
  if (ctl->rec) ctl_record(ctl, true);
  if (threadIdx.x != 0) return;
  double rcnvg = (ctl->icnvgopt == 2 || ctl->icnvgopt == 3 || ctl->icnvgopt == 4) ? ctl->l2norm
                                                                                : ctl->rmax;
  int icnvg = ctl->icnvg;
  d_testcnvg(ctl->icnvgopt, icnvg, ctl->iter, ctl->deltax, rcnvg, ctl->l2norm0, ctl->epfact,
             ctl->dvclose, ctl->rclose);
  if (rcnvg == 0.0) icnvg = 1;
  ctl->icnvg = icnvg;
  ctl->north_due = 0;
  if (ctl->nonfinite) {
    ctl->done = 1;
  } else if (icnvg != 0) {
    ctl->done = 1;
    ctl->exit_reason = (rcnvg == 0.0) ? kExitExact : kExitClosure;
  } else if (d_is_close(ctl->rho, ctl->rho0) || d_is_close(ctl->alpha, ctl->alpha0) ||
             d_is_close(ctl->omega, ctl->omega0)) {
    ctl->done = 1;
    ctl->exit_reason = kExitStagnation;
  } else {
    if (ctl->north > 0 && ((ctl->iter + 1) % ctl->north) == 0) ctl->north_due = 1;
    if (ctl->rho * ctl->omega == 0.0) {
      ctl->done = 1;
      ctl->exit_reason = kExitZeroRho;
    } else {
      ctl->rho0 = ctl->rho;
      ctl->alpha0 = ctl->alpha;
      ctl->omega0 = ctl->omega;
      if (ctl->iter >= ctl->itmax) {
        ctl->done = 1;
        ctl->exit_reason = kExitItmax;
      } else {
        ctl->iter += 1;
        ctl->first = 0;
      }
    }
  }
  if (ctl->done && ctl->icnvg < 0) ctl->icnvg = 0;
  set_loop(ctl, cond, use_cond);
}
__global__ void k_ctl_bcgs_cnvg(Ctl *ctl, const double *part, int G, unsigned long long cond,
                                int use_cond) {
  ctl_bcgs_cnvg(ctl, part, G, cond, use_cond);
}

// ---------------------------------------------------------------------------
// Mixed precision: FP64 iterative refinement around the FP32 inner loop
// ---------------------------------------------------------------------------

// End of a mixed inner iteration.  The IMS test runs on the recursive FP32
// residual; when it passes, or the recursive residual has dropped by
// refine_factor since the last refinement, the next true-residual check is
// requested (Ctl::north_due = 2) instead of stopping.
__device__ void ctl_mixed_inner(Ctl *ctl, const double *part, int G, int bcgs,
                                  double refine_factor) {
  if (ctl->done) return;
  ctl_finish_update(ctl, part, G);
  if (threadIdx.x != 0) return;
  double rcnvg = (ctl->icnvgopt == 2 || ctl->icnvgopt == 3 || ctl->icnvgopt == 4) ? ctl->l2norm
                                                                                : ctl->rmax;
  int icnvg = 0;
  d_testcnvg(ctl->icnvgopt, icnvg, ctl->iter, ctl->deltax, rcnvg, ctl->l2norm0, ctl->epfact,
             ctl->dvclose, ctl->rclose);
  if (rcnvg == 0.0) icnvg = 1;
  ctl->north_due = 0;
  // scratch[0]: L2 norm of the residual at the start of this refinement
  bool stag = d_is_close(ctl->rho, ctl->rho0);
  if (bcgs) stag = stag || d_is_close(ctl->alpha, ctl->alpha0) || d_is_close(ctl->omega, ctl->omega0);
  bool zero = bcgs ? (ctl->rho * ctl->omega == 0.0) : (ctl->rho == 0.0);
  if (ctl->nonfinite) {
    ctl->done = 1;
    return;
  }
  if (icnvg != 0 || ctl->l2norm <= refine_factor * ctl->scratch[0] || stag || zero) {
    ctl->north_due = 2;  // request the FP64 true residual
    // Every refinement restarts the recurrence from the true residual: with
    // FP32 search directions, continuing after a residual replacement costs
    // more iterations than a restart (measured on the 10M-cell case)
    (void)bcgs;
    ctl->restart_due = 1;
    ctl->scratch[1] = ctl->deltax;
    ctl->scratch[2] = (double)ctl->xloc;
  }
  ctl->rho0 = ctl->rho;
  ctl->alpha0 = ctl->alpha;
  ctl->omega0 = ctl->omega;
  if (ctl->north_due != 2) {
    if (ctl->iter >= ctl->itmax) {
      ctl->north_due = 2;  // final true-residual check at the iteration limit
      ctl->restart_due = 0;
      ctl->scratch[1] = ctl->deltax;
      ctl->scratch[2] = (double)ctl->xloc;
    } else {
      ctl->iter += 1;
      ctl->first = 0;
    }
  }
}
__global__ void k_ctl_mixed_inner(Ctl *ctl, const double *part, int G, int bcgs,
                                  double refine_factor) {
  ctl_mixed_inner(ctl, part, G, bcgs, refine_factor);
}

// True residual r = b - A x in FP64 with its max|r| and L2, only when
// requested; the FP32 residual is reset from it.
__global__ void __launch_bounds__(kRedBlock) k_true_resid_stats(int n, const double *__restrict__ r,
                                                                 float *__restrict__ d32,
                                                                 float *__restrict__ dhat32,
                                                                 double *__restrict__ dhat64,
                                                                 const double *__restrict__ dscale,
                                                                 double *__restrict__ part,
                                                                 const Ctl *__restrict__ ctl) {
  if (ctl->done || ctl->north_due != 2) return;
  double v[2] = {0.0, 0.0};
  unsigned nf = 0;
  MaxLoc m[2];
  m[0].val = 0.0; m[0].idx = -1; m[1].val = 0.0; m[1].idx = -1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double ri = r[i];
    if (d32) d32[i] = (float)ri;
    if (ctl->restart_due) {  // BiCGSTAB shadow residual, on a restart
      if (dhat32) dhat32[i] = (float)ri;
      if (dhat64) dhat64[i] = ri;
    }
    if (dscale) ri = ri / dscale[i];    // BiCGSTAB reports the unscaled residual
    if (absgt(ri, m[1].val)) { m[1].val = ri; m[1].idx = i; }
    v[0] = fma(ri, ri, v[0]);
    nf |= nonfinite(ri);
  }
  v[1] = (double)nf;
  block_sum<2>(v);
  block_maxloc<2>(m);
  if (threadIdx.x == 0) {
    int G = gridDim.x, b = blockIdx.x;
    part[b] = v[0];
    part[G + b] = 0.0; part[2 * G + b] = -1.0;
    part[3 * G + b] = m[1].val; part[4 * G + b] = (double)m[1].idx;
    part[5 * G + b] = v[1];
  }
}

// Closure test on the FP64 true residual; restart the inner loop if needed.
__device__ void ctl_refine(Ctl *ctl, const double *part, int G, unsigned long long cond,
                             int use_cond) {
  if (ctl->done || ctl->north_due != 2) {
    if (threadIdx.x == 0) set_loop(ctl, cond, use_cond);
    return;
  }
  double dsave = ctl->scratch[1];
  long long lsave = (long long)ctl->scratch[2];
  ctl_finish_update(ctl, part, G);
  if (threadIdx.x != 0) return;
  ctl->deltax = dsave;
  ctl->xloc = lsave;
  double rcnvg = (ctl->icnvgopt == 2 || ctl->icnvgopt == 3 || ctl->icnvgopt == 4) ? ctl->l2norm
                                                                                : ctl->rmax;
  int icnvg = 0;
  d_testcnvg(ctl->icnvgopt, icnvg, ctl->iter, ctl->deltax, rcnvg, ctl->l2norm0, ctl->epfact,
             ctl->dvclose, ctl->rclose);
  if (rcnvg == 0.0) icnvg = 1;
  ctl->north_due = 0;
  if (ctl->nonfinite) {
    ctl->done = 1;
  } else if (icnvg > 0) {
    ctl->icnvg = 1;
    ctl->done = 1;
    ctl->exit_reason = (rcnvg == 0.0) ? kExitExact : kExitClosure;
  } else if (ctl->iter >= ctl->itmax) {
    ctl->icnvg = 0;
    ctl->done = 1;
    ctl->exit_reason = kExitItmax;
  } else {
    // The FP32 recurrence residual is replaced by the FP64 true residual and
    // the recurrence restarts from it (restart_due); a recurrence that
    // carried on instead, like the reference's NORTH residual refresh
    // (ImsLinearBase.f90:221-227), would keep its search direction.
    ctl->scratch[0] = ctl->l2norm;
    ctl->scratch[3] += 1.0;  // refinement count
    if (ctl->restart_due) {
      ctl->first = 1;
      ctl->rho0 = 0.0;
      ctl->alpha0 = 0.0;
      ctl->omega0 = 0.0;
    } else {
      ctl->first = 0;
    }
    ctl->iter += 1;
  }
  set_loop(ctl, cond, use_cond);
}
__global__ void k_ctl_refine(Ctl *ctl, const double *part, int G, unsigned long long cond,
                             int use_cond) {
  ctl_refine(ctl, part, G, cond, use_cond);
}

// ---------------------------------------------------------------------------
// misc elementwise kernels
// ---------------------------------------------------------------------------
template <typename TD, typename TS>
__global__ void k_convert(int n, const TS *__restrict__ s, TD *__restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = (TD)s[i];
}

__device__ void ctl_set_l2norm0(Ctl *ctl, const double *part, int G) {
  double s = ctl_reduce_sum(part, G);
  if (threadIdx.x == 0) {
    ctl->l2norm0 = sqrt(s);
    ctl->scratch[0] = ctl->l2norm0;
    if (ctl->l2norm0 == 0.0 || ctl->itmax <= 0) {
      ctl->done = 1;
      if (ctl->l2norm0 == 0.0) {
        ctl->icnvg = 1;
        ctl->exit_reason = kExitExact;
      }
    }
    if (!isfinite(s)) {
      ctl->nonfinite = 1;
      ctl->done = 1;
    }
  }
}
__global__ void k_ctl_set_l2norm0(Ctl *ctl, const double *part, int G) {
  ctl_set_l2norm0(ctl, part, G);
}
// The L2 norm of the final residual, for a loop that did not take it.
__global__ void k_ctl_set_l2norm(Ctl *ctl, const double *part, int G) {
  double s = ctl_reduce_sum(part, G);
  if (threadIdx.x == 0 && ctl->l2norm0 != 0.0) ctl->l2norm = sqrt(s);
}

// ---------------------------------------------------------------------------
// Batched ensemble: independent systems ("members") concatenated into one
// block-diagonal system and iterated in lockstep.  Rows are cut into chunks
// that never straddle two members; one chunk is one block of the vector
// kernels and owns one reduction partial per slot.  Member m's partials are
// laid out like a single solve's (slot k of its b-th chunk at
// part[8*mc[m] + k*Gm + b], Gm = its chunk count), so the per-member control
// logic is exactly the single-solve code above, run by block m.  A member
// whose Ctl is done skips all of its chunks; the loop ends when every member
// is done.
// ---------------------------------------------------------------------------
struct ChunkRef {
  int m, b, G, r0, r1;
};

__device__ __forceinline__ ChunkRef chunk_of(const BatchDev &B, int c) {
  ChunkRef r;
  r.m = B.cm[c];
  const int c0 = B.mc[r.m];
  r.b = c - c0;
  r.G = B.mc[r.m + 1] - c0;
  r.r0 = B.cr[c];
  r.r1 = B.cr[c + 1];
  return r;
}

__device__ __forceinline__ double *member_part(double *part, const BatchDev &B, int m) {
  return part + 8LL * B.mc[m];
}

template <typename TA, typename TB>
__global__ void __launch_bounds__(kRedBlock) k_b_dot(BatchDev B, const TA *__restrict__ a,
                                                     const TB *__restrict__ b,
                                                     double *__restrict__ part) {
  const ChunkRef c = chunk_of(B, blockIdx.x);
  if (B.ctls[c.m].done) return;
  double v[1] = {0.0};
  for (int i = c.r0 + threadIdx.x; i < c.r1; i += blockDim.x) v[0] = fma(to_d(a[i]), to_d(b[i]), v[0]);
  block_sum<1>(v);
  if (threadIdx.x == 0) member_part(part, B, c.m)[c.b] = v[0];
}

__global__ void __launch_bounds__(kRedBlock) k_b_sumsq(BatchDev B, const double *__restrict__ a,
                                                       double *__restrict__ part) {
  const ChunkRef c = chunk_of(B, blockIdx.x);
  double v[1] = {0.0};
  for (int i = c.r0 + threadIdx.x; i < c.r1; i += blockDim.x) v[0] = fma(a[i], a[i], v[0]);
  block_sum<1>(v);
  if (threadIdx.x == 0) member_part(part, B, c.m)[c.b] = v[0];
}

template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_b_cg_pupdate(BatchDev B, const T *__restrict__ z,
                                                            T *__restrict__ p) {
  const ChunkRef c = chunk_of(B, blockIdx.x);
  const Ctl &ctl = B.ctls[c.m];
  if (ctl.done) return;
  const bool first = ctl.first;
  const double beta = ctl.beta;
  for (int i = c.r0 + threadIdx.x; i < c.r1; i += blockDim.x)
    p[i] = first ? z[i] : (T)fma((double)(T)beta, (double)p[i], (double)z[i]);
}

// x += alpha*p ; d -= alpha*q with the same partial slots as k_cg_update64.
__global__ void __launch_bounds__(kRedBlock) k_b_cg_update64(BatchDev B, double *__restrict__ x,
                                                             double *__restrict__ d,
                                                             const double *__restrict__ p,
                                                             const double *__restrict__ q,
                                                             double *__restrict__ part) {
  const ChunkRef c = chunk_of(B, blockIdx.x);
  const Ctl &ctl = B.ctls[c.m];
  if (ctl.done) return;
  const double alpha = ctl.alpha;
  double v[2] = {0.0, 0.0};
  unsigned nf = 0;
  MaxLoc m[2];
  m[0].val = 0.0; m[0].idx = -1; m[1].val = 0.0; m[1].idx = -1;
  const int row0 = B.mr[c.m];  // member-local row numbers for the maxima
  for (int i = c.r0 + threadIdx.x; i < c.r1; i += blockDim.x) {
    double tv = alpha * p[i];
    x[i] = x[i] + tv;
    if (absgt(tv, m[0].val)) { m[0].val = tv; m[0].idx = i - row0; }
    double di = fma(-alpha, q[i], d[i]);
    d[i] = di;
    if (absgt(di, m[1].val)) { m[1].val = di; m[1].idx = i - row0; }
    v[0] = fma(di, di, v[0]);
    nf |= nonfinite(di) | nonfinite(tv);
  }
  v[1] = (double)nf;
  block_sum<2>(v);
  block_maxloc<2>(m);
  if (threadIdx.x == 0) {
    double *pm = member_part(part, B, c.m);
    const int G = c.G, b = c.b;
    pm[b] = v[0];
    pm[G + b] = m[0].val; pm[2 * G + b] = (double)m[0].idx;
    pm[3 * G + b] = m[1].val; pm[4 * G + b] = (double)m[1].idx;
    pm[5 * G + b] = v[1];
  }
}

__global__ void k_b_ctl_set_l2norm0(BatchDev B, const double *part) {
  const int m = blockIdx.x;
  ctl_set_l2norm0(B.ctls + m, part + 8LL * B.mc[m], B.mc[m + 1] - B.mc[m]);
}
__global__ void k_b_ctl_cg_rho(BatchDev B, const double *part) {
  const int m = blockIdx.x;
  ctl_cg_rho(B.ctls + m, part + 8LL * B.mc[m], B.mc[m + 1] - B.mc[m]);
}
__global__ void k_b_ctl_alpha(BatchDev B, const double *part) {
  const int m = blockIdx.x;
  ctl_alpha(B.ctls + m, part + 8LL * B.mc[m], B.mc[m + 1] - B.mc[m]);
}
__global__ void k_b_ctl_cg_cnvg(BatchDev B, const double *part) {
  const int m = blockIdx.x;
  ctl_cg_cnvg(B.ctls + m, part + 8LL * B.mc[m], B.mc[m + 1] - B.mc[m], 0ULL, 0);
}

// The batch's own control block gets done = every member done; it gates the
// shared kernels (SpMV, preconditioner) and drives the WHILE condition.
__global__ void k_b_all_done(BatchDev B, Ctl *gctl, unsigned long long cond, int use_cond,
                            int count_body) {
  __shared__ int s_any;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  for (int m = threadIdx.x; m < B.nm; m += blockDim.x)
    if (!B.ctls[m].done) atomicOr(&s_any, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!s_any) gctl->done = 1;
    if (count_body) set_loop(gctl, cond, use_cond);
  }
}

// ---------------------------------------------------------------------------
// Batched mixed form: the single solve's FP32 inner loop and FP64
// refinement (k_dot32c, k_cg_pupdate32, k_cg_update_mixed,
// ctl_mixed_inner, k_true_resid_stats, ctl_refine) per member.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kRedBlock) k_b_dot32c(BatchDev B, const float *__restrict__ a,
                                                         const float *__restrict__ b,
                                                         double *__restrict__ part) {
  const ChunkRef c = chunk_of(B, blockIdx.x);
  if (B.ctls[c.m].done) return;
  CSum acc{0.f, 0.f};
  for (int i = c.r0 + threadIdx.x; i < c.r1; i += blockDim.x) csum_prod(acc, a[i], b[i]);
  double v[1] = {csum_value(acc)};
  block_sum<1>(v);
  if (threadIdx.x == 0) member_part(part, B, c.m)[c.b] = v[0];
}

__global__ void __launch_bounds__(kRedBlock) k_b_cg_pupdate32(BatchDev B, const float *__restrict__ z,
                                                               float *__restrict__ p) {
  const ChunkRef c = chunk_of(B, blockIdx.x);
  const Ctl &ctl = B.ctls[c.m];
  if (ctl.done) return;
  const bool first = ctl.first;
  const float beta = (float)ctl.beta;
  for (int i = c.r0 + threadIdx.x; i < c.r1; i += blockDim.x) p[i] = first ? z[i] : fmaf(beta, p[i], z[i]);
}

__global__ void __launch_bounds__(kRedBlock) k_b_cg_update_mixed(BatchDev B, double *__restrict__ x,
                                                                  float *__restrict__ d,
                                                                  const float *__restrict__ p,
                                                                  const float *__restrict__ q,
                                                                  double *__restrict__ part) {
  const ChunkRef c = chunk_of(B, blockIdx.x);
  const Ctl &ctl = B.ctls[c.m];
  if (ctl.done) return;
  const float alphaf = (float)ctl.alpha;
  const int row0 = B.mr[c.m];  // member-local row numbers for the maxima
  CSum l2{0.f, 0.f};
  unsigned nf = 0, bdx = 0, brr = 0;
  float vdx = 0.f, vrr = 0.f;
  int idx_dx = -1, idx_rr = -1;
  for (int i = c.r0 + threadIdx.x; i < c.r1; i += blockDim.x) {
    const float tv = __fmul_rn(alphaf, p[i]);
    x[i] = x[i] + (double)tv;
    const unsigned at = __float_as_uint(tv) & 0x7fffffffu;
    if (at > bdx) { bdx = at; vdx = tv; idx_dx = i - row0; }
    const float di = __fmaf_rn(-alphaf, q[i], d[i]);
    d[i] = di;
    const unsigned ad = __float_as_uint(di) & 0x7fffffffu;
    if (ad > brr) { brr = ad; vrr = di; idx_rr = i - row0; }
    csum_prod(l2, di, di);
    nf |= nonfinite(di) | nonfinite(tv);
  }
  double v[2] = {csum_value(l2), (double)nf};
  MaxLoc m[2];
  m[0].val = (double)vdx; m[0].idx = idx_dx;
  m[1].val = (double)vrr; m[1].idx = idx_rr;
  block_sum<2>(v);
  block_maxloc<2>(m);
  if (threadIdx.x == 0) {
    double *pm = member_part(part, B, c.m);
    const int G = c.G, b = c.b;
    pm[b] = v[0];
    pm[G + b] = m[0].val; pm[2 * G + b] = (double)m[0].idx;
    pm[3 * G + b] = m[1].val; pm[4 * G + b] = (double)m[1].idx;
    pm[5 * G + b] = v[1];
  }
}

__global__ void k_b_ctl_mixed_inner(BatchDev B, const double *part, double refine_factor) {
  const int m = blockIdx.x;
  ctl_mixed_inner(B.ctls + m, part + 8LL * B.mc[m], B.mc[m + 1] - B.mc[m], 0, refine_factor);
}

// The batch's own block asks for the FP64 true residual when any member
// does (the residual kernel is gated on it; members that are not due
// ignore it).
__global__ void k_b_any_due(BatchDev B, Ctl *gctl) {
  __shared__ int s_any;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  for (int m = threadIdx.x; m < B.nm; m += blockDim.x)
    if (!B.ctls[m].done && B.ctls[m].north_due == 2) atomicOr(&s_any, 1);
  __syncthreads();
  if (threadIdx.x == 0) gctl->north_due = s_any ? 2 : 0;
}

__global__ void __launch_bounds__(kRedBlock) k_b_true_resid_stats(BatchDev B,
                                                                   const double *__restrict__ r,
                                                                   float *__restrict__ d32,
                                                                   double *__restrict__ part) {
  const ChunkRef c = chunk_of(B, blockIdx.x);
  const Ctl &ctl = B.ctls[c.m];
  if (ctl.done || ctl.north_due != 2) return;
  const int row0 = B.mr[c.m];
  double v[2] = {0.0, 0.0};
  unsigned nf = 0;
  MaxLoc m[2];
  m[0].val = 0.0; m[0].idx = -1; m[1].val = 0.0; m[1].idx = -1;
  for (int i = c.r0 + threadIdx.x; i < c.r1; i += blockDim.x) {
    const double ri = r[i];
    d32[i] = (float)ri;
    if (absgt(ri, m[1].val)) { m[1].val = ri; m[1].idx = i - row0; }
    v[0] = fma(ri, ri, v[0]);
    nf |= nonfinite(ri);
  }
  v[1] = (double)nf;
  block_sum<2>(v);
  block_maxloc<2>(m);
  if (threadIdx.x == 0) {
    double *pm = member_part(part, B, c.m);
    const int G = c.G, b = c.b;
    pm[b] = v[0];
    pm[G + b] = 0.0; pm[2 * G + b] = -1.0;
    pm[3 * G + b] = m[1].val; pm[4 * G + b] = (double)m[1].idx;
    pm[5 * G + b] = v[1];
  }
}

__global__ void k_b_ctl_refine(BatchDev B, const double *part) {
  const int m = blockIdx.x;
  ctl_refine(B.ctls + m, part + 8LL * B.mc[m], B.mc[m + 1] - B.mc[m], 0ULL, 0);
}

// ---------------------------------------------------------------------------
// residual d = b - A x with its L2 norm and signed max|d| from CSR device
// arrays, one row per thread (ims_base_residual + dnrm2, ImsLinearBase.f90:
// 1291-1312; the row sum in amux order with FMA).  With one 256-row block per
// partial, the sum of squares rounds exactly like k_sumsq + k_ctl_set_l2norm0
// on a vector of at most kMaxRedBlocks * 256 rows.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kRedBlock) k_resid_rows(int n, const int *__restrict__ ia,
                                                           const int *__restrict__ ja, int base,
                                                           const double *__restrict__ amat,
                                                           const double *__restrict__ x,
                                                           const double *__restrict__ b,
                                                           double *__restrict__ resid,
                                                           double *__restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0};
  MaxLoc m[1];
  m[0].val = 0.0;
  m[0].idx = -1;
  if (i < n) {
    double t = 0.0;
    const int k1 = ia[i + 1] - base;
    for (int k = ia[i] - base; k < k1; ++k) t = fma(amat[k], x[ja[k] - base], t);
    const double d = b[i] - t;
    if (resid) resid[i] = d;
    v[0] = fma(d, d, v[0]);
    if (absgt(d, m[0].val)) { m[0].val = d; m[0].idx = i; }
  }
  block_sum<1>(v);
  block_maxloc<1>(m);
  if (threadIdx.x == 0) {
    const int G = gridDim.x;
    part[blockIdx.x] = v[0];
    part[G + blockIdx.x] = m[0].val;
    part[2 * G + blockIdx.x] = (double)m[0].idx;
  }
}

// out[0] = L2 norm, out[1] = signed max|d|, out[2] = its row.
__global__ void k_resid_final(const double *__restrict__ part, int G, double *__restrict__ out) {
  const double s = ctl_reduce_sum(part, G);
  const MaxLoc m = ctl_reduce_maxloc(part + G, part + 2 * G, G);
  if (threadIdx.x == 0) {
    out[0] = sqrt(s);
    out[1] = m.val;
    out[2] = (double)m.idx;
  }
}

// ---------------------------------------------------------------------------
// host launch wrappers
// ---------------------------------------------------------------------------
void kr_residual_rows(int n, const int *ia, const int *ja, int base, const double *amat,
                      const double *x, const double *b, double *resid, double *part,
                      double *out, cudaStream_t st) {
  const int G = (n + kRedBlock - 1) / kRedBlock;
  k_resid_rows<<<G, kRedBlock, 0, st>>>(n, ia, ja, base, amat, x, b, resid, part);
  k_resid_final<<<1, kRedBlock, 0, st>>>(part, G, out);
}
static inline int egrid(int n) { return std::max(1, (n + 255) / 256); }

void kr_dot64(int n, const double *a, const double *b, double *part, int G, const Ctl *ctl, cudaStream_t st) {
  k_dot<double, double><<<G, kRedBlock, 0, st>>>(n, a, b, part, ctl);
}
void kr_dot_tq_tt64(int n, const double *t, const double *q, double *part, int G, const Ctl *ctl, cudaStream_t st) {
  k_dot_tq_tt<double><<<G, kRedBlock, 0, st>>>(n, t, q, part, ctl);
}
void kr_dot32(int n, const float *a, const float *b, double *part, int G, const Ctl *ctl, cudaStream_t st) {
  k_dot32c<<<G, kRedBlock, 0, st>>>(n, a, b, part, ctl);
}
void kr_dot_tq_tt32(int n, const float *t, const float *q, double *part, int G, const Ctl *ctl, cudaStream_t st) {
  k_dot_tq_tt32c<<<G, kRedBlock, 0, st>>>(n, t, q, part, ctl);
}
void kr_sumsq64(int n, const double *a, double *part, int G, cudaStream_t st) {
  k_sumsq<double><<<G, kRedBlock, 0, st>>>(n, a, part);
}
void kr_ctl_set_l2norm0(Ctl *ctl, const double *part, int G, cudaStream_t st) {
  k_ctl_set_l2norm0<<<1, kRedBlock, 0, st>>>(ctl, part, G);
}
void kr_ctl_set_l2norm(Ctl *ctl, const double *part, int G, cudaStream_t st) {
  k_ctl_set_l2norm<<<1, kRedBlock, 0, st>>>(ctl, part, G);
}
void kr_ctl_cg_rho(Ctl *ctl, const double *part, int G, cudaStream_t st) {
  k_ctl_cg_rho<<<1, kRedBlock, 0, st>>>(ctl, part, G);
}
void kr_ctl_alpha(Ctl *ctl, const double *part, int G, cudaStream_t st) {
  k_ctl_alpha<<<1, kRedBlock, 0, st>>>(ctl, part, G);
}
void kr_cg_pupdate64(int n, const double *z, double *p, const Ctl *ctl, cudaStream_t st) {
  k_cg_pupdate64<<<egrid(n), 256, 0, st>>>(n, z, p, ctl);
}
void kr_cg_update64(int n, double *x, double *d, const double *p, const double *q, double *part,
                    int G, const Ctl *ctl, cudaStream_t st, bool l2) {
  if (l2) k_cg_update64<true><<<G, kRedBlock, 0, st>>>(n, x, d, p, q, part, ctl);
  else k_cg_update64<false><<<G, kRedBlock, 0, st>>>(n, x, d, p, q, part, ctl);
}
void kr_rec_models(bool bcgs, int nm, const int *modstart, const double *p, const double *q,
                   const double *d, const double *dscale, double *part, int G, const Ctl *ctl,
                   cudaStream_t st) {
  if (bcgs) k_rec_models<true><<<G, kRedBlock, 0, st>>>(nm, modstart, p, q, d, dscale, part, ctl);
  else k_rec_models<false><<<G, kRedBlock, 0, st>>>(nm, modstart, p, q, d, dscale, part, ctl);
}
void kr_cg_pupdate32(int n, const float *z, float *p, const Ctl *ctl, cudaStream_t st) {
  k_cg_pupdate32<<<egrid(n), 256, 0, st>>>(n, z, p, ctl);
}
void kr_cg_update_mixed(int n, double *x, float *d, const float *p, const float *q, double *part,
                        int G, const Ctl *ctl, cudaStream_t st) {
  k_cg_update_mixed<<<G, kRedBlock, 0, st>>>(n, x, d, p, q, part, ctl);
}
void kr_ctl_cg_cnvg(Ctl *ctl, const double *part, int G, unsigned long long cond, int use_cond,
                    cudaStream_t st) {
  k_ctl_cg_cnvg<<<1, kRedBlock, 0, st>>>(ctl, part, G, cond, use_cond);
}
void kr_ctl_bcgs_rho(Ctl *ctl, const double *part, int G, cudaStream_t st) {
  k_ctl_bcgs_rho<<<1, kRedBlock, 0, st>>>(ctl, part, G);
}
void kr_bcgs_p64(int n, const double *d, double *p, const double *v, const Ctl *ctl, cudaStream_t st) {
  k_bcgs_p<double><<<egrid(n), 256, 0, st>>>(n, d, p, v, ctl);
}
void kr_bcgs_q64(int n, const double *d, const double *v, double *q, const Ctl *ctl, cudaStream_t st) {
  k_bcgs_q<double><<<egrid(n), 256, 0, st>>>(n, d, v, q, ctl);
}
void kr_bcgs_p32(int n, const float *d, float *p, const float *v, const Ctl *ctl, cudaStream_t st) {
  k_bcgs_p<float><<<egrid(n), 256, 0, st>>>(n, d, p, v, ctl);
}
void kr_bcgs_q32(int n, const float *d, const float *v, float *q, const Ctl *ctl, cudaStream_t st) {
  k_bcgs_q<float><<<egrid(n), 256, 0, st>>>(n, d, v, q, ctl);
}
void kr_ctl_omega(Ctl *ctl, const double *part, int G, cudaStream_t st) {
  k_ctl_omega<<<1, kRedBlock, 0, st>>>(ctl, part, G);
}
void kr_bcgs_update64(int n, double *x, double *d, const double *phat, const double *qhat,
                      const double *q, const double *t, const double *dscale, double *part, int G,
                      const Ctl *ctl, cudaStream_t st, bool l2) {
  if (l2) k_bcgs_update<double, true><<<G, kRedBlock, 0, st>>>(n, x, d, phat, qhat, q, t, dscale, part, ctl);
  else k_bcgs_update<double, false><<<G, kRedBlock, 0, st>>>(n, x, d, phat, qhat, q, t, dscale, part, ctl);
}
void kr_bcgs_update32(int n, double *x, float *d, const float *phat, const float *qhat,
                      const float *q, const float *t, const double *dscale, double *part, int G,
                      const Ctl *ctl, cudaStream_t st) {
  k_bcgs_update<float, true><<<G, kRedBlock, 0, st>>>(n, x, d, phat, qhat, q, t, dscale, part, ctl);
}
void kr_ctl_bcgs_cnvg(Ctl *ctl, const double *part, int G, unsigned long long cond, int use_cond,
                      cudaStream_t st) {
  k_ctl_bcgs_cnvg<<<1, kRedBlock, 0, st>>>(ctl, part, G, cond, use_cond);
}
void kr_ctl_mixed_inner(Ctl *ctl, const double *part, int G, int bcgs, double refine_factor,
                        cudaStream_t st) {
  k_ctl_mixed_inner<<<1, kRedBlock, 0, st>>>(ctl, part, G, bcgs, refine_factor);
}
void kr_true_resid_stats(int n, const double *r, float *d32, float *dhat32, double *dhat64,
                         const double *dscale, double *part, int G, const Ctl *ctl,
                         cudaStream_t st) {
  k_true_resid_stats<<<G, kRedBlock, 0, st>>>(n, r, d32, dhat32, dhat64, dscale, part, ctl);
}
void kr_ctl_refine(Ctl *ctl, const double *part, int G, unsigned long long cond, int use_cond,
                   cudaStream_t st) {
  k_ctl_refine<<<1, kRedBlock, 0, st>>>(ctl, part, G, cond, use_cond);
}
void kr_f64_to_f32(int n, const double *s, float *d, cudaStream_t st) {
  k_convert<float, double><<<std::min(egrid(n), 4 * kNumSM), 256, 0, st>>>(n, s, d);
}
void kr_f32_to_f64(int n, const float *s, double *d, cudaStream_t st) {
  k_convert<double, float><<<std::min(egrid(n), 4 * kNumSM), 256, 0, st>>>(n, s, d);
}


// batched ensemble launchers
void kb_dot64(const BatchDev &B, const double *a, const double *b, double *part, cudaStream_t st) {
  k_b_dot<double, double><<<B.nchunks, kRedBlock, 0, st>>>(B, a, b, part);
}
void kb_sumsq64(const BatchDev &B, const double *a, double *part, cudaStream_t st) {
  k_b_sumsq<<<B.nchunks, kRedBlock, 0, st>>>(B, a, part);
}
void kb_cg_pupdate64(const BatchDev &B, const double *z, double *p, cudaStream_t st) {
  k_b_cg_pupdate<double><<<B.nchunks, kRedBlock, 0, st>>>(B, z, p);
}
void kb_cg_update64(const BatchDev &B, double *x, double *d, const double *p, const double *q,
                    double *part, cudaStream_t st) {
  k_b_cg_update64<<<B.nchunks, kRedBlock, 0, st>>>(B, x, d, p, q, part);
}
void kb_ctl_set_l2norm0(const BatchDev &B, const double *part, cudaStream_t st) {
  k_b_ctl_set_l2norm0<<<B.nm, kRedBlock, 0, st>>>(B, part);
}
void kb_ctl_cg_rho(const BatchDev &B, const double *part, cudaStream_t st) {
  k_b_ctl_cg_rho<<<B.nm, kRedBlock, 0, st>>>(B, part);
}
void kb_ctl_alpha(const BatchDev &B, const double *part, cudaStream_t st) {
  k_b_ctl_alpha<<<B.nm, kRedBlock, 0, st>>>(B, part);
}
void kb_ctl_cg_cnvg(const BatchDev &B, const double *part, cudaStream_t st) {
  k_b_ctl_cg_cnvg<<<B.nm, kRedBlock, 0, st>>>(B, part);
}
void kb_all_done(const BatchDev &B, Ctl *gctl, unsigned long long cond, int use_cond,
                 int count_body, cudaStream_t st) {
  k_b_all_done<<<1, kRedBlock, 0, st>>>(B, gctl, cond, use_cond, count_body);
}
void kb_dot32(const BatchDev &B, const float *a, const float *b, double *part, cudaStream_t st) {
  k_b_dot32c<<<B.nchunks, kRedBlock, 0, st>>>(B, a, b, part);
}
void kb_cg_pupdate32(const BatchDev &B, const float *z, float *p, cudaStream_t st) {
  k_b_cg_pupdate32<<<B.nchunks, kRedBlock, 0, st>>>(B, z, p);
}
void kb_cg_update_mixed(const BatchDev &B, double *x, float *d, const float *p, const float *q,
                        double *part, cudaStream_t st) {
  k_b_cg_update_mixed<<<B.nchunks, kRedBlock, 0, st>>>(B, x, d, p, q, part);
}
void kb_ctl_mixed_inner(const BatchDev &B, const double *part, double refine_factor,
                        cudaStream_t st) {
  k_b_ctl_mixed_inner<<<B.nm, kRedBlock, 0, st>>>(B, part, refine_factor);
}
void kb_any_due(const BatchDev &B, Ctl *gctl, cudaStream_t st) {
  k_b_any_due<<<1, kRedBlock, 0, st>>>(B, gctl);
}
void kb_true_resid_stats(const BatchDev &B, const double *r, float *d32, double *part,
                         cudaStream_t st) {
  k_b_true_resid_stats<<<B.nchunks, kRedBlock, 0, st>>>(B, r, d32, part);
}
void kb_ctl_refine(const BatchDev &B, const double *part, cudaStream_t st) {
  k_b_ctl_refine<<<B.nm, kRedBlock, 0, st>>>(B, part);
}

}  // namespace gb
