// k_dia7.cu -- structured ILU0 triangular sweeps for full DIS grids (7-point).
//
// Replaces the level-by-level sweeps of ims_base_ilu0a
// (src/Solution/LinearMethods/ImsLinearBase.f90:1049-1092) when the CSR
// pattern is that of a full DIS grid in natural order (node = j + i*ncol +
// k*nrow*ncol).  Row n then has at most three lower neighbours, (k-1,i,j),
// (k,i-1,j), (k,i,j-1), and three upper ones.
//
// Wavefront.  A "line" is the ncol cells of one grid row (k,i).  A CTA owns
// 32 consecutive lines of one layer (a "block").  Lane l of its compute warp
// walks line l of the block S steps behind lane l-1, so the value it needs
// from the neighbour line was produced S steps earlier and arrives by a
// register shuffle.  The neighbour block (line i0-1) and the neighbour layer
// are other CTAs.
//
// Skewed layout.  The factors and the results are stored per block as
// G x 32 tiles, row g = wavefront step, column l = lane (element (g,l) is
// the cell lane l handles at step g; slots outside the grid hold zero).  A
// chunk of C steps of one array is then one contiguous C*32 tile.
//
// Hand-over.  Every result goes to global memory as a word tagged with the
// epoch of its launch (k_llword.cuh): a consumer that reads the current
// epoch has the value, with no fence or progress counter in between.  Four
// warps per CTA, so that no wait stalls the dependent chain:
//  * copy: streams the block's own factor tiles (and, backward, its forward
//    result) into a ring of NS shared-memory buffers with bulk copies
//    (cp.async.bulk), one "full" mbarrier per buffer; it also writes each
//    chunk's own right-hand side (forward r read in natural order and split
//    into df64 pairs, backward dinv*y) into the buffer ("rdy" mbarrier): in
//    the layers with a layer neighbour the pre-compute warp was the slowest
//    warp with that work, and this warp idles between its copies;
//  * pre-compute: loads the layer neighbour's words (PF chunks ahead) and
//    folds the layer term into the right-hand side (forward r - Lz*zn,
//    backward dinv*y - Uz'*zn), released through a "prep" mbarrier;
//  * edge: loads the neighbour block's last line (PF chunks ahead) for the
//    first lane;
//  * compute: per step one shuffle and the two FMAs of the row and column
//    neighbours; writes each result word, and backward also the result in
//    natural order, then frees the buffer through its "empty" mbarrier.
// The compute and pre-compute warps sit on different SM sub-partitions, so
// that their FP64 instructions do not share a pipe.  Every wait is bounded
// by the global timer; a wait that runs out sets an error flag and
// Ctl::done, the copies in flight are drained, and the CTA returns.  CTAs
// take a ticket in launch order and depend only on smaller tickets, so the
// chain of waits always ends.
//
// Forward sweep: y = r - Lz*y(k-1) - Lx*y(j-1) - Ly*y(i-1).  Backward sweep:
// z = dinv*y - Uz'*z(k+1) - Ux'*z(j+1) - Uy'*z(i+1) with the upper factors
// pre-scaled by the inverse pivot (U' = dinv*U).  Both are equal in exact
// arithmetic to ilu0a's sums; the order puts the lane's own previous result
// first, so that a step's chain through its own line is two FMAs and the
// chain through the neighbour line (the shuffle) is one.
//
// Arithmetic.  The mixed form sweeps in FP32.  The FP64 form sweeps in df64
// (pairs of floats, k_df64.cuh) when every factor tile lies in the float
// exponent range, because GB300 issues a warp's FP64 FMA only every 64 cycles
// or so and a step carries two of them; otherwise, or when GBIMS_SWEEP_NATIVE
// is set, it sweeps in native FP64.  The df64 backward sweep converts its
// result to FP64 (one FP64 add per cell) in the compute warp, off the chain,
// on the FP64 pipe that the df64 chain leaves idle.
#include <algorithm>
#include <cstdlib>

#include "gbims_internal.cuh"
#include "k_llword.cuh"

namespace gb {

namespace {


__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for phase `parity` of an mbarrier, bounded; false if it ran out or
// the CTA is aborting.
__device__ __forceinline__ bool mbar_wait(unsigned long long *b, unsigned parity,
                                          volatile int *abort_flag) {
  if (mbar_test(b, parity)) return true;
  unsigned long long t0 = wclock();
  while (!mbar_test(b, parity)) {
    if (*abort_flag || wclock() - t0 > kWaitCycles) return false;
  }
  return true;
}
// 1-D bulk copy global -> shared (16-byte aligned addresses, size a multiple
// of 16), completion counted on the mbarrier.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         unsigned long long *b) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(b))
      : "memory");
}


// The arithmetic of a sweep: T is the element type of the tiles, the result
// words and the chain; V the type of the natural-order vectors r and z.
template <typename T>
struct Elem;
template <>
struct Elem<double> {
  using V = double;
  static __device__ __forceinline__ double zero() { return 0.0; }
  static __device__ __forceinline__ double fms(double a, double b, double c) { return fma(-a, b, c); }
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double shfl_up(double v, int d) {
    return __shfl_up_sync(0xffffffffu, v, d);
  }
  static __device__ __forceinline__ double from_vec(double v) { return v; }
  static __device__ __forceinline__ double to_vec(double v) { return v; }
  static __device__ __forceinline__ double from_factor(double v) { return v; }
};
template <>
struct Elem<float> {
  using V = float;
  static __device__ __forceinline__ float zero() { return 0.0f; }
  static __device__ __forceinline__ float fms(float a, float b, float c) { return fmaf(-a, b, c); }
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float shfl_up(float v, int d) {
    return __shfl_up_sync(0xffffffffu, v, d);
  }
  static __device__ __forceinline__ float from_vec(float v) { return v; }
  static __device__ __forceinline__ float to_vec(float v) { return v; }
  static __device__ __forceinline__ float from_factor(double v) { return (float)v; }
};
template <>
struct Elem<DF> {
  using V = double;
  static __device__ __forceinline__ DF zero() { return df_zero(); }
  static __device__ __forceinline__ DF fms(DF a, DF b, DF c) { return df_fms(a, b, c); }
  static __device__ __forceinline__ DF mul(DF a, DF b) { return df_mul(a, b); }
  static __device__ __forceinline__ DF shfl_up(DF v, int d) { return df_shfl_up(v, d); }
  static __device__ __forceinline__ DF from_vec(double v) { return df_from_double(v); }
  static __device__ __forceinline__ double to_vec(DF v) { return df_to_double(v); }
  static __device__ __forceinline__ DF from_factor(double v) { return df_from_double_fp64(v); }
};
__device__ __forceinline__ bool dinv_zero(double d) { return d == 0.0; }
__device__ __forceinline__ bool dinv_zero(float d) { return d == 0.0f; }
__device__ __forceinline__ bool dinv_zero(DF d) { return d.hi == 0.0f; }

template <typename T>
struct SweepArgs {
  const Dia7Geo *geo;  // members, in ticket order
  int nm;
  const Ctl *mctl;     // per-member control blocks (batched ensembles) or null
  const T *A, *B, *X, *D;  // skewed factors (forward: Lz Ly Lx -, backward: Uz' Uy' Ux' dinv)
  const typename Elem<T>::V *rnat;  // forward: right-hand side, natural order
  typename Elem<T>::V *znat;        // backward: result, natural order
  LLWord<T> *ysk;          // forward result, skewed (written forward, read backward)
  LLWord<T> *zsk;          // backward result, skewed (written and read backward)
  unsigned long long *ticket;  // this direction's ticket counter (zeroed once, never reset)
  int *err;
  Ctl *ctl;
};

// One ring buffer of a sweep CTA: C steps of the block's tiles (32 lanes).
template <typename T, int C, int DIR>
struct Stage;
// rv: the step's own right-hand side (forward r, backward dinv*y), written
// by the edge warp; the pre-compute warp folds the layer term into it.
template <typename T, int C>
struct alignas(16) Stage<T, C, 1> {
  T a[C * 32], b[C * 32], x[C * 32];
  T rv[C * 32];
  T yn[C];  // the neighbour block's last line, one value per step
};
template <typename T, int C>
struct alignas(16) Stage<T, C, -1> {
  T a[C * 32], b[C * 32], x[C * 32], d[C * 32];
  LLWord<T> y[C * 32];  // own forward result, steps descending
  T rv[C * 32];
  T yn[C];
};

// Warp roles of a sweep CTA.
// (numbered so that, with two CTAs on an SM, each compute warp shares its
// sub-partition with the other CTA's edge warp, the lightest role, and each
// pre-compute warp with the other CTA's copy warp; see the placement below)
enum { kRoleCompute = 0, kRolePre = 1, kRoleEdge = 2, kRoleCopy = 3 };

// Poll result words of the current epoch, bounded; warp-uniform result.
// `want` marks the lanes' words still missing (bit t = word t).  A round
// issues the loads of all missing words before it looks at any of them, so
// that their round trips overlap.
template <typename T, int C>
__device__ __forceinline__ bool ll_poll(const LLWord<T> *q, long long stride, unsigned want,
                                        unsigned ep, T (&v)[C], volatile int *abort_flag) {
  unsigned long long t0 = 0;
  while (true) {
    LLRaw r[C];
#pragma unroll
    for (int t = 0; t < C; ++t)
      if ((want >> t) & 1u) ll_issue(q + t * stride, r[t]);
#pragma unroll
    for (int t = 0; t < C; ++t)
      if (((want >> t) & 1u) && ll_ready<T>(r[t], ep)) {
        ll_take(r[t], v[t]);
        want &= ~(1u << t);
      }
    if (!__any_sync(0xffffffffu, want != 0)) return true;
    if (t0 == 0) t0 = wclock();
    if (__any_sync(0xffffffffu, *abort_flag != 0 || wclock() - t0 > kWaitCycles)) return false;
  }
}

// DIR = +1 forward, -1 backward.  A CTA is one block: 32 lines of one layer.
// PF: chunks of neighbour words whose loads are in flight ahead of use.
template <typename T, int S, int C, int NS, int DIR, int PF>
__global__ void __launch_bounds__(128) k_dia7_sweep(SweepArgs<T> p) {
  constexpr int W = 32;
  using St = Stage<T, C, DIR>;
  using E = Elem<T>;
  using V = typename E::V;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  St *stg = reinterpret_cast<St *>(smem_raw);
  unsigned long long *full = reinterpret_cast<unsigned long long *>(smem_raw + NS * sizeof(St));
  unsigned long long *empty = full + NS;
  unsigned long long *prep = full + 2 * NS;
  unsigned long long *rdy = full + 3 * NS;  // rv written (edge warp)
  __shared__ int s_id, s_abort, s_rot, s_m;
  __shared__ unsigned s_ep;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    // Every CTA of a launch takes its ticket, also one that returns at once,
    // so that launch e (from 0) owns tickets [e*grid, (e+1)*grid): the local
    // ticket orders the CTAs, the launch number is the epoch of its words.
    const unsigned long long tk = atomicAdd(p.ticket, 1ULL);
    s_id = (int)(tk % gridDim.x);
    s_ep = (unsigned)(tk / gridDim.x) + 1u;
    // the member this ticket belongs to (members own contiguous tickets)
    int lo = 0, hi = p.nm - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (p.geo[mid].ticket0 <= s_id) lo = mid;
      else hi = mid - 1;
    }
    s_m = lo;
    s_abort = 0;
    // Place the roles on the SM sub-partitions (each has its own issue
    // slots and FP64 pipe; warp w of the CTA is taken to sit on
    // sub-partition (slot of warp 0 + w) mod 4): compute on 2p, pre-compute
    // on 2p+1, edge on 2p+2 and copy on 2p+3 (mod 4), p the parity of the
    // CTA's 4-slot group.  Two co-resident CTAs then pair each compute warp
    // with the other's edge warp and each pre-compute warp with the other's
    // copy warp.  The roles are a rotation of the warps in any case.
    unsigned hw;
    asm volatile("mov.u32 %0, %%warpid;" : "=r"(hw));
    const int w0 = (int)(hw & 3u), par = (int)((hw >> 2) & 1u);
    s_rot = (2 * par - w0) & 3;  // the warp that computes
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
      mbar_init(&prep[s], 2);  // pre-compute warp + edge warp
      mbar_init(&rdy[s], 1);   // edge warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (p.ctl && p.ctl->done) return;
  // a member of a batch that has reached its closure is not swept; its CTAs
  // only depend on one another, so none of them waits for it
  if (p.mctl && p.mctl[s_m].done) return;
  const int role = (warp - s_rot) & 3;
  const int id = s_id;
  const unsigned ep = s_ep;
  const Dia7Geo geo = p.geo[s_m];
  const int lid = id - geo.ticket0;
  const int nlay = geo.nlay, nrow = geo.nrow, nb = geo.nb, G = geo.G;
  const int k = (DIR > 0) ? lid % nlay : nlay - 1 - (lid % nlay);
  const int b = (DIR > 0) ? lid / nlay : nb - 1 - lid / nlay;
  const int nch = G / C;
  const bool has_blk = (DIR > 0) ? (b > 0) : (b < nb - 1);
  const bool has_lay = (DIR > 0) ? (k > 0) : (k < nlay - 1);
  const long long slot0 = geo.slot0;
  auto tile = [&](int kk, int bb) -> long long { return slot0 + ((long long)kk * nb + bb) * G * W; };
  LLWord<T> *out = (DIR > 0) ? p.ysk : p.zsk;
  volatile int *v_abort = &s_abort;
  auto fail = [&]() {
    if (lane == 0) {
      *v_abort = 1;
      atomicExch(p.err, 1);
      if (p.ctl) p.ctl->done = 1;
    }
  };

  if (role == kRolePre) {
    // ---------------- pre-compute warp ----------------
    // The terms of a step that do not depend on the wavefront: forward
    // r - Lz*y(k-1), backward dinv*y - Uz'*z(k+1), in the same order and
    // rounding as the full step.  The neighbour layer's words are polled
    // straight from global memory; the sum is written over the stage's `a`
    // tile (each element read and written by one thread) and released
    // through the stage's prep mbarrier.
    const LLWord<T> *zsrc = has_lay ? out + tile(k - DIR, b) + lane : nullptr;
    // loads of chunk c sit in slot c % PF, issued PF chunks ahead
    LLRaw zr[PF][C];
    if (has_lay) {
#pragma unroll
      for (int j = 0; j < PF; ++j)
        if (j < nch)
#pragma unroll
          for (int t = 0; t < C; ++t) ll_issue(zsrc + (long long)(j * C + t) * W, zr[j][t]);
    }
    for (int c0 = 0; c0 < nch; c0 += PF) {
#pragma unroll
      for (int j = 0; j < PF; ++j) {
        const int c = c0 + j;
        if (c >= nch) break;
        const int s = c % NS;
        const bool got = mbar_wait(&full[s], (c / NS) & 1, v_abort) &&
                         mbar_wait(&rdy[s], (c / NS) & 1, v_abort);
        if (!__all_sync(0xffffffffu, got)) {
          if (lane == 0) *v_abort = 1;
          return;
        }
        St &st = stg[s];
        T zn[C];
        if (has_lay) {
          // words that were not yet written when their load was issued are
          // polled again
          unsigned want = 0;
#pragma unroll
          for (int t = 0; t < C; ++t) {
            if (ll_ready<T>(zr[j][t], ep)) ll_take(zr[j][t], zn[t]);
            else want |= 1u << t;
          }
          if (__any_sync(0xffffffffu, want != 0) &&
              !ll_poll<T, C>(zsrc + (long long)c * C * W, W, want, ep, zn, v_abort)) {
            fail();
            return;
          }
          if (c + PF < nch)
#pragma unroll
            for (int t = 0; t < C; ++t) ll_issue(zsrc + (long long)((c + PF) * C + t) * W, zr[j][t]);
        }
#pragma unroll
        for (int t = 0; t < C; ++t) {
          const int e = t * W + lane;
          T t0 = st.rv[e];
          if (has_lay) t0 = E::fms(st.a[e], zn[t], t0);
          st.a[e] = t0;
        }
        // the buffer is refilled by the async proxy after the compute warp
        // has released it: order these generic writes before that
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&prep[s]);
      }
    }
    return;
  }

  if (role == kRoleEdge) {
    // ---------------- edge warp ----------------
    // The neighbour block's last line: lane t < C polls the word of step t
    // of the chunk (the neighbour's lane 31 reaches column g at its step
    // g + S*31) and leaves it in the stage's `yn`.
    const LLWord<T> *ysrc = has_blk ? out + tile(k, b - DIR) + (W - 1) : nullptr;
    // lane t < C: the word of step t of a chunk; loads PF chunks ahead
    auto yrow_of = [&](int c) { return c * C + S * (W - 1) + lane; };
    auto needs = [&](int c) { return has_blk && lane < C && yrow_of(c) < G; };
    LLRaw yr[PF];
#pragma unroll
    for (int j = 0; j < PF; ++j)
      if (j < nch && needs(j)) ll_issue(ysrc + (long long)yrow_of(j) * W, yr[j]);
    for (int c0 = 0; c0 < nch; c0 += PF) {
#pragma unroll
      for (int j = 0; j < PF; ++j) {
        const int c = c0 + j;
        if (c >= nch) break;
        const int s = c % NS;
        if (c >= NS) {
          const bool got = mbar_wait(&empty[s], ((c / NS) - 1) & 1, v_abort);
          if (!__all_sync(0xffffffffu, got)) {
            if (lane == 0) *v_abort = 1;
            return;
          }
        }
        if (has_blk) {
          const bool need = needs(c);
          T v[1] = {E::zero()};
          unsigned want = 0;
          if (need) {
            if (ll_ready<T>(yr[j], ep)) ll_take(yr[j], v[0]);
            else want = 1u;
          }
          if (__any_sync(0xffffffffu, want != 0) &&
              !ll_poll<T, 1>(ysrc + (long long)(need ? yrow_of(c) : 0) * W, 0, want, ep, v,
                             v_abort)) {
            fail();
            return;
          }
          if (lane < C) stg[s].yn[lane] = need ? v[0] : E::zero();
          if (c + PF < nch && needs(c + PF)) ll_issue(ysrc + (long long)yrow_of(c + PF) * W, yr[j]);
        } else if (lane < C) {
          stg[s].yn[lane] = E::zero();  // an edge block of the layer: no neighbour line
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&prep[s]);
      }
    }
    return;
  }

  // the cells of the compute warp's lane `lane` at chunk c: line i, and for
  // step t the column g0 + t - S*lane of the sweep's direction
  const int i = (DIR > 0) ? (b * W + lane) : (b * W + (W - 1 - lane));
  const bool line_ok = i >= 0 && i < nrow;
  const int ncol = geo.ncol;
  V *zrow = (DIR < 0 && line_ok) ? p.znat + geo.row0 + ((long long)k * nrow + i) * ncol : nullptr;

  if (role == kRoleCopy) {
    // ---------------- copy warp ----------------
    // The block's own tiles have no producer in this launch: they stream
    // into the ring as fast as buffers free up.
    int issued = 0;
    bool ok = true;
    const unsigned tileb = C * W * sizeof(T);
    // It also writes each chunk's own right-hand side for the pre-compute
    // warp: forward r
    // from natural order (lane l walks line b*W + l; step g is column
    // g - S*l), kept as loaded until it is used (a conversion right after
    // the load would wait for it and the prefetch would hide nothing);
    // backward dinv*y from the stage's tiles
    const int ri = b * W + lane;
    const bool rline = (DIR > 0) && ri < nrow;
    const V *rrow = rline ? p.rnat + geo.row0 + ((long long)k * nrow + ri) * geo.ncol : nullptr;
    auto rload = [&](int c, V (&dst)[C]) {
#pragma unroll
      for (int t = 0; t < C; ++t) {
        const int jj = c * C + t - S * lane;
        dst[t] = (rline && (unsigned)jj < (unsigned)geo.ncol) ? __ldg(rrow + jj) : V(0);
      }
    };
    // r is loaded PR chunks ahead of its chunk (at least four: under the
    // load of a full grid its latency reaches several chunks)
    constexpr int PR = (PF < 4) ? 4 : PF;
    V rr[PR][C];
    if constexpr (DIR > 0) {
#pragma unroll
      for (int j = 0; j < PR; ++j)
        if (j < nch) rload(j, rr[j]);
    }
    // chunk q's rv: forward right after its tiles are issued (r has no
    // producer in the launch), backward once its tiles have landed, LB
    // chunks behind the copies (half the ring: the copies of LB chunks stay
    // in flight, and a chunk's tiles have had LB chunks' time to land).
    // LB <= NS - 1 keeps the waits acyclic: rv of chunk q is made after the
    // copy of q + LB, which waits for the compute warp's chunk q + LB - NS,
    // whose rv came LB chunks earlier still.
    constexpr int LB = (NS / 2 > 1) ? NS / 2 : 1;
    auto make_rv = [&](int q, int j) -> bool {
      St &st = stg[q % NS];
      if constexpr (DIR > 0) {
#pragma unroll
        for (int t = 0; t < C; ++t) st.rv[t * W + lane] = E::from_vec(rr[j][t]);
        if (q + PR < nch) rload(q + PR, rr[j]);
      } else {
        (void)j;
        if (!__all_sync(0xffffffffu, mbar_wait(&full[q % NS], (q / NS) & 1, v_abort))) return false;
#pragma unroll
        for (int t = 0; t < C; ++t) {
          const int e = t * W + lane;
          // the forward words of padding slots (dinv zero) may not have
          // been copied into this buffer: take zero, not 0 * stale bits
          const T dv = st.d[e];
          st.rv[e] = dinv_zero(dv) ? E::zero() : E::mul(dv, ll_val(st.y[C * W - 1 - e]));
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&rdy[q % NS]);
      return true;
    };
    for (int c0 = 0; ok && c0 < nch; c0 += PR) {
#pragma unroll
    for (int j = 0; j < PR; ++j) {
      const int c = c0 + j;
      if (c >= nch) break;
      const int s = c % NS;
      if (c >= NS) {
        const bool got = mbar_wait(&empty[s], ((c / NS) - 1) & 1, v_abort);
        ok = __all_sync(0xffffffffu, got);
        if (!ok) break;
      }
      if (lane == 0) {
        St &st = stg[s];
        const int g0 = c * C;
        const long long tb = tile(k, b) + (long long)g0 * W;
        if constexpr (DIR > 0) {
          mbar_expect_tx(&full[s], 3 * tileb);
        } else {
          // own forward result, steps P descending
          const int phi = geo.ncol - 1 + S * (W - 1) - g0;
          const int pl = phi - (C - 1);
          const int lo = max(pl, 0), hi = min(phi, G - 1);
          const int prows = max(0, hi - lo + 1);
          const int pskip = lo - pl;
          const unsigned ybytes = prows * W * (unsigned)sizeof(LLWord<T>);
          mbar_expect_tx(&full[s], 4 * tileb + ybytes);
          bulk_g2s(st.d, p.D + tb, tileb, &full[s]);
          if (prows > 0)
            bulk_g2s(st.y + pskip * W, p.ysk + tile(k, b) + (long long)lo * W, ybytes, &full[s]);
        }
        bulk_g2s(st.a, p.A + tb, tileb, &full[s]);
        bulk_g2s(st.b, p.B + tb, tileb, &full[s]);
        bulk_g2s(st.x, p.X + tb, tileb, &full[s]);
      }
      issued = c + 1;
      __syncwarp();
      if constexpr (DIR > 0) {
        ok = make_rv(c, j);
      } else {
        if (c >= LB) ok = make_rv(c - LB, 0);
      }
      if (!ok) break;
    }
    }
    if constexpr (DIR < 0) {
      for (int q = max(0, nch - LB); ok && q < nch; ++q) ok = make_rv(q, 0);
    }
    if (!ok) fail();
    if (lane == 0) {
      // every copy issued has landed before this warp, and so the CTA, ends
      // (the other warps may have left early on an abort)
      for (int c = max(0, issued - NS); c < issued; ++c) {
        unsigned long long t0 = wclock();
        while (!mbar_test(&full[c % NS], (c / NS) & 1))
          if (wclock() - t0 > kWaitCycles) break;
      }
    }
    return;
  }

  // ---------------- compute warp ----------------
  // Per step one shuffle and the two FMAs of the column and row neighbours,
  // on operands moved from the ring buffer into registers at the start of
  // the chunk; each result goes straight out as a word of this epoch.
  LLWord<T> *outt = out + tile(k, b) + lane;
  T h1 = E::zero(), h2 = E::zero();
  for (int c = 0; c < nch; ++c) {
    const int s = c % NS;
    const bool got = mbar_wait(&full[s], (c / NS) & 1, v_abort) &&
                     mbar_wait(&prep[s], (c / NS) & 1, v_abort);
    if (!__all_sync(0xffffffffu, got)) {
      if (lane == 0) *v_abort = 1;
      return;
    }
    St &st = stg[s];
    const int g0 = c * C;
    const int jc = g0 - S * lane;
    T ra[C], rb[C], rx[C], ryn[C];
#pragma unroll
    for (int t = 0; t < C; ++t) {
      ra[t] = st.a[t * W + lane];  // pre-computed r - Lz*zn (backward: dinv*y - Uz'*zn)
      rb[t] = st.b[t * W + lane];
      rx[t] = st.x[t * W + lane];
      ryn[t] = st.yn[t];
    }
#pragma unroll
    for (int t = 0; t < C; ++t) {
      T yv = E::shfl_up((S == 1) ? h1 : h2, 1);
      if (lane == 0) yv = ryn[t];
      // the coefficients of absent neighbours are zero (first line of the
      // grid, first column, padding slots) and every value is finite, so
      // both products are taken unconditionally and padding slots come out
      // zero: no divergent lanes and no select on the chain
      T tv = E::fms(rx[t], h1, ra[t]);
      tv = E::fms(rb[t], yv, tv);
      ll_put(outt + (long long)(g0 + t) * W, tv, ep);
      if constexpr (DIR < 0) {
        // the result in natural order (df64: widened and added in FP64, off
        // the chain, on this sub-partition's otherwise idle FP64 pipe)
        const int jj = jc + t;
        if (line_ok && (unsigned)jj < (unsigned)ncol) zrow[ncol - 1 - jj] = E::to_vec(tv);
      }
      h2 = h1;
      h1 = tv;
    }
    // the input buffer goes back to the copy and edge warps
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

// APC/JAPC -> skewed tiles.  Forward tiles hold Lz, Ly, Lx of the cell that
// lane l visits at step g; backward tiles hold dinv*Uz, dinv*Uy, dinv*Ux and
// dinv.  Slots outside the grid are zero.
// With an IDOMAIN-reduced grid (userred/nodeuser not null) the factor rows
// are those of the reduced nodes: a slot's cell reads the row of its reduced
// node (an inactive cell keeps zeros, dinv included) and recognises its
// neighbours by their user cells.
template <typename T>
__global__ void k_dia7_extract(const Dia7Geo *__restrict__ geos, int nm, long long nslot, int W,
                               int S, int dir, const int *__restrict__ iapc,
                               const int *__restrict__ japc, const double *__restrict__ apc,
                               const int *__restrict__ userred, const int *__restrict__ nodeuser,
                               T *A, T *B, T *X, T *D) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nslot;
       q += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = nm - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (geos[mid].slot0 <= q) lo = mid;
      else hi = mid - 1;
    }
    const Dia7Geo g = geos[lo];
    const long long lq = q - g.slot0;
    const long long nrc = (long long)g.nrow * g.ncol;
    const int l = (int)(lq % W);
    const long long r1 = lq / W;
    const int gg = (int)(r1 % g.G);
    const long long kb = r1 / g.G;
    const int b = (int)(kb % g.nb), k = (int)(kb / g.nb);
    const int jj = gg - S * l;
    const int i = (dir > 0) ? b * W + l : b * W + (W - 1 - l);
    double va = 0, vb = 0, vx = 0, vd = 0;
    const int j = (dir > 0) ? jj : g.ncol - 1 - jj;
    const long long n = g.row0 + k * nrc + (long long)i * g.ncol + j;
    const long long rn = (i < g.nrow && jj >= 0 && jj < g.ncol) ? (userred ? userred[n] : n) : -1;
    if (rn >= 0) {
      const double d = apc[rn];
      for (int pp = iapc[rn]; pp < iapc[rn + 1]; ++pp) {
        const long long c = nodeuser ? nodeuser[japc[pp]] : japc[pp];
        const double a = apc[pp];
        if (dir > 0) {
          if (k > 0 && c == n - nrc) va = a;
          else if (i > 0 && c == n - g.ncol) vb = a;
          else if (j > 0 && c == n - 1) vx = a;
        } else {
          if (k < g.nlay - 1 && c == n + nrc) va = d * a;
          else if (i < g.nrow - 1 && c == n + g.ncol) vb = d * a;
          else if (j < g.ncol - 1 && c == n + 1) vx = d * a;
        }
      }
      vd = d;
    }
    A[q] = Elem<T>::from_factor(va);
    B[q] = Elem<T>::from_factor(vb);
    X[q] = Elem<T>::from_factor(vx);
    if (D) D[q] = Elem<T>::from_factor(vd);
  }
}

// Sets *flag when a tile value is not finite or, being nonzero, lies outside
// [2^-100, 2^100]: such factors keep the native FP64 sweeps.
__global__ void k_dia7_range(long long nslot, const double *__restrict__ a0,
                             const double *__restrict__ a1, const double *__restrict__ a2,
                             const double *__restrict__ a3, const double *__restrict__ a4,
                             const double *__restrict__ a5, const double *__restrict__ a6,
                             int *flag) {
  const double *arr[7] = {a0, a1, a2, a3, a4, a5, a6};
  int bad = 0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nslot;
       q += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int t = 0; t < 7; ++t) {
      const unsigned long long u = (unsigned long long)__double_as_longlong(arr[t][q]);
      const int e = (int)((u >> 52) & 0x7ff);  // biased exponent; 0 for zero and denormals
      const bool zero = (u << 1) == 0ULL;
      if (!zero && (e < 1023 - 100 || e > 1023 + 100)) bad = 1;
    }
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// FP64 tile -> df64 tile in place (8 bytes each, element by element).
__global__ void k_dia7_to_df(long long nslot, double *a) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nslot;
       q += (long long)gridDim.x * blockDim.x) {
    const double v = a[q];
    reinterpret_cast<DF *>(a)[q] = df_from_double_fp64(v);
  }
}

// Wavefront shape: W = 32 lines per block (one warp), lane skew S = 1.  A
// sweep's chunk C (steps per ring buffer), ring depth NS and prefetch depth
// PF are run-time choices among the configurations below: the padded step
// count G is a multiple of 16, so every C fits the same layout, and
// gbims_autotune times them on the handle's own system.
// The FP32 lane skew can be set at build time (GB_DIA32_S, 1 or 2): with
// S = 2 the shuffle leaves a step's dependency chain at the price of twice
// the lag between neighbour blocks.
#ifndef GB_DIA32_S
#define GB_DIA32_S 1
#endif
constexpr int kW = 32, kGPad = 16;
template <typename T>
constexpr int kSOf = 1;
template <>
constexpr int kSOf<float> = GB_DIA32_S;
template <>
constexpr int kSOf<DF> = 1;
static_assert(GB_DIA32_S == 1 || GB_DIA32_S == 2, "lane skew 1 or 2");
// OCC 2: the CTA asks for enough shared memory that at most two share an
// SM, so that each compute warp has a sub-partition's FP64 pipe to itself.
struct SweepCfg {
  int C, NS, PF, OCC;
};
constexpr SweepCfg kSweepCfgs[] = {{8, 4, 1, 0},  {8, 4, 2, 0},  {4, 8, 1, 0},  {4, 8, 2, 0},
                                   {16, 2, 1, 0}, {16, 2, 2, 0}, {8, 4, 1, 2},  {8, 4, 2, 2},
                                   {4, 8, 1, 2},  {4, 8, 2, 2},  {16, 2, 1, 2}, {16, 2, 2, 2}};
constexpr size_t kOcc2Smem = 80 * 1024;
constexpr int kNumSweepCfgs = sizeof(kSweepCfgs) / sizeof(kSweepCfgs[0]);

template <typename T, int C, int NS, int DIR>
constexpr size_t stage_bytes() {
  return NS * sizeof(Stage<T, C, DIR>) + 4 * NS * sizeof(unsigned long long);
}
static_assert(stage_bytes<double, 16, 2, -1>() <= 72 * 1024 && stage_bytes<double, 4, 8, -1>() <= 72 * 1024 &&
                  stage_bytes<double, 8, 4, -1>() <= 72 * 1024,
              "three sweep CTAs per SM");

}  // namespace

bool dia7_matches(int nlay, int nrow, int ncol, int n, const std::vector<int> &ia,
                  const std::vector<int> &ja) {
  if ((long long)nlay * nrow * ncol != n) return false;
  long long nrc = (long long)nrow * ncol;
  for (int r = 0; r < n; ++r) {
    int k = (int)(r / nrc);
    int rem = (int)(r - k * nrc);
    int i = rem / ncol, j = rem - i * ncol;
    long long want[7];
    int w = 0;
    want[w++] = r;
    if (k > 0) want[w++] = r - nrc;
    if (i > 0) want[w++] = r - ncol;
    if (j > 0) want[w++] = r - 1;
    if (j < ncol - 1) want[w++] = r + 1;
    if (i < nrow - 1) want[w++] = r + ncol;
    if (k < nlay - 1) want[w++] = r + nrc;
    if (ia[r + 1] - ia[r] != w) return false;
    for (int q = 0; q < w; ++q)
      if (ja[ia[r] + q] != want[q]) return false;
  }
  return true;
}

// The pattern of a DIS grid whose inactive cells were removed (IDOMAIN):
// row r is user cell nodeuser[r] (strictly increasing), with the active
// ones of its six neighbours, in the full grid's JA order, renumbered.
bool dia7_matches_reduced(int nlay, int nrow, int ncol, int n, const std::vector<int> &ia,
                          const std::vector<int> &ja, const int *nodeuser) {
  const long long nrc = (long long)nrow * ncol, nu = nrc * nlay;
  if (n <= 0 || (long long)n > nu || (int)ia.size() != n + 1) return false;
  std::vector<int> red((size_t)nu, -1);
  for (int r = 0; r < n; ++r) {
    const long long u = nodeuser[r];
    if (u < 0 || u >= nu || (r > 0 && u <= nodeuser[r - 1])) return false;
    red[(size_t)u] = r;
  }
  for (int r = 0; r < n; ++r) {
    const long long u = nodeuser[r];
    const int k = (int)(u / nrc);
    const long long rem = u - k * nrc;
    const int i = (int)(rem / ncol), j = (int)(rem - (long long)i * ncol);
    long long nb[7];
    int w = 0;
    nb[w++] = u;
    if (k > 0) nb[w++] = u - nrc;
    if (i > 0) nb[w++] = u - ncol;
    if (j > 0) nb[w++] = u - 1;
    if (j < ncol - 1) nb[w++] = u + 1;
    if (i < nrow - 1) nb[w++] = u + ncol;
    if (k < nlay - 1) nb[w++] = u + nrc;
    int q = ia[r];
    for (int t = 0; t < w; ++t) {
      const int rr = red[(size_t)nb[t]];
      if (rr < 0) continue;
      if (q >= ia[r + 1] || ja[q] != rr) return false;
      ++q;
    }
    if (q != ia[r + 1]) return false;
  }
  return true;
}

namespace {
template <typename V>
__global__ void k_dia7_spread(long long nuser, const int *__restrict__ userred,
                              const V *__restrict__ r, V *__restrict__ rfull) {
  for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nuser;
       u += (long long)gridDim.x * blockDim.x) {
    const int rr = userred[u];
    rfull[u] = (rr >= 0) ? r[rr] : V(0);
  }
}
template <typename V>
__global__ void k_dia7_collect(int n, const int *__restrict__ nodeuser, const V *__restrict__ zfull,
                               V *__restrict__ z) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    z[q] = zfull[nodeuser[q]];
}
int vgrid(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8LL * kNumSM)); }
}  // namespace

void launch_dia7_spread(const Dia7 &D, int n, const double *r, double *rfull, cudaStream_t st) {
  (void)n;
  k_dia7_spread<double><<<vgrid(D.nuser), 256, 0, st>>>(D.nuser, D.d_userred, r, rfull);
}
void launch_dia7_spread32(const Dia7 &D, int n, const float *r, float *rfull, cudaStream_t st) {
  (void)n;
  k_dia7_spread<float><<<vgrid(D.nuser), 256, 0, st>>>(D.nuser, D.d_userred, r, rfull);
}
void launch_dia7_collect(const Dia7 &D, int n, const double *zfull, double *z, cudaStream_t st) {
  k_dia7_collect<double><<<vgrid(n), 256, 0, st>>>(n, D.d_nodeuser, zfull, z);
}
void launch_dia7_collect32(const Dia7 &D, int n, const float *zfull, float *z, cudaStream_t st) {
  k_dia7_collect<float><<<vgrid(n), 256, 0, st>>>(n, D.d_nodeuser, zfull, z);
}

bool dia7_detect(int n, const std::vector<int> &ia, const std::vector<int> &ja, int *nlay,
                 int *nrow, int *ncol) {
  if (n < 2 || (int)ia.size() != n + 1) return false;
  // row 0 of a natural-order DIS grid has only upper neighbours, at offsets
  // 1 (next column), ncol (next row) and nrow*ncol (next layer), each present
  // when its dimension exceeds one.  A grid with a dimension of one has the
  // pattern of a smaller-rank grid, which the sweeps treat alike.
  std::vector<long long> off;
  for (int q = ia[0] + 1; q < ia[1]; ++q) off.push_back(ja[q]);
  long long l = 1, r = 1, c = n;
  if (off.size() == 1 && off[0] == 1) {
    l = 1; r = 1; c = n;
  } else if (off.size() == 2 && off[0] == 1 && off[1] > 1 && n % off[1] == 0) {
    l = 1; r = n / off[1]; c = off[1];
  } else if (off.size() == 3 && off[0] == 1 && off[1] > 1 && off[2] > off[1] &&
             off[2] % off[1] == 0 && n % off[2] == 0) {
    l = n / off[2]; r = off[2] / off[1]; c = off[1];
  } else {
    return false;
  }
  if (!dia7_matches((int)l, (int)r, (int)c, n, ia, ja)) return false;
  *nlay = (int)l;
  *nrow = (int)r;
  *ncol = (int)c;
  return true;
}

// Geometry of the skewed layout of one precision.
void dia7_geometry(int nlay, int nrow, int ncol, bool fp32, int *nb, int *G, long long *slots) {
  const int S = fp32 ? kSOf<float> : kSOf<double>;
  *nb = (nrow + kW - 1) / kW;
  *G = ((ncol + S * (kW - 1) + kGPad - 1) / kGPad) * kGPad;
  *slots = (long long)nlay * (*nb) * (*G) * kW;
}

int dia7_num_cfgs() { return kNumSweepCfgs; }
void dia7_cfg(int i, int *C, int *NS, int *PF, int *OCC) {
  *C = kSweepCfgs[i].C;
  *NS = kSweepCfgs[i].NS;
  *PF = kSweepCfgs[i].PF;
  *OCC = kSweepCfgs[i].OCC;
}

void dia7_layout(Dia7 &D, const std::vector<int> &shapes, const std::vector<long long> &row0,
                 bool fp32) {
  D.nm = (int)row0.size();
  D.geo.resize(D.nm);
  long long slots = 0;
  int tickets = 0;
  for (int m = 0; m < D.nm; ++m) {
    Dia7Geo &g = D.geo[m];
    g.nlay = shapes[3 * m];
    g.nrow = shapes[3 * m + 1];
    g.ncol = shapes[3 * m + 2];
    long long ms = 0;
    dia7_geometry(g.nlay, g.nrow, g.ncol, fp32, &g.nb, &g.G, &ms);
    g.ticket0 = tickets;
    g.slot0 = slots;
    g.row0 = row0[m];
    tickets += g.nlay * g.nb;
    slots += ms;  // a multiple of 16*W elements: every member starts 16-byte aligned
  }
  D.slots = slots;
  D.ntickets = tickets;
  if (D.nm == 1) {
    D.nlay = D.geo[0].nlay;
    D.nrow = D.geo[0].nrow;
    D.ncol = D.geo[0].ncol;
    D.nb = D.geo[0].nb;
    D.G = D.geo[0].G;
  }
}

template <typename T>
static void extract_t(const Dia7 &D, const int *d_iapc, const int *d_japc, const double *d_apc,
                      T *const *arr, cudaStream_t st) {
  const long long nslot = D.slots;
  int grid = (int)std::min<long long>((nslot + 255) / 256, 8LL * kNumSM);
  k_dia7_extract<T><<<grid, 256, 0, st>>>(D.d_geo, D.nm, nslot, kW, kSOf<T>, 1, d_iapc, d_japc,
                                          d_apc, D.d_userred, D.d_nodeuser, arr[0], arr[1], arr[2],
                                          nullptr);
  k_dia7_extract<T><<<grid, 256, 0, st>>>(D.d_geo, D.nm, nslot, kW, kSOf<T>, -1, d_iapc, d_japc,
                                          d_apc, D.d_userred, D.d_nodeuser, arr[3], arr[4], arr[5],
                                          arr[6]);
}

int launch_dia7_extract(Dia7 &D, int n, const int *d_iapc, const int *d_japc,
                        const double *d_apc, bool mixed, cudaStream_t st) {
  (void)n;
  if (!mixed) {
    double *arr[7] = {D.d_lz, D.d_ly, D.d_lx, D.d_uz, D.d_uy, D.d_ux, D.d_dinv};
    extract_t<double>(D, d_iapc, d_japc, d_apc, arr, st);
    D.ext = 0;
    if (D.ext_allowed) {
      // df64 sweeps when every tile value lies in the float exponent range
      int *flag = D.d_err + 2;
      int bad = 1;
      const int grid = (int)std::min<long long>((D.slots + 255) / 256, 8LL * kNumSM);
      if (cudaMemsetAsync(flag, 0, sizeof(int), st) != cudaSuccess) return -1;
      k_dia7_range<<<grid, 256, 0, st>>>(D.slots, arr[0], arr[1], arr[2], arr[3], arr[4], arr[5],
                                        arr[6], flag);
      if (cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return -1;
      if (!bad) {
        for (double *a : arr) k_dia7_to_df<<<grid, 256, 0, st>>>(D.slots, a);
        D.ext = 1;
      }
    }
  } else {
    float *arr[7] = {D.f_lz, D.f_ly, D.f_lx, D.f_uz, D.f_uy, D.f_ux, D.f_dinv};
    extract_t<float>(D, d_iapc, d_japc, d_apc, arr, st);
  }
  return 0;
}

// One sweep of one configuration (opting in to more than 48 KB of dynamic
// shared memory once per kernel).
template <typename T, int C, int NS, int PF, int DIR>
static void sweep_one(const SweepArgs<T> &a, const Dia7 &D, int occ, cudaStream_t st) {
  constexpr size_t bytes = stage_bytes<T, C, NS, DIR>();
  static bool opted = false;
  if (!opted) {  // allow up to the two-per-SM request
    cudaFuncSetAttribute(k_dia7_sweep<T, kSOf<T>, C, NS, DIR, PF>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max(bytes, kOcc2Smem));
    opted = true;
  }
  const size_t sm = (occ == 2) ? std::max(bytes, kOcc2Smem) : bytes;
  k_dia7_sweep<T, kSOf<T>, C, NS, DIR, PF><<<D.ntickets, 128, sm, st>>>(a);
}

template <typename T, int DIR>
static void sweep_cfg(const SweepArgs<T> &a, const Dia7 &D, int cfg, cudaStream_t st) {
  const int occ = kSweepCfgs[cfg].OCC;
  switch (cfg % 6) {
    case 1: sweep_one<T, 8, 4, 2, DIR>(a, D, occ, st); break;
    case 2: sweep_one<T, 4, 8, 1, DIR>(a, D, occ, st); break;
    case 3: sweep_one<T, 4, 8, 2, DIR>(a, D, occ, st); break;
    case 4: sweep_one<T, 16, 2, 1, DIR>(a, D, occ, st); break;
    case 5: sweep_one<T, 16, 2, 2, DIR>(a, D, occ, st); break;
    default: sweep_one<T, 8, 4, 1, DIR>(a, D, occ, st); break;
  }
}

// One ILU0 application: the forward sweep reads r in natural order, the
// backward sweep writes z in natural order; between them the results live
// in the skewed layout as epoch-tagged words.  No memory is reset between
// applications: each sweep launch writes its words with a new epoch.  The
// two sweeps may use different tilings (D.cfg, D.cfg_b); D.only restricts
// an application to one of them (the autotuner's timing).
template <typename T>
static void apply_t(const Dia7 &D, const T *const *arr, const typename Elem<T>::V *r,
                    typename Elem<T>::V *z, const Ctl *ctl, cudaStream_t st) {
  SweepArgs<T> a;
  a.geo = D.d_geo;
  a.nm = D.nm;
  a.mctl = D.mctl;
  a.rnat = r;
  a.znat = z;
  a.ysk = static_cast<LLWord<T> *>(D.ll_y);
  a.zsk = static_cast<LLWord<T> *>(D.ll_z);
  a.err = D.d_err;
  a.ctl = const_cast<Ctl *>(ctl);
  if (D.only >= 0) {
    a.A = arr[0]; a.B = arr[1]; a.X = arr[2]; a.D = nullptr;
    a.ticket = reinterpret_cast<unsigned long long *>(D.d_flags);
    sweep_cfg<T, 1>(a, D, D.cfg, st);
  }
  if (D.only <= 0) {
    a.A = arr[3]; a.B = arr[4]; a.X = arr[5]; a.D = arr[6];
    a.ticket = reinterpret_cast<unsigned long long *>(D.d_flags + 32);
    sweep_cfg<T, -1>(a, D, D.cfg_b >= 0 ? D.cfg_b : D.cfg, st);
  }
}

void launch_dia7_apply64(const Dia7 &D, const double *r, double *z, const Ctl *ctl,
                         cudaStream_t st) {
  if (D.ext) {
    const DF *arr[7] = {reinterpret_cast<const DF *>(D.d_lz), reinterpret_cast<const DF *>(D.d_ly),
                        reinterpret_cast<const DF *>(D.d_lx), reinterpret_cast<const DF *>(D.d_uz),
                        reinterpret_cast<const DF *>(D.d_uy), reinterpret_cast<const DF *>(D.d_ux),
                        reinterpret_cast<const DF *>(D.d_dinv)};
    apply_t<DF>(D, arr, r, z, ctl, st);
    return;
  }
  const double *arr[7] = {D.d_lz, D.d_ly, D.d_lx, D.d_uz, D.d_uy, D.d_ux, D.d_dinv};
  apply_t<double>(D, arr, r, z, ctl, st);
}


void launch_dia7_apply32(const Dia7 &D, const float *r, float *z, const Ctl *ctl,
                         cudaStream_t st) {
  const float *arr[7] = {D.f_lz, D.f_ly, D.f_lx, D.f_uz, D.f_uy, D.f_ux, D.f_dinv};
  apply_t<float>(D, arr, r, z, ctl, st);
}

}  // namespace gb
