// k_dia7.cu -- structured ILU0 triangular sweeps for full DIS grids (7-point).
//
// Replaces the level-by-level sweeps of ims_base_ilu0a
// (src/Solution/LinearMethods/ImsLinearBase.f90:1049-1092) when the CSR
// pattern is that of a full DIS grid in natural order (node = j + i*ncol +
// k*nrow*ncol).  Row n then has at most three lower neighbours, (k-1,i,j),
// (k,i-1,j), (k,i,j-1), and three upper ones.
//
// Wavefront.  A "line" is the ncol cells of one grid row (k,i).  A CTA owns W
// consecutive lines of one layer (a "block").  Lane l of its compute warp
// walks line l of the block S steps behind lane l-1, so the value it needs
// from the neighbour line was produced S steps earlier and arrives by a
// register shuffle (with S >= 2 only the FMA with the lane's own previous
// column is on a step's dependency chain; with S = 1, the default, the
// shuffle and the row-neighbour FMA are too, but the blocks lag each other
// by half as many steps).  The neighbour block (line i0-1) and the
// neighbour layer are other CTAs.
//
// Skewed layout.  The factors and the intermediate results are stored per
// block as G x W tiles, row g = wavefront step, column l = lane (element
// (g,l) is the cell lane l handles at step g; slots outside the grid hold
// zero).  A chunk of C steps of one array is then one contiguous C*W tile.
//
// Four warps per CTA, so that no fence and no off-chain arithmetic ever
// stalls the dependent chain:
//  * copy: waits for the producer CTAs' progress words and stages the chunks
//    into a ring of NS shared-memory buffers with TMA bulk copies
//    (cp.async.bulk), one "full" mbarrier per buffer;
//  * pre-compute: once a buffer is full, folds the right-hand side and the
//    layer-neighbour term (r - Lz*zn; backward dinv*y - Uz'*zn) into one
//    tile and releases it through a "prep" mbarrier;
//  * compute: per step one shuffle and the two FMAs of the row and column
//    neighbours; writes the C x W result tile to a shared-memory ring and
//    frees the buffer through its "empty" mbarrier;
//  * store: sends finished result tiles out with bulk stores and publishes
//    the CTA's progress word (bulk-store completion, proxy fence, gpu-scope
//    fence, store).  On GB300 a gpu-scope fence costs on the order of a
//    microsecond, which is why it lives in a warp of its own.
// The roles rotate with the CTA's hardware warp slot so that compute warps
// of co-resident CTAs land on different SM sub-partitions (FP64 pipes).
// Every wait is bounded by the global timer; a wait that runs out sets an
// error flag and Ctl::done, drains the copies in flight and returns.  CTAs
// take a ticket in launch order and depend only on smaller tickets, so the
// chain of waits always ends.
//
// Forward sweep: y = r - Lz*y(k-1) - Ly*y(i-1) - Lx*y(j-1), in the reference's
// order (ascending column), so it rounds exactly like ilu0a with FMA.
// Backward sweep: z = dinv*y - Uz'*z(k+1) - Uy'*z(i+1) - Ux'*z(j+1) with the
// upper factors pre-scaled by the inverse pivot (U' = dinv*U), equal in exact
// arithmetic to the reference's (y - sum U z)*dinv with one FMA instead of two
// dependent operations on the critical path.  The forward input and the
// backward output are in natural order: k_dia7_skew / k_dia7_unskew permute
// them with coalesced row accesses.
#include "gbims_internal.cuh"

namespace gb {

namespace {

constexpr unsigned long long kWaitNs = 2000000000ULL;  // 2 s per wait

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
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
  unsigned long long t0 = gtimer();
  while (!mbar_test(b, parity)) {
    if (*abort_flag || gtimer() - t0 > kWaitNs) return false;
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

__device__ __forceinline__ void ll_put(LLWord<double> *p, double x, unsigned ep) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long f = (unsigned long long)ep << 32;
  asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(p), "l"((b & 0xffffffffULL) | f),
               "l"((b >> 32) | f)
               : "memory");
}
__device__ __forceinline__ void ll_put(LLWord<float> *p, float x, unsigned ep) {
  const unsigned long long v = (unsigned long long)__float_as_uint(x) | ((unsigned long long)ep << 32);
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
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

template <typename T>
struct SweepArgs {
  const Dia7Geo *geo;  // members, in ticket order
  int nm;
  const Ctl *mctl;     // per-member control blocks (batched ensembles) or null
  const T *A, *B, *X, *D;  // skewed factors (forward: Lz Ly Lx -, backward: Uz' Uy' Ux' dinv)
  const T *rsk;            // forward: right-hand side, skewed
  LLWord<T> *ysk;          // forward result, skewed (written forward, read backward)
  LLWord<T> *zsk;          // backward result, skewed (written and read backward)
  unsigned long long *ticket;  // this direction's ticket counter (zeroed once, never reset)
  int *err;
  Ctl *ctl;
};

// One ring buffer of a sweep CTA: C steps of the block's tiles (32 lanes).
template <typename T, int C, int DIR>
struct Stage;
template <typename T, int C>
struct alignas(16) Stage<T, C, 1> {
  T a[C * 32], b[C * 32], x[C * 32], r[C * 32];
  T yn[C];  // the neighbour block's last line, one value per step
};
template <typename T, int C>
struct alignas(16) Stage<T, C, -1> {
  T a[C * 32], b[C * 32], x[C * 32], d[C * 32];
  LLWord<T> y[C * 32];  // own forward result, steps descending
  T yn[C];
};

// Warp roles of a sweep CTA.
enum { kRoleCompute = 0, kRoleCopy = 1, kRoleEdge = 2, kRolePre = 3 };

// Poll result words of the current epoch, bounded; warp-uniform result.
// `want` marks the lanes' words still missing (bit t = word t).
template <typename T, int C>
__device__ __forceinline__ bool ll_poll(const LLWord<T> *q, long long stride, unsigned want,
                                        unsigned ep, T (&v)[C], volatile int *abort_flag) {
  unsigned long long t0 = 0;
  while (true) {
#pragma unroll
    for (int t = 0; t < C; ++t)
      if ((want >> t) & 1u)
        if (ll_get(q + t * stride, ep, v[t])) want &= ~(1u << t);
    if (!__any_sync(0xffffffffu, want != 0)) return true;
    if (t0 == 0) t0 = gtimer();
    if (__any_sync(0xffffffffu, *abort_flag != 0 || gtimer() - t0 > kWaitNs)) return false;
  }
}

// DIR = +1 forward, -1 backward.  A CTA is one block: 32 lines of one layer.
template <typename T, int S, int C, int NS, int DIR>
__global__ void __launch_bounds__(128) k_dia7_sweep(SweepArgs<T> p) {
  constexpr int W = 32;
  using St = Stage<T, C, DIR>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  St *stg = reinterpret_cast<St *>(smem_raw);
  unsigned long long *full = reinterpret_cast<unsigned long long *>(smem_raw + NS * sizeof(St));
  unsigned long long *empty = full + NS;
  unsigned long long *prep = full + 2 * NS;
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
    // Rotate the roles by the CTA's warp-slot group on the SM, so that the
    // compute warps of co-resident CTAs sit on different SM sub-partitions
    // (each has its own FP64 pipe).
    unsigned hw;
    asm volatile("mov.u32 %0, %%warpid;" : "=r"(hw));
    s_rot = (int)((hw >> 2) & 3u);
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
      mbar_init(&prep[s], 2);  // pre-compute warp + edge warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (p.ctl && p.ctl->done) return;
  // a member of a batch that has reached its closure is not swept; its CTAs
  // only depend on one another, so none of them waits for it
  if (p.mctl && p.mctl[s_m].done) return;
  const int role = (warp + s_rot) & 3;
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
    for (int c = 0; c < nch; ++c) {
      const int s = c % NS;
      const bool got = mbar_wait(&full[s], (c / NS) & 1, v_abort);
      if (!__all_sync(0xffffffffu, got)) {
        if (lane == 0) *v_abort = 1;
        return;
      }
      St &st = stg[s];
      T zn[C];
      if (has_lay && !ll_poll<T, C>(zsrc + (long long)c * C * W, W, (1u << C) - 1u, ep, zn, v_abort)) {
        fail();
        return;
      }
#pragma unroll
      for (int t = 0; t < C; ++t) {
        const int e = t * W + lane;
        T t0;
        if constexpr (DIR > 0) t0 = st.r[e];
        else t0 = st.d[e] * ll_val(st.y[C * W - 1 - e]);
        if (has_lay) t0 = fma(-st.a[e], zn[t], t0);
        st.a[e] = t0;
      }
      // the buffer is refilled by the async proxy after the compute warp
      // has released it: order these generic writes before that
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&prep[s]);
    }
    return;
  }

  if (role == kRoleEdge) {
    // ---------------- edge warp ----------------
    // The neighbour block's last line: lane t < C polls the word of step t
    // of the chunk (the neighbour's lane 31 reaches column g at its step
    // g + S*31) and leaves it in the stage's `yn`.
    const LLWord<T> *ysrc = has_blk ? out + tile(k, b - DIR) + (W - 1) : nullptr;
    for (int c = 0; c < nch; ++c) {
      const int s = c % NS;
      if (c >= NS) {
        const bool got = mbar_wait(&empty[s], ((c / NS) - 1) & 1, v_abort);
        if (!__all_sync(0xffffffffu, got)) {
          if (lane == 0) *v_abort = 1;
          return;
        }
      }
      if (has_blk) {
        const int yrow = c * C + S * (W - 1) + lane;
        T v[1] = {T(0)};
        const bool need = lane < C && yrow < G;
        if (!ll_poll<T, 1>(ysrc + (long long)(need ? yrow : 0) * W, 0, need ? 1u : 0u, ep, v,
                           v_abort)) {
          fail();
          return;
        }
        if (lane < C) stg[s].yn[lane] = need ? v[0] : T(0);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&prep[s]);
    }
    return;
  }

  if (role == kRoleCopy) {
    // ---------------- copy warp ----------------
    // The block's own tiles have no producer in this launch: they stream
    // into the ring as fast as buffers free up.
    int issued = 0;
    bool ok = true;
    const unsigned tileb = C * W * sizeof(T);
    for (int c = 0; c < nch; ++c) {
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
          mbar_expect_tx(&full[s], 4 * tileb);
          bulk_g2s(st.r, p.rsk + tb, tileb, &full[s]);
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
    }
    if (!ok) fail();
    if (lane == 0) {
      // every copy issued has landed before this warp, and so the CTA, ends
      // (the other warps may have left early on an abort)
      for (int c = max(0, issued - NS); c < issued; ++c) {
        unsigned long long t0 = gtimer();
        while (!mbar_test(&full[c % NS], (c / NS) & 1))
          if (gtimer() - t0 > kWaitNs) break;
      }
    }
    return;
  }

  // ---------------- compute warp ----------------
  // Per step one shuffle and the two FMAs of the row and column neighbours;
  // each result goes straight out as a word of this epoch.
  const int i = (DIR > 0) ? (b * W + lane) : (b * W + (W - 1 - lane));
  const bool line_ok = i >= 0 && i < nrow;
  const bool has_y = line_ok && ((DIR > 0) ? (i > 0) : (i + 1 < nrow));
  const int ncol = geo.ncol;
  LLWord<T> *outt = out + tile(k, b) + lane;
  T h1 = T(0), h2 = T(0);
  for (int c = 0; c < nch; ++c) {
    const int s = c % NS;
    const bool got = mbar_wait(&full[s], (c / NS) & 1, v_abort) &&
                     mbar_wait(&prep[s], (c / NS) & 1, v_abort);
    if (!__all_sync(0xffffffffu, got)) {
      if (lane == 0) *v_abort = 1;
      return;
    }
    const St &st = stg[s];
    const int g0 = c * C;
    const int jc = g0 - S * lane;
#pragma unroll
    for (int t = 0; t < C; ++t) {
      T yv = __shfl_up_sync(0xffffffffu, (S == 1) ? h1 : h2, 1);
      if (lane == 0) yv = st.yn[t];
      const int jj = jc + t;
      const bool v = line_ok && (unsigned)jj < (unsigned)ncol;
      T tv = st.a[t * W + lane];  // pre-computed r - Lz*zn (backward: dinv*y - Uz'*zn)
      if (has_y) tv = fma(-st.b[t * W + lane], yv, tv);
      if (jj > 0) tv = fma(-st.x[t * W + lane], h1, tv);
      if (!v) tv = T(0);
      ll_put(outt + (long long)(g0 + t) * W, tv, ep);
      h2 = h1;
      h1 = tv;
    }
    // the input buffer goes back to the copy and edge warps
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

// Natural order -> skewed tiles (forward input) and back (backward output).
// A 32 x 8 thread block covers 32 columns of 8 lines: the natural-order side
// is whole rows, and the skewed side falls in a few rows of one tile.
// The backward source holds result words (LLWord<TS>).
template <typename TS, typename TD, int W, int S, int DIR>
__global__ void k_dia7_permute(const Dia7Geo *__restrict__ geos, int nm, const void *__restrict__ src,
                               TD *__restrict__ dst, const Ctl *__restrict__ ctl,
                               const Ctl *__restrict__ mctl) {
  if (ctl && ctl->done) return;
  // member of this 32 x 8 tile
  const int t = blockIdx.x;
  int lo = 0, hi = nm - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (geos[mid].ptile0 <= t) lo = mid;
    else hi = mid - 1;
  }
  if (mctl && mctl[lo].done) return;
  const Dia7Geo g = geos[lo];
  const int tx = (g.ncol + 31) / 32, ty = (g.nrow + 7) / 8;
  const int lt = t - g.ptile0;
  const int k = lt / (tx * ty);
  const int rem = lt - k * tx * ty;
  const int j = (rem % tx) * 32 + threadIdx.x;
  const int i = (rem / tx) * 8 + threadIdx.y;
  if (j >= g.ncol || i >= g.nrow) return;
  const int b = i / W;
  const int l = (DIR > 0) ? (i - b * W) : (W - 1 - (i - b * W));
  const int gg = ((DIR > 0) ? j : (g.ncol - 1 - j)) + S * l;
  const long long sk = g.slot0 + (((long long)k * g.nb + b) * g.G + gg) * W + l;
  const long long nat = g.row0 + ((long long)k * g.nrow + i) * g.ncol + j;
  if (DIR > 0) dst[sk] = (TD)static_cast<const TS *>(src)[nat];  // skew (forward input)
  else dst[nat] = (TD)ll_val(static_cast<const LLWord<TS> *>(src)[sk]);  // unskew (backward output)
}

// APC/JAPC -> skewed tiles.  Forward tiles hold Lz, Ly, Lx of the cell that
// lane l visits at step g; backward tiles hold dinv*Uz, dinv*Uy, dinv*Ux and
// dinv.  Slots outside the grid are zero.
template <typename T>
__global__ void k_dia7_extract(const Dia7Geo *__restrict__ geos, int nm, long long nslot, int W,
                               int S, int dir, const int *__restrict__ iapc,
                               const int *__restrict__ japc, const double *__restrict__ apc,
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
    if (i < g.nrow && jj >= 0 && jj < g.ncol) {
      const int j = (dir > 0) ? jj : g.ncol - 1 - jj;
      const long long n = g.row0 + k * nrc + (long long)i * g.ncol + j;
      const double d = apc[n];
      for (int pp = iapc[n]; pp < iapc[n + 1]; ++pp) {
        const long long c = japc[pp];
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
    A[q] = (T)va;
    B[q] = (T)vb;
    X[q] = (T)vx;
    if (D) D[q] = (T)vd;
  }
}

// Wavefront shape per precision: lines per block W, lane skew S, chunk C,
// buffers NS.  The FP64 shape can be set at build time (GB_DIA64_W/S/NS) to
// tune it on a new part; W <= 32 (one warp), S >= 1, C a multiple of 2.
// Measured on GB300 (10M-cell case, one ILU0 application): W16/S2 1.83 ms,
// W16/S1 1.50 ms, W32/S1 (NS 4, three CTAs per SM) 1.20 ms -- the sweep is
// bound by the hand-off chain, so fewer, wider blocks win although each
// step then carries the y-term shuffle on its dependency chain.
#ifndef GB_DIA64_W
#define GB_DIA64_W 32
#endif
#ifndef GB_DIA64_S
#define GB_DIA64_S 1
#endif
#ifndef GB_DIA64_NS
#define GB_DIA64_NS 4
#endif
template <typename T>
struct Shape;
template <>
struct Shape<double> {
  static constexpr int W = GB_DIA64_W, S = GB_DIA64_S, C = 8, NS = GB_DIA64_NS;
};
template <>
struct Shape<float> { static constexpr int W = 32, S = 1, C = 8, NS = 5; };

template <typename T, int DIR>
constexpr size_t stage_bytes() {
  using P = Shape<T>;
  return P::NS * sizeof(Stage<T, P::C, DIR>) + 3 * P::NS * sizeof(unsigned long long);
}
static_assert(Shape<double>::W == 32 && Shape<float>::W == 32, "a sweep block is one warp of lines");
static_assert((Shape<double>::S == 1 || Shape<double>::S == 2) &&
                  (Shape<float>::S == 1 || Shape<float>::S == 2),
              "lane skew 1 or 2");
static_assert(stage_bytes<double, -1>() <= 200 * 1024, "FP64 stage ring too large");
static_assert(stage_bytes<float, -1>() <= 200 * 1024, "FP32 stage ring too large");

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

// Geometry of the skewed layout of one precision.
void dia7_geometry(int nlay, int nrow, int ncol, bool fp32, int *nb, int *G, long long *slots) {
  int W = fp32 ? Shape<float>::W : Shape<double>::W;
  int S = fp32 ? Shape<float>::S : Shape<double>::S;
  int C = fp32 ? Shape<float>::C : Shape<double>::C;
  *nb = (nrow + W - 1) / W;
  *G = ((ncol + S * (W - 1) + C - 1) / C) * C;
  *slots = (long long)nlay * (*nb) * (*G) * W;
}

void dia7_layout(Dia7 &D, const std::vector<int> &shapes, const std::vector<long long> &row0,
                 bool fp32) {
  D.nm = (int)row0.size();
  D.geo.resize(D.nm);
  long long slots = 0;
  int tickets = 0, ptiles = 0;
  for (int m = 0; m < D.nm; ++m) {
    Dia7Geo &g = D.geo[m];
    g.nlay = shapes[3 * m];
    g.nrow = shapes[3 * m + 1];
    g.ncol = shapes[3 * m + 2];
    long long ms = 0;
    dia7_geometry(g.nlay, g.nrow, g.ncol, fp32, &g.nb, &g.G, &ms);
    g.ticket0 = tickets;
    g.ptile0 = ptiles;
    g.slot0 = slots;
    g.row0 = row0[m];
    tickets += g.nlay * g.nb;
    ptiles += g.nlay * ((g.ncol + 31) / 32) * ((g.nrow + 7) / 8);
    slots += ms;  // a multiple of C*W elements: every member starts 16-byte aligned
  }
  D.slots = slots;
  D.ntickets = tickets;
  D.nptiles = ptiles;
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
  using P = Shape<T>;
  const long long nslot = D.slots;
  int grid = (int)std::min<long long>((nslot + 255) / 256, 8LL * kNumSM);
  k_dia7_extract<T><<<grid, 256, 0, st>>>(D.d_geo, D.nm, nslot, P::W, P::S, 1, d_iapc, d_japc,
                                          d_apc, arr[0], arr[1], arr[2], nullptr);
  k_dia7_extract<T><<<grid, 256, 0, st>>>(D.d_geo, D.nm, nslot, P::W, P::S, -1, d_iapc, d_japc,
                                          d_apc, arr[3], arr[4], arr[5], arr[6]);
}

void launch_dia7_extract(const Dia7 &D, int n, const int *d_iapc, const int *d_japc,
                         const double *d_apc, bool mixed, cudaStream_t st) {
  (void)n;
  if (!mixed) {
    double *arr[7] = {D.d_lz, D.d_ly, D.d_lx, D.d_uz, D.d_uy, D.d_ux, D.d_dinv};
    extract_t<double>(D, d_iapc, d_japc, d_apc, arr, st);
    cudaMemsetAsync(D.d_rsk, 0, sizeof(double) * D.slots, st);  // padding slots stay zero
  } else {
    float *arr[7] = {D.f_lz, D.f_ly, D.f_lx, D.f_uz, D.f_uy, D.f_ux, D.f_dinv};
    extract_t<float>(D, d_iapc, d_japc, d_apc, arr, st);
    cudaMemsetAsync(D.f_rsk, 0, sizeof(float) * D.slots, st);
  }
}

// One ILU0 application on the skewed layout: skew r (natural order, type TV)
// into the sweep type T, forward and backward wavefront sweeps, unskew z
// back to TV.
// No memory is reset between applications: each sweep launch writes its
// words with a new epoch.
template <typename T, typename TV = T>
static void apply_t(const Dia7 &D, const T *const *arr, T *rsk, const TV *r, TV *z, const Ctl *ctl,
                    cudaStream_t st) {
  using P = Shape<T>;
  const int nct = D.ntickets;
  constexpr size_t smf = stage_bytes<T, 1>(), smb = stage_bytes<T, -1>();
  const dim3 pb(32, 8);
  SweepArgs<T> a;
  a.geo = D.d_geo;
  a.nm = D.nm;
  a.mctl = D.mctl;
  a.rsk = rsk;
  a.ysk = static_cast<LLWord<T> *>(D.ll_y);
  a.zsk = static_cast<LLWord<T> *>(D.ll_z);
  a.err = D.d_err;
  a.ctl = const_cast<Ctl *>(ctl);
  a.A = arr[0]; a.B = arr[1]; a.X = arr[2]; a.D = nullptr;
  a.ticket = reinterpret_cast<unsigned long long *>(D.d_flags);
  {  // opt in to more than 48 KB of dynamic shared memory, once
    static bool opted = false;
    if (!opted) {
      if (smf > 48 * 1024)
        cudaFuncSetAttribute(k_dia7_sweep<T, P::S, P::C, P::NS, 1>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smf);
      if (smb > 48 * 1024)
        cudaFuncSetAttribute(k_dia7_sweep<T, P::S, P::C, P::NS, -1>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb);
      opted = true;
    }
  }
  k_dia7_permute<TV, T, P::W, P::S, 1><<<D.nptiles, pb, 0, st>>>(D.d_geo, D.nm, r, rsk, ctl, D.mctl);
  k_dia7_sweep<T, P::S, P::C, P::NS, 1><<<nct, 128, smf, st>>>(a);
  a.A = arr[3]; a.B = arr[4]; a.X = arr[5]; a.D = arr[6];
  a.ticket = reinterpret_cast<unsigned long long *>(D.d_flags + 32);
  k_dia7_sweep<T, P::S, P::C, P::NS, -1><<<nct, 128, smb, st>>>(a);
  k_dia7_permute<T, TV, P::W, P::S, -1><<<D.nptiles, pb, 0, st>>>(D.d_geo, D.nm, D.ll_z, z, ctl,
                                                                 D.mctl);
}

void launch_dia7_apply64(const Dia7 &D, const double *r, double *z, const Ctl *ctl,
                         cudaStream_t st) {
  const double *arr[7] = {D.d_lz, D.d_ly, D.d_lx, D.d_uz, D.d_uy, D.d_ux, D.d_dinv};
  apply_t<double>(D, arr, D.d_rsk, r, z, ctl, st);
}


void launch_dia7_apply32(const Dia7 &D, const float *r, float *z, const Ctl *ctl,
                         cudaStream_t st) {
  const float *arr[7] = {D.f_lz, D.f_ly, D.f_lx, D.f_uz, D.f_uy, D.f_ux, D.f_dinv};
  apply_t<float>(D, arr, D.f_rsk, r, z, ctl, st);
}

}  // namespace gb
