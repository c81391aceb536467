// k_dia7.cu -- structured ILU0 triangular sweeps for full DIS grids (7-point).
//
// Replaces the level-by-level sweeps of ims_base_ilu0a
// (src/Solution/LinearMethods/ImsLinearBase.f90:1049-1092) when the CSR
// pattern is that of a full DIS grid in natural order (node = j + i*ncol +
// k*nrow*ncol).  Row n then has at most three lower neighbours, (k-1,i,j),
// (k,i-1,j), (k,i,j-1), and three upper ones, so the factors are stored as
// seven length-n arrays (no index arrays).
//
// Wavefront: a "line" is the ncol cells of one grid row (k,i).  One warp
// (one CTA) owns W consecutive lines of one layer; lane l walks its line
// S steps behind lane l-1, so the value it needs from the neighbour line was
// produced S steps earlier by lane l-1 and arrives by a register shuffle.
// With S = 2 (FP64) the only operation on the critical path of a step is the
// FMA with the lane's own previous column; with S = 1 (FP32, short FMA
// latency) the neighbour-line FMA joins it.  Lines of the neighbour block and
// of the neighbour layer come through global memory: each warp publishes its
// progress after every chunk of C steps; a consumer reads the producers'
// progress words early (relaxed loads that complete behind a chunk of
// arithmetic) and spins only when they are short, with a wait bounded by the
// global timer (a wait that runs out sets an error flag and Ctl::done; it
// never hangs).  The factors, the right-hand side and the neighbour results
// of chunk c+1 are loaded at the start of chunk c through per-lane running
// pointers, so memory latency hides behind one chunk of arithmetic.  Warps
// take a ticket in launch order and depend only on smaller tickets, so the
// wait chain always ends.
//
// W < 32 leaves lanes idle on purpose: on GB300 the FP64 pipe of an SM
// sub-partition retires about half a lane-FMA per clock, so a 32-lane FP64
// FMA occupies it for ~67 cycles and the wavefront step time scales with the
// number of active lanes.
//
// Forward sweep: y = r - Lz*y(k-1) - Ly*y(i-1) - Lx*y(j-1), in the reference's
// order (ascending column), bit-identical to the level kernel.
// Backward sweep: z = dinv*y - Uz'*z(k+1) - Uy'*z(i+1) - Ux'*z(j+1) with the
// upper factors pre-scaled by the inverse pivot (U' = dinv*U), equal in exact
// arithmetic to the reference's (y - sum U z)*dinv with one FMA, not two
// dependent operations, on the critical path.
#include "gbims_internal.cuh"

namespace gb {

namespace {

constexpr unsigned long long kWaitNs = 2000000000ULL;  // 2 s per wait

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(int *p, int v) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
struct Fac {
  const T *lz, *ly, *lx, *ux, *uy, *uz, *dinv;
};

template <typename T, int C>
struct Chunk {
  T r[C], a[C], b[C], x[C], zn[C], yn[C];
};

// DIR = +1: forward sweep (lines ascending, columns left to right).
// DIR = -1: backward sweep (lines descending, columns right to left).
template <typename T, int W, int S, int C, int DIR>
__global__ void __launch_bounds__(32) k_dia7_sweep(int nlay, int nrow, int ncol, Fac<T> f,
                                                    const T *__restrict__ rin, T *out,
                                                    int *flags, int *err, Ctl *ctl) {
  if (ctl && ctl->done) return;
  const int lane = threadIdx.x;
  int id = 0;
  if (lane == 0) id = atomicAdd(&flags[0], 1);
  id = __shfl_sync(0xffffffffu, id, 0);
  const int nb = (nrow + W - 1) / W;
  const int k = (DIR > 0) ? id % nlay : nlay - 1 - (id % nlay);
  const int b = (DIR > 0) ? id / nlay : nb - 1 - id / nlay;
  const int i = (DIR > 0) ? (b * W + lane) : (b * W + (W - 1 - lane));
  const bool line_ok = lane < W && i >= 0 && i < nrow;
  const long long nrc = (long long)nrow * ncol;
  const int nch = (ncol + S * (W - 1) + C - 1) / C;
  const int total = nch * C;
  int *prog = flags + 1;
  const bool has_blk = (DIR > 0) ? (b > 0) : (b < nb - 1);
  const bool has_lay = (DIR > 0) ? (k > 0) : (k < nlay - 1);
  const int *pb = has_blk ? prog + (id - nlay) : nullptr;
  const int *pu = has_lay ? prog + (id - 1) : nullptr;
  // neighbour line exists for this lane (lane 0's lives in the other block)
  const bool has_y = line_ok && ((DIR > 0) ? (i > 0) : (i + 1 < nrow));
  const bool y_from_mem = has_y && lane == 0;
  const bool z_on = line_ok && has_lay;
  // element of step g: e(g) = e0 + DIR*g; walk index jj(g) = g - S*lane
  const long long base = k * nrc + (long long)(line_ok ? i : 0) * ncol;
  const long long e0 = (DIR > 0) ? base - (long long)S * lane : base + ncol - 1 + (long long)S * lane;
  const long long zoff = -(long long)DIR * nrc;
  const long long yoff = -(long long)DIR * ncol;
  const T *A = (DIR > 0) ? f.lz : f.uz;
  const T *B = (DIR > 0) ? f.ly : f.uy;
  const T *X = (DIR > 0) ? f.lx : f.ux;
  int seen_b = 0, seen_u = 0;

  // make sure the producers have published what chunk c needs
  auto ensure = [&](int c) -> bool {
    int ok = 1;
    if (lane == 0) {
      const int nb_need = min((c + 1) * C + S * (W - 1), total);
      const int nu_need = min((c + 1) * C, total);
      if (pb && seen_b < nb_need) {
        unsigned long long t0 = gtimer();
        while ((seen_b = ld_relaxed(pb)) < nb_need)
          if (gtimer() - t0 > kWaitNs) { ok = 0; break; }
      }
      if (ok && pu && seen_u < nu_need) {
        unsigned long long t0 = gtimer();
        while ((seen_u = ld_relaxed(pu)) < nu_need)
          if (gtimer() - t0 > kWaitNs) { ok = 0; break; }
      }
      if (!ok) {
        atomicExch(err, 1);
        if (ctl) ctl->done = 1;
      }
      // early reads for the next check; they complete behind a chunk of work
      if (ok && pb) seen_b = ld_relaxed(pb);
      if (ok && pu) seen_u = ld_relaxed(pu);
    }
    __syncwarp();
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
  };

  auto load = [&](int c, Chunk<T, C> &q) {
    const long long ec = e0 + (long long)DIR * c * C;
    const int jc = c * C - S * lane;
#pragma unroll
    for (int t = 0; t < C; ++t) {
      const long long e = ec + DIR * t;
      const bool v = line_ok && (unsigned)(jc + t) < (unsigned)ncol;
      T r = T(0), a = T(0), bb = T(0), x = T(0), zn = T(0), yn = T(0);
      if (v) {
        if (DIR > 0) r = __ldg(rin + e);
        else r = __ldg(f.dinv + e) * out[e];  // dinv * y: own cell, still the forward value
        bb = __ldg(B + e);
        x = __ldg(X + e);
        if (z_on) {
          a = __ldg(A + e);
          zn = __ldcg(out + e + zoff);
        }
        if (y_from_mem) yn = __ldcg(out + e + yoff);
      }
      q.r[t] = r; q.a[t] = a; q.b[t] = bb; q.x[t] = x; q.zn[t] = zn; q.yn[t] = yn;
    }
  };

  Chunk<T, C> cur, nxt;
  if (!ensure(0)) return;
  load(0, cur);
  T h1 = T(0), h2 = T(0);  // this lane's results of the last two steps
  for (int c = 0; c < nch; ++c) {
    const bool more = (c + 1 < nch);
    if (more) {
      if (!ensure(c + 1)) return;
      load(c + 1, nxt);
    }
    const long long ec = e0 + (long long)DIR * c * C;
    const int jc = c * C - S * lane;
#pragma unroll
    for (int t = 0; t < C; ++t) {
      // neighbour line, same column: lane-1's result S steps ago
      T yv = __shfl_up_sync(0xffffffffu, (S == 1) ? h1 : h2, 1);
      if (lane == 0) yv = cur.yn[t];
      const int jj = jc + t;
      T tv = cur.r[t];
      tv = fma(-cur.a[t], cur.zn[t], tv);
      if (has_y) tv = fma(-cur.b[t], yv, tv);
      if (jj > 0) tv = fma(-cur.x[t], h1, tv);
      const bool v = line_ok && (unsigned)jj < (unsigned)ncol;
      if (v) out[ec + DIR * t] = tv;
      else tv = T(0);
      h2 = h1;
      h1 = tv;
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      st_relaxed(prog + id, (c + 1) * C);
    }
    if (more) cur = nxt;
  }
}

// APC/JAPC -> seven arrays; U pre-scaled by the inverse pivot.
template <typename T>
__global__ void k_dia7_extract(int nlay, int nrow, int ncol, const int *__restrict__ iapc,
                               const int *__restrict__ japc, const double *__restrict__ apc,
                               T *lz, T *ly, T *lx, T *ux, T *uy, T *uz, T *dinv) {
  long long nn = (long long)nlay * nrow * ncol;
  long long nrc = (long long)nrow * ncol;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
       n += (long long)gridDim.x * blockDim.x) {
    int k = (int)(n / nrc);
    int rem = (int)(n - k * nrc);
    int i = rem / ncol, j = rem - i * ncol;
    double vz = 0, vy = 0, vx = 0, wx = 0, wy = 0, wz = 0;
    for (int p = iapc[n]; p < iapc[n + 1]; ++p) {
      long long c = japc[p];
      double a = apc[p];
      if (k > 0 && c == n - nrc) vz = a;
      else if (i > 0 && c == n - ncol) vy = a;
      else if (j > 0 && c == n - 1) vx = a;
      else if (j < ncol - 1 && c == n + 1) wx = a;
      else if (i < nrow - 1 && c == n + ncol) wy = a;
      else if (k < nlay - 1 && c == n + nrc) wz = a;
    }
    double d = apc[n];
    lz[n] = (T)vz; ly[n] = (T)vy; lx[n] = (T)vx;
    ux[n] = (T)(d * wx); uy[n] = (T)(d * wy); uz[n] = (T)(d * wz);
    dinv[n] = (T)d;
  }
}

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

void launch_dia7_extract(const Dia7 &D, int n, const int *d_iapc, const int *d_japc,
                         const double *d_apc, bool mixed, cudaStream_t st) {
  int grid = std::min((n + 255) / 256, 8 * kNumSM);
  if (!mixed)
    k_dia7_extract<double><<<grid, 256, 0, st>>>(D.nlay, D.nrow, D.ncol, d_iapc, d_japc, d_apc,
                                                 D.d_lz, D.d_ly, D.d_lx, D.d_ux, D.d_uy, D.d_uz,
                                                 D.d_dinv);
  else
    k_dia7_extract<float><<<grid, 256, 0, st>>>(D.nlay, D.nrow, D.ncol, d_iapc, d_japc, d_apc,
                                                D.f_lz, D.f_ly, D.f_lx, D.f_ux, D.f_uy, D.f_uz,
                                                D.f_dinv);
}

// Wavefront shape per precision: lines per warp W, lane skew S, chunk C.
template <typename T>
struct Shape;
template <>
struct Shape<double> { static constexpr int W = 16, S = 2, C = 8; };
template <>
struct Shape<float> { static constexpr int W = 32, S = 1, C = 8; };

template <typename T>
static void apply_t(const Dia7 &D, Fac<T> f, const T *r, T *z, const Ctl *ctl, cudaStream_t st) {
  using P = Shape<T>;
  int nb = (D.nrow + P::W - 1) / P::W;
  int nct = nb * D.nlay;
  cudaMemsetAsync(D.d_flags, 0, sizeof(int) * (nct + 1), st);
  k_dia7_sweep<T, P::W, P::S, P::C, 1><<<nct, 32, 0, st>>>(D.nlay, D.nrow, D.ncol, f, r, z,
                                                           D.d_flags, D.d_err,
                                                           const_cast<Ctl *>(ctl));
  cudaMemsetAsync(D.d_flags, 0, sizeof(int) * (nct + 1), st);
  k_dia7_sweep<T, P::W, P::S, P::C, -1><<<nct, 32, 0, st>>>(D.nlay, D.nrow, D.ncol, f, nullptr, z,
                                                            D.d_flags, D.d_err,
                                                            const_cast<Ctl *>(ctl));
}

void launch_dia7_apply64(const Dia7 &D, const double *r, double *z, const Ctl *ctl,
                         cudaStream_t st) {
  Fac<double> f{D.d_lz, D.d_ly, D.d_lx, D.d_ux, D.d_uy, D.d_uz, D.d_dinv};
  // the forward result is written into z and swept backwards in place
  apply_t<double>(D, f, r, z, ctl, st);
}

void launch_dia7_apply32(const Dia7 &D, const float *r, float *z, const Ctl *ctl,
                         cudaStream_t st) {
  Fac<float> f{D.f_lz, D.f_ly, D.f_lx, D.f_ux, D.f_uy, D.f_uz, D.f_dinv};
  apply_t<float>(D, f, r, z, ctl, st);
}

}  // namespace gb
