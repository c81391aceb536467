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
// (one CTA) owns W consecutive lines i0..i0+W-1 of one layer k; lane l walks
// its line in column order one step behind lane l-1, so the value it needs
// from line i-1 is the one lane l-1 produced in the previous step and
// arrives by a register shuffle.  Lines of the previous warp (i0-1) and of
// the layer above (k-1) come through global memory: every warp publishes its
// progress after each chunk of C steps with a release store; consumers wait
// with acquire loads bounded by the global timer (a wait that runs out sets
// an error flag and Ctl::done; it never hangs).  All loads of chunk c+1 --
// the local factors and right-hand side and the neighbour warps' results --
// are issued at the start of chunk c into registers, so memory latency is
// hidden behind one chunk of arithmetic; the price is a lag of one more
// chunk between a warp and the warps it depends on.  Warps take a ticket in
// launch order and depend only on smaller tickets, so the wait chain always
// ends.
//
// W < 32 leaves lanes idle on purpose: on GB300 the FP64 pipe of an SM
// sub-partition retires about half a lane-FMA per clock, so a 32-lane FP64
// FMA occupies it for ~67 cycles and the wavefront step time scales with
// the number of active lanes.
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

constexpr int kChunk = 8;
constexpr unsigned long long kWaitNs = 2000000000ULL;  // 2 s per wait

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait until *flag >= need; false if the wait ran out.
__device__ __forceinline__ bool wait_flag(const int *flag, int need) {
  if (ld_acquire(flag) >= need) return true;
  unsigned long long t0 = gtimer();
  while (ld_acquire(flag) < need) {
    if (gtimer() - t0 > kWaitNs) return false;
  }
  return true;
}

template <typename T>
struct Fac {
  const T *lz, *ly, *lx, *ux, *uy, *uz, *dinv;
};

// Loads of one chunk for one lane.
template <typename T>
struct Chunk {
  T r[kChunk], a[kChunk], b[kChunk], c[kChunk], zn[kChunk], yn[kChunk];
};

// DIR = +1: forward sweep (lines ascending, columns left to right).
// DIR = -1: backward sweep (lines descending, columns right to left).
template <typename T, int W, int DIR>
__global__ void __launch_bounds__(32) k_dia7_sweep(int nlay, int nrow, int ncol, Fac<T> f,
                                                    const T *__restrict__ rin, T *out,
                                                    int *flags, int *err, Ctl *ctl) {
  if (ctl && ctl->done) return;
  const int lane = threadIdx.x;
  int id = 0;
  if (lane == 0) id = atomicAdd(&flags[0], 1);
  id = __shfl_sync(0xffffffffu, id, 0);
  const int nb = (nrow + W - 1) / W;
  int k, b;
  if (DIR > 0) {
    k = id % nlay;
    b = id / nlay;
  } else {
    k = nlay - 1 - (id % nlay);
    b = nb - 1 - id / nlay;
  }
  // lane l walks line i: ascending lines for the forward sweep, descending
  // for the backward sweep, so lane l-1 always holds the line it depends on
  const int l = lane;
  const int i = (DIR > 0) ? (b * W + l) : (b * W + (W - 1 - l));
  const bool active = (l < W);
  const bool line_ok = active && i >= 0 && i < nrow;
  const long long nrc = (long long)nrow * ncol;
  const int nsteps = ncol + (W - 1);
  const int nchunks = (nsteps + kChunk - 1) / kChunk;
  const int total = nchunks * kChunk;
  int *prog = flags + 1;
  const bool has_blk = (DIR > 0) ? (b > 0) : (b < nb - 1);  // neighbour line block
  const bool has_lay = (DIR > 0) ? (k > 0) : (k < nlay - 1);  // neighbour layer
  const int *pb = has_blk ? prog + (id - nlay) : nullptr;
  const int *pu = has_lay ? prog + (id - 1) : nullptr;
  const long long base = k * nrc + (long long)i * ncol;
  const long long dz = DIR * nrc;      // neighbour in the next/previous layer
  const long long dyl = DIR * (long long)ncol;  // neighbour line
  // the neighbour line of lane 0 lives in the other block; it exists unless
  // this is the first line of the sweep
  const bool lane0_has_y = (DIR > 0) ? (i > 0) : (i + 1 < nrow);
  const bool y_exists = line_ok && ((DIR > 0) ? (i > 0) : (i + 1 < nrow));
  // per-lane element of step g: column index along the walk
  auto col_of = [&](int g) { int jj = g - l; return (DIR > 0) ? jj : (ncol - 1 - jj); };
  auto walk_of = [&](int g) { return g - l; };

  auto load_chunk = [&](int c, Chunk<T> &ch) {
#pragma unroll
    for (int t = 0; t < kChunk; ++t) {
      const int g = c * kChunk + t;
      const int jj = walk_of(g);
      const bool valid = line_ok && jj >= 0 && jj < ncol;
      T r = T(0), a = T(0), bb = T(0), cc = T(0), zn = T(0), yn = T(0);
      if (valid) {
        const int j = col_of(g);
        const long long n = base + j;
        if (DIR > 0) {
          r = __ldg(rin + n);
          a = __ldg(f.lz + n);
          bb = __ldg(f.ly + n);
          cc = __ldg(f.lx + n);
        } else {
          r = __ldg(f.dinv + n) * out[n];  // dinv * y (own cell, written by the forward sweep)
          a = __ldg(f.uz + n);
          bb = __ldg(f.uy + n);
          cc = __ldg(f.ux + n);
        }
        if (has_lay) zn = __ldcg(out + n - dz);
        if (lane == 0 && lane0_has_y) yn = __ldcg(out + n - dyl);
      }
      ch.r[t] = r; ch.a[t] = a; ch.b[t] = bb; ch.c[t] = cc; ch.zn[t] = zn; ch.yn[t] = yn;
    }
  };
  // data for chunk c needs: neighbour block progress >= (c+1)*C + W - 1 (its
  // last lane) ... capped by its total; neighbour layer progress >= (c+1)*C
  auto wait_for = [&](int c) -> bool {
    int ok = 1;
    if (lane == 0) {
      if (pb && !wait_flag(pb, min((c + 1) * kChunk + (W - 1), total))) ok = 0;
      if (ok && pu && !wait_flag(pu, min((c + 1) * kChunk, total))) ok = 0;
      if (!ok) {
        atomicExch(err, 1);
        if (ctl) ctl->done = 1;
      }
    }
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
  };

  Chunk<T> cur, nxt;
  if (!wait_for(0)) return;
  load_chunk(0, cur);
  T out1 = T(0);  // this lane's previous result (x neighbour)
  for (int c = 0; c < nchunks; ++c) {
    const bool more = (c + 1 < nchunks);
    if (more) {
      if (!wait_for(c + 1)) return;
      load_chunk(c + 1, nxt);
    }
#pragma unroll
    for (int t = 0; t < kChunk; ++t) {
      const int g = c * kChunk + t;
      const int jj = walk_of(g);
      const bool valid = line_ok && jj >= 0 && jj < ncol;
      T yprev = __shfl_up_sync(0xffffffffu, out1, 1);  // lane l-1, previous step = same column
      if (lane == 0) yprev = cur.yn[t];
      T tv = T(0);
      if (valid) {
        tv = cur.r[t];
        if (has_lay) tv = fma(-cur.a[t], cur.zn[t], tv);
        if (y_exists) tv = fma(-cur.b[t], yprev, tv);
        if (jj > 0) tv = fma(-cur.c[t], out1, tv);
        out[base + col_of(g)] = tv;
      }
      out1 = tv;
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      st_release(prog + id, (c + 1) * kChunk);
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

// Lines per warp: FP64 steps are bounded by the FP64 pipe (fewer lanes per
// warp, shorter steps), FP32 steps by latency (full warps).
template <typename T>
struct LinesPerWarp;
template <>
struct LinesPerWarp<double> { static constexpr int W = 16; };
template <>
struct LinesPerWarp<float> { static constexpr int W = 32; };

template <typename T>
static void apply_t(const Dia7 &D, Fac<T> f, const T *r, T *z, const Ctl *ctl, cudaStream_t st) {
  constexpr int W = LinesPerWarp<T>::W;
  int nb = (D.nrow + W - 1) / W;
  int nct = nb * D.nlay;
  cudaMemsetAsync(D.d_flags, 0, sizeof(int) * (nct + 1), st);
  k_dia7_sweep<T, W, 1><<<nct, 32, 0, st>>>(D.nlay, D.nrow, D.ncol, f, r, z, D.d_flags, D.d_err,
                                            const_cast<Ctl *>(ctl));
  cudaMemsetAsync(D.d_flags, 0, sizeof(int) * (nct + 1), st);
  k_dia7_sweep<T, W, -1><<<nct, 32, 0, st>>>(D.nlay, D.nrow, D.ncol, f, nullptr, z, D.d_flags,
                                             D.d_err, const_cast<Ctl *>(ctl));
}

int dia7_nflags(int nlay, int nrow) { return nlay * ((nrow + 15) / 16) + 2; }

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
