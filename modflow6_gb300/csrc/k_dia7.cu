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
// (one CTA) owns 32 consecutive lines i0..i0+31 of one layer k; lane l walks
// its line in column order, two steps behind lane l-1, so the value it needs
// from line i-1 was produced two steps earlier and arrives by a register
// shuffle, and the only dependency that is fresh at each step is the lane's
// own previous column (one FMA on the critical path).  Lines of the previous
// warp (i0-1) and of the layer above (k-1) come through global memory; each
// warp publishes its progress after every chunk of C steps with a release
// store, consumers wait with acquire loads bounded by the global timer (a
// wait that runs out sets an error flag and Ctl::done, it never hangs).
// Warps take a ticket in launch order and depend only on smaller tickets, so
// the wait chain always ends.
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

constexpr int kChunk = 16;
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

// Wait (lane 0) until *flag >= need; returns false if the wait ran out.
__device__ __forceinline__ bool wait_flag(const int *flag, int need) {
  if (ld_acquire(flag) >= need) return true;
  unsigned long long t0 = gtimer();
  while (ld_acquire(flag) < need) {
    if (gtimer() - t0 > kWaitNs) return false;
  }
  return true;
}

template <typename T>
__device__ __forceinline__ T ldc(const T *p) { return __ldcg(p); }

template <typename T>
struct Fac {
  const T *lz, *ly, *lx, *ux, *uy, *uz, *dinv;
};

template <typename T>
__global__ void __launch_bounds__(32) k_dia7_fwd(int nlay, int nrow, int ncol, Fac<T> f,
                                                  const T *__restrict__ r, T *y, int *flags,
                                                  int *err, Ctl *ctl) {
  if (ctl && ctl->done) return;
  const int lane = threadIdx.x;
  int id = 0;
  if (lane == 0) id = atomicAdd(&flags[0], 1);
  id = __shfl_sync(0xffffffffu, id, 0);
  const int k = id % nlay, b = id / nlay;
  const int i = 32 * b + lane;
  const long long nrc = (long long)nrow * ncol;
  const int nsteps = ncol + 62;
  const int nchunks = (nsteps + kChunk - 1) / kChunk;
  const int total = nchunks * kChunk;
  int *prog = flags + 1;
  const int *pb = (b > 0) ? prog + (id - nlay) : nullptr;
  const int *pu = (k > 0) ? prog + (id - 1) : nullptr;
  const bool line_ok = i < nrow;
  const long long base = k * nrc + (long long)i * ncol;
  T out1 = T(0), out2 = T(0);
  for (int c = 0; c < nchunks; ++c) {
    int ok = 1;
    if (lane == 0) {
      if (pb && !wait_flag(pb, min((c + 1) * kChunk + 62, total))) ok = 0;
      if (ok && pu && !wait_flag(pu, (c + 1) * kChunk)) ok = 0;
      if (!ok) {
        atomicExch(err, 1);
        if (ctl) ctl->done = 1;
      }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) return;
#pragma unroll 4
    for (int t = 0; t < kChunk; ++t) {
      const int g = c * kChunk + t;
      const int j = g - 2 * lane;
      const bool valid = line_ok && j >= 0 && j < ncol;
      T yb = __shfl_up_sync(0xffffffffu, out2, 1);
      T tv = T(0);
      if (valid) {
        const long long n = base + j;
        tv = r[n];
        if (k > 0) tv = fma(-__ldg(f.lz + n), ldc(y + n - nrc), tv);
        if (i > 0) {
          if (lane == 0) yb = ldc(y + n - ncol);
          tv = fma(-__ldg(f.ly + n), yb, tv);
        }
        if (j > 0) tv = fma(-__ldg(f.lx + n), out1, tv);
        y[n] = tv;
      }
      out2 = out1;
      out1 = tv;
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      st_release(prog + id, (c + 1) * kChunk);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(32) k_dia7_bwd(int nlay, int nrow, int ncol, Fac<T> f,
                                                  const T *y, T *z, int *flags, int *err,
                                                  Ctl *ctl) {
  if (ctl && ctl->done) return;
  const int lane = threadIdx.x;
  int id = 0;
  if (lane == 0) id = atomicAdd(&flags[0], 1);
  id = __shfl_sync(0xffffffffu, id, 0);
  const int nb = (nrow + 31) / 32;
  // tickets run from the last line block and the bottom layer upwards
  const int k = nlay - 1 - (id % nlay), b = nb - 1 - id / nlay;
  const int l = 31 - lane;  // lane 0 holds the highest line of the block
  const int i = 32 * b + l;
  const long long nrc = (long long)nrow * ncol;
  const int nsteps = ncol + 62;
  const int nchunks = (nsteps + kChunk - 1) / kChunk;
  const int total = nchunks * kChunk;
  int *prog = flags + 1;
  const int *pb = (b < nb - 1) ? prog + (id - nlay) : nullptr;  // block i0+32
  const int *pu = (k < nlay - 1) ? prog + (id - 1) : nullptr;   // layer k+1
  const bool line_ok = i < nrow;
  const bool has_next_line = (i + 1 < nrow);
  const long long base = k * nrc + (long long)i * ncol;
  T out1 = T(0), out2 = T(0);
  for (int c = 0; c < nchunks; ++c) {
    int ok = 1;
    if (lane == 0) {
      if (pb && !wait_flag(pb, min((c + 1) * kChunk + 62, total))) ok = 0;
      if (ok && pu && !wait_flag(pu, (c + 1) * kChunk)) ok = 0;
      if (!ok) {
        atomicExch(err, 1);
        if (ctl) ctl->done = 1;
      }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) return;
#pragma unroll 4
    for (int t = 0; t < kChunk; ++t) {
      const int g = c * kChunk + t;
      const int jj = g - 2 * lane;        // steps taken along the line
      const int j = ncol - 1 - jj;        // column, walked right to left
      const bool valid = line_ok && jj >= 0 && jj < ncol;
      T zb = __shfl_up_sync(0xffffffffu, out2, 1);
      T tv = T(0);
      if (valid) {
        const long long n = base + j;
        tv = __ldg(f.dinv + n) * y[n];
        if (k < nlay - 1) tv = fma(-__ldg(f.uz + n), ldc(z + n + nrc), tv);
        if (has_next_line) {
          if (lane == 0) zb = ldc(z + n + ncol);
          tv = fma(-__ldg(f.uy + n), zb, tv);
        }
        if (j < ncol - 1) tv = fma(-__ldg(f.ux + n), out1, tv);
        z[n] = tv;
      }
      out2 = out1;
      out1 = tv;
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      st_release(prog + id, (c + 1) * kChunk);
    }
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

template <typename T>
static void apply_t(const Dia7 &D, Fac<T> f, const T *r, T *z, T *ywork, const Ctl *ctl,
                    cudaStream_t st) {
  int nb = (D.nrow + 31) / 32;
  int nct = nb * D.nlay;
  cudaMemsetAsync(D.d_flags, 0, sizeof(int) * (nct + 1), st);
  k_dia7_fwd<T><<<nct, 32, 0, st>>>(D.nlay, D.nrow, D.ncol, f, r, ywork, D.d_flags, D.d_err,
                                    const_cast<Ctl *>(ctl));
  cudaMemsetAsync(D.d_flags, 0, sizeof(int) * (nct + 1), st);
  k_dia7_bwd<T><<<nct, 32, 0, st>>>(D.nlay, D.nrow, D.ncol, f, ywork, z, D.d_flags, D.d_err,
                                    const_cast<Ctl *>(ctl));
}

void launch_dia7_apply64(const Dia7 &D, const double *r, double *z, const Ctl *ctl,
                         cudaStream_t st) {
  Fac<double> f{D.d_lz, D.d_ly, D.d_lx, D.d_ux, D.d_uy, D.d_uz, D.d_dinv};
  // the forward result is written into z and swept backwards in place
  apply_t<double>(D, f, r, z, z, ctl, st);
}

void launch_dia7_apply32(const Dia7 &D, const float *r, float *z, const Ctl *ctl,
                         cudaStream_t st) {
  Fac<float> f{D.f_lz, D.f_ly, D.f_lx, D.f_ux, D.f_uy, D.f_uz, D.f_dinv};
  apply_t<float>(D, f, r, z, z, ctl, st);
}

}  // namespace gb
