// k_ilu.cu -- ILU0 / MILU0 factorisation and level-scheduled triangular sweeps.
//
// Factorisation: ims_base_pcilu0 (src/Solution/LinearMethods/ImsLinearBase.f90:928-1042)
// restated per row, one thread per row, rows of one dependency level in one
// launch.  The row's work vector W lives in registers, indexed by the row's
// sorted pattern (IAPC/JAPC from ims_base_pccrs); every update to a W slot and
// to the dropped-fill sum rs happens in the reference's order, and every
// operation is rounded separately (no FMA), so APC is bit-for-bit the
// reference's.
//
// Apply: ims_base_ilu0a (:1049-1092).  Forward sweep D = R - L*D (unit lower),
// backward sweep D = (D - U*D) * APC(n).  Rows of a level are independent; one
// launch per level.  Entries are summed in JAPC order with FMA.
#include "gbims_internal.cuh"
#include "k_llword.cuh"
#include <algorithm>
#include <climits>

namespace gb {

void levels_build_host(int n, const std::vector<int> &iapc, const std::vector<int> &japc,
                       bool forward, Levels &L) {
  std::vector<int> lev(n, 0);
  int nlev = 0;
  if (forward) {
    for (int r = 0; r < n; ++r) {
      int l = 0;
      for (int j = iapc[r]; j < japc[r]; ++j) l = std::max(l, lev[japc[j]] + 1);
      lev[r] = l;
      nlev = std::max(nlev, l + 1);
    }
  } else {
    for (int r = n - 1; r >= 0; --r) {
      int l = 0;
      for (int j = japc[r]; j < iapc[r + 1]; ++j) l = std::max(l, lev[japc[j]] + 1);
      lev[r] = l;
      nlev = std::max(nlev, l + 1);
    }
  }
  L.nlev = nlev;
  L.ptr.assign(nlev + 1, 0);
  for (int r = 0; r < n; ++r) L.ptr[lev[r] + 1]++;
  for (int l = 0; l < nlev; ++l) L.ptr[l + 1] += L.ptr[l];
  std::vector<int> rows(n), fill(L.ptr.begin(), L.ptr.end() - 1);
  for (int r = 0; r < n; ++r) rows[fill[lev[r]]++] = r;
  L.maxwidth = 0;
  for (int l = 0; l < nlev; ++l) L.maxwidth = std::max(L.maxwidth, L.ptr[l + 1] - L.ptr[l]);
  if (L.d_rows) cudaFree(L.d_rows);
  L.d_rows = nullptr;
  if (n > 0) {
    cudaMalloc(&L.d_rows, sizeof(int) * n);
    cudaMemcpy(L.d_rows, rows.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  }
}

// Position of column c in the sorted off-diagonal pattern japc[i0:i1), or -1.
__device__ __forceinline__ int find_sorted(const int *__restrict__ japc, int i0, int i1, int c) {
  int lo = i0, hi = i1 - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    int v = japc[mid];
    if (v == c) return mid - i0;
    if (v < c) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

__global__ void k_ilu0_factor_level(const int *__restrict__ rows, int nrows,
                                    const int *__restrict__ ia, const int *__restrict__ ja,
                                    const double *__restrict__ amat,
                                    const int *__restrict__ iapc,
                                    const int *__restrict__ japc, double *apc,
                                    double relax, double delta, int ipcflag, Ctl *ctl) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  if (ctl->pivot_fail != INT_MAX) return;  // a lower row failed: the attempt is void
  int n = rows[t];
  int ic0 = iapc[n], ic1 = iapc[n + 1], iu = japc[n];
  int len = ic1 - ic0;
  // w[0..len) : off-diagonal slots in JAPC order; wd : the diagonal slot
  double w[kMaxRowLen];
#pragma unroll 8
  for (int k = 0; k < kMaxRowLen; ++k)
    if (k < len) w[k] = 0.0;
  double wd = 0.0;
  // W(jcol) = W(jcol) + AMAT(j) over the CSR row (ImsLinearBase.f90:985-989)
  for (int j = ia[n]; j < ia[n + 1]; ++j) {
    int c = ja[j];
    if (c == n) {
      wd = __dadd_rn(wd, amat[j]);
    } else {
      int k = find_sorted(japc, ic0, ic1, c);
      if (k >= 0) w[k] = __dadd_rn(w[k], amat[j]);
    }
  }
  double rs = 0.0;
  // LOWER loop (:993-1007)
  for (int j = ic0; j < iu; ++j) {
    int jcol = japc[j];
    int kj = j - ic0;
    int iic1 = iapc[jcol + 1];
    int iiu = japc[jcol];
    double tl = __dmul_rn(w[kj], apc[jcol]);
    w[kj] = tl;
    for (int jj = iiu; jj < iic1; ++jj) {
      int jjcol = japc[jj];
      double prod = __dmul_rn(tl, apc[jj]);
      if (jjcol == n) {
        wd = __dsub_rn(wd, prod);
      } else {
        int k = find_sorted(japc, ic0, ic1, jjcol);
        if (k >= 0) w[k] = __dsub_rn(w[k], prod);
        else rs = __dadd_rn(rs, prod);
      }
    }
  }
  // DIAGONAL (:1010-1037)
  double d = wd;
  double tl = __dsub_rn(__dmul_rn(__dadd_rn(1.0, delta), d), __dmul_rn(relax, rs));
  double sd1 = copysign(fabs(d), tl);
  if (sd1 != d) {
    if (ipcflag > 1) tl = copysign(1.0e-6, d);
    else {
      atomicMin(&ctl->pivot_fail, n);
      return;
    }
  }
  if (fabs(tl) == 0.0) {
    if (ipcflag > 1) tl = copysign(1.0e-6, d);
    else {
      atomicMin(&ctl->pivot_fail, n);
      return;
    }
  }
  apc[n] = __drcp_rn(tl);
  for (int k = 0; k < len; ++k) apc[ic0 + k] = w[k];
}

void launch_ilu_factor(int n, const int *d_ia, const int *d_ja, const double *d_amat,
                       const int *d_iapc, const int *d_japc, double *d_apc, const Levels &L,
                       double relax, double delta, int ipcflag, Ctl *ctl, cudaStream_t st) {
  for (int l = 0; l < L.nlev; ++l) {
    int nr = L.ptr[l + 1] - L.ptr[l];
    k_ilu0_factor_level<<<(nr + 127) / 128, 128, 0, st>>>(L.d_rows + L.ptr[l], nr, d_ia, d_ja,
                                                          d_amat, d_iapc, d_japc, d_apc, relax,
                                                          delta, ipcflag, ctl);
  }
  (void)n;
}

template <typename T>
__device__ __forceinline__ T fms(T a, T b, T c);  // c - a*b with one rounding
template <>
__device__ __forceinline__ double fms<double>(double a, double b, double c) { return fma(-a, b, c); }
template <>
__device__ __forceinline__ float fms<float>(float a, float b, float c) { return fmaf(-a, b, c); }

template <typename T>
__global__ void k_ilu_fwd_level(const int *__restrict__ rows, int nrows,
                                const int *__restrict__ iapc, const int *__restrict__ japc,
                                const T *__restrict__ apc, const T *__restrict__ r, T *d,
                                const Ctl *__restrict__ ctl) {
  if (ctl && ctl->done) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  int n = rows[t];
  T tv = r[n];
  for (int j = iapc[n]; j < japc[n]; ++j) tv = fms<T>(apc[j], d[japc[j]], tv);
  d[n] = tv;
}

template <typename T>
__global__ void k_ilu_bwd_level(const int *__restrict__ rows, int nrows,
                                const int *__restrict__ iapc, const int *__restrict__ japc,
                                const T *__restrict__ apc, T *d,
                                const Ctl *__restrict__ ctl) {
  if (ctl && ctl->done) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  int n = rows[t];
  T tv = d[n];
  for (int j = japc[n]; j < iapc[n + 1]; ++j) tv = fms<T>(apc[j], d[japc[j]], tv);
  d[n] = tv * apc[n];
}

// Sync-free sweeps: one launch per sweep instead of one per level.  The
// warps walk the level-ordered row list with a grid stride, 32 consecutive
// rows per warp; a row reads the rows it depends on as result words tagged
// with the launch's epoch.  The polling is warp-synchronous: in each round
// every unfinished lane loads all its dependencies' words (up to kDeps in
// flight at once), and a lane whose words are all of this epoch finishes its
// row; the warp repeats the round until all its lanes are done.  A lane may
// depend on a lane of its own warp (a warp can straddle two levels): that
// row is written in one round and seen in the next.  Rows depend only on
// rows of lower levels, which come earlier in the list, and the grid is
// sized so that all of its CTAs are resident: the lowest unfinished row of
// the list can always proceed, so every wait ends (and is bounded besides).
// Each row sums its entries in JAPC order with FMA, as the per-level kernels
// do (bit-identical results).
template <typename T, int DIR>
__global__ void __launch_bounds__(256) k_ilu_sweep_sf(int n, const int *__restrict__ rows,
                                                      const int *__restrict__ iapc,
                                                      const int *__restrict__ japc,
                                                      const T *__restrict__ apc,
                                                      const T *__restrict__ r,
                                                      const LLWord<T> *__restrict__ yin,
                                                      LLWord<T> *out, T *d,
                                                      unsigned long long *ticket, int *err,
                                                      Ctl *ctl, int active) {
  __shared__ unsigned s_ep;
  if (threadIdx.x == 0) {
    // every CTA takes a ticket, so launch e owns tickets [e*grid, (e+1)*grid)
    const unsigned long long tk = atomicAdd(ticket, 1ULL);
    s_ep = (unsigned)(tk / gridDim.x) + 1u;
  }
  __syncthreads();
  if (ctl && ctl->done) return;
  // the launch always has the same (resident) grid, so that its tickets and
  // epochs line up with every other launch; CTAs past `active` only take
  // their ticket
  if ((int)blockIdx.x >= active) return;
  const unsigned ep = s_ep;
  const int lane = threadIdx.x & 31;
  volatile int *vdone = ctl ? &ctl->done : nullptr;
  constexpr int kDeps = 8;
  const int stride = active * blockDim.x;
  for (int q0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); q0 < n; q0 += stride) {
    const int q = q0 + lane;
    bool done = q >= n;
    int row = 0, j0 = 0, j1 = 0;
    T tv0 = T(0);
    if (!done) {
      row = rows[q];
      if (DIR > 0) {
        tv0 = r[row];
        j0 = iapc[row];
        j1 = japc[row];
      } else {
        tv0 = ll_val(yin[row]);
        j0 = japc[row];
        j1 = iapc[row + 1];
      }
    }
    const unsigned long long t0 = wclock();
    while (true) {
      if (!done) {
        T tv = tv0;
        bool ok = true;
        for (int jb = j0; ok && jb < j1; jb += kDeps) {
          LLRaw w[kDeps];
          const int nd = min(kDeps, j1 - jb);
#pragma unroll
          for (int q2 = 0; q2 < kDeps; ++q2)
            if (q2 < nd) ll_issue(out + japc[jb + q2], w[q2]);
#pragma unroll
          for (int q2 = 0; q2 < kDeps; ++q2) {
            if (q2 >= nd || !ok) break;
            if (!ll_ready<T>(w[q2], ep)) {
              ok = false;
            } else {
              T v;
              ll_take(w[q2], v);
              tv = fms<T>(apc[jb + q2], v, tv);
            }
          }
        }
        if (ok) {
          if (DIR < 0) {
            tv = tv * apc[row];
            d[row] = tv;
          }
          ll_put(out + row, tv, ep);
          done = true;
        }
      }
      if (!__any_sync(0xffffffffu, !done)) break;
      if (__any_sync(0xffffffffu, (vdone && *vdone) || wclock() - t0 > kWaitCycles)) {
        if (lane == 0) {
          atomicExch(err, 1);
          if (ctl) ctl->done = 1;
        }
        return;
      }
    }
  }
}

// Grid of the sync-free sweeps: every CTA that can be resident (always the
// same, see the kernel); `mult` threads per row of the widest level work,
// the rest return after their ticket.  Threads that run several levels
// ahead of the front have their rows' indices and operands loaded by the
// time the front reaches them: on GB300, 8 threads per row of the widest
// level sweep a 250k-cell hexagon grid in 2.57 ms against 3.66 ms with one
// (the default; gbims_autotune picks among 1 to 16).
template <typename T, int DIR>
static int sf_grid() {
  static int per_sm = -1;
  if (per_sm < 0) {
    per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ilu_sweep_sf<T, DIR>, 256, 0);
    per_sm = std::max(1, per_sm);
  }
  return per_sm * kNumSM;
}
static int sf_active(int grid, int n, int maxwidth, int mult) {
  const long long want = ((long long)std::max(1, std::min(n, maxwidth)) * std::max(1, mult) + 255) / 256;
  return (int)std::max<long long>(1, std::min<long long>(want, grid));
}

template <typename T>
static void apply_sf(int n, const int *d_iapc, const int *d_japc, const T *d_apc, const Levels &F,
                     const Levels &B, const LevelWords &Wd, const T *r, T *d, Ctl *ctl,
                     cudaStream_t st) {
  LLWord<T> *yf = static_cast<LLWord<T> *>(Wd.fwd);
  LLWord<T> *zb = static_cast<LLWord<T> *>(Wd.bwd);
  const int gf = sf_grid<T, 1>(), gb = sf_grid<T, -1>();
  k_ilu_sweep_sf<T, 1><<<gf, 256, 0, st>>>(n, F.d_rows, d_iapc, d_japc, d_apc, r, nullptr, yf,
                                           nullptr, Wd.ticket, Wd.err, ctl,
                                           sf_active(gf, n, F.maxwidth, Wd.sf_mult));
  k_ilu_sweep_sf<T, -1><<<gb, 256, 0, st>>>(n, B.d_rows, d_iapc, d_japc, d_apc, nullptr, yf, zb,
                                            d, Wd.ticket + 16, Wd.err, ctl,
                                            sf_active(gb, n, B.maxwidth, Wd.sf_mult));
}

template <typename T>
static void apply_levels(const int *d_iapc, const int *d_japc, const T *d_apc,
                         const Levels &F, const Levels &B, const T *r, T *d, const Ctl *ctl,
                         cudaStream_t st) {
  for (int l = 0; l < F.nlev; ++l) {
    int nr = F.ptr[l + 1] - F.ptr[l];
    k_ilu_fwd_level<T><<<(nr + 127) / 128, 128, 0, st>>>(F.d_rows + F.ptr[l], nr, d_iapc,
                                                          d_japc, d_apc, r, d, ctl);
  }
  for (int l = 0; l < B.nlev; ++l) {
    int nr = B.ptr[l + 1] - B.ptr[l];
    k_ilu_bwd_level<T><<<(nr + 127) / 128, 128, 0, st>>>(B.d_rows + B.ptr[l], nr, d_iapc,
                                                          d_japc, d_apc, d, ctl);
  }
}

void launch_ilu_apply_levels(int n, const int *d_iapc, const int *d_japc, const double *d_apc,
                             const Levels &F, const Levels &B, const LevelWords &Wd,
                             const double *r, double *d, const Ctl *ctl, cudaStream_t st) {
  if (Wd.mode == 1)
    apply_sf<double>(n, d_iapc, d_japc, d_apc, F, B, Wd, r, d, const_cast<Ctl *>(ctl), st);
  else
    apply_levels<double>(d_iapc, d_japc, d_apc, F, B, r, d, ctl, st);
}

void launch_ilu_apply_levels32(int n, const int *d_iapc, const int *d_japc,
                               const float *d_apc32, const Levels &F, const Levels &B,
                               const LevelWords &Wd, const float *r, float *d, const Ctl *ctl,
                               cudaStream_t st) {
  if (Wd.mode == 1)
    apply_sf<float>(n, d_iapc, d_japc, d_apc32, F, B, Wd, r, d, const_cast<Ctl *>(ctl), st);
  else
    apply_levels<float>(d_iapc, d_japc, d_apc32, F, B, r, d, ctl, st);
}

}  // namespace gb
