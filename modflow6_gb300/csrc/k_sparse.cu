// k_sparse.cu -- SELL-32 sparse matrix-vector products.
//
// Replaces amux (src/Utilities/Libraries/sparsekit/sparsekit.f90:1-59) and
// ims_base_residual (src/Solution/LinearMethods/ImsLinearBase.f90:1291-1312).
// One thread per row, one warp per 32-row slice; the k-th entry of every row
// of a slice is contiguous, so each entry column of a slice is one coalesced
// 256-byte value load and one 128-byte index load.  Entries are summed in CSR
// (JA) order with fused multiply-adds, t = fma(a, x, t) from t = 0, the order
// of amux with FMA contraction.
#include "gbims_internal.cuh"

namespace gb {

void sell_build_host(int n, const std::vector<int> &ia, const std::vector<int> &ja,
                     std::vector<int> &ptr, std::vector<int> &col, std::vector<int> &src) {
  int nslices = (n + kSell - 1) / kSell;
  ptr.assign(nslices + 1, 0);
  long long total = 0;
  for (int s = 0; s < nslices; ++s) {
    int w = 0;
    for (int r = s * kSell; r < std::min(n, (s + 1) * kSell); ++r) w = std::max(w, ia[r + 1] - ia[r]);
    ptr[s] = (int)total;
    total += (long long)w * kSell;
  }
  ptr[nslices] = (int)total;
  col.assign(total, 0);
  src.assign(total, -1);
  for (int s = 0; s < nslices; ++s) {
    int w = (ptr[s + 1] - ptr[s]) / kSell;
    for (int l = 0; l < kSell; ++l) {
      int r = s * kSell + l;
      for (int k = 0; k < w; ++k) {
        long long p = ptr[s] + (long long)k * kSell + l;
        if (r < n && k < ia[r + 1] - ia[r]) {
          col[p] = ja[ia[r] + k];
          src[p] = ia[r] + k;
        } else {
          col[p] = (r < n) ? r : 0;  // padding: zero value times x[row]
          src[p] = -1;
        }
      }
    }
  }
}

__global__ void k_sell_fill(long long nstored, const int *__restrict__ src,
                            const double *__restrict__ amat, double *__restrict__ val,
                            float *__restrict__ val32) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nstored;
       p += (long long)gridDim.x * blockDim.x) {
    int s = src[p];
    double v = (s >= 0) ? amat[s] : 0.0;
    val[p] = v;
    if (val32) val32[p] = (float)v;
  }
}

void launch_sell_fill(const Sell &S, const double *d_amat, cudaStream_t st) {
  if (S.nstored == 0) return;
  int grid = (int)std::min<long long>((S.nstored + 255) / 256, 8LL * kNumSM);
  k_sell_fill<<<grid, 256, 0, st>>>(S.nstored, S.d_src, d_amat, S.d_val, S.d_val32);
}

// Streaming loads for matrix data (read once per product) keep the L2 for
// the gathered vector.
template <typename T>
__device__ __forceinline__ T ld_stream(const T *p) { return __ldcs(p); }

template <typename T>
__device__ __forceinline__ T mac(T a, T x, T t);
template <>
__device__ __forceinline__ double mac<double>(double a, double x, double t) { return fma(a, x, t); }
template <>
__device__ __forceinline__ float mac<float>(float a, float x, float t) { return fmaf(a, x, t); }

// y = A*x (MODE 0), or d = b - A*x (MODE 1).
template <typename T, int MODE, typename TM = T>
__global__ void __launch_bounds__(256) k_sell_spmv(int n, const int *__restrict__ ptr,
                                                    const int *__restrict__ col,
                                                    const TM *__restrict__ val,
                                                    const T *__restrict__ x,
                                                    const T *__restrict__ b, T *__restrict__ y,
                                                    const Ctl *__restrict__ ctl,
                                                    int only_if_north_due,
                                                    const int *__restrict__ slm,
                                                    const int *__restrict__ mrow, int nm,
                                                    const Ctl *__restrict__ mctl) {
  if (ctl) {
    if (ctl->done) return;
    if (only_if_north_due && !ctl->north_due) return;
  }
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  int s = row / kSell, lane = row % kSell;
  if (mctl) {  // batched ensemble: rows of a member that is done are skipped
    int m = slm[s];
    if (m < 0) {
      int lo = 0, hi = nm - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (mrow[mid] <= row) lo = mid;
        else hi = mid - 1;
      }
      m = lo;
    }
    if (mctl[m].done) return;
  }
  int p0 = ptr[s];
  int w = (ptr[s + 1] - p0) / kSell;
  const int *c = col + p0 + lane;
  const TM *v = val + p0 + lane;
  T t = T(0);
  if (w <= 8) {
    // the common 5/7-point case: issue all loads first, then the gathers
    int cc[8];
    TM vv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < w) {
        cc[k] = ld_stream(c + k * kSell);
        vv[k] = ld_stream(v + k * kSell);
      }
    }
    T xx[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k < w) xx[k] = __ldg(x + cc[k]);
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k < w) t = mac<T>((T)vv[k], xx[k], t);
  } else {
    for (int k = 0; k < w; ++k)
      t = mac<T>((T)ld_stream(v + k * kSell), __ldg(x + ld_stream(c + k * kSell)), t);
  }
  if (MODE == 0) y[row] = t;
  else y[row] = b[row] - t;
}

static inline int rows_grid(int n) { return (n + 255) / 256; }

// ---------------------------------------------------------------------------
// Full DIS grids (7-point, natural order): the same products without index
// arrays.  Value slot s of row r sits at v[s*n + r], slots in CSR (JA) order
// (diagonal, k-1, i-1, j-1, j+1, i+1, k+1); absent neighbours hold zero and
// are skipped, so every row sums exactly the entries of its CSR row in JA
// order, like the SELL kernel.
// ---------------------------------------------------------------------------
__global__ void k_dia7_vfill(int nlay, int nrow, int ncol, const int *__restrict__ ia,
                             const double *__restrict__ amat, double *__restrict__ v,
                             float *__restrict__ v32) {
  const long long nrc = (long long)nrow * ncol, n = nrc * nlay;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(r / nrc);
    const int rem = (int)(r - k * nrc);
    const int i = rem / ncol, j = rem - i * ncol;
    const bool has[7] = {true, k > 0, i > 0, j > 0, j < ncol - 1, i < nrow - 1, k < nlay - 1};
    int p = ia[r];
#pragma unroll
    for (int s = 0; s < 7; ++s) {
      const double a = has[s] ? amat[p++] : 0.0;
      if (v) v[s * n + r] = a;
      if (v32) v32[s * n + r] = (float)a;
    }
  }
}

template <typename T, int MODE, typename TM = T>
__global__ void __launch_bounds__(256) k_dia7_spmv(int nlay, int nrow, int ncol,
                                                   const TM *__restrict__ v,
                                                   const T *__restrict__ x,
                                                   const T *__restrict__ b, T *__restrict__ y,
                                                   const Ctl *__restrict__ ctl,
                                                   int only_if_north_due) {
  if (ctl) {
    if (ctl->done) return;
    if (only_if_north_due && !ctl->north_due) return;
  }
  const int nrc = nrow * ncol, n = nrc * nlay;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int k = r / nrc;
  const int rem = r - k * nrc;
  const int i = rem / ncol, j = rem - i * ncol;
  const bool has[7] = {true, k > 0, i > 0, j > 0, j < ncol - 1, i < nrow - 1, k < nlay - 1};
  const int off[7] = {0, -nrc, -ncol, -1, 1, ncol, nrc};
  TM vv[7];
  T xx[7];
#pragma unroll
  for (int s = 0; s < 7; ++s)
    if (has[s]) vv[s] = ld_stream(v + (size_t)s * n + r);
#pragma unroll
  for (int s = 0; s < 7; ++s)
    if (has[s]) xx[s] = __ldg(x + r + off[s]);
  T t = T(0);
#pragma unroll
  for (int s = 0; s < 7; ++s)
    if (has[s]) t = mac<T>((T)vv[s], xx[s], t);
  if (MODE == 0) y[r] = t;
  else y[r] = b[r] - t;
}

void launch_dia7_vfill(const Dia7 &D, const int *d_ia, const double *d_amat, cudaStream_t st) {
  const long long n = (long long)D.nlay * D.nrow * D.ncol;
  const int grid = (int)std::min<long long>((n + 255) / 256, 8LL * kNumSM);
  k_dia7_vfill<<<grid, 256, 0, st>>>(D.nlay, D.nrow, D.ncol, d_ia, d_amat, D.d_sv, D.f_sv);
}

void launch_dia7_spmv64(const Dia7 &D, const double *x, double *y, const Ctl *ctl,
                        cudaStream_t st) {
  const int n = D.nlay * D.nrow * D.ncol;
  k_dia7_spmv<double, 0><<<rows_grid(n), 256, 0, st>>>(D.nlay, D.nrow, D.ncol, D.d_sv, x,
                                                        nullptr, y, ctl, 0);
}

void launch_dia7_spmv32(const Dia7 &D, const float *x, float *y, const Ctl *ctl,
                        cudaStream_t st) {
  const int n = D.nlay * D.nrow * D.ncol;
  k_dia7_spmv<float, 0><<<rows_grid(n), 256, 0, st>>>(D.nlay, D.nrow, D.ncol, D.f_sv, x,
                                                       nullptr, y, ctl, 0);
}

void launch_dia7_residual64(const Dia7 &D, const double *x, const double *b, double *d,
                            const Ctl *ctl, int only_if_north_due, cudaStream_t st) {
  const int n = D.nlay * D.nrow * D.ncol;
  k_dia7_spmv<double, 1><<<rows_grid(n), 256, 0, st>>>(D.nlay, D.nrow, D.ncol, D.d_sv, x, b,
                                                        d, ctl, only_if_north_due);
}

void launch_spmv64(const Sell &S, const double *x, double *y, const Ctl *ctl, cudaStream_t st) {
  if (S.n == 0) return;
  k_sell_spmv<double, 0><<<rows_grid(S.n), 256, 0, st>>>(S.n, S.d_ptr, S.d_col, S.d_val, x,
                                                          nullptr, y, ctl, 0, S.d_slm, S.d_mrow,
                                                          S.nm, S.mctl);
}

void launch_spmv32(const Sell &S, const float *x, float *y, const Ctl *ctl, cudaStream_t st) {
  if (S.n == 0) return;
  k_sell_spmv<float, 0><<<rows_grid(S.n), 256, 0, st>>>(S.n, S.d_ptr, S.d_col, S.d_val32, x,
                                                         nullptr, y, ctl, 0, S.d_slm, S.d_mrow,
                                                         S.nm, S.mctl);
}

void launch_residual64(const Sell &S, const double *x, const double *b, double *d,
                       const Ctl *ctl, int only_if_north_due, cudaStream_t st) {
  if (S.n == 0) return;
  k_sell_spmv<double, 1><<<rows_grid(S.n), 256, 0, st>>>(S.n, S.d_ptr, S.d_col, S.d_val, x, b,
                                                          d, ctl, only_if_north_due, S.d_slm,
                                                          S.d_mrow, S.nm, S.mctl);
}

}  // namespace gb
