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
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_sell_spmv(int n, const int *__restrict__ ptr,
                                                    const int *__restrict__ col,
                                                    const T *__restrict__ val,
                                                    const T *__restrict__ x,
                                                    const T *__restrict__ b, T *__restrict__ y,
                                                    const Ctl *__restrict__ ctl,
                                                    int only_if_north_due) {
  if (ctl) {
    if (ctl->done) return;
    if (only_if_north_due && !ctl->north_due) return;
  }
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  int s = row / kSell, lane = row % kSell;
  int p0 = ptr[s];
  int w = (ptr[s + 1] - p0) / kSell;
  const int *c = col + p0 + lane;
  const T *v = val + p0 + lane;
  T t = T(0);
  if (w <= 8) {
    // the common 5/7-point case: issue all loads first, then the gathers
    int cc[8];
    T vv[8];
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
      if (k < w) t = mac<T>(vv[k], xx[k], t);
  } else {
    for (int k = 0; k < w; ++k) t = mac<T>(ld_stream(v + k * kSell), __ldg(x + ld_stream(c + k * kSell)), t);
  }
  if (MODE == 0) y[row] = t;
  else y[row] = b[row] - t;
}

static inline int rows_grid(int n) { return (n + 255) / 256; }

void launch_spmv64(const Sell &S, const double *x, double *y, const Ctl *ctl, cudaStream_t st) {
  if (S.n == 0) return;
  k_sell_spmv<double, 0><<<rows_grid(S.n), 256, 0, st>>>(S.n, S.d_ptr, S.d_col, S.d_val, x,
                                                          nullptr, y, ctl, 0);
}

void launch_spmv32(const Sell &S, const float *x, float *y, const Ctl *ctl, cudaStream_t st) {
  if (S.n == 0) return;
  k_sell_spmv<float, 0><<<rows_grid(S.n), 256, 0, st>>>(S.n, S.d_ptr, S.d_col, S.d_val32, x,
                                                         nullptr, y, ctl, 0);
}

void launch_residual64(const Sell &S, const double *x, const double *b, double *d,
                       const Ctl *ctl, int only_if_north_due, cudaStream_t st) {
  if (S.n == 0) return;
  k_sell_spmv<double, 1><<<rows_grid(S.n), 256, 0, st>>>(S.n, S.d_ptr, S.d_col, S.d_val, x, b,
                                                          d, ctl, only_if_north_due);
}

}  // namespace gb
