// k_scale.cu -- matrix scaling of the IMS linear solve, ims_base_scale
// (src/Solution/LinearMethods/ImsLinearBase.f90:619-757).
//
// SCALING_METHOD DIAGONAL (ISCL 1): DSCALE = DSCALE2 = 1/sqrt(|a_nn|) and
// A <- DSCALE(row) * A * DSCALE2(col).  SCALING_METHOD L2NORM (ISCL 2): every
// row scaled to unit L2 norm, then every column.  X <- X / DSCALE2 and
// B <- B * DSCALE before the solve, X <- X * DSCALE2 after it.
//
// Every operation is explicitly rounded (no FMA contraction) and every sum
// runs in the reference's order: row sums in CSR order, column sums over the
// rows in ascending order (a column-major position map built at create), so
// the scaled system is bit-identical to the reference's.
#include "gbims_internal.cuh"
#include <algorithm>

namespace gb {

namespace {

__global__ void k_scale_diag(int n, const int *__restrict__ ia, const double *__restrict__ amat,
                             double *__restrict__ dscale, double *__restrict__ dscale2) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const double c1 = __ddiv_rn(1.0, __dsqrt_rn(fabs(amat[ia[r]])));
    dscale[r] = c1;
    dscale2[r] = c1;
  }
}

// AMAT = DSCALE(row) * AMAT(i) * DSCALE2(col), evaluated left to right.
__global__ void k_scale_sym(int n, const int *__restrict__ ia, const int *__restrict__ ja,
                            double *__restrict__ amat, const double *__restrict__ dscale,
                            const double *__restrict__ dscale2) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const double c1 = dscale[r];
    for (int i = ia[r]; i < ia[r + 1]; ++i)
      amat[i] = __dmul_rn(__dmul_rn(c1, amat[i]), dscale2[ja[i]]);
  }
}

// Row L2 norms; AMAT = DSCALE(row) * AMAT(i).
__global__ void k_scale_rows(int n, const int *__restrict__ ia, double *__restrict__ amat,
                             double *__restrict__ dscale) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    double c1 = 0.0;
    for (int i = ia[r]; i < ia[r + 1]; ++i) c1 = __dadd_rn(c1, __dmul_rn(amat[i], amat[i]));
    c1 = __dsqrt_rn(c1);
    c1 = (c1 == 0.0) ? 1.0 : __ddiv_rn(1.0, c1);
    dscale[r] = c1;
    for (int i = ia[r]; i < ia[r + 1]; ++i) amat[i] = __dmul_rn(c1, amat[i]);
  }
}

// Column L2 norms of the row-scaled matrix, summed over the rows in
// ascending order: cpos[cptr[c] .. cptr[c+1]) are the positions of column c.
__global__ void k_scale_colnorm(int n, const int *__restrict__ cptr, const int *__restrict__ cpos,
                                const double *__restrict__ amat, double *__restrict__ dscale2) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int q = cptr[c]; q < cptr[c + 1]; ++q) {
      const double a = amat[cpos[q]];
      s = __dadd_rn(s, __dmul_rn(a, a));
    }
    dscale2[c] = (s == 0.0) ? 1.0 : __ddiv_rn(1.0, __dsqrt_rn(s));
  }
}

// AMAT = DSCALE2(col) * AMAT(i).
__global__ void k_scale_cols(int n, const int *__restrict__ ia, const int *__restrict__ ja,
                             double *__restrict__ amat, const double *__restrict__ dscale2) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    for (int i = ia[r]; i < ia[r + 1]; ++i) amat[i] = __dmul_rn(dscale2[ja[i]], amat[i]);
}

__global__ void k_scale_xb(int n, double *__restrict__ x, double *__restrict__ b,
                           const double *__restrict__ dscale, const double *__restrict__ dscale2) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    x[r] = __ddiv_rn(x[r], dscale2[r]);
    b[r] = __dmul_rn(b[r], dscale[r]);
  }
}

__global__ void k_unscale_x(int n, double *__restrict__ x, const double *__restrict__ dscale2) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    x[r] = __dmul_rn(x[r], dscale2[r]);
}

}  // namespace

void scale_colmap_host(int n, const std::vector<int> &ia, const std::vector<int> &ja,
                       std::vector<int> &cptr, std::vector<int> &cpos) {
  cptr.assign(n + 1, 0);
  for (int k = 0; k < ia[n]; ++k) cptr[ja[k] + 1]++;
  for (int c = 0; c < n; ++c) cptr[c + 1] += cptr[c];
  cpos.assign(ia[n], 0);
  std::vector<int> fill(cptr.begin(), cptr.end() - 1);
  for (int r = 0; r < n; ++r)  // rows in ascending order: each column list is row-sorted
    for (int k = ia[r]; k < ia[r + 1]; ++k) cpos[fill[ja[k]]++] = k;
}

int launch_scale(int iscl, int n, const int *ia, const int *ja, const int *cptr, const int *cpos,
                 double *amat, double *x, double *b, double *dscale, double *dscale2,
                 cudaStream_t st) {
  const int g = std::max(1, std::min(8 * kNumSM, (n + 255) / 256));
  if (iscl == 1) {
    k_scale_diag<<<g, 256, 0, st>>>(n, ia, amat, dscale, dscale2);
    k_scale_sym<<<g, 256, 0, st>>>(n, ia, ja, amat, dscale, dscale2);
    k_scale_xb<<<g, 256, 0, st>>>(n, x, b, dscale, dscale2);
    return 3;
  }
  k_scale_rows<<<g, 256, 0, st>>>(n, ia, amat, dscale);
  k_scale_colnorm<<<g, 256, 0, st>>>(n, cptr, cpos, amat, dscale2);
  k_scale_cols<<<g, 256, 0, st>>>(n, ia, ja, amat, dscale2);
  k_scale_xb<<<g, 256, 0, st>>>(n, x, b, dscale, dscale2);
  return 4;
}

void launch_unscale_x(int n, double *x, const double *dscale2, cudaStream_t st) {
  const int g = std::max(1, std::min(8 * kNumSM, (n + 255) / 256));
  k_unscale_x<<<g, 256, 0, st>>>(n, x, dscale2);
}

}  // namespace gb
