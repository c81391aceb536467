// gbims_noalloc.cu -- gbims_residual_noalloc: the initial residual of an IMS
// solve (d = b - A x, its L2 norm and signed max|d|; ims_base_residual and
// dnrm2, src/Solution/LinearMethods/ImsLinearBase.f90:1291-1312) from the
// caller's device arrays, allocating nothing.  It serves hosts whose device
// memory is owned by their own memory manager (the GPU's memory reserved up
// front and handed out in pieces), where a cudaMalloc by a library would fail
// or fragment that pool.  The call copies its three results to the host and
// synchronizes its stream before it returns.
//
// The reduction partials live in a file-scope device array sized for
// kNoAllocBlocks blocks of 256 rows, so the call serves systems of at most
// kNoAllocMaxRows rows and rejects larger ones.  The array's address is looked
// up once per device (cudaGetSymbolAddress); that first call also loads the
// library's device code, so it must come before any stream capture.  Every
// scratch slot a call reads is written earlier in the same call: nothing has
// to start at zero and nothing carries over.  The scratch is shared by all
// callers on a device, so overlapping calls (two host threads, or two streams
// in flight at once) race on it.
#include <cmath>
#include <mutex>

#include "gbims_internal.cuh"
#include "k_krylov.cuh"

using namespace gb;

namespace {

constexpr int kNoAllocBlocks = 608;                         // reduction blocks of 256 rows
constexpr int kNoAllocMaxRows = kNoAllocBlocks * kRedBlock;  // 155,648
constexpr int kNoAllocOut = 3 * kNoAllocBlocks;              // offset of the 3 results
static_assert(kNoAllocBlocks <= kMaxRedBlocks, "one row per thread, as in the handle's reductions");
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_noalloc_scratch[3 * kNoAllocBlocks + 4];

std::mutex g_addr_mu;
double *g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.
int scratch_address(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBIMS_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return GBIMS_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_addr_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GBIMS_ERR_CUDA;
    g_addr[dev] = static_cast<double *>(p);
  }
  *out = g_addr[dev];
  return GBIMS_OK;
}

}  // namespace

extern "C" int gbims_residual_noalloc(int neq, int nja, const int *d_ia, const int *d_ja,
                                      const double *d_amat, const double *d_x,
                                      const double *d_rhs, double *d_resid, int index_base,
                                      void *stream, double *l2norm, double *rmax, int *locr) {
  if (neq <= 0 || neq > kNoAllocMaxRows || nja < neq) return GBIMS_ERR_ARG;
  if (!d_ia || !d_ja || !d_amat || !d_x || !d_rhs || !l2norm || !rmax || !locr) return GBIMS_ERR_ARG;
  if (index_base != 0 && index_base != 1) return GBIMS_ERR_ARG;
  double *scr = nullptr;
  int rc = scratch_address(&scr);
  if (rc != GBIMS_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  kr_residual_rows(neq, d_ia, d_ja, index_base, d_amat, d_x, d_rhs, d_resid, scr,
                   scr + kNoAllocOut, st);
  if (cudaGetLastError() != cudaSuccess) return GBIMS_ERR_CUDA;
  double res[3];
  if (cudaMemcpyAsync(res, scr + kNoAllocOut, sizeof(res), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return GBIMS_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return GBIMS_ERR_CUDA;
  *l2norm = res[0];
  *rmax = res[1];
  *locr = (int)res[2];
  return std::isfinite(res[0]) ? GBIMS_OK : GBIMS_ERR_NONFINITE;
}
