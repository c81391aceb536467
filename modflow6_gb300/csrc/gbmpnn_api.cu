// gbmpnn_api.cu -- C ABI of the learned warm start (include/gbims.h,
// gbmpnn_*): a message-passing network over the IMS matrix graph, trained and
// evaluated on the GPU by the kernels of k_mpnn.cu.
#include <cstring>
#include <new>
#include <random>
#include <string>

#include <cmath>
#include <vector>

#include "k_mpnn.cuh"

using namespace gb;

struct gbmpnn_handle {
  MpnnDev D;
  int n = 0, nja = 0, hidden = 0, layers = 0, features = 0;
  long long np = 0;
  int *d_ia = nullptr, *d_ja = nullptr;
  cudaStream_t st = nullptr;
  std::string err;
};

#define MP_CUDA(h, call)                                                        \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      if (h) (h)->err = std::string(#call) + ": " + cudaGetErrorString(e_);     \
      return GBIMS_ERR_CUDA;                                                    \
    }                                                                           \
  } while (0)

template <typename T>
static cudaError_t alloc(T **p, size_t count) {
  *p = nullptr;
  return cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
}

extern "C" long long gbmpnn_param_count(void) { return mpnn_param_count(); }

extern "C" int gbmpnn_create(int nodes, int nja, const int *ia, const int *ja,
                             unsigned long long seed, gbmpnn_handle **out) {
  if (!out) return GBIMS_ERR_ARG;
  *out = nullptr;
  if (nodes <= 0 || nja < nodes || !ia || !ja) return GBIMS_ERR_ARG;
  gbmpnn_handle *h = new (std::nothrow) gbmpnn_handle();
  if (!h) return GBIMS_ERR_NOMEM;
  *out = h;
  h->n = nodes;
  h->nja = nja;
  h->hidden = kMpnnHidden;
  h->layers = kMpnnLayers;
  h->features = kMpnnFeatures;
  h->np = mpnn_param_count();
  const int H = h->hidden, L = h->layers;
  (void)L;
  const size_t n = (size_t)nodes;
  MpnnDev &D = h->D;
  D.n = nodes;
  MP_CUDA(h, cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  MP_CUDA(h, alloc(&h->d_ia, n + 1));
  MP_CUDA(h, alloc(&h->d_ja, (size_t)nja));
  MP_CUDA(h, cudaMemcpy(h->d_ia, ia, sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
  MP_CUDA(h, cudaMemcpy(h->d_ja, ja, sizeof(int) * nja, cudaMemcpyHostToDevice));
  D.ia = h->d_ia;
  D.ja = h->d_ja;
  MP_CUDA(h, alloc(&D.w, (size_t)nja));
  MP_CUDA(h, alloc(&D.deg, n));
  MP_CUDA(h, alloc(&D.p, (size_t)h->np));
  MP_CUDA(h, alloc(&D.g, (size_t)h->np));
  MP_CUDA(h, alloc(&D.m, (size_t)h->np));
  MP_CUDA(h, alloc(&D.v, (size_t)h->np));
  MP_CUDA(h, alloc(&D.bt0, (size_t)h->features * H));
  MP_CUDA(h, alloc(&D.wbf0, (size_t)h->features * H));
  for (int l = 0; l < L; ++l) {
    MP_CUDA(h, alloc(&D.bt[l], (size_t)2 * H * H));
    MP_CUDA(h, alloc(&D.wbf[l], (size_t)2 * H * H));
  }
  MP_CUDA(h, alloc(&D.xbf, n * h->features));
  for (int l = 0; l <= L; ++l) {
    MP_CUDA(h, alloc(&D.H[l], n * H));
    MP_CUDA(h, alloc(&D.Hbf[l], n * H));
    MP_CUDA(h, alloc(&D.Abf[l], n * H));
    MP_CUDA(h, alloc(&D.mask[l], n * H));
  }
  MP_CUDA(h, alloc(&D.A, n * H));
  MP_CUDA(h, alloc(&D.y, n));
  MP_CUDA(h, alloc(&D.dy, n));
  MP_CUDA(h, alloc(&D.loss, 1));
  MP_CUDA(h, alloc(&D.dH, n * H));
  MP_CUDA(h, alloc(&D.dHp, n * H));
  MP_CUDA(h, alloc(&D.dX, n * 2 * H));
  MP_CUDA(h, alloc(&D.dZ, n * H));
  D.nja = nja;
  MP_CUDA(h, alloc(&D.amat, (size_t)nja));
  MP_CUDA(h, cudaMemset(D.amat, 0, sizeof(double) * nja));
  MP_CUDA(h, alloc(&D.ee, n));
  MP_CUDA(h, alloc(&D.tt, n));
  MP_CUDA(h, alloc(&D.we, n));
  MP_CUDA(h, alloc(&D.epart, (size_t)2 * kMpnnRedBlocks));
  // initial weights: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)), zero biases
  // except the output, from a seeded host generator
  std::vector<float> p((size_t)h->np, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](long long off, int fan_in, int count, float gain) {
    const float a = gain / std::sqrt((float)fan_in);
    std::uniform_real_distribution<float> u(-a, a);
    for (int i = 0; i < count; ++i) p[(size_t)off + i] = u(rng);
  };
  long long off = 0;
  fill(off, h->features, h->features * H, 1.f);
  off += (long long)h->features * H + H;
  for (int l = 0; l < L; ++l) {
    fill(off, 2 * H, 2 * H * H, 0.5f);  // damped residual branches
    off += 2LL * H * H + H;
  }
  fill(off, H, H, 0.1f);  // small initial output
  MP_CUDA(h, cudaMemcpy(D.p, p.data(), sizeof(float) * p.size(), cudaMemcpyHostToDevice));
  MP_CUDA(h, cudaMemset(D.m, 0, sizeof(float) * h->np));
  MP_CUDA(h, cudaMemset(D.v, 0, sizeof(float) * h->np));
  mpnn_refresh_bf16(D, h->st);
  MP_CUDA(h, cudaStreamSynchronize(h->st));
  MP_CUDA(h, cudaGetLastError());
  return GBIMS_OK;
}

extern "C" int gbmpnn_set_graph(gbmpnn_handle *h, const double *d_amat) {
  if (!h || !d_amat) return GBIMS_ERR_ARG;
  mpnn_set_graph(h->D, d_amat, h->st);
  MP_CUDA(h, cudaStreamSynchronize(h->st));
  MP_CUDA(h, cudaGetLastError());
  return GBIMS_OK;
}

extern "C" int gbmpnn_set_loss(gbmpnn_handle *h, int mode, const gbmpnn_scaling *sc,
                               float mse_weight) {
  if (!h || (mode != 0 && mode != 1) || !(mse_weight >= 0.f)) return GBIMS_ERR_ARG;
  if (mode == 1 && (!sc || !(sc->dh_soft > 0.0) || !(sc->dh_scale > 0.0))) return GBIMS_ERR_ARG;
  MP_CUDA(h, cudaStreamSynchronize(h->st));
  h->D.energy = mode;
  h->D.mse_w = (mode == 1) ? mse_weight : 1.f;
  if (mode == 1) {
    h->D.dh_soft = sc->dh_soft;
    h->D.dh_scale = sc->dh_scale;
  }
  return GBIMS_OK;
}

extern "C" int gbsln_warm_guess(gbsln_handle *sln, gbmpnn_handle *h, const float *d_static,
                                const gbmpnn_scaling *sc, int first_step, double *d_guess,
                                float *device_ms) {
  if (!sln || !h || !d_static || !sc || !d_guess) return GBIMS_ERR_ARG;
  SlnView v;
  if (sln_view(sln, &v) != GBIMS_OK || v.n != h->n) return GBIMS_ERR_ARG;
  if (!(sc->head_scale != 0.0) || !(sc->dh_soft > 0.0) || !(sc->dh_scale > 0.0))
    return GBIMS_ERR_ARG;
  const GuessScaling g{sc->head_ref, sc->head_scale, sc->dh_soft, sc->dh_scale, sc->unit_max};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (device_ms) {
    MP_CUDA(h, cudaEventCreate(&e0));
    MP_CUDA(h, cudaEventCreate(&e1));
    MP_CUDA(h, cudaEventRecord(e0, v.st));
  }
  // on the time step's own stream: the step that reads the guess follows in
  // stream order, with no host synchronisation in between
  mpnn_guess(h->D, d_static, v.x, v.xold, first_step, v.ibound, g, d_guess, v.st);
  MP_CUDA(h, cudaGetLastError());
  if (device_ms) {
    MP_CUDA(h, cudaEventRecord(e1, v.st));
    MP_CUDA(h, cudaEventSynchronize(e1));
    MP_CUDA(h, cudaEventElapsedTime(device_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  return GBIMS_OK;
}

extern "C" int gbmpnn_forward(gbmpnn_handle *h, const float *d_x, float *d_y) {
  if (!h || !d_x || !d_y) return GBIMS_ERR_ARG;
  mpnn_forward(h->D, d_x, nullptr, nullptr, 0.f, h->st);
  MP_CUDA(h, cudaMemcpyAsync(d_y, h->D.y, sizeof(float) * h->n, cudaMemcpyDeviceToDevice, h->st));
  MP_CUDA(h, cudaStreamSynchronize(h->st));
  MP_CUDA(h, cudaGetLastError());
  return GBIMS_OK;
}

// Forward + backward; the loss and, if grad is not NULL, the gradients
// (gbmpnn_param_count floats) come back to the host.  inv_count scales the
// masked squared error.
static int fwd_bwd(gbmpnn_handle *h, const float *d_x, const float *d_t, const float *d_mask,
                   float inv_count, float *loss) {
  mpnn_forward(h->D, d_x, d_t, d_mask, inv_count, h->st);
  mpnn_backward(h->D, h->st);
  if (loss) MP_CUDA(h, cudaMemcpyAsync(loss, h->D.loss, sizeof(float), cudaMemcpyDeviceToHost, h->st));
  return GBIMS_OK;
}

extern "C" int gbmpnn_gradients(gbmpnn_handle *h, const float *d_x, const float *d_target,
                                const float *d_mask, float inv_count, float *loss, float *grad) {
  if (!h || !d_x || !d_target || !d_mask) return GBIMS_ERR_ARG;
  int rc = fwd_bwd(h, d_x, d_target, d_mask, inv_count, loss);
  if (rc) return rc;
  if (grad) MP_CUDA(h, cudaMemcpyAsync(grad, h->D.g, sizeof(float) * h->np, cudaMemcpyDeviceToHost, h->st));
  MP_CUDA(h, cudaStreamSynchronize(h->st));
  MP_CUDA(h, cudaGetLastError());
  return GBIMS_OK;
}

extern "C" int gbmpnn_train_step(gbmpnn_handle *h, const float *d_x, const float *d_target,
                                 const float *d_mask, float inv_count, float lr, float *loss) {
  if (!h || !d_x || !d_target || !d_mask || !(lr > 0.f)) return GBIMS_ERR_ARG;
  int rc = fwd_bwd(h, d_x, d_target, d_mask, inv_count, loss);
  if (rc) return rc;
  mpnn_adam(h->D, lr, h->st);
  MP_CUDA(h, cudaStreamSynchronize(h->st));
  MP_CUDA(h, cudaGetLastError());
  return GBIMS_OK;
}

extern "C" int gbmpnn_get_params(gbmpnn_handle *h, float *params) {
  if (!h || !params) return GBIMS_ERR_ARG;
  MP_CUDA(h, cudaStreamSynchronize(h->st));
  MP_CUDA(h, cudaMemcpy(params, h->D.p, sizeof(float) * h->np, cudaMemcpyDeviceToHost));
  return GBIMS_OK;
}

extern "C" int gbmpnn_set_params(gbmpnn_handle *h, const float *params) {
  if (!h || !params) return GBIMS_ERR_ARG;
  MP_CUDA(h, cudaMemcpy(h->D.p, params, sizeof(float) * h->np, cudaMemcpyHostToDevice));
  mpnn_refresh_bf16(h->D, h->st);
  MP_CUDA(h, cudaStreamSynchronize(h->st));
  return GBIMS_OK;
}

extern "C" const char *gbmpnn_last_error(const gbmpnn_handle *h) {
  return h ? h->err.c_str() : "null handle";
}

extern "C" int gbmpnn_destroy(gbmpnn_handle *h) {
  if (!h) return GBIMS_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  MpnnDev &D = h->D;
  std::vector<void *> ptrs = {h->d_ia, h->d_ja, D.w, D.deg, D.p, D.g, D.m, D.v, D.bt0, D.wbf0,
                              D.xbf, D.A, D.y, D.dy, D.loss, D.dH, D.dHp, D.dX, D.dZ,
                              D.amat, D.ee, D.tt, D.we, D.epart};
  for (int l = 0; l < kMpnnLayers; ++l) {
    ptrs.push_back(D.bt[l]);
    ptrs.push_back(D.wbf[l]);
  }
  for (int l = 0; l <= kMpnnLayers; ++l) {
    ptrs.push_back(D.H[l]);
    ptrs.push_back(D.Hbf[l]);
    ptrs.push_back(D.Abf[l]);
    ptrs.push_back(D.mask[l]);
  }
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return GBIMS_OK;
}
