// k_mpnn.cuh -- device state and launchers of the warm-start network
// (k_mpnn.cu), shared with its C ABI (gbmpnn_api.cu).
#pragma once
#include <cuda_bf16.h>

#include "gbims_internal.cuh"

namespace gb {

constexpr int kMpnnHidden = 64;    // hidden width
constexpr int kMpnnFeatures = 16;  // node features (one k16 slice)
constexpr int kMpnnLayers = 8;     // message-passing layers

struct MpnnDev {
  int n = 0;
  const int *ia = nullptr, *ja = nullptr;     // matrix graph (CSR, diagonal first)
  float *w = nullptr, *deg = nullptr;         // normalised edge weights, degrees
  float *p = nullptr, *g = nullptr;           // FP32 parameters and gradients
  float *m = nullptr, *v = nullptr;           // Adam moments
  __nv_bfloat16 *bt0 = nullptr, *wbf0 = nullptr;                    // W0 as BF16
  __nv_bfloat16 *bt[kMpnnLayers] = {}, *wbf[kMpnnLayers] = {};      // W_l as BF16
  __nv_bfloat16 *xbf = nullptr;                                     // features, BF16
  float *H[kMpnnLayers + 1] = {};             // residual stream per layer (FP32)
  __nv_bfloat16 *Hbf[kMpnnLayers + 1] = {};
  float *A = nullptr;                         // aggregation scratch (FP32)
  __nv_bfloat16 *Abf[kMpnnLayers + 1] = {};   // aggregations (BF16, for dW)
  unsigned char *mask[kMpnnLayers + 1] = {};  // relu masks
  float *y = nullptr, *dy = nullptr, *loss = nullptr;
  float *dH = nullptr, *dHp = nullptr, *dX = nullptr;
  __nv_bfloat16 *dZ = nullptr;
  int steps = 0;                              // Adam steps taken
  // energy loss (mode 1): the matrix of the last set_graph, the errors and
  // true changes in head units, W*e, and per-block partials of e'We, t'Wt
  int nja = 0;
  int energy = 0;
  float mse_w = 1.f;
  double dh_soft = 1.0, dh_scale = 1.0;
  double *amat = nullptr, *ee = nullptr, *tt = nullptr, *we = nullptr, *epart = nullptr;
};
constexpr int kMpnnRedBlocks = 1024;  // grid of the energy-loss reductions

long long mpnn_param_count();
void mpnn_set_graph(MpnnDev &D, const double *d_amat, cudaStream_t st);
void mpnn_refresh_bf16(MpnnDev &D, cudaStream_t st);
void mpnn_forward(MpnnDev &D, const float *d_x, const float *target, const float *mask,
                  float inv_count, cudaStream_t st);
void mpnn_backward(MpnnDev &D, cudaStream_t st);
void mpnn_adam(MpnnDev &D, float lr, cudaStream_t st);
// The warm start's guess on the device: features from the last two steps'
// heads (x, xold; xold ignored when first), the forward pass, and
// guess = x + the predicted change on active cells.
struct GuessScaling {
  double head_ref, head_scale, dh_soft, dh_scale, unit_max;
};
void mpnn_guess(MpnnDev &D, const float *d_static, const double *x, const double *xold,
                int first, const int *ibound, const GuessScaling &sc, double *guess,
                cudaStream_t st);

}  // namespace gb
