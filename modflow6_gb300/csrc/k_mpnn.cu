// k_mpnn.cu -- learned warm start: a message-passing network over the IMS
// matrix graph that predicts a time step's head change, trained and run on
// the GPU by the kernels below (no counterpart in the reference, which
// starts every time step from the previous heads).
//
// Network (hidden width H = 64, L = 8 message-passing layers):
//   H0   = relu(X W0 + b0)                        X: N x 16 node features
//   A_l  = S H_{l-1}                               S: normalised conductances
//   Z_l  = [H_{l-1}, A_l] W_l + b_l                (N x 128) (128 x 64)
//   H_l  = H_{l-1} + relu(Z_l)                     l = 1..L
//   y    = H_L w_out + b_out                       predicted scaled head change
// S_ij = c_ij / sqrt(d_i d_j), c_ij = -a_ij the off-diagonal conductance of
// the assembled matrix and d_i = sum_j c_ij, so S is symmetric and the same
// kernel serves the forward and the backward pass.
//
// GEMM operands are BF16, accumulation FP32, on the tensor cores
// (mma.sync m16n8k16 BF16 -> FP32); the residual stream, the loss, the
// gradients and the Adam state are FP32.
#include <algorithm>

#include "k_mpnn.cuh"

namespace gb {

namespace {

constexpr int kH = kMpnnHidden;
constexpr int kIn = kMpnnFeatures;
constexpr int kL = kMpnnLayers;
constexpr int kCat = 2 * kH;

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4],
                                         const unsigned (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}


// ---------------------------------------------------------------------------
// Y[M x N] = [X1 | X2] (M x (K1 + K2), BF16 row-major) * B ((K1+K2) x N,
// given transposed: Bt N x (K1+K2), BF16), + bias.  64 rows per block, each
// of the 4 warps 16 rows x N columns.  Epilogue:
//   EPI 0: Y = acc + bias                       (FP32 out)
//   EPI 1: Y = relu(acc + bias), also BF16 copy, mask of acc + bias > 0
//   EPI 2: Y = Hold + relu(acc + bias), BF16 copy, mask
// ---------------------------------------------------------------------------
template <int K1, int K2, int N, int EPI>
__global__ void __launch_bounds__(128) k_gemm_rows(int M, const __nv_bfloat16 *__restrict__ X1,
                                                   const __nv_bfloat16 *__restrict__ X2,
                                                   const __nv_bfloat16 *__restrict__ Bt,
                                                   const float *__restrict__ bias,
                                                   const float *__restrict__ Hold,
                                                   float *__restrict__ Y,
                                                   __nv_bfloat16 *__restrict__ Ybf,
                                                   unsigned char *__restrict__ mask) {
  constexpr int K = K1 + K2;
  constexpr int KP = K + 8;  // padded row (bank spread)
  __shared__ __align__(16) __nv_bfloat16 xs[64][KP];
  __shared__ __align__(16) __nv_bfloat16 bs[N][KP];
  const int row0 = blockIdx.x * 64;
  for (int e = threadIdx.x; e < N * K; e += blockDim.x) bs[e / K][e % K] = Bt[e];
  for (int e = threadIdx.x; e < 64 * K; e += blockDim.x) {
    const int r = e / K, c = e % K, gr = row0 + r;
    __nv_bfloat16 v = __float2bfloat16(0.f);
    if (gr < M) v = (c < K1) ? X1[(size_t)gr * K1 + c] : X2[(size_t)gr * K2 + (c - K1)];
    xs[r][c] = v;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int r0 = warp * 16;
  float acc[N / 8][4];
#pragma unroll
  for (int nt = 0; nt < N / 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
  for (int ks = 0; ks < K / 16; ++ks) {
    const int k0 = ks * 16 + 2 * t;
    unsigned a[4];
    a[0] = *reinterpret_cast<const unsigned *>(&xs[r0 + g][k0]);
    a[1] = *reinterpret_cast<const unsigned *>(&xs[r0 + g + 8][k0]);
    a[2] = *reinterpret_cast<const unsigned *>(&xs[r0 + g][k0 + 8]);
    a[3] = *reinterpret_cast<const unsigned *>(&xs[r0 + g + 8][k0 + 8]);
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
      unsigned b[2];
      b[0] = *reinterpret_cast<const unsigned *>(&bs[nt * 8 + g][k0]);
      b[1] = *reinterpret_cast<const unsigned *>(&bs[nt * 8 + g][k0 + 8]);
      mma_bf16(acc[nt], a, b);
    }
  }
#pragma unroll
  for (int nt = 0; nt < N / 8; ++nt) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = row0 + r0 + g + 8 * h;
      if (r >= M) continue;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int c = nt * 8 + 2 * t + q;
        const size_t o = (size_t)r * N + c;
        float z = acc[nt][2 * h + q] + (bias ? bias[c] : 0.f);
        if (EPI == 0) {
          Y[o] = z;
        } else {
          const bool pos = z > 0.f;
          float yv = pos ? z : 0.f;
          if (EPI == 2) yv += Hold[o];
          Y[o] = yv;
          Ybf[o] = __float2bfloat16(yv);
          mask[o] = pos ? 1 : 0;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// G[K x N] += X^T dZ over a chunk of 64 rows: X (M x K, BF16), dZ (M x N,
// BF16); the block's partial sums go to G with atomicAdd.  Each warp owns
// K/4 rows of G.
// ---------------------------------------------------------------------------
template <int K1, int K2, int N>
__global__ void __launch_bounds__(128) k_gemm_xtdz(int M, const __nv_bfloat16 *__restrict__ X1,
                                                   const __nv_bfloat16 *__restrict__ X2,
                                                   const __nv_bfloat16 *__restrict__ dZ,
                                                   float *__restrict__ G) {
  constexpr int K = K1 + K2;
  constexpr int MC = 64, MP = MC + 8;
  __shared__ __align__(16) __nv_bfloat16 xt[K][MP];   // X^T chunk
  __shared__ __align__(16) __nv_bfloat16 dzt[N][MP];  // dZ^T chunk
  const int m0 = blockIdx.x * MC;
  for (int e = threadIdx.x; e < MC * K; e += blockDim.x) {
    const int m = e / K, c = e % K, gm = m0 + m;
    __nv_bfloat16 v = __float2bfloat16(0.f);
    if (gm < M) v = (c < K1) ? X1[(size_t)gm * K1 + c] : X2[(size_t)gm * K2 + (c - K1)];
    xt[c][m] = v;
  }
  for (int e = threadIdx.x; e < MC * N; e += blockDim.x) {
    const int m = e / N, c = e % N, gm = m0 + m;
    dzt[c][m] = (gm < M) ? dZ[(size_t)gm * N + c] : __float2bfloat16(0.f);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  constexpr int FT = K / 16 / 4 > 0 ? K / 16 / 4 : 1;  // m16 tiles of G rows per warp
  if (warp * FT * 16 >= K) return;
  float acc[FT][N / 8][4];
#pragma unroll
  for (int f = 0; f < FT; ++f)
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) acc[f][nt][0] = acc[f][nt][1] = acc[f][nt][2] = acc[f][nt][3] = 0.f;
#pragma unroll
  for (int ks = 0; ks < MC / 16; ++ks) {
    const int k0 = ks * 16 + 2 * t;
    unsigned b[N / 8][2];
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
      b[nt][0] = *reinterpret_cast<const unsigned *>(&dzt[nt * 8 + g][k0]);
      b[nt][1] = *reinterpret_cast<const unsigned *>(&dzt[nt * 8 + g][k0 + 8]);
    }
#pragma unroll
    for (int f = 0; f < FT; ++f) {
      const int fr = (warp * FT + f) * 16;
      unsigned a[4];
      a[0] = *reinterpret_cast<const unsigned *>(&xt[fr + g][k0]);
      a[1] = *reinterpret_cast<const unsigned *>(&xt[fr + g + 8][k0]);
      a[2] = *reinterpret_cast<const unsigned *>(&xt[fr + g][k0 + 8]);
      a[3] = *reinterpret_cast<const unsigned *>(&xt[fr + g + 8][k0 + 8]);
#pragma unroll
      for (int nt = 0; nt < N / 8; ++nt) mma_bf16(acc[f][nt], a, b[nt]);
    }
  }
#pragma unroll
  for (int f = 0; f < FT; ++f)
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int r = (warp * FT + f) * 16 + g + 8 * h, c = nt * 8 + 2 * t + q;
          atomicAdd(&G[r * N + c], acc[f][nt][2 * h + q]);
        }
}

// A = S H over the CSR pattern (off-diagonals), FP32 in, BF16 and FP32 out.
__global__ void k_aggregate(int n, const int *__restrict__ ia, const int *__restrict__ ja,
                            const float *__restrict__ w, const float *__restrict__ H,
                            float *__restrict__ A, __nv_bfloat16 *__restrict__ Abf) {
  // one warp per node, 2 features per lane
  const int node = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (node >= n) return;
  float a0 = 0.f, a1 = 0.f;
  for (int p = ia[node] + 1; p < ia[node + 1]; ++p) {
    const float wv = w[p];
    const float2 h = reinterpret_cast<const float2 *>(H + (size_t)ja[p] * kH)[lane];
    a0 = fmaf(wv, h.x, a0);
    a1 = fmaf(wv, h.y, a1);
  }
  reinterpret_cast<float2 *>(A + (size_t)node * kH)[lane] = make_float2(a0, a1);
  if (Abf) reinterpret_cast<__nv_bfloat162 *>(Abf + (size_t)node * kH)[lane] = __floats2bfloat162_rn(a0, a1);
}

// Edge weights S_ij = c_ij / sqrt(d_i d_j) from the assembled matrix.
__global__ void k_edge_deg(int n, const int *__restrict__ ia, const double *__restrict__ amat,
                           float *__restrict__ deg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int p = ia[i] + 1; p < ia[i + 1]; ++p) d += fmax(-amat[p], 0.0);
    deg[i] = (float)d;
  }
}
__global__ void k_edge_w(int n, const int *__restrict__ ia, const int *__restrict__ ja,
                         const double *__restrict__ amat, const float *__restrict__ deg,
                         float *__restrict__ w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    w[ia[i]] = 0.f;
    for (int p = ia[i] + 1; p < ia[i + 1]; ++p) {
      const float c = (float)fmax(-amat[p], 0.0);
      const float dd = deg[i] * deg[ja[p]];
      w[p] = dd > 0.f ? c * rsqrtf(dd) : 0.f;
    }
  }
}

__global__ void k_f32_to_bf16(long long n, const float *__restrict__ s, __nv_bfloat16 *__restrict__ d) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    d[i] = __float2bfloat16(s[i]);
}

// y = H wout + bout (one warp per node); optional loss and dy.
__global__ void k_readout(int n, const float *__restrict__ H, const float *__restrict__ wout,
                          const float *__restrict__ bout, float *__restrict__ y,
                          const float *__restrict__ target, const float *__restrict__ mask,
                          float inv_count, float *__restrict__ dy, float *__restrict__ loss) {
  const int node = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (node >= n) return;
  const float2 h = reinterpret_cast<const float2 *>(H + (size_t)node * kH)[lane];
  float s = h.x * wout[2 * lane] + h.y * wout[2 * lane + 1];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    const float yv = s + bout[0];
    y[node] = yv;
    if (target) {
      const float m = mask[node];
      const float e = (yv - target[node]) * m;
      dy[node] = 2.f * e * inv_count;
      atomicAdd(loss, e * e * inv_count);
    }
  }
}

// Readout backward: dH = dy wout^T (overwrites dH), dwout += H^T dy, dbout += sum dy.
__global__ void k_readout_bwd(int n, const float *__restrict__ H, const float *__restrict__ wout,
                              const float *__restrict__ dy, float *__restrict__ dH,
                              float *__restrict__ dwout, float *__restrict__ dbout) {
  __shared__ float sw[kH];
  __shared__ float sb;
  if (threadIdx.x < kH) sw[threadIdx.x] = 0.f;
  if (threadIdx.x == 0) sb = 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  float g0 = 0.f, g1 = 0.f, gb = 0.f;
  for (int node = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; node < n; node += warps) {
    const float d = dy[node];
    const float2 h = reinterpret_cast<const float2 *>(H + (size_t)node * kH)[lane];
    reinterpret_cast<float2 *>(dH + (size_t)node * kH)[lane] =
        make_float2(d * wout[2 * lane], d * wout[2 * lane + 1]);
    g0 = fmaf(d, h.x, g0);
    g1 = fmaf(d, h.y, g1);
    if (lane == 0) gb += d;
  }
  atomicAdd(&sw[2 * lane], g0);
  atomicAdd(&sw[2 * lane + 1], g1);
  if (lane == 0) atomicAdd(&sb, gb);
  __syncthreads();
  if (threadIdx.x < kH) atomicAdd(&dwout[threadIdx.x], sw[threadIdx.x]);
  if (threadIdx.x == 0) atomicAdd(dbout, sb);
}

// dZ = dH (x) mask, as BF16 for the GEMMs, and the bias gradient db += sum dZ.
__global__ void k_relu_bwd(int n, const float *__restrict__ dH,
                           const unsigned char *__restrict__ mask, __nv_bfloat16 *__restrict__ dZ,
                           float *__restrict__ db) {
  __shared__ float sb[kH];
  if (threadIdx.x < kH) sb[threadIdx.x] = 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  float b0 = 0.f, b1 = 0.f;
  for (int node = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; node < n; node += warps) {
    const size_t o = (size_t)node * kH + 2 * lane;
    const float d0 = mask[o] ? dH[o] : 0.f, d1 = mask[o + 1] ? dH[o + 1] : 0.f;
    reinterpret_cast<__nv_bfloat162 *>(dZ)[o / 2] = __floats2bfloat162_rn(d0, d1);
    b0 += d0;
    b1 += d1;
  }
  atomicAdd(&sb[2 * lane], b0);
  atomicAdd(&sb[2 * lane + 1], b1);
  __syncthreads();
  if (threadIdx.x < kH) atomicAdd(&db[threadIdx.x], sb[threadIdx.x]);
}

// dH_prev = dH (residual) + dXcat[:, :64] + S dXcat[:, 64:]
__global__ void k_layer_bwd_combine(int n, const int *__restrict__ ia, const int *__restrict__ ja,
                                    const float *__restrict__ w, const float *__restrict__ dH,
                                    const float *__restrict__ dX, float *__restrict__ dHprev) {
  const int node = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (node >= n) return;
  float a0 = 0.f, a1 = 0.f;
  for (int p = ia[node] + 1; p < ia[node + 1]; ++p) {
    const float wv = w[p];
    const float2 d = reinterpret_cast<const float2 *>(dX + (size_t)ja[p] * kCat + kH)[lane];
    a0 = fmaf(wv, d.x, a0);
    a1 = fmaf(wv, d.y, a1);
  }
  const float2 r = reinterpret_cast<const float2 *>(dH + (size_t)node * kH)[lane];
  const float2 x = reinterpret_cast<const float2 *>(dX + (size_t)node * kCat)[lane];
  reinterpret_cast<float2 *>(dHprev + (size_t)node * kH)[lane] =
      make_float2(r.x + x.x + a0, r.y + x.y + a1);
}

// Adam (bias-corrected), FP32 master weights.
__global__ void k_adam(int n, float *__restrict__ p, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr, float b1, float b2,
                       float c1, float c2, float eps) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// W (K x N, FP32 master) -> Bt (N x K, BF16) for the forward GEMM and
// Wbf (K x N, BF16) for the backward one.
__global__ void k_weights_bf16(int K, int N, const float *__restrict__ W, __nv_bfloat16 *__restrict__ Bt,
                               __nv_bfloat16 *__restrict__ Wbf) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < K * N; e += gridDim.x * blockDim.x) {
    const int k = e / N, c = e % N;
    const __nv_bfloat16 v = __float2bfloat16(W[e]);
    Bt[c * K + k] = v;
    Wbf[e] = v;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Parameter layout (FP32): W0 (kIn x kH), b0 (kH), then per layer
// W_l (kCat x kH), b_l (kH), then wout (kH), bout (1).
struct MpnnLayout {
  static constexpr long long w0 = 0, b0 = w0 + kIn * kH;
  static constexpr long long layer0 = b0 + kH, layer_sz = kCat * kH + kH;
  static constexpr long long wout = layer0 + kL * layer_sz, bout = wout + kH;
  static constexpr long long total = bout + 1;
  static constexpr long long W(int l) { return layer0 + (l - 1) * layer_sz; }
  static constexpr long long B(int l) { return W(l) + kCat * kH; }
};

long long mpnn_param_count() { return MpnnLayout::total; }

static int ngrid(long long work, int block) {
  return (int)std::max<long long>(1, std::min<long long>((work + block - 1) / block, 16LL * gb::kNumSM));
}

void mpnn_set_graph(MpnnDev &D, const double *d_amat, cudaStream_t st) {
  k_edge_deg<<<ngrid(D.n, 256), 256, 0, st>>>(D.n, D.ia, d_amat, D.deg);
  k_edge_w<<<ngrid(D.n, 256), 256, 0, st>>>(D.n, D.ia, D.ja, d_amat, D.deg, D.w);
  if (D.amat) cudaMemcpyAsync(D.amat, d_amat, sizeof(double) * D.nja, cudaMemcpyDeviceToDevice, st);
}

// ---- energy loss (mode 1) ----
// e = mask*(dh(y) - dh(t)), tt = mask*dh(t) in head units, dh(u) = soft*sinh(u*scale).
__global__ void k_energy_err(int n, const float *__restrict__ y, const float *__restrict__ t,
                             const float *__restrict__ mask, double soft, double scale,
                             double *__restrict__ ee, double *__restrict__ tt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double m = mask[i] > 0.f ? 1.0 : 0.0;
    const double dt = soft * sinh((double)t[i] * scale);
    const double dy = soft * sinh((double)y[i] * scale);
    ee[i] = m * (dy - dt);
    tt[i] = m * dt;
  }
}

// we = -A e over the active rows, and per-block partials of e'(-A e) and
// t'(-A t) (epart[2b], epart[2b+1]).
__global__ void k_energy_dots(int n, const int *__restrict__ ia, const int *__restrict__ ja,
                              const double *__restrict__ amat, const float *__restrict__ mask,
                              const double *__restrict__ ee, const double *__restrict__ tt,
                              double *__restrict__ we, double *__restrict__ epart) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double ae = 0.0, at = 0.0;
    if (mask[i] > 0.f) {
      for (int k = ia[i]; k < ia[i + 1]; ++k) {
        const int j = ja[k];
        ae = fma(-amat[k], ee[j], ae);
        at = fma(-amat[k], tt[j], at);
      }
    }
    we[i] = ae;
    s1 = fma(ee[i], ae, s1);
    s2 = fma(tt[i], at, s2);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  __shared__ double sh[2][32];
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = s1;
    sh[1][threadIdx.x >> 5] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += sh[0][w];
      b += sh[1][w];
    }
    epart[2 * blockIdx.x] = a;
    epart[2 * blockIdx.x + 1] = b;
  }
}

// dy += 2 (W e)_i / t'Wt * dh'(y_i) on active cells and loss += e'We / t'Wt,
// the partials summed in block order by every block.
__global__ void k_energy_grad(int n, int G, const double *__restrict__ epart,
                              const double *__restrict__ we, const float *__restrict__ y,
                              const float *__restrict__ mask, double soft, double scale,
                              float *__restrict__ dy, float *__restrict__ loss) {
  __shared__ double s_inv;
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int q = 0; q < G; ++q) {
      a += epart[2 * q];
      b += epart[2 * q + 1];
    }
    s_inv = (b > 0.0) ? 1.0 / b : 0.0;
    if (blockIdx.x == 0) atomicAdd(loss, (float)(a * s_inv));
  }
  __syncthreads();
  const double inv = s_inv;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!(mask[i] > 0.f)) continue;
    const double d = soft * scale * cosh((double)y[i] * scale);
    dy[i] += (float)(2.0 * we[i] * inv * d);
  }
}

void mpnn_refresh_bf16(MpnnDev &D, cudaStream_t st) {
  using P = MpnnLayout;
  k_weights_bf16<<<ngrid(kIn * kH, 256), 256, 0, st>>>(kIn, kH, D.p + P::w0, D.bt0, D.wbf0);
  for (int l = 1; l <= kL; ++l)
    k_weights_bf16<<<ngrid(kCat * kH, 256), 256, 0, st>>>(kCat, kH, D.p + P::W(l), D.bt[l - 1],
                                                          D.wbf[l - 1]);
}

// The network's input for a warm-start guess, written as BF16: the static
// columns of `stat` (n x kIn: standardised ln K, well rate, CHD mask, layer
// position, bias), column 1 the previous heads (x - head_ref) / head_scale,
// column 6 the previous step's head change in network units
// asinh(dh / dh_soft) / dh_scale (zero on the first step and on inactive
// cells).
__global__ void k_guess_features(int n, const float *__restrict__ stat, const double *__restrict__ x,
                                 const double *__restrict__ xold, int first,
                                 const int *__restrict__ ibound, GuessScaling sc,
                                 __nv_bfloat16 *__restrict__ xbf) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)n * kIn;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q / kIn), f = (int)(q % kIn);
    float v;
    if (f == 1) {
      v = (float)((x[i] - sc.head_ref) / sc.head_scale);
    } else if (f == 6) {
      const double dh = (first || ibound[i] <= 0) ? 0.0 : x[i] - xold[i];
      v = (float)(asinh(dh / sc.dh_soft) / sc.dh_scale);
    } else {
      v = stat[q];
    }
    xbf[q] = __float2bfloat16(v);
  }
}

// guess = x + sinh(clamp(y) * dh_scale) * dh_soft on active cells, x elsewhere
__global__ void k_guess_out(int n, const float *__restrict__ y, const double *__restrict__ x,
                            const int *__restrict__ ibound, GuessScaling sc,
                            double *__restrict__ guess) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double u = (double)y[i];
    if (sc.unit_max > 0.0) u = fmin(fmax(u, -sc.unit_max), sc.unit_max);
    const double dh = sinh(u * sc.dh_scale) * sc.dh_soft;
    guess[i] = (ibound[i] > 0) ? x[i] + dh : x[i];
  }
}

static void forward_from_xbf(MpnnDev &D, const float *target, const float *mask, float inv_count,
                             cudaStream_t st);

void mpnn_guess(MpnnDev &D, const float *d_static, const double *x, const double *xold,
                int first, const int *ibound, const GuessScaling &sc, double *guess,
                cudaStream_t st) {
  const int n = D.n;
  k_guess_features<<<ngrid((long long)n * kIn, 256), 256, 0, st>>>(n, d_static, x, xold, first,
                                                                    ibound, sc, D.xbf);
  forward_from_xbf(D, nullptr, nullptr, 0.f, st);
  k_guess_out<<<ngrid(n, 256), 256, 0, st>>>(n, D.y, x, ibound, sc, guess);
}

// Forward pass from features (N x kIn FP32); y (N) written.  With a target,
// the loss and dy are produced too.
void mpnn_forward(MpnnDev &D, const float *d_x, const float *target, const float *mask,
                  float inv_count, cudaStream_t st) {
  const int n = D.n;
  k_f32_to_bf16<<<ngrid((long long)n * kIn, 256), 256, 0, st>>>((long long)n * kIn, d_x, D.xbf);
  forward_from_xbf(D, target, mask, inv_count, st);
}

static void forward_from_xbf(MpnnDev &D, const float *target, const float *mask, float inv_count,
                             cudaStream_t st) {
  using P = MpnnLayout;
  const int n = D.n;
  const int gb = (n + 63) / 64;
  k_gemm_rows<kIn, 0, kH, 1><<<gb, 128, 0, st>>>(n, D.xbf, nullptr, D.bt0, D.p + P::b0, nullptr,
                                                  D.H[0], D.Hbf[0], D.mask[0]);
  const int ga = (int)(((long long)n * 32 + 255) / 256);
  for (int l = 1; l <= kL; ++l) {
    k_aggregate<<<ga, 256, 0, st>>>(n, D.ia, D.ja, D.w, D.H[l - 1], D.A, D.Abf[l]);
    k_gemm_rows<kH, kH, kH, 2><<<gb, 128, 0, st>>>(n, D.Hbf[l - 1], D.Abf[l], D.bt[l - 1],
                                                    D.p + P::B(l), D.H[l - 1], D.H[l], D.Hbf[l],
                                                    D.mask[l]);
  }
  if (target) cudaMemsetAsync(D.loss, 0, sizeof(float), st);
  const bool energy = target && D.energy;
  k_readout<<<ga, 256, 0, st>>>(n, D.H[kL], D.p + P::wout, D.p + P::bout, D.y, target, mask,
                                energy ? inv_count * D.mse_w : inv_count, D.dy, D.loss);
  if (energy) {
    const int G = std::min(kMpnnRedBlocks, (n + 255) / 256);
    k_energy_err<<<ngrid(n, 256), 256, 0, st>>>(n, D.y, target, mask, D.dh_soft, D.dh_scale, D.ee, D.tt);
    k_energy_dots<<<G, 256, 0, st>>>(n, D.ia, D.ja, D.amat, mask, D.ee, D.tt, D.we, D.epart);
    k_energy_grad<<<ngrid(n, 256), 256, 0, st>>>(n, G, D.epart, D.we, D.y, mask, D.dh_soft,
                                                 D.dh_scale, D.dy, D.loss);
  }
}

// Backward pass after mpnn_forward with a target: gradients into D.g.
void mpnn_backward(MpnnDev &D, cudaStream_t st) {
  using P = MpnnLayout;
  const int n = D.n;
  const int ga = (int)(((long long)n * 32 + 255) / 256);
  const int gr = ngrid((long long)n * 32, 256);
  const int gb = (n + 63) / 64;
  const int gc = (n + 63) / 64;
  cudaMemsetAsync(D.g, 0, sizeof(float) * P::total, st);
  k_readout_bwd<<<gr, 256, 0, st>>>(n, D.H[kL], D.p + P::wout, D.dy, D.dH, D.g + P::wout,
                                    D.g + P::bout);
  for (int l = kL; l >= 1; --l) {
    k_relu_bwd<<<gr, 256, 0, st>>>(n, D.dH, D.mask[l], D.dZ, D.g + P::B(l));
    // dW_l = [H_{l-1}, A_l]^T dZ
    k_gemm_xtdz<kH, kH, kH><<<gc, 128, 0, st>>>(n, D.Hbf[l - 1], D.Abf[l], D.dZ, D.g + P::W(l));
    // d[H_{l-1}, A_l] = dZ W_l^T  (W_l as BF16, kCat x kH; transposed use: Bt = W_l)
    k_gemm_rows<kH, 0, kCat, 0><<<gb, 128, 0, st>>>(n, D.dZ, nullptr, D.wbf[l - 1], nullptr,
                                                     nullptr, D.dX, nullptr, nullptr);
    k_layer_bwd_combine<<<ga, 256, 0, st>>>(n, D.ia, D.ja, D.w, D.dH, D.dX, D.dHp);
    std::swap(D.dH, D.dHp);
  }
  k_relu_bwd<<<gr, 256, 0, st>>>(n, D.dH, D.mask[0], D.dZ, D.g + P::b0);
  k_gemm_xtdz<kIn, 0, kH><<<gc, 128, 0, st>>>(n, D.xbf, nullptr, D.dZ, D.g + P::w0);
}

void mpnn_adam(MpnnDev &D, float lr, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  D.steps += 1;
  const float c1 = 1.f - powf(b1, (float)D.steps), c2 = 1.f - powf(b2, (float)D.steps);
  k_adam<<<ngrid(MpnnLayout::total, 256), 256, 0, st>>>((int)MpnnLayout::total, D.p, D.g, D.m, D.v,
                                                        lr, b1, b2, c1, c2, 1e-8f);
  mpnn_refresh_bf16(D, st);
}

}  // namespace gb
