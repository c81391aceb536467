// gbsln_api.cu -- NPF fill and the device-resident solution (C ABI).
//
// gbnpf_*: the NPF package's fill (npf_cf/npf_fc/npf_fn, gwf-npf.f90:444-698)
//          on caller-owned device arrays.
// gbsln_*: one GWF DIS model and its NumericalSolution outer loop
//          (NumericalSolution.f90:1482-1837) with x, amat and rhs resident in
//          HBM: prepareSolve (gwf_ad, chd_ad), sln_buildsystem (the fill),
//          sln_calc_ptc, sln_ls (fix-ups, pseudo-transient continuation, IMS
//          apply), sln_get_dxmax, sln_underrelax and npf_nur.  The host only
//          reads back a few scalars per outer iteration.
#include "gbims_internal.cuh"
#include "k_gwf.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

using namespace gb;

namespace {

template <typename T>
cudaError_t up(T **d, const T *h, size_t n) {
  *d = nullptr;
  cudaError_t e = cudaMalloc((void **)d, sizeof(T) * std::max<size_t>(n, 1));
  if (e != cudaSuccess || n == 0 || !h) return e;
  return cudaMemcpy(*d, h, sizeof(T) * n, cudaMemcpyHostToDevice);
}

// Full-grid DIS connectivity (Connections.f90:463-698 with the JA sort of
// Sparse.f90:217-239 and fillisym/filljas :1205-1268), 0-based.
struct Conn {
  std::vector<int> ia, ja, isym, jas, ihc;
  std::vector<double> cl1, cl2, hwva;
  int njas = 0;
};

void build_connections(int nlay, int nrow, int ncol, const double *delr, const double *delc,
                       const std::vector<double> &top, const std::vector<double> &bot, Conn &c) {
  const long long nrc = (long long)nrow * ncol;
  const int n = (int)(nlay * nrc);
  c.ia.assign(n + 1, 0);
  c.ja.clear();
  c.ja.reserve((size_t)n * 7);
  for (int k = 0; k < nlay; ++k)
    for (int i = 0; i < nrow; ++i)
      for (int j = 0; j < ncol; ++j) {
        int p = (int)(j + (long long)i * ncol + k * nrc);
        c.ia[p] = (int)c.ja.size();
        c.ja.push_back(p);
        if (k > 0) c.ja.push_back((int)(p - nrc));
        if (i > 0) c.ja.push_back(p - ncol);
        if (j > 0) c.ja.push_back(p - 1);
        if (j < ncol - 1) c.ja.push_back(p + 1);
        if (i < nrow - 1) c.ja.push_back(p + ncol);
        if (k < nlay - 1) c.ja.push_back((int)(p + nrc));
      }
  c.ia[n] = (int)c.ja.size();
  const size_t nja = c.ja.size();
  c.isym.assign(nja, -1);
  c.jas.assign(nja, -1);
  for (int p = 0; p < n; ++p)
    for (int q = c.ia[p]; q < c.ia[p + 1]; ++q) {
      int m = c.ja[q];
      if (m == p) { c.isym[q] = q; continue; }
      for (int r = c.ia[m]; r < c.ia[m + 1]; ++r)
        if (c.ja[r] == p) { c.isym[q] = r; break; }
    }
  int ipos = 0;
  for (int p = 0; p < n; ++p)
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q)
      if (c.ja[q] > p) c.jas[q] = ipos++;
  for (int p = 0; p < n; ++p)
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q)
      if (c.ja[q] < p) c.jas[q] = c.jas[c.isym[q]];
  c.njas = ipos;
  c.ihc.assign(ipos, 0);
  c.cl1.assign(ipos, 0.0);
  c.cl2.assign(ipos, 0.0);
  c.hwva.assign(ipos, 0.0);
  int s = 0;
  for (int k = 0; k < nlay; ++k)
    for (int i = 0; i < nrow; ++i)
      for (int j = 0; j < ncol; ++j) {
        long long p = j + (long long)i * ncol + k * nrc;
        if (j < ncol - 1) { c.ihc[s] = 1; c.cl1[s] = 0.5 * delr[j]; c.cl2[s] = 0.5 * delr[j + 1]; c.hwva[s] = delc[i]; ++s; }
        if (i < nrow - 1) { c.ihc[s] = 1; c.cl1[s] = 0.5 * delc[i]; c.cl2[s] = 0.5 * delc[i + 1]; c.hwva[s] = delr[j]; ++s; }
        if (k < nlay - 1) {
          long long m = p + nrc;
          c.ihc[s] = 0; c.cl1[s] = 0.5 * (top[p] - bot[p]); c.cl2[s] = 0.5 * (top[m] - bot[m]);
          c.hwva[s] = delr[j] * delc[i]; ++s;
        }
      }
}

struct NpfStore {
  int *ia = nullptr, *ja = nullptr, *jas = nullptr, *isym = nullptr, *ihc = nullptr, *icelltype = nullptr;
  double *cl1 = nullptr, *cl2 = nullptr, *hwva = nullptr, *top = nullptr, *bot = nullptr,
         *k11 = nullptr, *k33 = nullptr, *condsat = nullptr, *sat = nullptr;
  NpfDev view() const {
    NpfDev g;
    g.ia = ia; g.ja = ja; g.jas = jas; g.isym = isym; g.ihc = ihc;
    g.cl1 = cl1; g.cl2 = cl2; g.hwva = hwva; g.top = top; g.bot = bot; g.k11 = k11; g.k33 = k33;
    g.icelltype = icelltype;
    g.inewton = 0; g.ivarcv = 0; g.idewatcv = 0; g.icellavg = 0; g.satomega = 1.0e-6;
    return g;
  }
  void release() {
    void *p[] = {ia, ja, jas, isym, ihc, icelltype, cl1, cl2, hwva, top, bot, k11, k33, condsat, sat};
    for (void *q : p)
      if (q) cudaFree(q);
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// gbnpf
// ---------------------------------------------------------------------------
struct gbnpf_handle {
  gbnpf_options o{};
  int nodes = 0, nja = 0, njas = 0;
  NpfStore d;
  NpfDev g{};
  int *zero_ptr = nullptr;  // nodes+1 zeros: empty boundary lists
  cudaStream_t st = nullptr;
  std::string err;
};

extern "C" int gbnpf_create(const gbnpf_options *opt, int nodes, int nja, int njas, const int *ia,
                            const int *ja, const int *jas, const int *isym, const int *ihc,
                            const double *cl1, const double *cl2, const double *hwva,
                            const double *top, const double *bot, const double *k11,
                            const double *k33, const int *icelltype, gbnpf_handle **out) {
  if (!out) return GBIMS_ERR_ARG;
  *out = nullptr;
  if (!opt || nodes <= 0 || nja < nodes || njas < 0 || !ia || !ja || !jas || !isym || !ihc ||
      !cl1 || !cl2 || !hwva || !top || !bot || !k11 || !k33 || !icelltype)
    return GBIMS_ERR_ARG;
  if (opt->index_base != 0 && opt->index_base != 1) return GBIMS_ERR_ARG;
  gbnpf_handle *h = new (std::nothrow) gbnpf_handle();
  if (!h) return GBIMS_ERR_NOMEM;
  *out = h;
  h->o = *opt;
  h->nodes = nodes;
  h->nja = nja;
  h->njas = njas;
  int b = opt->index_base;
  std::vector<int> ia0(ia, ia + nodes + 1), ja0(ja, ja + nja), jas0(jas, jas + nja), isym0(isym, isym + nja);
  for (auto &v : ia0) v -= b;
  for (auto &v : ja0) v -= b;
  for (auto &v : jas0) v -= b;  // the diagonal's 0 (Fortran) becomes -1
  for (auto &v : isym0) v -= b;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (x != cudaSuccess && e == cudaSuccess) e = x; };
  chk(up(&h->d.ia, ia0.data(), ia0.size()));
  chk(up(&h->d.ja, ja0.data(), ja0.size()));
  chk(up(&h->d.jas, jas0.data(), jas0.size()));
  chk(up(&h->d.isym, isym0.data(), isym0.size()));
  chk(up(&h->d.ihc, ihc, (size_t)njas));
  chk(up(&h->d.cl1, cl1, (size_t)njas));
  chk(up(&h->d.cl2, cl2, (size_t)njas));
  chk(up(&h->d.hwva, hwva, (size_t)njas));
  chk(up(&h->d.top, top, (size_t)nodes));
  chk(up(&h->d.bot, bot, (size_t)nodes));
  chk(up(&h->d.k11, k11, (size_t)nodes));
  chk(up(&h->d.k33, k33, (size_t)nodes));
  chk(up(&h->d.icelltype, icelltype, (size_t)nodes));
  chk(up<double>(&h->d.condsat, nullptr, (size_t)njas));
  chk(up<double>(&h->d.sat, nullptr, (size_t)nodes));
  chk(up<int>(&h->zero_ptr, nullptr, (size_t)nodes + 1));
  if (h->zero_ptr) chk(cudaMemset(h->zero_ptr, 0, sizeof(int) * (nodes + 1)));
  chk(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  if (e != cudaSuccess) {
    h->err = cudaGetErrorString(e);
    return GBIMS_ERR_CUDA;
  }
  h->g = h->d.view();
  h->g.inewton = opt->inewton;
  h->g.ivarcv = opt->ivarcv;
  h->g.idewatcv = opt->idewatcv;
  h->g.icellavg = opt->icellavg;
  h->g.satomega = opt->satomega > 0 ? opt->satomega : 1.0e-6;
  {
    // npf_ar's initial saturation: 1 in every cell; npf_cf updates the
    // convertible ones (gwf-npf.f90:1853-1884)
    std::vector<double> one((size_t)nodes, 1.0);
    cudaMemcpy(h->d.sat, one.data(), sizeof(double) * nodes, cudaMemcpyHostToDevice);
  }
  gwf_condsat(nodes, h->g, h->d.condsat, h->st);
  e = cudaStreamSynchronize(h->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->err = cudaGetErrorString(e);
    return GBIMS_ERR_CUDA;
  }
  return GBIMS_OK;
}

extern "C" int gbnpf_fill(gbnpf_handle *h, const int *d_ibound, const double *d_hnew,
                          double *d_amat, double *d_rhs) {
  if (!h || !d_ibound || !d_hnew || !d_amat || !d_rhs) return GBIMS_ERR_ARG;
  // NPF terms only (with the Newton terms of a Newton model): no storage,
  // empty boundary lists
  FillDev f{};
  f.bnd_ptr = h->zero_ptr;
  gwf_npf_cf(h->nodes, h->g, d_ibound, d_hnew, h->d.sat, h->st);
  gwf_fill(h->nodes, h->g, f, d_ibound, d_hnew, d_hnew, h->d.sat, h->d.condsat, d_amat, d_rhs, h->st);
  cudaError_t e = cudaStreamSynchronize(h->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->err = cudaGetErrorString(e);
    return GBIMS_ERR_CUDA;
  }
  return GBIMS_OK;
}

extern "C" int gbnpf_get_condsat(gbnpf_handle *h, double *condsat) {
  if (!h || !condsat) return GBIMS_ERR_ARG;
  if (cudaMemcpy(condsat, h->d.condsat, sizeof(double) * h->njas, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GBIMS_ERR_CUDA;
  return GBIMS_OK;
}

extern "C" int gbnpf_destroy(gbnpf_handle *h) {
  if (!h) return GBIMS_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  h->d.release();
  if (h->zero_ptr) cudaFree(h->zero_ptr);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return GBIMS_OK;
}

// ---------------------------------------------------------------------------
// gbsln
// ---------------------------------------------------------------------------
struct gbsln_handle {
  int nlay = 0, nrow = 0, ncol = 0, n = 0, nja = 0;
  gbsln_nonlinear nl{};
  bool inewtonur = false;  // NEWTON UNDER_RELAXATION
  gbims_settings ims_s{};
  NpfStore d;
  NpfDev g{};
  double *strt = nullptr;  // initial heads (IC STRT), kept for gbsln_restart
  double *ss = nullptr, *sy = nullptr, *area = nullptr, *vol = nullptr, *xold = nullptr,
         *xtemp = nullptr, *wsave = nullptr, *hchold = nullptr, *deold = nullptr,
         *dxold = nullptr, *part = nullptr, *bnd_val = nullptr, *chd_head = nullptr;
  int *ibound = nullptr, *bnd_ptr = nullptr, *chd_node = nullptr, *flag = nullptr;
  int *bnd_kind = nullptr;  // per boundary entry: 0 WEL, 1 RCH
  int *ibotnode = nullptr;  // NEWTON UNDER_RELAXATION: the lowest cell below each cell
  // the matrix pattern: the model's connections, or with XT3D the wider one
  const int *s_ia = nullptr, *s_ja = nullptr;
  Xt3dDev xt{};             // XT3D on the device (xt.on 0: off)
  int njas = 0;
  int nja_m = 0;            // the model's connections (FLOW-JA-FACE entries)
  // boundary entries in bnd_ptr order: their package list index and kind
  std::vector<int> bnd_list, bnd_kind_h, chd_node_h;
  int nwel = 0, nrch = 0;
  void *xt_mem[16] = {};    // XT3D device arrays, freed by gbsln_destroy
  double *galpha = nullptr; // the last warm step's projection factors (2)
  double *dprev = nullptr;  // the last step's head change (valid when have_prev)
  double *gpart = nullptr;  // projection partials (5 per block)
  bool have_prev = false;
  double *bpart = nullptr;  // budget partials (kGwfBudgetSlots per block)
  int nchd = 0, G = 1;
  bool has_sto = false;
  double last_delt = 0.0;   // the last time step (or formulate) the budget refers to
  gbims_handle *ims = nullptr;
  double *amat = nullptr, *rhs = nullptr, *x = nullptr;  // inside the IMS handle
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  // outer-loop state
  double bigch = 0, bigchold = 0, relaxold = 0, l2norm0_ptc = 0, ptcdel = 0;
  double res_prev = 0, res_new = 0;  // backtracking residual norms
  std::vector<double> hpart;
  std::string err;
};

#define SLN_CUDA(h, call)                                                   \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      (h)->err = std::string(#call) + ": " + cudaGetErrorString(e_);        \
      return GBIMS_ERR_CUDA;                                                \
    }                                                                       \
  } while (0)

// Warm start: the first outer iterate of active cells from a guess.
__global__ void k_apply_guess(int n, const int *__restrict__ ibound, const double *__restrict__ guess,
                              double *__restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (ibound[i] > 0) x[i] = guess[i];
}

// Energy projection of the first iterate (no counterpart in the
// reference).  With d1 = the previous step's head change (zero when there
// is none), d2 = guess - xold (zero without a guess), both zero off the
// active cells, and r = rhs - A*xold, the per-block partials (part[5b..])
// of d1.r, d2.r, d1.(A d1), d1.(A d2), d2.(A d2).  For the symmetric
// (negative definite) GWF matrix, x0 = xold + a1*d1 + a2*d2 with
// (a1, a2) = (D'AD)^-1 D'r is the point of the plane through xold spanned
// by d1 and d2 closest to the solution in the energy norm: never farther
// from it than the previous heads, nor than the better of the two
// directions alone.
__global__ void k_guess_dots(int n, const int *__restrict__ ia, const int *__restrict__ ja,
                             const double *__restrict__ amat, const double *__restrict__ rhs,
                             const int *__restrict__ ibound, const double *__restrict__ dprev,
                             const double *__restrict__ guess, const double *__restrict__ xold,
                             double *part) {
  double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (ibound[i] < 1) continue;
    double ax = 0.0, a1 = 0.0, a2 = 0.0;
    for (int k = ia[i]; k < ia[i + 1]; ++k) {
      const int j = ja[k];
      const double xj = xold[j];
      const bool act = ibound[j] > 0;
      const double d1 = (act && dprev) ? dprev[j] : 0.0;
      const double d2 = (act && guess) ? guess[j] - xj : 0.0;
      ax = fma(amat[k], xj, ax);
      a1 = fma(amat[k], d1, a1);
      a2 = fma(amat[k], d2, a2);
    }
    const double r = rhs[i] - ax;
    const double d1 = dprev ? dprev[i] : 0.0;
    const double d2 = guess ? guess[i] - xold[i] : 0.0;
    s[0] = fma(d1, r, s[0]);
    s[1] = fma(d2, r, s[1]);
    s[2] = fma(d1, a1, s[2]);
    s[3] = fma(d1, a2, s[3]);
    s[4] = fma(d2, a2, s[4]);
  }
  __shared__ double sh[5][32];
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    double v = s[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[q][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double a = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += sh[threadIdx.x][w];
    part[5 * blockIdx.x + threadIdx.x] = a;
  }
}

// The 2x2 projection from the G blocks' partials, summed in block order by
// every block (the same factors everywhere): the plane when its Gram matrix
// is well conditioned, else the better single direction; factors that are
// not finite, or beyond +-4, give the previous heads.  Then
// x = xold + a1*d1 + a2*d2 on active cells; block 0 writes (a1, a2).
__global__ void k_guess_blend(int n, int G, const double *__restrict__ part,
                              const int *__restrict__ ibound, const double *__restrict__ dprev,
                              const double *__restrict__ guess, const double *__restrict__ xold,
                              double *__restrict__ x, double *alpha_out) {
  __shared__ double s_a1, s_a2;
  if (threadIdx.x == 0) {
    double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int q = 0; q < G; ++q)
      for (int c = 0; c < 5; ++c) t[c] += part[5 * q + c];
    const double b1 = t[0], b2 = t[1], m11 = t[2], m12 = t[3], m22 = t[4];
    double a1 = 0.0, a2 = 0.0;
    const double det = m11 * m22 - m12 * m12;
    if (m11 != 0.0 && m22 != 0.0 && det > 1e-10 * m11 * m22) {
      a1 = (m22 * b1 - m12 * b2) / det;
      a2 = (m11 * b2 - m12 * b1) / det;
    } else {
      // one direction: the one that removes more energy (b^2/|m|)
      const double g1 = (m11 != 0.0) ? b1 * b1 / fabs(m11) : 0.0;
      const double g2 = (m22 != 0.0) ? b2 * b2 / fabs(m22) : 0.0;
      if (g1 >= g2 && m11 != 0.0) a1 = b1 / m11;
      else if (m22 != 0.0) a2 = b2 / m22;
    }
    if (!(fabs(a1) <= 4.0) || !(fabs(a2) <= 4.0)) a1 = a2 = 0.0;
    s_a1 = a1;
    s_a2 = a2;
    if (blockIdx.x == 0) {
      alpha_out[0] = a1;
      alpha_out[1] = a2;
    }
  }
  __syncthreads();
  const double a1 = s_a1, a2 = s_a2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (ibound[i] < 1) continue;
    double v = xold[i];
    if (dprev) v = fma(a1, dprev[i], v);
    if (guess) v = fma(a2, guess[i] - xold[i], v);
    x[i] = v;
  }
}

// The head change of the step just taken (x - xold) on active cells, zero
// elsewhere: the first direction of the next warm step's projection.
__global__ void k_prev_change(int n, const int *__restrict__ ibound, const double *__restrict__ x,
                              const double *__restrict__ xold, double *__restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    d[i] = (ibound[i] > 0) ? x[i] - xold[i] : 0.0;
}

__global__ void k_set_chd(int nchd, const int *__restrict__ node, const double *__restrict__ head,
                          double *x, double *xold) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nchd) {
    x[node[i]] = head[i];
    xold[node[i]] = head[i];
  }
}

namespace {

// The lowest cell reached from each cell by following, from cell to cell,
// the vertical connection to a higher-numbered cell with the lowest bottom
// (gwf-npf.f90:1904-1939, the cell NEWTON UNDER_RELAXATION relaxes toward).
std::vector<int> bottom_nodes(int n, const Conn &c, const std::vector<double> &bot) {
  std::vector<int> ib(n);
  for (int p = 0; p < n; ++p) {
    double minbot = bot[p];
    int nn = p;
    for (;;) {
      int next = -1;
      for (int q = c.ia[nn] + 1; q < c.ia[nn + 1]; ++q) {
        const int m = c.ja[q];
        if (c.ihc[c.jas[q]] == 0 && m > nn && bot[m] < minbot) {
          next = m;
          minbot = bot[m];
        }
      }
      if (next < 0) break;
      nn = next;
    }
    ib[p] = nn;
  }
  return ib;
}

// Everything of gbsln_create after the grid: boundaries, device arrays,
// the IMS handle and the saturated conductances.
// XT3D setup on a full DIS grid (Xt3dInterface.f90: xt3d_ac :124-189 for
// the wider pattern, xt3d_mc :191-271 for the positions of the extended
// neighbours, xt3d_iallpc :1109-1179, xt3d_fillrmatck :1577-1613 and the
// tensor of xt3d_load :1230-1237; the DIS connection geometry of Dis.f90:
// 1039-1160).  Fills the solution pattern sia/sja and the host arrays of
// the device view.
struct Xt3dHost {
  std::vector<int> sia, sja, idxglo, iallpc, pair_n, pair_il0, pair_il10;
  std::vector<unsigned char> sflag;
  std::vector<double> ck, geo;
  int lamatsaved = 0, nozee = 0, vcentre = 0, rhsform = 0;
};

int xt3d_host(const gbsln_model *m, const gbsln_ktensor *xt, const gbsln_geometry *geom,
              const Conn &c, const std::vector<int> &ibound, Xt3dHost &o, std::string &err) {
  const int n = (int)c.ia.size() - 1;
  if ((xt->angle2 == nullptr) != (xt->angle3 == nullptr)) {
    err = "XT3D: ANGLE2 and ANGLE3 must be given both or neither";
    return GBIMS_ERR_ARG;
  }
  for (int p = 0; p < n; ++p)
    if (c.ia[p + 1] - c.ia[p] - 1 > kXtNb) {
      err = "XT3D: more neighbours per cell than supported";
      return GBIMS_ERR_UNSUPPORTED;
    }
  o.nozee = (xt->angle2 == nullptr) ? 1 : 0;
  // the tensor per cell, angles from degrees (DPIO180 = atan(1)/45)
  const double dpio180 = std::atan(1.0) / 45.0;
  o.ck.assign((size_t)9 * n, 0.0);
  for (int p = 0; p < n; ++p) {
    const double ang1 = xt->angle1 ? xt->angle1[p] * dpio180 : 0.0;
    const double ang2 = (!o.nozee) ? xt->angle2[p] * dpio180 : 0.0;
    const double ang3 = (!o.nozee) ? xt->angle3[p] * dpio180 : 0.0;
    const double s1 = std::sin(ang1), c1 = std::cos(ang1), s2 = std::sin(ang2), c2 = std::cos(ang2),
                 s3 = std::sin(ang3), c3 = std::cos(ang3);
    double r[3][3];
    r[0][0] = c1 * c2;
    r[0][1] = c1 * s2 * s3 - s1 * c3;
    r[0][2] = -c1 * s2 * c3 - s1 * s3;
    r[1][0] = s1 * c2;
    r[1][1] = s1 * s2 * s3 + c1 * c3;
    r[1][2] = -s1 * s2 * c3 + c1 * s3;
    r[2][0] = s2;
    r[2][1] = -c2 * s3;
    r[2][2] = c2 * c3;
    const double kd[3] = {m->k11[p], xt->k22 ? xt->k22[p] : m->k11[p], m->k33[p]};
    double t[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc = acc + r[i][k] * (k == j ? kd[k] : 0.0);
        t[i][j] = acc;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc = acc + t[i][k] * r[j][k];
        o.ck[(size_t)9 * p + 3 * i + j] = acc;
      }
  }
  // horizontal geometry of each connection n < m, from n to m and from m
  // to n: the displacement (x2 - x1, y2 - y1) and the face normal.  Right
  // neighbour (j+1): (ds, 0), (1, 0); back from it (left): (-ds, 0),
  // (-1, 0); front neighbour (i+1): (0, -ds), (0, -1); back from it:
  // (0, ds), (0, 1); ds = cl1 + cl2
  o.geo.assign((size_t)8 * c.njas, 0.0);
  if (geom) {
    // a grid given by its cell centres and face-normal angles (DISV
    // connection_normal/vector, Disv.f90:979-1080; DISU, Disu.f90:1062-1164):
    // the displacement between the centres (for DISU vertical connections
    // too) and the normal cos/sin(anglex) times +1 or -1
    for (int p = 0; p < n; ++p)
      for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q) {
        const int mm = c.ja[q], sidx = c.jas[q];
        if (mm < p) continue;
        if (c.ihc[sidx] == 0 && !geom->centre_vertical) continue;
        double *gg = &o.geo[(size_t)8 * sidx];
        gg[0] = geom->xc[mm] - geom->xc[p];
        gg[1] = geom->yc[mm] - geom->yc[p];
        gg[4] = geom->xc[p] - geom->xc[mm];
        gg[5] = geom->yc[p] - geom->yc[mm];
        if (c.ihc[sidx] != 0) {
          const double angle = geom->anglex[sidx];
          gg[2] = std::cos(angle) * 1.0;
          gg[3] = std::sin(angle) * 1.0;
          gg[6] = std::cos(angle) * -1.0;
          gg[7] = std::sin(angle) * -1.0;
        }
      }
    o.vcentre = geom->centre_vertical ? 1 : 0;
  }
  for (int p = 0; p < n && !geom; ++p)
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q) {
      const int mm = c.ja[q], sidx = c.jas[q];
      if (mm < p || c.ihc[sidx] == 0) continue;
      const double ds = c.cl1[sidx] + c.cl2[sidx];
      double *gg = &o.geo[(size_t)8 * sidx];
      if (mm == p + 1) {
        gg[0] = ds;
        gg[2] = 1.0;
        gg[4] = -ds;
        gg[6] = -1.0;
      } else {
        gg[1] = -ds;
        gg[3] = -1.0;
        gg[5] = ds;
        gg[7] = 1.0;
      }
    }
  // XT3D RHS: the model's own pattern (xt3d_ac adds nothing, :139)
  o.rhsform = (xt->xt3d == 2) ? 1 : 0;
  if (o.rhsform) {
    o.sia = c.ia;
    o.sja = c.ja;
    o.sflag.assign(c.ja.size(), 1);
    o.idxglo.resize(c.ja.size());
    for (size_t q = 0; q < c.ja.size(); ++q) o.idxglo[q] = (int)q;
  }
  // the solution pattern: each row the connections and the neighbours of
  // the neighbours, diagonal first, the rest ascending; flags 1 (a model
  // connection) and 2 (an extended neighbour, xt3d_ac)
  if (!o.rhsform) {
    o.sia.assign(n + 1, 0);
    o.sja.clear();
    o.sflag.clear();
    o.idxglo.assign(c.ja.size(), -1);
  }
  std::vector<int> row;
  for (int p = 0; p < n && !o.rhsform; ++p) {
    row.clear();
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q) {
      row.push_back(c.ja[q]);
      const int j = c.ja[q];
      for (int k = c.ia[j] + 1; k < c.ia[j + 1]; ++k) row.push_back(c.ja[k]);
    }
    std::sort(row.begin(), row.end());
    row.erase(std::unique(row.begin(), row.end()), row.end());
    row.erase(std::remove(row.begin(), row.end(), p), row.end());
    row.insert(row.begin(), p);
    if ((int)row.size() > kXtRow) {
      err = "XT3D: a matrix row is longer than supported";
      return GBIMS_ERR_UNSUPPORTED;
    }
    o.sia[p] = (int)o.sja.size();
    for (int col : row) {
      unsigned char f = 0;
      for (int q = c.ia[p]; q < c.ia[p + 1]; ++q)
        if (c.ja[q] == col) {
          f |= 1;
          o.idxglo[q] = (int)o.sja.size();
        }
      for (int q = c.ia[p] + 1; q < c.ia[p + 1] && !(f & 2); ++q) {
        const int j = c.ja[q];
        for (int k = c.ia[j] + 1; k < c.ia[j + 1]; ++k)
          if (c.ja[k] == col) {
            f |= 2;
            break;
          }
      }
      o.sja.push_back(col);
      o.sflag.push_back(f);
    }
  }
  if (!o.rhsform) o.sia[n] = (int)o.sja.size();
  // xt3d_iallpc: every cell the terms of whose connections never change
  o.iallpc.assign(n, 1);
  for (int p = 0; p < n; ++p) {
    if (m->icelltype[p] != 0) {
      o.iallpc[p] = 0;
      continue;
    }
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q) {
      const int mm = ibound[c.ja[q]] != 0 ? c.ja[q] : -1;
      if (mm < p) continue;
      if (m->icelltype[mm] != 0) {
        o.iallpc[p] = 0;
        o.iallpc[mm] = 0;
        continue;
      }
      for (int k = c.ia[mm] + 1; k < c.ia[mm + 1]; ++k) {
        const int qq = ibound[c.ja[k]] != 0 ? c.ja[k] : -1;
        if (qq >= 0 && m->icelltype[qq] != 0) {
          o.iallpc[p] = 0;
          o.iallpc[mm] = 0;
          o.iallpc[qq] = 0;
        }
      }
    }
  }
  o.lamatsaved = 0;
  for (int p = 0; p < n && !o.rhsform; ++p)
    if (o.iallpc[p] == 1) o.lamatsaved = 1;
  // each connection n < m: n, m's slot in n's row, n's slot in m's row
  o.pair_n.assign(c.njas, 0);
  o.pair_il0.assign(c.njas, 0);
  o.pair_il10.assign(c.njas, 0);
  for (int p = 0; p < n; ++p)
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q) {
      const int mm = c.ja[q];
      if (mm < p) continue;
      const int sidx = c.jas[q];
      o.pair_n[sidx] = p;
      o.pair_il0[sidx] = q - c.ia[p] - 1;
      o.pair_il10[sidx] = c.isym[q] - c.ia[mm] - 1;
    }
  return GBIMS_OK;
}

// hy_eff (gwf-npf.f90:2280-2357) with hyeff (HGeoUtil.f90:29-108) for every
// connection n < m, from n toward m and from m toward n.  The connection
// normal is DIS's (from the cells' rows and columns, Dis.f90:1039-1087) or,
// with a geometry, cos/sin of anglex flipped for the reverse direction
// (Disv.f90:979-1018, Disu.f90:1062-1102).
std::vector<double> npf_hy_host(const gbsln_model *m, const gbsln_ktensor *kt,
                                const gbsln_geometry *geom, const Conn &c, int nrow, int ncol) {
  const int n = (int)c.ia.size() - 1;
  const double dpio180 = std::atan(1.0) / 45.0;
  auto rad = [&](const double *a, int p) { return a ? a[p] * dpio180 : 0.0; };
  auto normal = [&](int a, int b, int ihc, int sidx, double v[3]) {
    v[0] = 0.0;
    v[1] = 0.0;
    v[2] = 0.0;
    if (ihc == 0) {
      v[2] = (b < a) ? 1.0 : -1.0;
    } else if (geom) {
      const double angle = geom->anglex[sidx];
      const double dmult = (b < a) ? -1.0 : 1.0;
      v[0] = std::cos(angle) * dmult;
      v[1] = std::sin(angle) * dmult;
    } else {
      const int nrc = nrow * ncol;
      const int ra = a % nrc, rb = b % nrc;
      const int i1 = ra / ncol, j1 = ra % ncol, i2 = rb / ncol, j2 = rb % ncol;
      if (i2 < i1) v[1] = 1.0;
      else if (j2 < j1) v[0] = -1.0;
      else if (j2 > j1) v[0] = 1.0;
      else v[1] = -1.0;
    }
  };
  auto hyeff = [&](double k11, double k22, double k33, double ang1, double ang2, double ang3,
                   const double *vg) {
    const double s1 = std::sin(ang1), c1 = std::cos(ang1), s2 = std::sin(ang2),
                 c2 = std::cos(ang2), s3 = std::sin(ang3), c3 = std::cos(ang3);
    double r[3][3];
    r[0][0] = c1 * c2;
    r[0][1] = c1 * s2 * s3 - s1 * c3;
    r[0][2] = -c1 * s2 * c3 - s1 * s3;
    r[1][0] = s1 * c2;
    r[1][1] = s1 * s2 * s3 + c1 * c3;
    r[1][2] = -s1 * s2 * c3 + c1 * s3;
    r[2][0] = s2;
    r[2][1] = -c2 * s3;
    r[2][2] = c2 * c3;
    const double ve1 = r[0][0] * vg[0] + r[1][0] * vg[1] + r[2][0] * vg[2];
    const double ve2 = r[0][1] * vg[0] + r[1][1] * vg[1] + r[2][1] * vg[2];
    const double ve3 = r[0][2] * vg[0] + r[1][2] * vg[1] + r[2][2] * vg[2];
    double k = 0.0;
    if (kt->iavgkeff == 0) {
      double dnum = 1.0, d1 = ve1 * ve1, d2 = ve2 * ve2, d3 = ve3 * ve3;
      if (ve1 != 0.0) { dnum = dnum * k11; d2 = d2 * k11; d3 = d3 * k11; }
      if (ve2 != 0.0) { dnum = dnum * k22; d1 = d1 * k22; d3 = d3 * k22; }
      if (ve3 != 0.0) { dnum = dnum * k33; d1 = d1 * k33; d2 = d2 * k33; }
      const double denom = d1 + d2 + d3;
      if (denom > 0.0) k = dnum / denom;
    } else if (kt->iavgkeff == 1) {
      k = ve1 * ve1 * k11 + ve2 * ve2 * k22 + ve3 * ve3 * k33;
    }
    return k;
  };
  auto hy_eff = [&](int a, int b, int ihc, int sidx) {
    const double hy11 = m->k11[a], hy22 = kt->k22 ? kt->k22[a] : m->k11[a], hy33 = m->k33[a];
    double v[3];
    if (ihc == 0) {
      if (!kt->angle2) return hy33;
      normal(a, b, ihc, sidx, v);
      return hyeff(hy11, hy22, hy33, rad(kt->angle1, a), rad(kt->angle2, a), rad(kt->angle3, a), v);
    }
    if (!kt->k22) return hy11;
    normal(a, b, ihc, sidx, v);
    double ang1 = 0.0, ang2 = 0.0, ang3 = 0.0;
    if (kt->angle1) {
      ang1 = rad(kt->angle1, a);
      if (kt->angle2) {
        ang2 = rad(kt->angle2, a);
        if (kt->angle3) ang3 = rad(kt->angle3, a);
      }
    }
    return hyeff(hy11, hy22, hy33, ang1, ang2, ang3, v);
  };
  std::vector<double> hy((size_t)2 * c.njas, 0.0);
  for (int p = 0; p < n; ++p)
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q) {
      const int mm = c.ja[q];
      if (mm < p) continue;
      const int sidx = c.jas[q];
      hy[2 * (size_t)sidx] = hy_eff(p, mm, c.ihc[sidx], sidx);
      hy[2 * (size_t)sidx + 1] = hy_eff(mm, p, c.ihc[sidx], sidx);
    }
  return hy;
}

int sln_setup(gbsln_handle *h, const gbsln_model *m, const gbnpf_options *npf, const double *strt,
              const Conn &c, const std::vector<double> &top, const std::vector<double> &bot,
              const std::vector<double> &area, const gbsln_ktensor *xt = nullptr,
              const gbsln_geometry *geom = nullptr) {
  const int n = h->n;
  std::vector<double> vol(n);
  for (int p = 0; p < n; ++p) vol[p] = area[p] * (top[p] - bot[p]);
  h->nja = (int)c.ja.size();
  h->nja_m = h->nja;
  h->njas = c.njas;
  std::vector<int> ibound(n, 1);
  for (int i = 0; i < m->nchd; ++i) {
    int node = m->chd_node[i];
    if (node < 0 || node >= n) { h->err = "CHD node out of range"; return GBIMS_ERR_ARG; }
    ibound[node] = -1;
  }
  // boundary values per node: WEL q, then RCH rate*area (package order)
  struct BndEntry { double v; int kind, list; };
  std::vector<std::vector<BndEntry>> per(n);
  for (int i = 0; i < m->nwel; ++i) {
    int node = m->wel_node[i];
    if (node < 0 || node >= n) { h->err = "WEL node out of range"; return GBIMS_ERR_ARG; }
    per[node].push_back({m->wel_q[i], 0, i});
  }
  for (int i = 0; i < m->nrch; ++i) {
    int node = m->rch_node[i];
    if (node < 0 || node >= n) { h->err = "RCH node out of range"; return GBIMS_ERR_ARG; }
    per[node].push_back({m->rch_rate[i] * area[node], 1, i});
  }
  std::vector<int> bptr(n + 1, 0), bkind;
  std::vector<double> bval;
  h->bnd_list.clear();
  h->bnd_kind_h.clear();
  for (int p = 0; p < n; ++p) {
    bptr[p] = (int)bval.size();
    for (const auto &v : per[p]) {
      bval.push_back(v.v);
      bkind.push_back(v.kind);
      h->bnd_list.push_back(v.list);
      h->bnd_kind_h.push_back(v.kind);
    }
  }
  h->nwel = m->nwel;
  h->nrch = m->nrch;
  h->chd_node_h.assign(m->chd_node, m->chd_node + m->nchd);
  bptr[n] = (int)bval.size();
  h->inewtonur = npf->inewton && npf->inewtonur;
  Xt3dHost xh;
  std::vector<double> hyv;
  if (xt && xt->xt3d == 0) {
    if (xt->angle2 && !xt->angle1) {
      h->err = "ANGLE2 SPECIFIED BUT NOT ANGLE1";
      return GBIMS_ERR_ARG;
    }
    if ((xt->angle2 == nullptr) != (xt->angle3 == nullptr)) {
      h->err = "ANGLE2 and ANGLE3 must be given both or neither";
      return GBIMS_ERR_ARG;
    }
    if (xt->k22 || xt->angle2) hyv = npf_hy_host(m, xt, geom, c, h->nrow, h->ncol);
    xt = nullptr;  // the standard formulation
  }
  if (xt) {
    if (npf->icellavg != 0) {
      h->err = "ALTERNATIVE_CELL_AVERAGING cannot be used with XT3D";
      return GBIMS_ERR_ARG;
    }
    int rc = xt3d_host(m, xt, geom, c, ibound, xh, h->err);
    if (rc < 0) return rc;
    h->nja = (int)xh.sja.size();
    h->ims_s.nlay = -1;  // the wider pattern: the level-scheduled sweeps
  }
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (x != cudaSuccess && e == cudaSuccess) e = x; };
  chk(up(&h->d.ia, c.ia.data(), c.ia.size()));
  chk(up(&h->d.ja, c.ja.data(), c.ja.size()));
  chk(up(&h->d.jas, c.jas.data(), c.jas.size()));
  chk(up(&h->d.isym, c.isym.data(), c.isym.size()));
  chk(up(&h->d.ihc, c.ihc.data(), c.ihc.size()));
  chk(up(&h->d.cl1, c.cl1.data(), c.cl1.size()));
  chk(up(&h->d.cl2, c.cl2.data(), c.cl2.size()));
  chk(up(&h->d.hwva, c.hwva.data(), c.hwva.size()));
  chk(up(&h->d.top, top.data(), top.size()));
  chk(up(&h->d.bot, bot.data(), bot.size()));
  chk(up(&h->d.k11, m->k11, (size_t)n));
  chk(up(&h->d.k33, m->k33, (size_t)n));
  chk(up(&h->d.icelltype, m->icelltype, (size_t)n));
  chk(up<double>(&h->d.condsat, nullptr, c.cl1.size()));
  chk(up<double>(&h->d.sat, nullptr, (size_t)n));
  if (h->inewtonur) {
    std::vector<int> ib = bottom_nodes(n, c, bot);
    chk(up(&h->ibotnode, ib.data(), ib.size()));
  }
  double *d_hy = nullptr;
  if (!hyv.empty()) {
    chk(up(&d_hy, hyv.data(), hyv.size()));
    h->xt_mem[14] = d_hy;
  }
  h->has_sto = (m->ss != nullptr && m->sy != nullptr);
  if (h->has_sto) {
    chk(up(&h->ss, m->ss, (size_t)n));
    chk(up(&h->sy, m->sy, (size_t)n));
  }
  chk(up(&h->area, area.data(), area.size()));
  chk(up(&h->vol, vol.data(), vol.size()));
  chk(up(&h->ibound, ibound.data(), ibound.size()));
  chk(up(&h->bnd_ptr, bptr.data(), bptr.size()));
  chk(up(&h->bnd_val, bval.data(), bval.size()));
  chk(up(&h->bnd_kind, bkind.data(), bkind.size()));
  h->nchd = m->nchd;
  chk(up(&h->chd_node, m->chd_node, (size_t)m->nchd));
  chk(up(&h->chd_head, m->chd_head, (size_t)m->nchd));
  double **wv[] = {&h->xold, &h->xtemp, &h->wsave, &h->hchold, &h->deold, &h->dxold};
  for (double **p : wv) chk(up<double>(p, nullptr, (size_t)n));
  h->G = std::max(1, std::min(2 * kNumSM * 2, (n + 255) / 256));
  chk(up<double>(&h->part, nullptr, (size_t)h->G * 2));
  chk(up<int>(&h->flag, nullptr, 4));
  chk(up<double>(&h->galpha, nullptr, 2));
  chk(up<double>(&h->dprev, nullptr, (size_t)n));
  chk(up<double>(&h->gpart, nullptr, (size_t)h->G * 5));
  chk(up(&h->strt, strt, (size_t)n));
  if (xt) {
    Xt3dDev &x = h->xt;
    int *d_sia = nullptr, *d_sja = nullptr, *d_idx = nullptr, *d_pc = nullptr, *d_pn = nullptr,
        *d_p0 = nullptr, *d_p1 = nullptr;
    unsigned char *d_fl = nullptr;
    double *d_ck = nullptr, *d_geo = nullptr, *d_coef = nullptr, *d_pcval = nullptr,
           *d_ones = nullptr;
    chk(up(&d_sia, xh.sia.data(), xh.sia.size()));
    chk(up(&d_sja, xh.sja.data(), xh.sja.size()));
    chk(up(&d_idx, xh.idxglo.data(), xh.idxglo.size()));
    chk(up(&d_fl, xh.sflag.data(), xh.sflag.size()));
    chk(up(&d_pc, xh.iallpc.data(), xh.iallpc.size()));
    chk(up(&d_ck, xh.ck.data(), xh.ck.size()));
    chk(up(&d_geo, xh.geo.data(), xh.geo.size()));
    chk(up(&d_pn, xh.pair_n.data(), xh.pair_n.size()));
    chk(up(&d_p0, xh.pair_il0.data(), xh.pair_il0.size()));
    chk(up(&d_p1, xh.pair_il10.data(), xh.pair_il10.size()));
    chk(up<double>(&d_coef, nullptr, (size_t)c.njas * kXtStride));
    chk(up<double>(&d_pcval, nullptr, xh.sja.size()));
    std::vector<double> ones(n, 1.0);
    chk(up(&d_ones, ones.data(), ones.size()));
    void *mem[] = {d_sia, d_sja, d_idx, d_fl, d_pc, d_ck, d_geo, d_pn, d_p0, d_p1, d_coef, d_pcval,
                   d_ones};
    for (int i = 0; i < 13; ++i) h->xt_mem[i] = mem[i];
    x.on = 1;
    x.lamatsaved = xh.lamatsaved;
    x.nozee = xh.nozee;
    x.vcentre = xh.vcentre;
    x.rhsform = xh.rhsform;
    x.sia = d_sia;
    x.sja = d_sja;
    x.idxglo = d_idx;
    x.sflag = d_fl;
    x.iallpc = d_pc;
    x.ck = d_ck;
    x.geo = d_geo;
    x.pair_n = d_pn;
    x.pair_il0 = d_p0;
    x.pair_il10 = d_p1;
    x.coef = d_coef;
    x.pcval = d_pcval;
    h->s_ia = d_sia;
    h->s_ja = d_sja;
  } else {
    h->s_ia = h->d.ia;
    h->s_ja = h->d.ja;
  }
  if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return GBIMS_ERR_CUDA; }
  for (double **p : wv) cudaMemset(*p, 0, sizeof(double) * n);
  {
    // npf_ar's initial saturation: 1 in every cell; npf_cf updates the
    // convertible ones (gwf-npf.f90:1853-1884)
    std::vector<double> one((size_t)n, 1.0);
    cudaMemcpy(h->d.sat, one.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  }
  h->hpart.resize((size_t)h->G * 2);
  // IMS handle (imslinear_allocate) on the same connectivity
  int rc = xt ? gbims_create(&h->ims_s, n, h->nja, xh.sia.data(), xh.sja.data(), &h->ims)
              : gbims_create(&h->ims_s, n, h->nja, c.ia.data(), c.ja.data(), &h->ims);
  if (rc < 0) {
    h->err = std::string("IMS: ") + (h->ims ? gbims_last_error(h->ims) : "create failed");
    return rc;
  }
  ims_buffers(h->ims, &h->amat, &h->rhs, &h->x);
  h->st = ims_stream(h->ims);
  SLN_CUDA(h, cudaEventCreate(&h->e0));
  SLN_CUDA(h, cudaEventCreate(&h->e1));
  SLN_CUDA(h, cudaEventCreate(&h->e2));
  h->g = h->d.view();
  h->g.inewton = npf->inewton;
  h->g.ivarcv = npf->ivarcv;
  h->g.idewatcv = npf->idewatcv;
  h->g.icellavg = npf->icellavg;
  h->g.satomega = npf->satomega > 0 ? npf->satomega : 1.0e-6;
  h->g.hy = d_hy;
  SLN_CUDA(h, cudaMemcpyAsync(h->x, strt, sizeof(double) * n, cudaMemcpyHostToDevice, h->st));
  gwf_condsat(n, h->g, h->d.condsat, h->st);
  if (xt && h->xt.lamatsaved) {
    // the permanently confined coefficients, once, with every saturation 1
    // (npf_ar's initial sat, xt3d_ar :366-367)
    const double *ones = (const double *)h->xt_mem[12];
    xt3d_pairs(h->njas, h->g, h->xt, h->ibound, ones, h->x, 1, h->st);
    xt3d_pcrows(n, h->g, h->xt, h->ibound, (double *)h->xt_mem[11], h->st);
  }
  SLN_CUDA(h, cudaStreamSynchronize(h->st));
  SLN_CUDA(h, cudaGetLastError());
  return GBIMS_OK;
}

bool model_props_ok(const gbsln_model *m) {
  return m->k11 && m->k33 && m->icelltype && m->nchd >= 0 && m->nwel >= 0 && m->nrch >= 0 &&
         (m->nchd == 0 || (m->chd_node && m->chd_head)) &&
         (m->nwel == 0 || (m->wel_node && m->wel_q)) &&
         (m->nrch == 0 || (m->rch_node && m->rch_rate));
}

}  // namespace

static int create_dis(const gbsln_model *m, const gbsln_ktensor *xt, const gbnpf_options *npf,
                      const gbims_settings *ims, const gbsln_nonlinear *nl, const double *strt,
                      gbsln_handle **out) {
  if (!out) return GBIMS_ERR_ARG;
  *out = nullptr;
  if (!m || !npf || !ims || !nl || !strt || m->nlay <= 0 || m->nrow <= 0 || m->ncol <= 0 ||
      !m->delr || !m->delc || !m->top || !m->botm || !model_props_ok(m))
    return GBIMS_ERR_ARG;
  gbsln_handle *h = new (std::nothrow) gbsln_handle();
  if (!h) return GBIMS_ERR_NOMEM;
  *out = h;
  h->nlay = m->nlay; h->nrow = m->nrow; h->ncol = m->ncol;
  const long long nrc = (long long)m->nrow * m->ncol;
  const long long nn = nrc * m->nlay;
  if (nn > 400000000LL) { h->err = "grid too large"; return GBIMS_ERR_UNSUPPORTED; }
  const int n = (int)nn;
  h->n = n;
  h->nl = *nl;
  h->ims_s = *ims;
  h->ims_s.index_base = 0;
  h->ims_s.nlay = m->nlay; h->ims_s.nrow = m->nrow; h->ims_s.ncol = m->ncol;
  // cell geometry (Dis.f90: top of layer 1 is TOP, of layer k>1 the bottom above)
  std::vector<double> top(n), bot(m->botm, m->botm + n), area(n);
  for (long long p = 0; p < nn; ++p) {
    top[p] = (p < nrc) ? m->top[p] : m->botm[p - nrc];
    long long rem = p % nrc;
    int i = (int)(rem / m->ncol), j = (int)(rem % m->ncol);
    area[p] = m->delc[i] * m->delr[j];
  }
  Conn c;
  build_connections(m->nlay, m->nrow, m->ncol, m->delr, m->delc, top, bot, c);
  return sln_setup(h, m, npf, strt, c, top, bot, area, xt);
}

extern "C" int gbsln_create(const gbsln_model *m, const gbnpf_options *npf,
                            const gbims_settings *ims, const gbsln_nonlinear *nl,
                            const double *strt, gbsln_handle **out) {
  return create_dis(m, nullptr, npf, ims, nl, strt, out);
}

extern "C" int gbsln_create_tensor(const gbsln_model *m, const gbsln_ktensor *xt,
                                 const gbnpf_options *npf, const gbims_settings *ims,
                                 const gbsln_nonlinear *nl, const double *strt,
                                 gbsln_handle **out) {
  if (!xt) {
    if (out) *out = nullptr;
    return GBIMS_ERR_ARG;
  }
  return create_dis(m, xt, npf, ims, nl, strt, out);
}

static int create_grid(const gbsln_grid *grid, const gbsln_model *m, const gbsln_ktensor *xt,
                       const gbsln_geometry *geom, const gbnpf_options *npf,
                       const gbims_settings *ims, const gbsln_nonlinear *nl, const double *strt,
                       gbsln_handle **out) {
  if (!out) return GBIMS_ERR_ARG;
  *out = nullptr;
  if (!grid || !m || !npf || !ims || !nl || !strt || grid->nodes <= 0 ||
      grid->nja < grid->nodes || !grid->ia || !grid->ja || !grid->ihc || !grid->cl1 ||
      !grid->cl2 || !grid->hwva || !grid->top || !grid->bot || !grid->area ||
      !model_props_ok(m))
    return GBIMS_ERR_ARG;
  gbsln_handle *h = new (std::nothrow) gbsln_handle();
  if (!h) return GBIMS_ERR_NOMEM;
  *out = h;
  const int n = grid->nodes, nja = grid->nja;
  h->n = n;
  h->nl = *nl;
  h->ims_s = *ims;
  h->ims_s.index_base = 0;
  // no shape given: a DIS pattern is found from IA/JA, any other takes the
  // general-pattern path
  h->ims_s.nlay = 0; h->ims_s.nrow = 0; h->ims_s.ncol = 0;
  if (grid->ia[0] != 0 || grid->ia[n] != nja) { h->err = "IA does not span JA"; return GBIMS_ERR_ARG; }
  Conn c;
  c.ia.assign(grid->ia, grid->ia + n + 1);
  c.ja.assign(grid->ja, grid->ja + nja);
  // con_finalize's checks (Connections.f90:203-247): the diagonal first,
  // the off-diagonals ascending, every connection with its counterpart
  for (int p = 0; p < n; ++p) {
    if (c.ia[p + 1] <= c.ia[p] || c.ja[c.ia[p]] != p) {
      h->err = "JA: the first entry of row " + std::to_string(p) + " is not its diagonal";
      return GBIMS_ERR_ARG;
    }
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q) {
      const int m2 = c.ja[q];
      if (m2 < 0 || m2 >= n || m2 == p || (q + 1 < c.ia[p + 1] && m2 >= c.ja[q + 1])) {
        h->err = "JA: row " + std::to_string(p) + " is not sorted or names a bad node";
        return GBIMS_ERR_ARG;
      }
    }
  }
  // fillisym / filljas (Connections.f90:1205-1268), 0-based
  c.isym.assign(nja, -1);
  c.jas.assign(nja, -1);
  for (int p = 0; p < n; ++p)
    for (int q = c.ia[p]; q < c.ia[p + 1]; ++q) {
      const int m2 = c.ja[q];
      if (m2 == p) { c.isym[q] = q; continue; }
      for (int r = c.ia[m2]; r < c.ia[m2 + 1]; ++r)
        if (c.ja[r] == p) { c.isym[q] = r; break; }
      if (c.isym[q] < 0) {
        h->err = "JA: connection " + std::to_string(p) + "-" + std::to_string(m2) +
                 " has no symmetric counterpart";
        return GBIMS_ERR_ARG;
      }
    }
  int ipos = 0;
  for (int p = 0; p < n; ++p)
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q)
      if (c.ja[q] > p) c.jas[q] = ipos++;
  for (int p = 0; p < n; ++p)
    for (int q = c.ia[p] + 1; q < c.ia[p + 1]; ++q)
      if (c.ja[q] < p) c.jas[q] = c.jas[c.isym[q]];
  c.njas = ipos;
  c.ihc.assign(grid->ihc, grid->ihc + ipos);
  for (int s2 = 0; s2 < ipos; ++s2)
    if (c.ihc[s2] < 0 || c.ihc[s2] > 2) { h->err = "IHC must be 0, 1, or 2"; return GBIMS_ERR_ARG; }
  c.cl1.assign(grid->cl1, grid->cl1 + ipos);
  c.cl2.assign(grid->cl2, grid->cl2 + ipos);
  c.hwva.assign(grid->hwva, grid->hwva + ipos);
  std::vector<double> top(grid->top, grid->top + n), bot(grid->bot, grid->bot + n),
      area(grid->area, grid->area + n);
  return sln_setup(h, m, npf, strt, c, top, bot, area, xt, geom);
}

extern "C" int gbsln_create_grid(const gbsln_grid *grid, const gbsln_model *m,
                                 const gbnpf_options *npf, const gbims_settings *ims,
                                 const gbsln_nonlinear *nl, const double *strt,
                                 gbsln_handle **out) {
  return create_grid(grid, m, nullptr, nullptr, npf, ims, nl, strt, out);
}

extern "C" int gbsln_create_grid_tensor(const gbsln_grid *grid, const gbsln_model *m,
                                      const gbsln_ktensor *xt, const gbsln_geometry *geom,
                                      const gbnpf_options *npf, const gbims_settings *ims,
                                      const gbsln_nonlinear *nl, const double *strt,
                                      gbsln_handle **out) {
  if (!xt || !geom || !geom->anglex || (xt->xt3d != 0 && (!geom->xc || !geom->yc))) {
    if (out) *out = nullptr;
    return GBIMS_ERR_ARG;
  }
  return create_grid(grid, m, xt, geom, npf, ims, nl, strt, out);
}

static int read_dxmax(gbsln_handle *h, double *hncg, int *loc) {
  gwf_dxmax(h->n, h->ibound, h->x, h->xtemp, h->part, h->G, h->st);
  SLN_CUDA(h, cudaMemcpyAsync(h->hpart.data(), h->part, sizeof(double) * 2 * h->G,
                              cudaMemcpyDeviceToHost, h->st));
  SLN_CUDA(h, cudaStreamSynchronize(h->st));
  double best = 0.0;
  long long bi = -1;
  for (int b = 0; b < h->G; ++b) {
    double v = h->hpart[2 * b];
    long long i = (long long)h->hpart[2 * b + 1];
    if (i < 0) continue;
    if (fabs(v) > fabs(best) || (fabs(v) == fabs(best) && (bi < 0 || i < bi))) {
      best = v;
      bi = i;
    }
  }
  *hncg = best;
  if (loc) *loc = (int)bi;
  return GBIMS_OK;
}

static int reduce_host(gbsln_handle *h, bool max_not_sum, double *out) {
  SLN_CUDA(h, cudaMemcpyAsync(h->hpart.data(), h->part, sizeof(double) * h->G,
                              cudaMemcpyDeviceToHost, h->st));
  SLN_CUDA(h, cudaStreamSynchronize(h->st));
  double a = 0.0;
  for (int b = 0; b < h->G; ++b) a = max_not_sum ? std::max(a, h->hpart[b]) : a + h->hpart[b];
  *out = a;
  return GBIMS_OK;
}

static int timestep_core(gbsln_handle *h, int kper, int kstp, double delt, const double *d_guess,
                         gbsln_stats *st, int inner_cap = 0, bool project = false);
// timestep_core's status when a guessed step has used its inner-iteration
// budget without closing (internal; gbsln_timestep_warm falls back on it)
constexpr int kCapReached = 1000;

extern "C" int gbsln_timestep(gbsln_handle *h, int kper, int kstp, double delt, gbsln_stats *st) {
  return timestep_core(h, kper, kstp, delt, nullptr, st);
}

extern "C" int gbsln_timestep_guess(gbsln_handle *h, int kper, int kstp, double delt,
                                    const double *d_guess, gbsln_stats *st) {
  if (!d_guess) return GBIMS_ERR_ARG;
  return timestep_core(h, kper, kstp, delt, d_guess, st);
}

extern "C" int gbsln_timestep_warm(gbsln_handle *h, int kper, int kstp, double delt,
                                   const double *d_guess, int inner_cap, gbsln_stats *st) {
  if (!h || inner_cap < 1) return GBIMS_ERR_ARG;
  gbsln_stats a;
  memset(&a, 0, sizeof(a));
  int rc = timestep_core(h, kper, kstp, delt, d_guess, &a, inner_cap, true);
  if (rc != kCapReached) {
    if (st) *st = a;
    return rc;
  }
  // fall back: the step again from the previous heads (xold still holds
  // them: the projection only ever replaced the first iterate)
  SLN_CUDA(h, cudaMemcpyAsync(h->x, h->xold, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st));
  gbsln_stats b;
  memset(&b, 0, sizeof(b));
  rc = timestep_core(h, kper, kstp, delt, nullptr, &b);
  b.guess_alpha = a.guess_alpha;
  b.prev_alpha = a.prev_alpha;
  b.inner_total += a.inner_total;
  b.fill_ms += a.fill_ms;
  b.solve_ms += a.solve_ms;
  b.total_ms += a.total_ms;
  b.pivot_retries += a.pivot_retries;
  b.backtracks += a.backtracks;
  if (st) *st = b;
  return rc < 0 ? rc : GBIMS_WARN_FALLBACK;
}

static int timestep_core(gbsln_handle *h, int kper, int kstp, double delt, const double *d_guess,
                         gbsln_stats *st, int inner_cap, bool project) {
  if (!h || !h->ims) return GBIMS_ERR_ARG;
  const int n = h->n;
  const bool transient = (delt > 0.0) && h->has_sto;
  h->last_delt = delt;
  gbsln_stats s;
  memset(&s, 0, sizeof(s));
  float fill_ms = 0.f;
  SLN_CUDA(h, cudaEventRecord(h->e0, h->st));
  // prepareSolve: gwf_ad (xold = x) and chd_ad (x = xold = head)
  SLN_CUDA(h, cudaMemcpyAsync(h->xold, h->x, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->st));
  // warm start: the guess replaces the previous heads as the first iterate
  // (xold, the storage reference, keeps the previous heads)
  if (d_guess && !project)
    k_apply_guess<<<std::min(4 * kNumSM, (n + 255) / 256), 256, 0, h->st>>>(n, h->ibound, d_guess, h->x);
  if (h->nchd > 0)
    k_set_chd<<<(h->nchd + 255) / 256, 256, 0, h->st>>>(h->nchd, h->chd_node, h->chd_head, h->x, h->xold);
  FillDev f{};
  f.transient = transient ? 1 : 0;
  f.tled = transient ? 1.0 / delt : 0.0;
  f.ss = h->ss;
  f.sy = h->sy;
  f.area = h->area;
  f.bnd_ptr = h->bnd_ptr;
  f.bnd_val = h->bnd_val;
  f.xt = h->xt;
  const int isymmetric = (h->ims_s.ilinmeth == 1) ? 1 : 0;
  const bool steady_newton = !transient && h->g.inewton;
  bool converged = false;
  double hncg = 0.0;
  // the system without Newton terms (sln_buildsystem with inewton = 0) and
  // the L2 norm of its residual over active cells (sln_l2norm)
  auto build_l2_nonewton = [&](double *l2) -> int {
    FillDev f0 = f;
    f0.fn = 0;
    SLN_CUDA(h, cudaMemsetAsync(h->amat, 0, sizeof(double) * h->nja, h->st));
    SLN_CUDA(h, cudaMemsetAsync(h->rhs, 0, sizeof(double) * n, h->st));
    gwf_npf_cf(n, h->g, h->ibound, h->x, h->d.sat, h->st);
    if (f0.xt.on) xt3d_pairs(h->njas, h->g, f0.xt, h->ibound, h->d.sat, h->x, 0, h->st);
    gwf_fill(n, h->g, f0, h->ibound, h->x, h->xold, h->d.sat, h->d.condsat, h->amat, h->rhs, h->st);
    gwf_l2_resid(n, h->s_ia, h->s_ja, h->amat, h->x, h->rhs, h->ibound, h->part, h->G, h->st);
    double ss = 0.0;
    int rc = reduce_host(h, false, &ss);
    *l2 = sqrt(ss);
    return rc;
  };
  const double *dprev = h->have_prev ? h->dprev : nullptr;
  const bool projected = project && (d_guess || dprev);
  if (projected) {
    // the first iterate in the plane through the previous heads spanned by
    // the last step's change and the guess's, at its energy-norm optimum
    // for the step's first system (built at the previous heads, as the
    // plain step's first outer iteration is)
    SLN_CUDA(h, cudaMemsetAsync(h->amat, 0, sizeof(double) * h->nja, h->st));
    SLN_CUDA(h, cudaMemsetAsync(h->rhs, 0, sizeof(double) * n, h->st));
    gwf_npf_cf(n, h->g, h->ibound, h->x, h->d.sat, h->st);
    if (f.xt.on) xt3d_pairs(h->njas, h->g, f.xt, h->ibound, h->d.sat, h->x, 0, h->st);
    gwf_fill(n, h->g, f, h->ibound, h->x, h->xold, h->d.sat, h->d.condsat, h->amat, h->rhs, h->st);
    k_guess_dots<<<h->G, 256, 0, h->st>>>(n, h->s_ia, h->s_ja, h->amat, h->rhs, h->ibound, dprev,
                                            d_guess, h->xold, h->gpart);
    k_guess_blend<<<std::min(4 * kNumSM, (n + 255) / 256), 256, 0, h->st>>>(
        n, h->G, h->gpart, h->ibound, dprev, d_guess, h->xold, h->x, h->galpha);
    SLN_CUDA(h, cudaGetLastError());
  }
  auto read_alphas = [&]() -> int {
    double al[2] = {0.0, 0.0};
    if (projected) SLN_CUDA(h, cudaMemcpy(al, h->galpha, sizeof(al), cudaMemcpyDeviceToHost));
    else if (d_guess) al[1] = 1.0;
    s.prev_alpha = al[0];
    s.guess_alpha = al[1];
    return GBIMS_OK;
  };
  for (int kiter = 1; kiter <= h->nl.mxiter; ++kiter) {
    if (d_guess && inner_cap > 0 && kiter > 1 && s.inner_total >= inner_cap) {
      // the guessed step has used its budget without closing
      SLN_CUDA(h, cudaEventRecord(h->e1, h->st));
      SLN_CUDA(h, cudaEventSynchronize(h->e1));
      float tot = 0.f;
      cudaEventElapsedTime(&tot, h->e0, h->e1);
      s.total_ms = tot;
      if (int rc = read_alphas()) return rc;
      if (st) *st = s;
      return kCapReached;
    }
    if (h->nl.numtrack > 0) {
      // sln_backtracking (NumericalSolution.f90:2680-2760): from the second
      // outer iteration on, while the residual norm exceeds BTOL times the
      // previous one, the last change is cut by BREDUC
      // (get_backtracking_flag :2795-2817, apply_backtracking :2823-2838)
      double l2 = 0.0;
      if (int rc = build_l2_nonewton(&l2)) return rc;
      if (kiter == 1) {
        h->res_prev = l2;
      } else {
        h->res_new = l2;
        if (h->res_new > h->res_prev * h->nl.btol) {
          for (int nb = 1; nb <= h->nl.numtrack; ++nb) {
            double dxm = 0.0;
            if (int rc = read_dxmax(h, &dxm, nullptr)) return rc;
            if (!(h->nl.breduc * fabs(dxm) >= h->nl.dvclose)) break;
            gwf_backtrack(n, h->nl.breduc, h->ibound, h->x, h->xtemp, h->st);
            s.backtracks += 1;
            if (int rc = build_l2_nonewton(&h->res_new)) return rc;
            if (nb == h->nl.numtrack) break;
            if (h->res_new < h->res_prev * h->nl.btol) break;
            if (h->res_new < h->nl.res_lim) break;
          }
        }
        h->res_prev = h->res_new;
      }
    }
    cudaEvent_t f0, f1;
    cudaEventCreate(&f0);
    cudaEventCreate(&f1);
    cudaEventRecord(f0, h->st);
    // sln_buildsystem: amat = rhs = 0, npf_cf, gwf_fc
    SLN_CUDA(h, cudaMemsetAsync(h->amat, 0, sizeof(double) * h->nja, h->st));
    SLN_CUDA(h, cudaMemsetAsync(h->rhs, 0, sizeof(double) * n, h->st));
    gwf_npf_cf(n, h->g, h->ibound, h->x, h->d.sat, h->st);
    if (f.xt.on) xt3d_pairs(h->njas, h->g, f.xt, h->ibound, h->d.sat, h->x, 0, h->st);
    gwf_fill(n, h->g, f, h->ibound, h->x, h->xold, h->d.sat, h->d.condsat, h->amat, h->rhs, h->st);
    cudaEventRecord(f1, h->st);
    // sln_calc_ptc -> gwf_ptc (steady-state Newton models)
    int iptc = 0;
    double ptcf = 0.0;
    if (steady_newton) {
      gwf_ptc_resid(n, h->s_ia, h->s_ja, h->amat, h->x, h->rhs, h->ibound, h->vol, h->part, h->G, h->st);
      int rc = reduce_host(h, true, &ptcf);
      if (rc < 0) return rc;
      if (ptcf == 0.0) ptcf = 1.0 / (delt * 10.0);
      iptc = 1;
    }
    // sln_ls: loose ends, then pseudo-transient continuation
    gwf_fixups(n, h->s_ia, h->s_ja, h->ibound, isymmetric, h->amat, h->rhs, h->x, h->xtemp, h->st);
    int iallowptc = h->nl.iallowptc;
    if (iallowptc < 0) iallowptc = (kper > 1) ? 1 : 0;
    if (iptc * iallowptc != 0) {
      gwf_l2_resid(n, h->s_ia, h->s_ja, h->amat, h->x, h->rhs, h->ibound, h->part, h->G, h->st);
      double ss2 = 0.0;
      int rc = reduce_host(h, false, &ss2);
      if (rc < 0) return rc;
      double l2norm = sqrt(ss2);
      if (kiter == 1) {
        if ((kper > 1 || kstp > 1) && l2norm <= h->l2norm0_ptc) iptc = 0;
      } else {
        double a = l2norm, b = h->l2norm0_ptc;
        bool same = (a == b) || fabs(a - b) <= 100.0 * 2.220446049250313e-16 * std::max(fabs(a), fabs(b));
        if (same) iptc = 0;
      }
      if (iptc * iallowptc != 0) {
        if (kiter == 1) h->ptcdel = 1.0 / ptcf;
        else h->ptcdel = (l2norm > 0.0) ? h->ptcdel * (h->l2norm0_ptc / l2norm) : 0.0;
        double ptcval = (h->ptcdel > 0.0) ? 1.0 / h->ptcdel : 1.0;
        gwf_ptc_apply(n, h->s_ia, h->ibound, ptcval, h->amat, h->rhs, h->x, h->st);
        h->l2norm0_ptc = l2norm;
      }
    }
    // IMS apply (in place on the handle's buffers)
    int icnvg = 0, in_iter = 0;
    gbims_summary sm;
    int rc = ims_apply_inplace(h->ims, kstp, kiter, &icnvg, &in_iter, &sm);
    cudaEventElapsedTime(&fill_ms, f0, f1);
    cudaEventDestroy(f0);
    cudaEventDestroy(f1);
    s.fill_ms += fill_ms;
    s.solve_ms += sm.solve_ms;
    if (rc < 0) {
      h->err = std::string("IMS: ") + ims_error(h->ims);
      return rc;
    }
    s.inner_total += in_iter;
    s.pivot_retries += sm.pivot_retries;
    s.outer = kiter;
    rc = read_dxmax(h, &hncg, nullptr);
    if (rc < 0) return rc;
    bool cnvg = fabs(hncg) <= h->nl.dvclose;
    if (!cnvg) {
      if (h->nl.nonmeth == 1 || h->nl.nonmeth == 3) {
        gwf_underrelax(n, h->nl.nonmeth, kiter, h->nl.theta, h->nl.akappa, h->nl.gamma,
                       h->nl.amomentum, h->ibound, h->x, h->xtemp, h->wsave, h->hchold, h->deold,
                       h->dxold, h->st);
      } else if (h->nl.nonmeth == 2) {
        double relax;
        h->bigch = hncg;
        if (kiter == 1) {
          relax = 1.0;
          h->relaxold = 1.0;
          h->bigchold = hncg;
        } else {
          double es = h->bigch / (h->bigchold * h->relaxold);
          double aes = fabs(es);
          relax = (es < -1.0) ? 0.5 / aes : (3.0 + es) / (3.0 + aes);
        }
        h->relaxold = relax;
        h->bigchold = (1.0 - h->nl.gamma) * h->bigch + h->nl.gamma * h->bigchold;
        if (relax < 1.0) gwf_relax_scale(n, relax, h->ibound, h->x, h->xtemp, h->dxold, h->st);
      } else {
        gwf_calcdx(n, h->ibound, h->x, h->xtemp, h->dxold, h->st);
      }
      if (h->inewtonur) {  // gwf_nur (gwf.f90:717): NEWTON UNDER_RELAXATION only
        SLN_CUDA(h, cudaMemsetAsync(h->flag, 0, sizeof(int), h->st));
        gwf_npf_nur(n, h->ibotnode, h->g, h->ibound, h->x, h->xtemp, h->dxold, h->flag, h->st);
        int flag = 0;
        SLN_CUDA(h, cudaMemcpyAsync(&flag, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->st));
        SLN_CUDA(h, cudaStreamSynchronize(h->st));
        if (flag) {
          // sln_maxval over dxold, then sln_nur_has_converged
          std::vector<double> dx(n);
          SLN_CUDA(h, cudaMemcpy(dx.data(), h->dxold, sizeof(double) * n, cudaMemcpyDeviceToHost));
          double vmax = dx[0];
          for (int q = 1; q < n; ++q) {
            double denom = fabs(vmax);
            if (denom == 0.0) denom = 2.220446049250313e-16;
            if (fabs(dx[q]) / denom > 1.0) vmax = dx[q];
          }
          if (fabs(vmax) <= h->nl.dvclose && fabs(hncg) <= h->nl.dvclose) {
            cnvg = true;
            rc = read_dxmax(h, &hncg, nullptr);
            if (rc < 0) return rc;
          }
        }
      }
    }
    if (cnvg) {
      converged = true;
      break;
    }
  }
  SLN_CUDA(h, cudaEventRecord(h->e1, h->st));
  SLN_CUDA(h, cudaEventSynchronize(h->e1));
  float tot = 0.f;
  cudaEventElapsedTime(&tot, h->e0, h->e1);
  s.total_ms = tot;
  s.converged = converged ? 1 : 0;
  s.dxmax = hncg;
  if (int rc = read_alphas()) return rc;
  // the step's head change, the first direction of the next warm step
  if (converged)
    k_prev_change<<<std::min(4 * kNumSM, (n + 255) / 256), 256, 0, h->st>>>(n, h->ibound, h->x,
                                                                           h->xold, h->dprev);
  h->have_prev = converged;
  SLN_CUDA(h, cudaGetLastError());
  if (st) *st = s;
  return GBIMS_OK;
}

extern "C" int gbsln_formulate(gbsln_handle *h, double delt, const double *hold, double *amat,
                               double *rhs) {
  if (!h || !amat || !rhs) return GBIMS_ERR_ARG;
  const int n = h->n;
  const bool transient = (delt > 0.0) && h->has_sto;
  if (transient && !hold) return GBIMS_ERR_ARG;
  h->last_delt = delt;
  if (hold) SLN_CUDA(h, cudaMemcpyAsync(h->xold, hold, sizeof(double) * n, cudaMemcpyHostToDevice, h->st));
  FillDev f{};
  f.transient = transient ? 1 : 0;
  f.tled = transient ? 1.0 / delt : 0.0;
  f.ss = h->ss;
  f.sy = h->sy;
  f.area = h->area;
  f.bnd_ptr = h->bnd_ptr;
  f.bnd_val = h->bnd_val;
  f.xt = h->xt;
  SLN_CUDA(h, cudaMemsetAsync(h->amat, 0, sizeof(double) * h->nja, h->st));
  SLN_CUDA(h, cudaMemsetAsync(h->rhs, 0, sizeof(double) * n, h->st));
  gwf_npf_cf(n, h->g, h->ibound, h->x, h->d.sat, h->st);
  if (f.xt.on) xt3d_pairs(h->njas, h->g, f.xt, h->ibound, h->d.sat, h->x, 0, h->st);
  gwf_fill(n, h->g, f, h->ibound, h->x, h->xold, h->d.sat, h->d.condsat, h->amat, h->rhs, h->st);
  SLN_CUDA(h, cudaGetLastError());
  SLN_CUDA(h, cudaMemcpyAsync(amat, h->amat, sizeof(double) * h->nja, cudaMemcpyDeviceToHost, h->st));
  SLN_CUDA(h, cudaMemcpyAsync(rhs, h->rhs, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
  SLN_CUDA(h, cudaStreamSynchronize(h->st));
  return GBIMS_OK;
}

extern "C" int gbsln_budget(gbsln_handle *h, double *flowja, gbsln_budget_table *out) {
  if (!h || !out) return GBIMS_ERR_ARG;
  const int n = h->n;
  const bool transient = (h->last_delt > 0.0) && h->has_sto;
  if (!h->bpart) SLN_CUDA(h, cudaMalloc((void **)&h->bpart, sizeof(double) * kGwfBudgetSlots * h->G));
  double *dflow = nullptr;
  if (flowja) SLN_CUDA(h, cudaMallocAsync((void **)&dflow, sizeof(double) * h->nja_m, h->st));
  FillDev f{};
  f.transient = transient ? 1 : 0;
  f.tled = transient ? 1.0 / h->last_delt : 0.0;
  f.ss = h->ss;
  f.sy = h->sy;
  f.area = h->area;
  f.bnd_ptr = h->bnd_ptr;
  f.bnd_val = h->bnd_val;
  f.xt = h->xt;
  if (f.xt.on) xt3d_pairs(h->njas, h->g, f.xt, h->ibound, h->d.sat, h->x, 2, h->st);
  gwf_budget(n, h->g, f, h->bnd_kind, nullptr, h->ibound, h->x, h->xold, h->d.sat, h->d.condsat,
             dflow, h->bpart, h->G, h->st);
  std::vector<double> part((size_t)kGwfBudgetSlots * h->G);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(part.data(), h->bpart, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess && flowja)
    e = cudaMemcpyAsync(flowja, dflow, sizeof(double) * h->nja_m, cudaMemcpyDeviceToHost, h->st);
  if (dflow) cudaFreeAsync(dflow, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) {
    h->err = std::string("gbsln_budget: ") + cudaGetErrorString(e);
    return GBIMS_ERR_CUDA;
  }
  // block partials in block order, then the entries in budget order
  double t[10] = {0};
  double best = 0.0, row = -1.0;
  for (int b = 0; b < h->G; ++b) {
    const double *pb = part.data() + (size_t)b * kGwfBudgetSlots;
    for (int k = 0; k < 10; ++k) t[k] += pb[k];
    if (pb[10] > best) {
      best = pb[10];
      row = pb[11];
    }
  }
  memset(out, 0, sizeof(*out));
  for (int k = 0; k < 5; ++k) {
    out->rate_in[k] = t[2 * k];
    out->rate_out[k] = t[2 * k + 1];
    out->total_in += t[2 * k];
    out->total_out += t[2 * k + 1];
  }
  const double avg = (out->total_in + out->total_out) / 2.0;
  out->percent_discrepancy = (avg != 0.0) ? 100.0 * (out->total_in - out->total_out) / avg : 0.0;
  out->max_cell_imbalance = best;
  out->max_cell = (int)row;
  return GBIMS_OK;
}

extern "C" int gbsln_budget_cells(gbsln_handle *h, double *sto_ss, double *sto_sy,
                                  double *chd_rate, double *wel_rate, double *rch_rate) {
  if (!h) return GBIMS_ERR_ARG;
  const int n = h->n;
  const size_t nb = h->bnd_list.size();
  const bool transient = (h->last_delt > 0.0) && h->has_sto;
  if (!h->bpart) SLN_CUDA(h, cudaMalloc((void **)&h->bpart, sizeof(double) * kGwfBudgetSlots * h->G));
  double *dcells = nullptr;
  SLN_CUDA(h, cudaMallocAsync((void **)&dcells, sizeof(double) * (3 * (size_t)n + nb + 1), h->st));
  FillDev f{};
  f.transient = transient ? 1 : 0;
  f.tled = transient ? 1.0 / h->last_delt : 0.0;
  f.ss = h->ss;
  f.sy = h->sy;
  f.area = h->area;
  f.bnd_ptr = h->bnd_ptr;
  f.bnd_val = h->bnd_val;
  f.xt = h->xt;
  if (f.xt.on) xt3d_pairs(h->njas, h->g, f.xt, h->ibound, h->d.sat, h->x, 2, h->st);
  gwf_budget(n, h->g, f, h->bnd_kind, dcells, h->ibound, h->x, h->xold, h->d.sat, h->d.condsat,
             nullptr, h->bpart, h->G, h->st);
  std::vector<double> c(3 * (size_t)n + nb);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c.data(), dcells, sizeof(double) * c.size(), cudaMemcpyDeviceToHost, h->st);
  cudaFreeAsync(dcells, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) {
    h->err = std::string("gbsln_budget_cells: ") + cudaGetErrorString(e);
    return GBIMS_ERR_CUDA;
  }
  if (sto_ss) std::copy(c.begin(), c.begin() + n, sto_ss);
  if (sto_sy) std::copy(c.begin() + n, c.begin() + 2 * (size_t)n, sto_sy);
  if (chd_rate)
    for (size_t i = 0; i < h->chd_node_h.size(); ++i) chd_rate[i] = c[2 * (size_t)n + h->chd_node_h[i]];
  for (size_t e2 = 0; e2 < nb; ++e2) {
    double *dst = (h->bnd_kind_h[e2] == 0) ? wel_rate : rch_rate;
    if (dst) dst[h->bnd_list[e2]] = c[3 * (size_t)n + e2];
  }
  return GBIMS_OK;
}

extern "C" const char *gbsln_last_error(const gbsln_handle *h) {
  return h ? h->err.c_str() : "null handle";
}

extern "C" int gbsln_restart(gbsln_handle *h) {
  if (!h) return GBIMS_ERR_ARG;
  SLN_CUDA(h, cudaMemcpyAsync(h->x, h->strt, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st));
  SLN_CUDA(h, cudaStreamSynchronize(h->st));
  h->bigch = h->bigchold = h->relaxold = h->l2norm0_ptc = h->ptcdel = 0.0;
  h->res_prev = h->res_new = 0.0;
  h->have_prev = false;
  return GBIMS_OK;
}

extern "C" int gbsln_get_heads(gbsln_handle *h, double *x) {
  if (!h || !x) return GBIMS_ERR_ARG;
  SLN_CUDA(h, cudaStreamSynchronize(h->st));
  SLN_CUDA(h, cudaMemcpy(x, h->x, sizeof(double) * h->n, cudaMemcpyDeviceToHost));
  return GBIMS_OK;
}

extern "C" int gbsln_set_heads(gbsln_handle *h, const double *x) {
  if (!h || !x) return GBIMS_ERR_ARG;
  SLN_CUDA(h, cudaStreamSynchronize(h->st));
  SLN_CUDA(h, cudaMemcpy(h->x, x, sizeof(double) * h->n, cudaMemcpyHostToDevice));
  h->have_prev = false;
  return GBIMS_OK;
}

extern "C" gbims_handle *gbsln_ims(gbsln_handle *h) { return h ? h->ims : nullptr; }

namespace gb {
int sln_view(gbsln_handle *h, SlnView *v) {
  if (!h || !v || !h->ims) return GBIMS_ERR_ARG;
  v->n = h->n;
  v->x = h->x;
  v->xold = h->xold;
  v->ibound = h->ibound;
  v->st = h->st;
  return GBIMS_OK;
}
}  // namespace gb

extern "C" int gbsln_destroy(gbsln_handle *h) {
  if (!h) return GBIMS_OK;
  if (h->ims) gbims_destroy(h->ims);
  h->d.release();
  void *p[] = {h->strt, h->ss, h->sy, h->area, h->vol, h->xold, h->xtemp, h->wsave, h->hchold, h->deold,
               h->dxold, h->part, h->bnd_val, h->chd_head, h->ibound, h->bnd_ptr, h->chd_node,
               h->bnd_kind, h->bpart, h->ibotnode,
               h->flag, h->galpha, h->dprev, h->gpart};
  for (void *q : p)
    if (q) cudaFree(q);
  for (void *q : h->xt_mem)
    if (q) cudaFree(q);
  if (h->e0) cudaEventDestroy(h->e0);
  if (h->e1) cudaEventDestroy(h->e1);
  if (h->e2) cudaEventDestroy(h->e2);
  delete h;
  return GBIMS_OK;
}
