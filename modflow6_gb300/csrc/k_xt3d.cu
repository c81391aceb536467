// k_xt3d.cu -- XT3D coefficient kernels.
//
// The reference walks cell n and its upper neighbours m > n and, for each
// connection, computes the "conductances" chat01 (cells 0 and 1),
// chati0 (cell 0's other neighbours) and chat1j (cell 1's), then scatters
// them into up to 4 + 4*nnbr matrix positions (xt3d_fc,
// Xt3dInterface.f90:371-497).  Here one thread computes the coefficients of
// one connection into coef (k_xt3d_pairs); the fill kernel then gathers
// them row by row in the reference's order (k_gwf.cu).  The coefficients of
// connections whose cells are all permanently confined are made once, with
// saturated areas, and summed per position as the reference's amatpc and
// amatpcx (k_xt3d_pcrows, xt3d_fcpc :499-571).
#include "k_xt3d.cuh"

namespace gb {

// xt3d_areas (Xt3dInterface.f90:1300-1379)
__device__ inline void xt_areas(const NpfDev &g, const double *sat, const double *h, int n, int m,
                                int jjs01, bool lsat, double &ar01, double &ar10) {
  if (g.ihc[jjs01] == 0) {
    ar01 = g.hwva[jjs01];
    ar10 = ar01;
    return;
  }
  const double topn = g.top[n], botn = g.bot[n], topm = g.top[m], botm = g.bot[m];
  double thksatn = XSUB(topn, botn), thksatm = XSUB(topm, botm);
  if (g.inewton != 0) {
    if (lsat) {
      if (g.ihc[jjs01] == 2) {
        const double sill_top = fmin(topn, topm), sill_bot = fmax(botn, botm);
        const double tpn = XADD(botn, thksatn), tpm = XADD(botm, thksatm);
        thksatn = fmax(XSUB(fmin(tpn, sill_top), sill_bot), 0.0);
        thksatm = fmax(XSUB(fmin(tpm, sill_top), sill_bot), 0.0);
      }
      ar01 = XMUL(XMUL(g.hwva[jjs01], 0.5), XADD(thksatn, thksatm));
    } else {
      const double satups = (h[m] < h[n]) ? sat[n] : sat[m];
      ar01 = XMUL(ar01, satups);
    }
    ar10 = ar01;
    return;
  }
  if (!lsat) {
    thksatn = XMUL(sat[n], thksatn);
    thksatm = XMUL(sat[m], thksatm);
  }
  if (g.ihc[jjs01] == 2) {
    const double sill_top = fmin(topn, topm), sill_bot = fmax(botn, botm);
    const double tpn = XADD(botn, thksatn), tpm = XADD(botm, thksatm);
    thksatn = fmax(XSUB(fmin(tpn, sill_top), sill_bot), 0.0);
    thksatm = fmax(XSUB(fmin(tpm, sill_top), sill_bot), 0.0);
  }
  ar01 = XMUL(g.hwva[jjs01], thksatn);
  ar10 = XMUL(g.hwva[jjs01], thksatm);
}

// One thread per connection n < m.  mode 0: the fill's connections (both
// cells active; n not permanently confined when lamatsaved), with the
// current saturation and, under Newton, the saturated flow qsat and the
// scaling by the actual area.  mode 1: the permanently confined cells'
// connections with saturated areas.
__global__ void k_xt3d_pairs(int njas, NpfDev g, Xt3dDev x, const int *__restrict__ ibound,
                             const double *__restrict__ sat, const double *__restrict__ h,
                             int mode) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < njas; s += gridDim.x * blockDim.x) {
    const int n = x.pair_n[s], il0 = x.pair_il0[s], il10 = x.pair_il10[s];
    const int ii01 = g.ia[n] + 1 + il0;
    const int m = g.ja[ii01];
    const bool pc = x.lamatsaved && x.iallpc[n] == 1;
    const bool use = ibound[n] != 0 && ibound[m] != 0 && (mode == 2 || (mode == 1 ? pc : !pc));
    if (!use) continue;  // never read
    XtCell c0, c1;
    xt_load(g, x, ibound, sat, n, c0);
    xt_load(g, x, ibound, sat, m, c1);
    const int jjs01 = g.jas[ii01];
    double ar01 = 0.0, ar10 = 0.0;
    if (mode == 2) {
      // xt3d_flowja's areas: under Newton the saturated area scaled by the
      // upstream saturation
      if (g.inewton != 0) xt_areas(g, sat, h, n, m, jjs01, true, ar01, ar10);
      xt_areas(g, sat, h, n, m, jjs01, false, ar01, ar10);
    } else if (mode == 1) {
      xt_areas(g, sat, h, n, m, jjs01, true, ar01, ar10);
    } else if (g.inewton != 0) {
      ar01 = 1.0;
      ar10 = 1.0;
    } else {
      xt_areas(g, sat, h, n, m, jjs01, false, ar01, ar10);
    }
    double chat01, chati0[kXtNb], chat1j[kXtNb];
    xt_qconds(c0, il0, x.ck + 9 * (size_t)n, c1, il10, x.ck + 9 * (size_t)m, ar01, ar10, 1e-10,
              chat01, chati0, chat1j);
    double qsat = 0.0;
    if (mode == 2) {
      double qnm = XMUL(chat01, XSUB(h[m], h[n]));
      double qn = 0.0;
      for (int iil = 0; iil < c0.nnbr; ++iil)
        if (c0.nb[iil] >= 0) qn = XADD(qn, XMUL(chati0[iil], XSUB(h[c0.nb[iil]], h[n])));
      qnm = XADD(qnm, qn);
      qn = 0.0;
      for (int iil = 0; iil < c1.nnbr; ++iil)
        if (c1.nb[iil] >= 0) qn = XADD(qn, XMUL(chat1j[iil], XSUB(h[c1.nb[iil]], h[m])));
      x.coef[(size_t)s * kXtStride] = XSUB(qnm, qn);
      continue;
    }
    if (mode == 0 && g.inewton != 0) {
      // xt3d_qnbrs (:1548-1575) on both sides, then the saturated and the
      // actual areas
      double qnm = XMUL(chat01, XSUB(h[m], h[n]));
      double qn = 0.0;
      for (int iil = 0; iil < c0.nnbr; ++iil)
        if (c0.nb[iil] >= 0) qn = XADD(qn, XMUL(chati0[iil], XSUB(h[c0.nb[iil]], h[n])));
      qnm = XADD(qnm, qn);
      qn = 0.0;
      for (int iil = 0; iil < c1.nnbr; ++iil)
        if (c1.nb[iil] >= 0) qn = XADD(qn, XMUL(chat1j[iil], XSUB(h[c1.nb[iil]], h[m])));
      qnm = XSUB(qnm, qn);
      xt_areas(g, sat, h, n, m, jjs01, true, ar01, ar10);
      qsat = XMUL(qnm, ar01);
      xt_areas(g, sat, h, n, m, jjs01, false, ar01, ar10);
      chat01 = XMUL(chat01, ar01);
      for (int i = 0; i < kXtNb; ++i) {
        chati0[i] = XMUL(chati0[i], ar01);
        chat1j[i] = XMUL(chat1j[i], ar01);
      }
    }
    double *out = x.coef + (size_t)s * kXtStride;
    out[0] = chat01;
    for (int i = 0; i < kXtNb; ++i) {
      out[1 + i] = chati0[i];
      out[1 + kXtNb + i] = chat1j[i];
    }
    out[1 + 2 * kXtNb] = qsat;
  }
}

// One thread per row: amatpc and amatpcx of the row's positions in the order
// xt3d_fcpc makes them (its connections n < m by n, then m; for each, the
// four primary terms, xt3d_amatpc_nbrs and xt3d_amatpcx_nbrnbrs of both
// cells over every neighbour slot), then their sum as xt3d_fc adds them to
// the zeroed matrix: amatpc first, amatpcx after.
__global__ void k_xt3d_pcrows(int nodes, NpfDev g, Xt3dDev x, const int *__restrict__ ibound,
                              double *pcval) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nodes; r += gridDim.x * blockDim.x) {
    const int s0 = x.sia[r], len = x.sia[r + 1] - s0;
    double A[kXtRow], B[kXtRow];
    for (int k = 0; k < len; ++k) {
      A[k] = 0.0;
      B[k] = 0.0;
    }
    const int r0 = g.ia[r], r1 = g.ia[r + 1];
    // connections (n, r), n < r: r is cell 1
    for (int ii = r0 + 1; ii < r1; ++ii) {
      const int n = g.ja[ii];
      if (n > r) break;
      if (!(x.iallpc[n] == 1 && ibound[n] != 0 && ibound[r] != 0)) continue;
      const double *cf = x.coef + (size_t)g.jas[ii] * kXtStride;
      const int q10 = x.idxglo[ii] - s0;
      A[0] = XSUB(A[0], cf[0]);
      A[q10] = XADD(A[q10], cf[0]);
      const double *c1j = cf + 1 + kXtNb;
      for (int iil = 0; iil < r1 - r0 - 1; ++iil) {
        A[0] = XSUB(A[0], c1j[iil]);
        const int q = x.idxglo[r0 + 1 + iil] - s0;
        A[q] = XADD(A[q], c1j[iil]);
      }
      const double *ci0 = cf + 1;
      const int n0 = g.ia[n], nn = g.ia[n + 1] - n0 - 1;
      for (int iil = 0; iil < nn; ++iil) {
        A[q10] = XADD(A[q10], ci0[iil]);
        const int q = xt_pos(x, s0, len, g.ja[n0 + 1 + iil]);
        if (q < 0) continue;
        if (x.sflag[s0 + q] & 2) B[q] = XSUB(B[q], ci0[iil]);
        else A[q] = XSUB(A[q], ci0[iil]);
      }
    }
    // connections (r, m), m > r: r is cell 0
    if (x.iallpc[r] == 1 && ibound[r] != 0) {
      for (int ii = r0 + 1; ii < r1; ++ii) {
        const int m = g.ja[ii];
        if (m < r || ibound[m] == 0) continue;
        const double *cf = x.coef + (size_t)g.jas[ii] * kXtStride;
        const int q01 = x.idxglo[ii] - s0;
        A[0] = XSUB(A[0], cf[0]);
        A[q01] = XADD(A[q01], cf[0]);
        const double *ci0 = cf + 1;
        for (int iil = 0; iil < r1 - r0 - 1; ++iil) {
          A[0] = XSUB(A[0], ci0[iil]);
          const int q = x.idxglo[r0 + 1 + iil] - s0;
          A[q] = XADD(A[q], ci0[iil]);
        }
        const double *c1j = cf + 1 + kXtNb;
        const int m0 = g.ia[m], nm = g.ia[m + 1] - m0 - 1;
        for (int iil = 0; iil < nm; ++iil) {
          A[q01] = XADD(A[q01], c1j[iil]);
          const int q = xt_pos(x, s0, len, g.ja[m0 + 1 + iil]);
          if (q < 0) continue;
          if (x.sflag[s0 + q] & 2) B[q] = XSUB(B[q], c1j[iil]);
          else A[q] = XSUB(A[q], c1j[iil]);
        }
      }
    }
    for (int k = 0; k < len; ++k) {
      double v = 0.0;
      if (x.sflag[s0 + k] & 1) v = XADD(v, A[k]);
      if (x.sflag[s0 + k] & 2) v = XADD(v, B[k]);
      pcval[s0 + k] = v;
    }
  }
}

static inline int xt_grid(int n) { return std::max(1, std::min((n + 127) / 128, 8 * kNumSM)); }

void xt3d_pairs(int njas, const NpfDev &g, const Xt3dDev &x, const int *ibound, const double *sat,
                const double *h, int mode, cudaStream_t st) {
  if (njas > 0) k_xt3d_pairs<<<xt_grid(njas), 128, 0, st>>>(njas, g, x, ibound, sat, h, mode);
}

void xt3d_pcrows(int nodes, const NpfDev &g, const Xt3dDev &x, const int *ibound, double *pcval,
                 cudaStream_t st) {
  k_xt3d_pcrows<<<xt_grid(nodes), 128, 0, st>>>(nodes, g, x, ibound, pcval);
}

}  // namespace gb
