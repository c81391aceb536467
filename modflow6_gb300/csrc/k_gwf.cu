// k_gwf.cu -- GWF assembly and outer-loop kernels for one DIS model.
//
// The reference fills the solution matrix in scatter form: npf_fc
// (src/Model/GroundWaterFlow/gwf-npf.f90:474-574) walks node n and its upper
// connections m > n and adds +cond to (n,m) and (m,n) and -cond to both
// diagonals.  Because JA is sorted (diagonal first, then ascending columns,
// src/Utilities/Sparse.f90:217-239), row p receives its -cond terms in JA
// order: lower neighbours first (while their rows are processed), then its
// own upper neighbours.  The kernels here are the gather form of the same
// computation, one thread per row, visiting the row in JA order and applying
// the terms of every package in the reference's package order (gwf_fc,
// gwf.f90:466-555: NPF fc, STO fc, BND fc, NPF fn, STO fn).  Every operation
// is rounded on its own (__dadd_rn / __dmul_rn / __ddiv_rn, no FMA), so amat
// and rhs are bit-for-bit those of the Fortran compiled without contraction.
#include "gbims_internal.cuh"
#include "k_gwf.cuh"
#include "k_xt3d.cuh"
#include <cfloat>

namespace gb {

#define DADD __dadd_rn
#define DSUB __dsub_rn
#define DMUL __dmul_rn
#define DDIV __ddiv_rn

// GwfConductanceUtils.f90:290-305, logmean
__device__ double d_logmean(double d1, double d2) {
  double drat = DDIV(d2, d1);
  if (drat <= 0.995 || drat >= 1.005) return DDIV(DSUB(d2, d1), log(drat));
  return DMUL(0.5, DADD(d1, d2));
}

// GwfConductanceUtils.f90:226-284, condmean
__device__ double d_condmean(double k1, double k2, double thick1, double thick2, double cl1,
                             double cl2, double width, int iavgmeth) {
  double t1 = DMUL(k1, thick1);
  double t2 = DMUL(k2, thick2);
  if (iavgmeth == 0) {
    if (DMUL(t1, t2) > 0.0) return DDIV(DMUL(DMUL(width, t1), t2), DADD(DMUL(t1, cl2), DMUL(t2, cl1)));
    return 0.0;
  } else if (iavgmeth == 1) {
    double tmean = (DMUL(t1, t2) > 0.0) ? d_logmean(t1, t2) : 0.0;
    return DDIV(DMUL(tmean, width), DADD(cl1, cl2));
  } else if (iavgmeth == 2) {
    double kmean = (DMUL(k1, k2) > 0.0) ? d_logmean(k1, k2) : 0.0;
    return DDIV(DMUL(DMUL(DMUL(kmean, 0.5), DADD(thick1, thick2)), width), DADD(cl1, cl2));
  } else {
    double denom = DADD(DMUL(k1, cl2), DMUL(k2, cl1));
    double kmean = (denom > 0.0) ? DDIV(DMUL(k1, k2), denom) : 0.0;
    return DMUL(DMUL(DMUL(kmean, 0.5), DADD(thick1, thick2)), width);
  }
}

// GwfConductanceUtils.f90:375-393, staggered_thkfrac: the wetted part of a
// cell that lies within the vertical overlap (sill) of the two cells
__device__ double d_staggered_thk(double top, double bot, double sat, double topc,
                                  double botc) {
  const double sill_top = fmin(top, topc);
  const double sill_bot = fmax(bot, botc);
  const double tp = DADD(bot, DMUL(sat, DSUB(top, bot)));
  return fmax(DSUB(fmin(tp, sill_top), sill_bot), 0.0);
}

// GwfConductanceUtils.f90:43-145, hcond and convertible_standard; ihc 2 is a
// horizontal connection between vertically staggered cells
__device__ double d_hcond(int ibdn, int ibdm, int ictn, int ictm, int iupstream, int ihc,
                          int icellavg, double condsat, double hn, double hm, double satn,
                          double satm, double hkn, double hkm, double topn, double topm,
                          double botn, double botm, double cln, double clm, double fawidth) {
  if (ibdn == 0 || ibdm == 0) return 0.0;
  if (ictn == 0 && ictm == 0) return condsat;
  if (iupstream == 1) {
    double sat_up = (hn > hm) ? satn : satm;
    return DMUL(sat_up, condsat);
  }
  double thksatn, thksatm;
  if (ihc == 2) {
    thksatn = d_staggered_thk(topn, botn, satn, topm, botm);
    thksatm = d_staggered_thk(topm, botm, satm, topn, botn);
  } else {
    thksatn = DMUL(satn, DSUB(topn, botn));
    thksatm = DMUL(satm, DSUB(topm, botm));
  }
  return d_condmean(hkn, hkm, thksatn, thksatm, cln, clm, fawidth, icellavg);
}

// GwfConductanceUtils.f90:149-222, vcond
__device__ double d_vcond(int ibdn, int ibdm, int ictn, int ictm, int ivarcv, int idewatcv,
                          double condsat, double hn, double hm, double vkn, double vkm,
                          double satn, double satm, double topn, double topm, double botn,
                          double botm, double flowarea) {
  if (ibdn == 0 || ibdm == 0) return 0.0;
  if (ivarcv == 0) return condsat;
  if (ictn == 0 && ictm == 0) return condsat;
  if (hn >= topn && hm >= topm) return condsat;
  double satntmp = satn, satmtmp = satm;
  if (idewatcv == 0) {
    if (botn > botm) satmtmp = 1.0;
    else satntmp = 1.0;
  }
  double bovk1 = DDIV(DMUL(DMUL(satntmp, DSUB(topn, botn)), 0.5), vkn);
  double bovk2 = DDIV(DMUL(DMUL(satmtmp, DSUB(topm, botm)), 0.5), vkm);
  double denom = DADD(bovk1, bovk2);
  if (denom != 0.0) return DDIV(flowarea, denom);
  return 0.0;
}

// SmoothingFunctions.f90:275-324, sQuadraticSaturation
__device__ double d_sqsat(double top, double bot, double x, double eps) {
  double b = DSUB(top, bot);
  if (b > 0.0) {
    double br;
    if (x < bot) br = 0.0;
    else if (x > top) br = 1.0;
    else br = DDIV(DSUB(x, bot), b);
    double av = DDIV(1.0, DSUB(1.0, eps));
    double bri = DSUB(1.0, br);
    if (br < eps) return DDIV(DMUL(DMUL(av, 0.5), DMUL(br, br)), eps);
    if (br < DSUB(1.0, eps)) return DADD(DMUL(av, br), DMUL(0.5, DSUB(1.0, av)));
    if (br < 1.0) return DSUB(1.0, DDIV(DMUL(DMUL(av, 0.5), DMUL(bri, bri)), eps));
    return 1.0;
  }
  return (x < bot) ? 0.0 : 1.0;
}

// SmoothingFunctions.f90:364-406, sQuadraticSaturationDerivative
__device__ double d_sqsat_derv(double top, double bot, double x, double eps) {
  double b = DSUB(top, bot);
  double br;
  if (x < bot) br = 0.0;
  else if (x > top) br = 1.0;
  else br = DDIV(DSUB(x, bot), b);
  double av = DDIV(1.0, DSUB(1.0, eps));
  double bri = DSUB(1.0, br);
  double y;
  if (br < eps) y = DDIV(DMUL(av, br), eps);
  else if (br < DSUB(1.0, eps)) y = av;
  else if (br < 1.0) y = DDIV(DMUL(av, bri), eps);
  else y = 0.0;
  return DDIV(y, b);
}

// the effective K of connection jj (n < m) at its lower- (hy_n) and higher-
// numbered (hy_m) cell: hy_eff (gwf-npf.f90:2280-2357)
__device__ __forceinline__ double hy_n(const NpfDev &g, int jj, int n, bool vert) {
  return g.hy ? g.hy[2 * jj] : (vert ? g.k33[n] : g.k11[n]);
}
__device__ __forceinline__ double hy_m(const NpfDev &g, int jj, int m, bool vert) {
  return g.hy ? g.hy[2 * jj + 1] : (vert ? g.k33[m] : g.k11[m]);
}

// calc_condsat (gwf-npf.f90:1950-2044) for every upper connection, with the
// default initial saturation of one.
__global__ void k_condsat(int nodes, NpfDev g, double *condsat) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    for (int ii = g.ia[n] + 1; ii < g.ia[n + 1]; ++ii) {
      int m = g.ja[ii];
      if (m < n) continue;
      int jj = g.jas[ii];
      double csat;
      if (g.ihc[jj] == 0) {
        csat = d_vcond(1, 1, 1, 1, 1, 1, 1.0, g.bot[n], g.bot[m], hy_n(g, jj, n, true),
                       hy_m(g, jj, m, true), 1.0, 1.0, g.top[n], g.top[m], g.bot[n], g.bot[m],
                       g.hwva[jj]);
      } else {
        csat = d_hcond(1, 1, 1, 1, 0, g.ihc[jj], g.icellavg, 1.0, g.top[n], g.top[m], 1.0, 1.0,
                       hy_n(g, jj, n, false), hy_m(g, jj, m, false), g.top[n], g.top[m],
                       g.bot[n], g.bot[m], g.cl1[jj], g.cl2[jj], g.hwva[jj]);
      }
      condsat[jj] = csat;
    }
  }
}

// npf_cf + thksat (gwf-npf.f90:444-470, 775-794)
__global__ void k_npf_cf(int nodes, NpfDev g, const int *__restrict__ ibound,
                         const double *__restrict__ hnew, double *sat) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (g.icelltype[n] != 0) {
      double s;
      if (ibound[n] == 0) {
        s = 0.0;
      } else if (g.inewton != 0) {
        s = d_sqsat(g.top[n], g.bot[n], hnew[n], g.satomega);
      } else {
        s = (hnew[n] >= g.top[n]) ? 1.0
                                  : DDIV(DSUB(hnew[n], g.bot[n]), DSUB(g.top[n], g.bot[n]));
      }
      sat[n] = s;
    }
  }
}

// Conductance of connection (n, m), n < m (npf_fc, gwf-npf.f90:495-543).
__device__ __forceinline__ double conn_cond(const NpfDev &g, const int *ibound, const double *h,
                                            const double *sat, const double *condsat, int n, int m,
                                            int jj) {
  if (g.ihc[jj] == 0) {
    return d_vcond(ibound[n], ibound[m], g.icelltype[n], g.icelltype[m], g.ivarcv, g.idewatcv,
                   condsat[jj], h[n], h[m], hy_n(g, jj, n, true), hy_m(g, jj, m, true), sat[n],
                   sat[m], g.top[n], g.top[m], g.bot[n], g.bot[m], g.hwva[jj]);
  }
  return d_hcond(ibound[n], ibound[m], g.icelltype[n], g.icelltype[m], g.inewton, g.ihc[jj],
                 g.icellavg, condsat[jj], h[n], h[m], sat[n], sat[m], hy_n(g, jj, n, false),
                 hy_m(g, jj, m, false), g.top[n], g.top[m], g.bot[n], g.bot[m], g.cl1[jj],
                 g.cl2[jj], g.hwva[jj]);
}

// One row of gwf_fc in gather form: NPF fc, STO fc, BND fc, NPF fn, STO fn.
// XT3D fc of row p (xt3d_fc, Xt3dInterface.f90:371-497) in gather form:
// the row's positions start from the permanently confined part (amatpc and
// amatpcx, already summed) or zero, then take the terms of the connections
// (n, p), n < p, by n (p is cell 1: its primary terms, xt3d_amat_nbrs over
// p's neighbours, xt3d_amat_nbrnbrs over n's), then of (p, m), m > p, by m
// (p is cell 0), which is the order in which the reference adds them.
__device__ inline void xt_row_fc(const NpfDev &g, const Xt3dDev &x, const int *ibound,
                                 const double *h, int p, int s0, int len, double *val,
                                 double &r) {
  for (int k = 0; k < len; ++k) val[k] = x.lamatsaved ? x.pcval[s0 + k] : 0.0;
  const int r0 = g.ia[p], r1 = g.ia[p + 1], np = r1 - r0 - 1;
  if (ibound[p] == 0) return;
  if (x.rhsform) {
    // XT3D RHS: the primary terms in the matrix, the neighbours' terms into
    // the right-hand side at the current heads (xt3d_rhs, :1522-1546)
    for (int ii = r0 + 1; ii < r1; ++ii) {
      const int q = g.ja[ii];
      if (ibound[q] == 0) continue;
      const bool lower = q < p;
      if (!lower && (x.lamatsaved && x.iallpc[p] == 1)) continue;
      if (lower && (x.lamatsaved && x.iallpc[q] == 1)) continue;
      const double *cf = x.coef + (size_t)g.jas[ii] * kXtStride;
      const int qp = x.idxglo[ii] - s0;
      val[0] = DADD(val[0], -cf[0]);
      val[qp] = DADD(val[qp], cf[0]);
      const int n = lower ? q : p, m = lower ? p : q;
      const double *ci0 = cf + 1, *c1j = cf + 1 + kXtNb;
      const int n0 = g.ia[n], nn = g.ia[n + 1] - n0 - 1;
      const int m0 = g.ia[m], nm = g.ia[m + 1] - m0 - 1;
      // cell 0's neighbours: -term to n, +term to m
      for (int iil = 0; iil < nn; ++iil) {
        const int jjj = g.ja[n0 + 1 + iil];
        if (ibound[jjj] == 0) continue;
        const double term = DMUL(ci0[iil], DSUB(h[jjj], h[n]));
        r = lower ? DADD(r, term) : DSUB(r, term);
      }
      // cell 1's neighbours: -term to m, +term to n
      for (int iil = 0; iil < nm; ++iil) {
        const int jjj = g.ja[m0 + 1 + iil];
        if (ibound[jjj] == 0) continue;
        const double term = DMUL(c1j[iil], DSUB(h[jjj], h[m]));
        r = lower ? DSUB(r, term) : DADD(r, term);
      }
    }
    return;
  }
  for (int ii = r0 + 1; ii < r1; ++ii) {
    const int n = g.ja[ii];
    if (n > p) break;
    if (ibound[n] == 0 || (x.lamatsaved && x.iallpc[n] == 1)) continue;
    const double *cf = x.coef + (size_t)g.jas[ii] * kXtStride;
    const int q10 = x.idxglo[ii] - s0;
    val[0] = DADD(val[0], -cf[0]);
    val[q10] = DADD(val[q10], cf[0]);
    const double *c1j = cf + 1 + kXtNb;
    for (int iil = 0; iil < np; ++iil) {
      if (ibound[g.ja[r0 + 1 + iil]] == 0) continue;
      const int q = x.idxglo[r0 + 1 + iil] - s0;
      val[0] = DADD(val[0], -c1j[iil]);
      val[q] = DADD(val[q], c1j[iil]);
    }
    const double *ci0 = cf + 1;
    const int n0 = g.ia[n], nn = g.ia[n + 1] - n0 - 1;
    for (int iil = 0; iil < nn; ++iil) {
      const int jjj = g.ja[n0 + 1 + iil];
      if (ibound[jjj] == 0) continue;
      val[q10] = DADD(val[q10], ci0[iil]);
      const int q = xt_pos(x, s0, len, jjj);
      if (q >= 0) val[q] = DADD(val[q], -ci0[iil]);
    }
  }
  if (x.lamatsaved && x.iallpc[p] == 1) return;
  for (int ii = r0 + 1; ii < r1; ++ii) {
    const int m = g.ja[ii];
    if (m < p || ibound[m] == 0) continue;
    const double *cf = x.coef + (size_t)g.jas[ii] * kXtStride;
    const int q01 = x.idxglo[ii] - s0;
    val[0] = DADD(val[0], -cf[0]);
    val[q01] = DADD(val[q01], cf[0]);
    const double *ci0 = cf + 1;
    for (int iil = 0; iil < np; ++iil) {
      if (ibound[g.ja[r0 + 1 + iil]] == 0) continue;
      const int q = x.idxglo[r0 + 1 + iil] - s0;
      val[0] = DADD(val[0], -ci0[iil]);
      val[q] = DADD(val[q], ci0[iil]);
    }
    const double *c1j = cf + 1 + kXtNb;
    const int m0 = g.ia[m], nm = g.ia[m + 1] - m0 - 1;
    for (int iil = 0; iil < nm; ++iil) {
      const int jjj = g.ja[m0 + 1 + iil];
      if (ibound[jjj] == 0) continue;
      val[q01] = DADD(val[q01], c1j[iil]);
      const int q = xt_pos(x, s0, len, jjj);
      if (q >= 0) val[q] = DADD(val[q], -c1j[iil]);
    }
  }
}

// XT3D fn of row p (xt3d_fn, Xt3dInterface.f90:693-795) in the same order;
// the saturation derivative takes its default smoothing 1e-6
__device__ inline void xt_row_fn(const NpfDev &g, const Xt3dDev &x, const int *ibound,
                                 const double *h, int p, int s0, double *val, double &r) {
  const int r0 = g.ia[p], r1 = g.ia[p + 1];
  if (ibound[p] == 0) return;
  for (int ii = r0 + 1; ii < r1; ++ii) {
    const int q = g.ja[ii];
    const bool lower = q < p;
    const int n = lower ? q : p, m = lower ? p : q;
    if (ibound[q] == 0) continue;
    if (x.lamatsaved && x.iallpc[n] == 1) continue;
    const int jjs = g.jas[ii];
    const int iups = (h[m] < h[n]) ? n : m;
    if (g.icelltype[iups] == 0 && !x.rhsform) continue;
    double topup = g.top[iups], botup = g.bot[iups];
    if (g.ihc[jjs] == 2) {
      topup = fmin(g.top[n], g.top[m]);
      botup = fmax(g.bot[n], g.bot[m]);
    }
    const double derv = d_sqsat_derv(topup, botup, h[iups], 1.0e-6);
    const double term = DMUL(x.coef[(size_t)jjs * kXtStride + 1 + 2 * kXtNb], derv);
    const int qp = x.idxglo[ii] - s0;
    if (!lower) {  // p is cell 0
      if (iups == n) {
        val[0] = DADD(val[0], term);
        r = DADD(r, DMUL(term, h[n]));
      } else {
        val[qp] = DADD(val[qp], term);
        r = DADD(r, DMUL(term, h[m]));
      }
    } else {  // p is cell 1
      if (iups == n) {
        val[qp] = DADD(val[qp], -term);
        r = DSUB(r, DMUL(term, h[n]));
      } else {
        val[0] = DADD(val[0], -term);
        r = DSUB(r, DMUL(term, h[m]));
      }
    }
  }
}

template <bool XT>
__global__ void k_gwf_fill(int nodes, NpfDev g, FillDev f, const int *__restrict__ ibound,
                           const double *__restrict__ h, const double *__restrict__ hold,
                           const double *__restrict__ sat, const double *__restrict__ condsat,
                           double *amat, double *rhs) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nodes; p += gridDim.x * blockDim.x) {
    const int i0 = XT ? f.xt.sia[p] : g.ia[p], i1 = g.ia[p + 1];
    double val[XT ? kXtRow : 1];
    const int xlen = XT ? f.xt.sia[p + 1] - i0 : 0;
    double diag;
    double r = rhs[p];
    if constexpr (XT) {
      xt_row_fc(g, f.xt, ibound, h, p, i0, xlen, val, r);
      diag = val[0];
    } else {
      diag = amat[i0];
      // NPF fc: row p in JA order
      for (int ii = i0 + 1; ii < i1; ++ii) {
        int q = g.ja[ii];
        int n = min(p, q), m = max(p, q);
        double cond = conn_cond(g, ibound, h, sat, condsat, n, m, g.jas[ii]);
        amat[ii] = DADD(amat[ii], cond);
        diag = DADD(diag, -cond);
      }
    }
    // STO fc (gwf-sto.f90:226-345)
    if (f.transient && ibound[p] >= 1) {
      double tp = g.top[p], bt = g.bot[p];
      int iconvert = g.icelltype[p];
      double snold = 1.0, snnew = 1.0;
      if (iconvert != 0) {
        snold = d_sqsat(tp, bt, hold[p], g.satomega);
        snnew = d_sqsat(tp, bt, h[p], g.satomega);
      }
      double sc1 = DMUL(DMUL(f.ss[p], DSUB(tp, bt)), f.area[p]);
      double rho1 = DMUL(sc1, f.tled);
      double aterm = DMUL(-rho1, snnew);
      double rhsterm;
      if (iconvert != 0) {
        double tthk = DSUB(tp, bt);
        double zold = DADD(bt, DMUL(DMUL(0.5, tthk), snold));
        double znew = DADD(bt, DMUL(DMUL(0.5, tthk), snnew));
        rhsterm = DSUB(DMUL(DMUL(-rho1, snold), DSUB(hold[p], zold)), DMUL(DMUL(rho1, snnew), znew));
      } else {
        rhsterm = DMUL(DMUL(-rho1, snold), hold[p]);
      }
      diag = DADD(diag, aterm);
      r = DADD(r, rhsterm);
      if (iconvert != 0) {
        double rho2 = DMUL(DMUL(f.sy[p], f.area[p]), f.tled);
        double tthk = DSUB(tp, bt);
        aterm = 0.0;
        if (snnew < 1.0) {
          if (snnew > 0.0) {
            aterm = -rho2;
            rhsterm = DSUB(DMUL(DMUL(-rho2, tthk), snold), DMUL(rho2, bt));
          } else {
            rhsterm = DMUL(tthk, DSUB(0.0, DMUL(rho2, snold)));
          }
        } else {
          rhsterm = DMUL(tthk, DSUB(DMUL(rho2, snnew), DMUL(rho2, snold)));
        }
        diag = DADD(diag, aterm);
        r = DADD(r, rhsterm);
      }
    }
    // BND fc: per-node boundary entries in package and list order
    for (int e = f.bnd_ptr[p]; e < f.bnd_ptr[p + 1]; ++e) {
      double v = f.bnd_val[e];
      r = DADD(r, (ibound[p] <= 0) ? 0.0 : -v);
      diag = DADD(diag, 0.0);
    }
    if constexpr (XT) {
      if (g.inewton && f.fn) {
        val[0] = diag;
        xt_row_fn(g, f.xt, ibound, h, p, i0, val, r);
        diag = val[0];
      }
    }
    // NPF fn (gwf-npf.f90:578-698), gather form
    if (!XT && g.inewton && f.fn) {
      for (int ii = i0 + 1; ii < i1; ++ii) {
        int q = g.ja[ii];
        int n = min(p, q), m = max(p, q);
        int jj = g.jas[ii];
        if (g.ihc[jj] == 0 && g.ivarcv == 0) continue;
        int iups = (h[m] < h[n]) ? n : m;
        int idn = (iups == n) ? m : n;
        if (g.icelltype[iups] == 0) continue;
        // the upstream cell's top and bottom; for a staggered connection the
        // overlap of the two cells
        double topup = g.top[iups], botup = g.bot[iups];
        if (g.ihc[jj] == 2) {
          topup = fmin(g.top[n], g.top[m]);
          botup = fmax(g.bot[n], g.bot[m]);
        }
        double cond = condsat[jj];
        double consterm = DMUL(-cond, DSUB(h[iups], h[idn]));
        double derv = d_sqsat_derv(topup, botup, h[iups], g.satomega);
        if (p == n) {  // p is the lower-numbered end: the "n" updates
          if (iups == n) {
            double term = DMUL(consterm, derv);
            r = DADD(r, DMUL(term, h[n]));
            diag = DADD(diag, term);
          } else {
            double term = DMUL(-consterm, derv);
            r = DADD(r, DMUL(term, h[m]));
            if (ibound[n] > 0) amat[ii] = DADD(amat[ii], term);
          }
        } else {  // p is the upper end: the "m" updates
          if (iups == n) {
            double term = DMUL(consterm, derv);
            r = DSUB(r, DMUL(term, h[n]));
            if (ibound[m] > 0) amat[ii] = DADD(amat[ii], -term);
          } else {
            double term = DMUL(-consterm, derv);
            r = DSUB(r, DMUL(term, h[m]));
            diag = DADD(diag, -term);
          }
        }
      }
    }
    // STO fn (gwf-sto.f90:353-439)
    if (g.inewton && f.fn && f.transient && ibound[p] > 0 && g.icelltype[p] != 0) {
      double tp = g.top[p], bt = g.bot[p];
      double tthk = DSUB(tp, bt);
      double hp = h[p];
      double snnew = d_sqsat(tp, bt, hp, 1.0e-6);
      double rho1 = DMUL(DMUL(DMUL(f.ss[p], DSUB(tp, bt)), f.area[p]), f.tled);
      double rho2 = DMUL(DMUL(f.sy[p], f.area[p]), f.tled);
      double derv = d_sqsat_derv(tp, bt, hp, 1.0e-6);
      double drterm = DADD(DMUL(DMUL(-rho1, derv), DSUB(hp, bt)), DMUL(DMUL(DMUL(rho1, tthk), snnew), derv));
      diag = DADD(diag, drterm);
      r = DADD(r, DMUL(drterm, hp));
      if (snnew < 1.0 && snnew > 0.0) {
        double rterm = DMUL(DMUL(-rho2, tthk), snnew);
        drterm = DMUL(DMUL(-rho2, tthk), derv);
        diag = DADD(diag, DADD(drterm, rho2));
        r = DADD(DADD(DSUB(r, rterm), DMUL(drterm, hp)), DMUL(rho2, bt));
      }
    }
    amat[i0] = diag;
    if constexpr (XT)
      for (int k = 1; k < xlen; ++k) amat[i0 + k] = val[k];
    rhs[p] = r;
  }
}

// Cell-by-cell flows and the model budget of one time step (gwf_cq and
// gwf_bd, gwf.f90:741-830), one row per thread in gather form:
//  * sto_cq (gwf-sto.f90:447-564, SsTerms/SyTerms rates,
//    GwfStorageUtils.f90:32-134) into the flowja diagonal;
//  * bnd_cq_simrate (BoundaryPackage.f90:583-619) for WEL then RCH:
//    rate = hcof*h - rhs with hcof = 0, for active cells;
//  * npf_cq (gwf-npf.f90:745-770, qcalc :800-865): q = cond*(h_m - h_n)
//    into the lower-numbered cell n, -q into m; csr_diagsum
//    (Sparse.f90:262-281) adds the row's flows to the diagonal in JA order;
//  * calc_chd_rate (gwf-chd.f90:264-320) for CHD cells: rate = -sum q, and
//    the in/out split over connections to active cells.
// Per block: the in/out sums of STO-SS, STO-SY, CHD, WEL, RCH (the
// rate_accumulator of Budget.f90:631-648) and the largest |flowja diagonal|
// of an active cell (its row as a double).  flowja may be null.
__global__ void __launch_bounds__(256) k_gwf_budget(int nodes, NpfDev g, FillDev f,
                                                    const int *__restrict__ bnd_kind,
                                                    const int *__restrict__ ibound,
                                                    const double *__restrict__ h,
                                                    const double *__restrict__ hold,
                                                    const double *__restrict__ sat,
                                                    const double *__restrict__ condsat,
                                                    double *flowja, double *part,
                                                    double *cells) {
  double acc[kGwfBudgetSlots];
#pragma unroll
  for (int t = 0; t < kGwfBudgetSlots; ++t) acc[t] = 0.0;
  acc[11] = -1.0;
  auto inout = [&](int slot, double r) {
    if (r < 0.0) acc[2 * slot + 1] = DSUB(acc[2 * slot + 1], r);
    else acc[2 * slot] = DADD(acc[2 * slot], r);
  };
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nodes; p += gridDim.x * blockDim.x) {
    const int i0 = g.ia[p], i1 = g.ia[p + 1];
    double diag = 0.0;
    // STO
    if (f.transient && ibound[p] > 0) {
      const double tp = g.top[p], bt = g.bot[p];
      const int iconvert = g.icelltype[p];
      double snold = 1.0, snnew = 1.0;
      if (iconvert != 0) {
        snold = d_sqsat(tp, bt, hold[p], g.satomega);
        snnew = d_sqsat(tp, bt, h[p], g.satomega);
      }
      const double sc1 = DMUL(DMUL(f.ss[p], DSUB(tp, bt)), f.area[p]);
      const double rho1 = DMUL(sc1, f.tled);
      const double aterm = DMUL(-rho1, snnew);
      double rhsterm;
      if (iconvert != 0) {
        const double tthk = DSUB(tp, bt);
        const double zold = DADD(bt, DMUL(DMUL(0.5, tthk), snold));
        const double znew = DADD(bt, DMUL(DMUL(0.5, tthk), snnew));
        rhsterm = DSUB(DMUL(DMUL(-rho1, snold), DSUB(hold[p], zold)), DMUL(DMUL(rho1, snnew), znew));
      } else {
        rhsterm = DMUL(DMUL(-rho1, snold), hold[p]);
      }
      const double rss = DSUB(DMUL(aterm, h[p]), rhsterm);
      diag = DADD(diag, rss);
      inout(0, rss);
      if (cells) cells[p] = rss;
      double rsy = 0.0;
      if (iconvert != 0) {
        const double rho2 = DMUL(DMUL(f.sy[p], f.area[p]), f.tled);
        const double tthk = DSUB(tp, bt);
        rsy = DSUB(DMUL(DMUL(rho2, tthk), snold), DMUL(DMUL(rho2, tthk), snnew));
      }
      diag = DADD(diag, rsy);
      inout(1, rsy);
      if (cells) cells[nodes + p] = rsy;
    } else if (cells) {
      cells[p] = 0.0;
      cells[nodes + p] = 0.0;
    }
    // WEL, RCH: rhs = -v, hcof = 0
    for (int e = f.bnd_ptr[p]; e < f.bnd_ptr[p + 1]; ++e) {
      double rr = 0.0;
      if (ibound[p] > 0) rr = DSUB(DMUL(0.0, h[p]), -f.bnd_val[e]);
      diag = DADD(diag, rr);
      inout(3 + bnd_kind[e], rr);
      if (cells) cells[3 * (size_t)nodes + e] = rr;
    }
    // NPF flows, diagonal sum, CHD
    const bool chd = ibound[p] < 0;
    double crate = 0.0, cin = 0.0, cout = 0.0;
    for (int ii = i0 + 1; ii < i1; ++ii) {
      const int q = g.ja[ii];
      const int n = min(p, q), m = max(p, q);
      double fj;
      if (f.xt.on) {
        // xt3d_flowja (Xt3dInterface.f90:797-875): the connection's flow,
        // added to zero with its sign for each end
        if (ibound[n] == 0 || ibound[m] == 0) {
          fj = 0.0;
        } else {
          const double qx = f.xt.coef[(size_t)g.jas[ii] * kXtStride];
          fj = (p == n) ? DADD(0.0, qx) : DSUB(0.0, qx);
        }
      } else {
        const double cond = conn_cond(g, ibound, h, sat, condsat, n, m, g.jas[ii]);
        const double qnm = DMUL(cond, DSUB(h[m], h[n]));
        fj = (p == n) ? qnm : -qnm;
      }
      if (flowja) flowja[ii] = fj;
      diag = DADD(diag, fj);
      if (chd) {
        crate = DSUB(crate, fj);
        if (ibound[q] > 0) {
          if (fj < 0.0) cin = DSUB(cin, fj);
          else cout = DADD(cout, fj);
        }
      }
    }
    if (chd) {
      diag = DADD(diag, crate);
      acc[4] = DADD(acc[4], cin);
      acc[5] = DADD(acc[5], cout);
    }
    if (cells) cells[2 * (size_t)nodes + p] = crate;
    if (flowja) flowja[i0] = diag;
    if (ibound[p] > 0 && fabs(diag) > acc[10]) {
      acc[10] = fabs(diag);
      acc[11] = (double)p;
    }
  }
  // block reduction: sums of slots 0-9, max (with row) of slot 10
  __shared__ double sh[8][kGwfBudgetSlots];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < 10; ++t)
    for (int o = 16; o > 0; o >>= 1) acc[t] += __shfl_xor_sync(0xffffffffu, acc[t], o);
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, acc[10], o);
    const double r = __shfl_xor_sync(0xffffffffu, acc[11], o);
    if (v > acc[10] || (v == acc[10] && r >= 0.0 && (acc[11] < 0.0 || r < acc[11]))) {
      acc[10] = v;
      acc[11] = r;
    }
  }
  if (lane == 0)
    for (int t = 0; t < kGwfBudgetSlots; ++t) sh[w][t] = acc[t];
  __syncthreads();
  if (threadIdx.x == 0) {
    double out[kGwfBudgetSlots];
    for (int t = 0; t < kGwfBudgetSlots; ++t) out[t] = sh[0][t];
    for (int v = 1; v < (int)(blockDim.x >> 5); ++v) {
      for (int t = 0; t < 10; ++t) out[t] += sh[v][t];
      if (sh[v][10] > out[10]) {
        out[10] = sh[v][10];
        out[11] = sh[v][11];
      }
    }
    for (int t = 0; t < kGwfBudgetSlots; ++t) part[(size_t)blockIdx.x * kGwfBudgetSlots + t] = out[t];
  }
}

// sln_calc_residual + gwf_ptc (NumericalSolution.f90:2966-2982, gwf.f90:625-687):
// per block, max over active cells of |A x - b| / cell volume.
__global__ void k_ptc_resid(int nodes, const int *__restrict__ ia, const int *__restrict__ ja,
                            const double *__restrict__ amat, const double *__restrict__ x,
                            const double *__restrict__ rhs, const int *__restrict__ ibound,
                            const double *__restrict__ vol, double *part) {
  double best = 0.0;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (ibound[n] < 1) continue;
    double t = 0.0;
    for (int k = ia[n]; k < ia[n + 1]; ++k) t = DADD(t, DMUL(amat[k], x[ja[k]]));
    double v = DDIV(fabs(DSUB(t, rhs[n])), vol[n]);
    best = fmax(best, v);
  }
  for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b = fmax(b, sh[w]);
    part[blockIdx.x] = b;
  }
}

// ||A x - b||_2 over active rows (sln_l2norm, NumericalSolution.f90:2855-2871)
__global__ void k_l2_resid(int nodes, const int *__restrict__ ia, const int *__restrict__ ja,
                           const double *__restrict__ amat, const double *__restrict__ x,
                           const double *__restrict__ rhs, const int *__restrict__ ibound,
                           double *part) {
  double s = 0.0;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (ibound[n] < 1) continue;
    double t = 0.0;
    for (int k = ia[n]; k < ia[n + 1]; ++k) t = DADD(t, DMUL(amat[k], x[ja[k]]));
    double r = DSUB(t, rhs[n]);
    s = DADD(s, DMUL(r, r));
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += sh[w];
    part[blockIdx.x] = b;
  }
}

// sln_ls loose ends (NumericalSolution.f90:2434-2478), one row per thread;
// also xtemp = x.
__global__ void k_sln_fixups(int nodes, const int *__restrict__ ia, const int *__restrict__ ja,
                             const int *__restrict__ active, int isymmetric, double *amat,
                             double *rhs, const double *__restrict__ x, double *xtemp) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    xtemp[n] = x[n];
    const int i0 = ia[n], i1 = ia[n + 1];
    if (active[n] > 0) {
      if (fabs(amat[i0]) < 1.0e-15) {
        amat[i0] = -1.0;
        rhs[n] = DADD(rhs[n], DMUL(-1.0, x[n]));
      }
      if (isymmetric) {
        double r = rhs[n];
        for (int p = i0 + 1; p < i1; ++p) {
          int c = ja[p];
          if (active[c] < 0) {
            r = DSUB(r, DMUL(amat[p], x[c]));
            amat[p] = 0.0;
          }
        }
        rhs[n] = r;
      }
    } else {
      amat[i0] = 1.0;
      for (int p = i0 + 1; p < i1; ++p) amat[p] = 0.0;
      rhs[n] = x[n];
    }
  }
}

// PTC terms on active rows (NumericalSolution.f90:2563-2575)
__global__ void k_ptc_apply(int nodes, const int *__restrict__ ia, const int *__restrict__ ibound,
                            double ptcval, double *amat, double *rhs, const double *__restrict__ x) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (ibound[n] > 0) {
      amat[ia[n]] = DADD(amat[ia[n]], -ptcval);
      rhs[n] = DSUB(rhs[n], DMUL(ptcval, x[n]));
    }
  }
}

// sln_get_dxmax (NumericalSolution.f90:3122-3153): per block max |x - xtemp|
// over active cells with its first location.
__global__ void k_dxmax(int nodes, const int *__restrict__ active, const double *__restrict__ x,
                        const double *__restrict__ xtemp, double *part) {
  MaxLoc m;
  m.val = 0.0;
  m.idx = -1;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (active[n] < 1) continue;
    double d = DSUB(x[n], xtemp[n]);
    if (absgt(d, m.val)) { m.val = d; m.idx = n; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    MaxLoc b;
    b.val = __shfl_xor_sync(0xffffffffu, m.val, o);
    b.idx = __shfl_xor_sync(0xffffffffu, m.idx, o);
    maxloc_merge(m, b);
  }
  __shared__ double sv[32];
  __shared__ long long si[32];
  if ((threadIdx.x & 31) == 0) { sv[threadIdx.x >> 5] = m.val; si[threadIdx.x >> 5] = m.idx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    MaxLoc b = {0.0, -1};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      MaxLoc c = {sv[w], si[w]};
      maxloc_merge(b, c);
    }
    part[2 * blockIdx.x] = b.val;
    part[2 * blockIdx.x + 1] = (double)b.idx;
  }
}

// sln_underrelax (NumericalSolution.f90:2989-3114), nonmeth 1 (simple) and
// 3 (delta-bar-delta); Cooley (2) is a scalar relaxation done on the host
// with k_relax_scale.
__global__ void k_underrelax(int nodes, int nonmeth, int kiter, double theta, double akappa,
                             double gamma, double amomentum, const int *__restrict__ active,
                             double *x, const double *__restrict__ xtemp, double *wsave,
                             double *hchold, double *deold, double *dxold) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (active[n] < 1) continue;
    double delx = DSUB(x[n], xtemp[n]);
    if (nonmeth == 1) {
      dxold[n] = delx;
      x[n] = DADD(xtemp[n], DMUL(gamma, delx));
    } else {
      if (kiter == 1) {
        wsave[n] = 1.0;
        hchold[n] = 1.0e-20;
        deold[n] = 0.0;
      }
      double ww;
      if (DMUL(deold[n], delx) < 0.0) ww = DMUL(theta, wsave[n]);
      else ww = DADD(wsave[n], akappa);
      if (ww > 1.0) ww = 1.0;
      wsave[n] = ww;
      if (kiter == 1) hchold[n] = delx;
      else hchold[n] = DADD(DMUL(DSUB(1.0, gamma), delx), DMUL(gamma, hchold[n]));
      deold[n] = delx;
      dxold[n] = delx;
      double amom = (kiter > 4) ? amomentum : 0.0;
      delx = DADD(DMUL(delx, ww), DMUL(amom, hchold[n]));
      x[n] = DADD(xtemp[n], delx);
    }
  }
}

__global__ void k_relax_scale(int nodes, double relax, const int *__restrict__ active, double *x,
                              const double *__restrict__ xtemp, double *dxold) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (active[n] < 1) continue;
    double delx = DSUB(x[n], xtemp[n]);
    dxold[n] = delx;
    x[n] = DADD(xtemp[n], DMUL(relax, delx));
  }
}

__global__ void k_calcdx(int nodes, const int *__restrict__ active, const double *__restrict__ x,
                         const double *__restrict__ xtemp, double *dx) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x)
    dx[n] = (active[n] < 1) ? 0.0 : DSUB(x[n], xtemp[n]);
}

// npf_nur (gwf-npf.f90:705-741); flag[0] set when any cell was relaxed.
// ibotnode: the lowest cell below each cell (gwf-npf.f90:1904-1939).
__global__ void k_npf_nur(int nodes, const int *__restrict__ ibotnode, NpfDev g,
                          const int *__restrict__ ibound, double *x,
                          const double *__restrict__ xtemp, double *dx, int *flag) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (ibound[n] < 1 || g.icelltype[n] <= 0) continue;
    double botm = g.bot[ibotnode[n]];
    if (x[n] < botm) {
      flag[0] = 1;
      x[n] = DADD(DMUL(xtemp[n], DSUB(1.0, 0.9)), DMUL(botm, 0.9));
      dx[n] = 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
static inline int g_grid(int n) { return std::max(1, std::min((n + 255) / 256, 8 * kNumSM)); }

void gwf_condsat(int nodes, const NpfDev &g, double *condsat, cudaStream_t st) {
  k_condsat<<<g_grid(nodes), 256, 0, st>>>(nodes, g, condsat);
}
void gwf_npf_cf(int nodes, const NpfDev &g, const int *ibound, const double *h, double *sat,
                cudaStream_t st) {
  k_npf_cf<<<g_grid(nodes), 256, 0, st>>>(nodes, g, ibound, h, sat);
}
void gwf_fill(int nodes, const NpfDev &g, const FillDev &f, const int *ibound, const double *h,
              const double *hold, const double *sat, const double *condsat, double *amat,
              double *rhs, cudaStream_t st) {
  if (f.xt.on)
    k_gwf_fill<true><<<g_grid(nodes), 128, 0, st>>>(nodes, g, f, ibound, h, hold, sat, condsat,
                                                    amat, rhs);
  else
    k_gwf_fill<false><<<g_grid(nodes), 256, 0, st>>>(nodes, g, f, ibound, h, hold, sat, condsat,
                                                     amat, rhs);
}
void gwf_ptc_resid(int nodes, const int *ia, const int *ja, const double *amat, const double *x,
                   const double *rhs, const int *ibound, const double *vol, double *part, int G,
                   cudaStream_t st) {
  k_ptc_resid<<<G, 256, 0, st>>>(nodes, ia, ja, amat, x, rhs, ibound, vol, part);
}
void gwf_l2_resid(int nodes, const int *ia, const int *ja, const double *amat, const double *x,
                  const double *rhs, const int *ibound, double *part, int G, cudaStream_t st) {
  k_l2_resid<<<G, 256, 0, st>>>(nodes, ia, ja, amat, x, rhs, ibound, part);
}
void gwf_fixups(int nodes, const int *ia, const int *ja, const int *active, int isymmetric,
                double *amat, double *rhs, const double *x, double *xtemp, cudaStream_t st) {
  k_sln_fixups<<<g_grid(nodes), 256, 0, st>>>(nodes, ia, ja, active, isymmetric, amat, rhs, x, xtemp);
}
void gwf_ptc_apply(int nodes, const int *ia, const int *ibound, double ptcval, double *amat,
                   double *rhs, const double *x, cudaStream_t st) {
  k_ptc_apply<<<g_grid(nodes), 256, 0, st>>>(nodes, ia, ibound, ptcval, amat, rhs, x);
}
void gwf_dxmax(int nodes, const int *active, const double *x, const double *xtemp, double *part,
               int G, cudaStream_t st) {
  k_dxmax<<<G, 256, 0, st>>>(nodes, active, x, xtemp, part);
}
void gwf_underrelax(int nodes, int nonmeth, int kiter, double theta, double akappa, double gamma,
                    double amomentum, const int *active, double *x, const double *xtemp,
                    double *wsave, double *hchold, double *deold, double *dxold, cudaStream_t st) {
  k_underrelax<<<g_grid(nodes), 256, 0, st>>>(nodes, nonmeth, kiter, theta, akappa, gamma,
                                              amomentum, active, x, xtemp, wsave, hchold, deold,
                                              dxold);
}
void gwf_relax_scale(int nodes, double relax, const int *active, double *x, const double *xtemp,
                     double *dxold, cudaStream_t st) {
  k_relax_scale<<<g_grid(nodes), 256, 0, st>>>(nodes, relax, active, x, xtemp, dxold);
}
void gwf_calcdx(int nodes, const int *active, const double *x, const double *xtemp, double *dx,
                cudaStream_t st) {
  k_calcdx<<<g_grid(nodes), 256, 0, st>>>(nodes, active, x, xtemp, dx);
}
void gwf_npf_nur(int nodes, const int *ibotnode, const NpfDev &g, const int *ibound, double *x,
                 const double *xtemp, double *dx, int *flag, cudaStream_t st) {
  k_npf_nur<<<g_grid(nodes), 256, 0, st>>>(nodes, ibotnode, g, ibound, x, xtemp, dx, flag);
}

// apply_backtracking (NumericalSolution.f90:2823-2838), the same two
// roundings as the reference: delx = breduc*(x - xtemp); x = xtemp + delx.
__global__ void k_backtrack(int nodes, double breduc, const int *__restrict__ active, double *x,
                            const double *__restrict__ xtemp) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nodes; n += gridDim.x * blockDim.x) {
    if (active[n] < 1) continue;
    const double delx = DMUL(breduc, DSUB(x[n], xtemp[n]));
    x[n] = DADD(xtemp[n], delx);
  }
}
void gwf_backtrack(int nodes, double breduc, const int *active, double *x, const double *xtemp,
                   cudaStream_t st) {
  k_backtrack<<<g_grid(nodes), 256, 0, st>>>(nodes, breduc, active, x, xtemp);
}

void gwf_budget(int nodes, const NpfDev &g, const FillDev &f, const int *bnd_kind, double *cells,
                const int *ibound, const double *h, const double *hold, const double *sat,
                const double *condsat, double *flowja, double *part, int G, cudaStream_t st) {
  k_gwf_budget<<<G, 256, 0, st>>>(nodes, g, f, bnd_kind, ibound, h, hold, sat, condsat, flowja, part,
                                  cells);
}

}  // namespace gb
