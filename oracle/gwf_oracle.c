/*
 * gwf_oracle.c -- CPU restatement of the MODFLOW 6 GWF assembly and the
 * NumericalSolution outer loop around IMS, for a single DIS model with the
 * NPF, STO, CHD, WEL and RCH packages.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  The product never links this file.
 *
 * Summation order follows the Fortran exactly (add_value_pos sequences), so
 * with -ffp-contract=off the assembled matrix is bit-for-bit the reference's.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#include "gwf_oracle.h"

#define DEM6 1.0e-6
#define DEM15 1.0e-15
#define DEM20 1.0e-20
#define DP9 0.9
#define DPREC DBL_EPSILON

/* ------------------------------------------------------------------------ */
/* Grid connectivity                                                         */
/* ------------------------------------------------------------------------ */

/* Connections.f90:463-698 (disconnections, full grid, no IDOMAIN) plus
 * Sparse.f90:217-239 (diagonal first, remaining columns ascending) and
 * fillisym/filljas (Connections.f90:1205-1268).  Node numbering follows
 * GeomUtil.f90:82-95 (column fastest, then row, then layer), 0-based.
 * Arrays must be sized by or_dis_sizes(). */
void or_dis_sizes(int nlay, int nrow, int ncol, int *nodes, int *nja, int *njas) {
  long long n = (long long)nlay * nrow * ncol;
  long long nh = (long long)nlay * nrow * (ncol - 1) + (long long)nlay * (nrow - 1) * ncol;
  long long nv = (long long)(nlay - 1) * nrow * ncol;
  *nodes = (int)n;
  *njas = (int)(nh + nv);
  *nja = (int)(n + 2 * (nh + nv));
}

void or_dis_connect(int nlay, int nrow, int ncol, const double *delr, const double *delc,
                    const double *top, const double *bot, int *ia, int *ja, int *isym,
                    int *jas, int *ihc, double *cl1, double *cl2, double *hwva) {
  int nrc = nrow * ncol;
  int pos = 0;
  for (int k = 0; k < nlay; ++k)
    for (int i = 0; i < nrow; ++i)
      for (int j = 0; j < ncol; ++j) {
        int n = j + i * ncol + k * nrc;
        ia[n] = pos;
        ja[pos++] = n; /* diagonal first */
        if (k > 0) ja[pos++] = n - nrc;
        if (i > 0) ja[pos++] = n - ncol;
        if (j > 0) ja[pos++] = n - 1;
        if (j < ncol - 1) ja[pos++] = n + 1;
        if (i < nrow - 1) ja[pos++] = n + ncol;
        if (k < nlay - 1) ja[pos++] = n + nrc;
      }
  int nodes = nlay * nrc;
  ia[nodes] = pos;
  /* fillisym */
  for (int n = 0; n < nodes; ++n)
    for (int ii = ia[n]; ii < ia[n + 1]; ++ii) {
      int m = ja[ii];
      if (m != n) {
        isym[ii] = -1;
        for (int jj = ia[m]; jj < ia[m + 1]; ++jj)
          if (ja[jj] == n) {
            isym[ii] = jj;
            break;
          }
      } else {
        isym[ii] = ii;
      }
    }
  /* filljas: 0-based symmetric index, -1 on the diagonal */
  int ipos = 0;
  for (int n = 0; n < nodes; ++n) {
    jas[ia[n]] = -1;
    for (int ii = ia[n] + 1; ii < ia[n + 1]; ++ii)
      if (ja[ii] > n) jas[ii] = ipos++;
  }
  for (int n = 0; n < nodes; ++n)
    for (int ii = ia[n]; ii < ia[n + 1]; ++ii)
      if (ja[ii] < n) jas[ii] = jas[isym[ii]];
  /* symmetric geometry arrays in (right, front, down) order per node */
  int isympos = 0;
  for (int k = 0; k < nlay; ++k)
    for (int i = 0; i < nrow; ++i)
      for (int j = 0; j < ncol; ++j) {
        int nr = j + i * ncol + k * nrc;
        if (j < ncol - 1) {
          ihc[isympos] = 1;
          cl1[isympos] = 0.5 * delr[j];
          cl2[isympos] = 0.5 * delr[j + 1];
          hwva[isympos] = delc[i];
          isympos++;
        }
        if (i < nrow - 1) {
          ihc[isympos] = 1;
          cl1[isympos] = 0.5 * delc[i];
          cl2[isympos] = 0.5 * delc[i + 1];
          hwva[isympos] = delr[j];
          isympos++;
        }
        if (k < nlay - 1) {
          int mr = nr + nrc;
          ihc[isympos] = 0;
          cl1[isympos] = 0.5 * (top[nr] - bot[nr]);
          cl2[isympos] = 0.5 * (top[mr] - bot[mr]);
          hwva[isympos] = delr[j] * delc[i];
          isympos++;
        }
      }
}

/* ------------------------------------------------------------------------ */
/* Conductance utilities                                                     */
/* ------------------------------------------------------------------------ */

/* GwfConductanceUtils.f90:226-284, condmean (harmonic, CCOND_HMEAN, and the
 * logarithmic/arithmetic variants). */
static double logmean(double d1, double d2) {
  double drat = d2 / d1;
  if (drat <= 0.995 || drat >= 1.005) return (d2 - d1) / log(drat);
  return 0.5 * (d1 + d2);
}

static double condmean(double k1, double k2, double thick1, double thick2, double cl1,
                       double cl2, double width, int iavgmeth) {
  double t1 = k1 * thick1;
  double t2 = k2 * thick2;
  switch (iavgmeth) {
  case 0:
    if (t1 * t2 > 0.0) return width * t1 * t2 / (t1 * cl2 + t2 * cl1);
    return 0.0;
  case 1: {
    double tmean = (t1 * t2 > 0.0) ? logmean(t1, t2) : 0.0;
    return tmean * width / (cl1 + cl2);
  }
  case 2: {
    double kmean = (k1 * k2 > 0.0) ? logmean(k1, k2) : 0.0;
    return kmean * 0.5 * (thick1 + thick2) * width / (cl1 + cl2);
  }
  default: {
    double denom = (k1 * cl2 + k2 * cl1);
    double kmean = (denom > 0.0) ? k1 * k2 / denom : 0.0;
    return kmean * 0.5 * (thick1 + thick2) * width;
  }
  }
}

/* GwfConductanceUtils.f90:375-393, staggered_thkfrac. */
static double staggered_thkfrac(double top, double bot, double sat, double topc, double botc) {
  double sill_top = (top < topc) ? top : topc;
  double sill_bot = (bot > botc) ? bot : botc;
  double tp = bot + sat * (top - bot);
  double t = ((tp < sill_top) ? tp : sill_top) - sill_bot;
  return (t > 0.0) ? t : 0.0;
}

/* GwfConductanceUtils.f90:43-145, hcond with convertible_standard (ihc 2:
 * vertically staggered cells). */
static double hcond(int ibdn, int ibdm, int ictn, int ictm, int iupstream, int ihc,
                    int icellavg, double condsat, double hn, double hm, double satn,
                    double satm, double hkn, double hkm, double topn, double topm, double botn,
                    double botm, double cln, double clm, double fawidth) {
  if (ibdn == 0 || ibdm == 0) return 0.0;
  if (ictn == 0 && ictm == 0) return condsat;
  if (iupstream == 1) {
    double sat_up = (hn > hm) ? satn : satm;
    return sat_up * condsat;
  }
  double thksatn, thksatm;
  if (ihc == 2) {
    thksatn = staggered_thkfrac(topn, botn, satn, topm, botm);
    thksatm = staggered_thkfrac(topm, botm, satm, topn, botn);
  } else {
    thksatn = satn * (topn - botn);
    thksatm = satm * (topm - botm);
  }
  return condmean(hkn, hkm, thksatn, thksatm, cln, clm, fawidth, icellavg);
}

/* GwfConductanceUtils.f90:149-222, vcond. */
static double vcond(int ibdn, int ibdm, int ictn, int ictm, int ivarcv, int idewatcv,
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
  double bovk1 = satntmp * (topn - botn) * 0.5 / vkn;
  double bovk2 = satmtmp * (topm - botm) * 0.5 / vkm;
  double denom = (bovk1 + bovk2);
  if (denom != 0.0) return flowarea / denom;
  return 0.0;
}

/* SmoothingFunctions.f90:275-324, sQuadraticSaturation. */
double or_squadratic_sat(double top, double bot, double x, double eps) {
  double teps = eps;
  double b = top - bot;
  double y;
  if (b > 0.0) {
    double br;
    if (x < bot) br = 0.0;
    else if (x > top) br = 1.0;
    else br = (x - bot) / b;
    double av = 1.0 / (1.0 - teps);
    double bri = 1.0 - br;
    if (br < teps) y = av * 0.5 * (br * br) / teps;
    else if (br < (1.0 - teps)) y = av * br + 0.5 * (1.0 - av);
    else if (br < 1.0) y = 1.0 - ((av * 0.5 * (bri * bri)) / teps);
    else y = 1.0;
  } else {
    y = (x < bot) ? 0.0 : 1.0;
  }
  return y;
}

/* SmoothingFunctions.f90:364-406, sQuadraticSaturationDerivative. */
double or_squadratic_sat_derv(double top, double bot, double x, double eps) {
  double teps = eps;
  double b = top - bot;
  double br;
  if (x < bot) br = 0.0;
  else if (x > top) br = 1.0;
  else br = (x - bot) / b;
  double av = 1.0 / (1.0 - teps);
  double bri = 1.0 - br;
  double y;
  if (br < teps) y = av * br / teps;
  else if (br < (1.0 - teps)) y = av;
  else if (br < 1.0) y = av * bri / teps;
  else y = 0.0;
  return y / b;
}

/* hy_eff (gwf-npf.f90:2280-2357) of connection jas from its lower- (HYN)
 * and higher-numbered (HYM) cell: the per-connection values when K22 or the
 * angles are given, else K11 (horizontal) or K33 (vertical). */
#define HYN(m, jj, n, vert) ((m)->hy ? (m)->hy[2 * (jj)] : ((vert) ? (m)->k33[n] : (m)->k11[n]))
#define HYM(m, jj, mm, vert) ((m)->hy ? (m)->hy[2 * (jj) + 1] : ((vert) ? (m)->k33[mm] : (m)->k11[mm]))

/* The solution's pattern: the model's, or with XT3D the wider one. */
#define SIA(m) ((m)->ixt3d ? (m)->sia : (m)->ia)
#define SJA(m) ((m)->ixt3d ? (m)->sja : (m)->ja)
#define SNJA(m) ((m)->ixt3d ? (m)->nja_sln : (m)->nja)

/* ------------------------------------------------------------------------ */
/* DISU connectivity                                                         */
/* ------------------------------------------------------------------------ */

static int cmp_int(const void *a, const void *b);
static void disv_shared_edge(const int *l1, int nv1, const int *l2, int nv2, int *iv1, int *iv2);

/* disuconnections (Connections.f90:801-928) then con_finalize (:160-316),
 * 0-based.  A full grid copies IA/JA; a reduced one builds each kept row as
 * the sparse matrix does (the diagonal, then every kept neighbour once, the
 * neighbours sorted, Sparse.f90:217-239) and compresses the per-entry arrays
 * in input order. */
int or_disu_connect(int nodesuser, const int *iainp, const int *jainp, const int *ihcinp,
                    const double *cl12inp, const double *hwvainp, const double *angldegxinp,
                    const int *nodereduced, int cap, int *nodes_out, int *ia, int *ja, int *isym,
                    int *jas, int *ihc, double *cl1, double *cl2, double *hwva, double *anglex) {
  int nodes = nodesuser;
  if (nodereduced) {
    nodes = 0;
    for (int u = 0; u < nodesuser; ++u)
      if (nodereduced[u] >= 0) nodes++;
  }
  *nodes_out = nodes;
  if (nodes == 0) return -8;
  int nja = 0;
  double *cl12t = NULL, *hwvat = NULL, *angt = NULL;
  int *ihcti = NULL;
  if (!nodereduced) {
    nja = iainp[nodesuser];
    if (nja > cap) return -1;
    ihcti = (int *)malloc(sizeof(int) * (nja + 1));
    cl12t = (double *)malloc(sizeof(double) * (nja + 1));
    hwvat = (double *)malloc(sizeof(double) * (nja + 1));
    angt = (double *)malloc(sizeof(double) * (nja + 1));
    for (int n = 0; n <= nodes; ++n) ia[n] = iainp[n];
    for (int q = 0; q < nja; ++q) {
      int v = jainp[q];
      ja[q] = (v < 0 ? -v : v) - 1; /* negative JA made positive */
      ihcti[q] = ihcinp[q];
      cl12t[q] = cl12inp[q];
      hwvat[q] = hwvainp[q];
      angt[q] = angldegxinp ? angldegxinp[q] : 0.0;
    }
  } else {
    /* rows of the sparse matrix, in reduced order */
    int total = 0;
    ia[0] = 0;
    for (int u = 0; u < nodesuser; ++u) {
      int nr = nodereduced[u];
      if (nr < 0) continue;
      int start = total;
      if (total >= cap) return -1;
      ja[total++] = nr;
      for (int q = iainp[u] + 1; q < iainp[u + 1]; ++q) {
        int mu = (jainp[q] < 0 ? -jainp[q] : jainp[q]) - 1;
        int mr = nodereduced[mu];
        if (mr < 0) continue;
        int dup = 0;
        for (int t = start; t < total; ++t)
          if (ja[t] == mr) dup = 1;
        if (dup) continue;
        if (total >= cap) return -1;
        ja[total++] = mr;
      }
      qsort(ja + start + 1, total - start - 1, sizeof(int), cmp_int);
      ia[nr + 1] = total;
    }
    nja = total;
    ihcti = (int *)malloc(sizeof(int) * (nja + 1));
    cl12t = (double *)malloc(sizeof(double) * (nja + 1));
    hwvat = (double *)malloc(sizeof(double) * (nja + 1));
    angt = (double *)malloc(sizeof(double) * (nja + 1));
    int iposr = 0;
    for (int u = 0; u < nodesuser; ++u) {
      int nr = nodereduced[u];
      for (int q = iainp[u]; q < iainp[u + 1]; ++q) {
        int mu = (jainp[q] < 0 ? -jainp[q] : jainp[q]) - 1;
        int mr = nodereduced[mu];
        if (nr < 0 || mr < 0) continue;
        if (iposr >= nja) { /* a duplicated entry: the arrays would overrun */
          free(ihcti); free(cl12t); free(hwvat); free(angt);
          return -3;
        }
        ihcti[iposr] = ihcinp[q];
        cl12t[iposr] = cl12inp[q];
        hwvat[iposr] = hwvainp[q];
        angt[iposr] = angldegxinp ? angldegxinp[q] : 0.0;
        iposr++;
      }
    }
  }
  int rc = nja;
  /* con_finalize: the diagonal first, the rest ascending */
  for (int n = 0; n < nodes && rc >= 0; ++n) {
    if (ja[ia[n]] != n) rc = -2;
    for (int q = ia[n] + 1; q < ia[n + 1] - 1 && rc >= 0; ++q)
      if (ja[q] > ja[q + 1]) rc = -3;
  }
  /* fillisym */
  for (int n = 0; n < nodes && rc >= 0; ++n)
    for (int q = ia[n]; q < ia[n + 1]; ++q) {
      int m = ja[q];
      if (m == n) { isym[q] = q; continue; }
      isym[q] = -1;
      for (int r = ia[m]; r < ia[m + 1]; ++r)
        if (ja[r] == n) { isym[q] = r; break; }
      if (isym[q] < 0) rc = -4;
    }
  if (rc >= 0) {
    /* filljas */
    int ipos = 0;
    for (int n = 0; n < nodes; ++n) {
      jas[ia[n]] = -1;
      for (int q = ia[n] + 1; q < ia[n + 1]; ++q)
        if (ja[q] > n) jas[q] = ipos++;
    }
    for (int n = 0; n < nodes; ++n)
      for (int q = ia[n]; q < ia[n + 1]; ++q)
        if (ja[q] < n) jas[q] = jas[isym[q]];
    /* ihc, cl12 and hwva into the symmetric arrays */
    for (int n = 0; n < nodes && rc >= 0; ++n)
      for (int q = ia[n] + 1; q < ia[n + 1]; ++q) {
        if (ihcti[q] != ihcti[isym[q]]) { rc = -5; break; }
        ihc[jas[q]] = ihcti[q];
      }
    for (int n = 0; n < nodes && rc >= 0; ++n)
      for (int q = ia[n] + 1; q < ia[n + 1]; ++q) {
        int m = ja[q];
        if (m > n) cl1[jas[q]] = cl12t[q];
        else if (n > m) cl2[jas[q]] = cl12t[q];
      }
    for (int n = 0; n < nodes && rc >= 0; ++n)
      for (int q = ia[n] + 1; q < ia[n + 1]; ++q) {
        if (hwvat[q] != hwvat[isym[q]]) { rc = -6; break; }
        if (ihcti[q] < 0 || ihcti[q] > 2) { rc = -7; break; }
        hwva[jas[q]] = hwvat[q];
      }
    /* anglex: the upper triangle's ANGLDEGX in radians (:300-307) */
    if (rc >= 0 && anglex) {
      const double dpio180 = atan(1.0) / 45.0;
      for (int n = 0; n < nodes; ++n)
        for (int q = ia[n] + 1; q < ia[n + 1]; ++q)
          if (ja[q] > n) anglex[jas[q]] = angt[q] * dpio180;
    }
  }
  free(ihcti); free(cl12t); free(hwvat); free(angt);
  return rc;
}

void or_disv_anglex(int nodes, int ncpl, const double *vx, const double *vy, const int *iavert,
                    const int *javert, const int *nodeuser, const int *ia, const int *ja,
                    const int *jas, const int *ihc, double *anglex) {
  const double dpi = 4.0 * atan(1.0);
  for (int n = 0; n < nodes; ++n) {
    const int jn = (nodeuser ? nodeuser[n] : n) % ncpl;
    for (int ii = ia[n] + 1; ii < ia[n + 1]; ++ii) {
      const int m = ja[ii];
      if (m < n) continue;
      const int s = jas[ii];
      anglex[s] = 0.0;
      if (ihc[s] == 0) continue;
      const int jm = (nodeuser ? nodeuser[m] : m) % ncpl;
      int a, b;
      disv_shared_edge(javert + iavert[jn], iavert[jn + 1] - iavert[jn], javert + iavert[jm],
                       iavert[jm + 1] - iavert[jm], &a, &b);
      if (a < 0 || b < 0) continue;
      double dx = vx[b] - vx[a], dy = vy[b] - vy[a];
      double ax = atan2(dx, -dy);
      if (ax < 0.0) ax = 2.0 * dpi + ax;
      anglex[s] = ax;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* NPF                                                                       */
/* ------------------------------------------------------------------------ */

/* gwf-npf.f90:1950-2044, calc_condsat(node, upperOnly=.true.) for every node,
 * with the default initial saturation of one (no THICKSTRT). */
void or_npf_condsat(const or_gwf_model *m, double *condsat) {
  for (int n = 0; n < m->nodes; ++n) {
    for (int ii = m->ia[n] + 1; ii < m->ia[n + 1]; ++ii) {
      int mm = m->ja[ii];
      if (mm < n) continue;
      int jj = m->jas[ii];
      int ihc = m->ihc[jj];
      double csat;
      if (ihc == 0) {
        double hyn = HYN(m, jj, n, 1), hym = HYM(m, jj, mm, 1);
        csat = vcond(1, 1, 1, 1, 1, 1, 1.0, m->bot[n], m->bot[mm], hyn, hym, 1.0, 1.0,
                     m->top[n], m->top[mm], m->bot[n], m->bot[mm], m->hwva[jj]);
      } else {
        double hyn = HYN(m, jj, n, 0), hym = HYM(m, jj, mm, 0);
        csat = hcond(1, 1, 1, 1, 0, ihc, m->icellavg, 1.0, m->top[n], m->top[mm], 1.0, 1.0,
                     hyn, hym, m->top[n], m->top[mm], m->bot[n], m->bot[mm],
                     m->cl1[jj], m->cl2[jj], m->hwva[jj]);
      }
      condsat[jj] = csat;
    }
  }
}

/* gwf-npf.f90:444-470 (npf_cf) and 775-794 (thksat). */
void or_npf_cf(const or_gwf_model *m, const int *ibound, const double *hnew, double *sat) {
  for (int n = 0; n < m->nodes; ++n) {
    if (m->icelltype[n] != 0) {
      double satn;
      if (ibound[n] == 0) {
        satn = 0.0;
      } else {
        if (hnew[n] >= m->top[n]) satn = 1.0;
        else satn = (hnew[n] - m->bot[n]) / (m->top[n] - m->bot[n]);
        if (m->inewton != 0)
          satn = or_squadratic_sat(m->top[n], m->bot[n], hnew[n], m->satomega);
      }
      sat[n] = satn;
    }
  }
}

/* gwf-npf.f90:474-574, npf_fc (no XT3D, no perched). */
void or_npf_fc(const or_gwf_model *m, const int *ibound, const double *condsat,
               const double *sat, const double *hnew, double *amat, double *rhs) {
  (void)rhs;
  for (int n = 0; n < m->nodes; ++n) {
    for (int ii = m->ia[n] + 1; ii < m->ia[n + 1]; ++ii) {
      int mm = m->ja[ii];
      if (mm < n) continue;
      int jj = m->jas[ii];
      int ihc = m->ihc[jj];
      double cond;
      if (ihc == 0) {
        cond = vcond(ibound[n], ibound[mm], m->icelltype[n], m->icelltype[mm],
                     m->ivarcv, m->idewatcv, condsat[jj], hnew[n], hnew[mm], HYN(m, jj, n, 1),
                     HYM(m, jj, mm, 1), sat[n], sat[mm], m->top[n], m->top[mm], m->bot[n],
                     m->bot[mm], m->hwva[jj]);
      } else {
        cond = hcond(ibound[n], ibound[mm], m->icelltype[n], m->icelltype[mm],
                     m->inewton, ihc, m->icellavg, condsat[jj], hnew[n], hnew[mm], sat[n],
                     sat[mm], HYN(m, jj, n, 0), HYM(m, jj, mm, 0), m->top[n], m->top[mm], m->bot[n],
                     m->bot[mm], m->cl1[jj], m->cl2[jj], m->hwva[jj]);
      }
      int idiag = m->ia[n];
      amat[ii] = amat[ii] + cond;
      amat[idiag] = amat[idiag] + (-cond);
      int isymcon = m->isym[ii];
      int idiagm = m->ia[mm];
      amat[isymcon] = amat[isymcon] + cond;
      amat[idiagm] = amat[idiagm] + (-cond);
    }
  }
}

/* gwf-npf.f90:578-698, npf_fn (no XT3D).  The get/set pairs of the Fortran
 * that store a value back unchanged are no-ops and are omitted. */
void or_npf_fn(const or_gwf_model *m, const int *ibound, const double *condsat,
               const double *hnew, double *amat, double *rhs) {
  for (int n = 0; n < m->nodes; ++n) {
    int idiag = m->ia[n];
    for (int ii = m->ia[n] + 1; ii < m->ia[n + 1]; ++ii) {
      int mm = m->ja[ii];
      int isymcon = m->isym[ii];
      if (mm < n) continue;
      int jj = m->jas[ii];
      if (m->ihc[jj] == 0 && m->ivarcv == 0) continue;
      int iups = (hnew[mm] < hnew[n]) ? n : mm;
      int idn = (iups == n) ? mm : n;
      if (m->icelltype[iups] == 0) continue;
      double topup = m->top[iups];
      double botup = m->bot[iups];
      if (m->ihc[jj] == 2) { /* the overlap of the two cells */
        topup = (m->top[n] < m->top[mm]) ? m->top[n] : m->top[mm];
        botup = (m->bot[n] > m->bot[mm]) ? m->bot[n] : m->bot[mm];
      }
      double cond = condsat[jj];
      double consterm = -cond * (hnew[iups] - hnew[idn]);
      double derv = or_squadratic_sat_derv(topup, botup, hnew[iups], m->satomega);
      int idiagm = m->ia[mm];
      if (iups == n) {
        double term = consterm * derv;
        rhs[n] = rhs[n] + term * hnew[n];
        rhs[mm] = rhs[mm] - term * hnew[n];
        amat[idiag] = amat[idiag] + term;
        if (ibound[mm] > 0) amat[isymcon] = amat[isymcon] + (-term);
      } else {
        double term = -consterm * derv;
        rhs[n] = rhs[n] + term * hnew[mm];
        rhs[mm] = rhs[mm] - term * hnew[mm];
        if (ibound[n] > 0) amat[ii] = amat[ii] + term;
        amat[idiagm] = amat[idiagm] + (-term);
      }
    }
  }
}

/* gwf-npf.f90:705-741, npf_nur. */
void or_npf_nur(const or_gwf_model *m, const int *ibound, double *x, const double *xtemp,
                double *dx, int *inewtonur, double *dxmax, int *locmax) {
  for (int n = 0; n < m->nodes; ++n) {
    if (ibound[n] < 1) continue;
    if (m->icelltype[n] > 0) {
      /* ibotnode (gwf-npf.f90:1904-1939): follow the vertical connection to
       * a higher-numbered cell with the lowest bottom while there is one */
      double minbot = m->bot[n];
      int ibot = n;
      for (;;) {
        int nextn = -1;
        for (int ii = m->ia[ibot] + 1; ii < m->ia[ibot + 1]; ++ii) {
          int mm = m->ja[ii];
          if (m->ihc[m->jas[ii]] == 0 && mm > ibot && m->bot[mm] < minbot) {
            nextn = mm;
            minbot = m->bot[mm];
          }
        }
        if (nextn < 0) break;
        ibot = nextn;
      }
      double botm = m->bot[ibot];
      if (x[n] < botm) {
        *inewtonur = 1;
        double xx = xtemp[n] * (1.0 - DP9) + botm * DP9;
        double dxx = x[n] - xx;
        if (fabs(dxx) > fabs(*dxmax)) {
          *locmax = n;
          *dxmax = dxx;
        }
        x[n] = xx;
        dx[n] = 0.0;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* DISV connectivity                                                         */
/* ------------------------------------------------------------------------ */

/* DisvGeom.f90:416-427, distance */
static double disv_distance(double x1, double y1, double x2, double y2) {
  double d = (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2);
  return sqrt(d);
}

/* DisvGeom.f90:432-445, distance_normal */
static double disv_distance_normal(double x0, double y0, double x1, double y1, double x2,
                                   double y2) {
  double d = fabs((x2 - x1) * (y1 - y0) - (x1 - x0) * (y2 - y1));
  return d / disv_distance(x1, y1, x2, y2);
}

/* DisvGeom.f90:302-332, shared_edge: the first consecutive pair of cell 1's
 * (closed) vertex list found reversed in cell 2's list. */
static void disv_shared_edge(const int *l1, int nv1, const int *l2, int nv2, int *iv1, int *iv2) {
  *iv1 = -1;
  *iv2 = -1;
  for (int a = 0; a < nv1 - 1; ++a) {
    for (int b = nv2 - 1; b >= 1; --b) {
      if (l1[a] == l2[b] && l1[a + 1] == l2[b - 1]) {
        *iv1 = l1[a];
        *iv2 = l1[a + 1];
        return;
      }
    }
  }
}

/* DisvGeom.f90:339-386, get_area (shoelace over the closed vertex list) */
static double disv_area(int j, const int *iavert, const int *javert, const double *vx,
                        const double *vy) {
  double area = 0.0;
  const int i0 = iavert[j], i1 = iavert[j + 1];
  const int nvert = i1 - i0;
  const double x1 = vx[javert[i0]], y1 = vy[javert[i0]];
  int icount = 1;
  for (int iv = i0; iv < i1; ++iv) {
    double x = vx[javert[iv]];
    double y = (icount < nvert) ? vy[javert[iv + 1]] : vy[javert[i0]];
    area = area + (x - x1) * (y - y1);
    icount++;
  }
  icount = 1;
  for (int iv = i0; iv < i1; ++iv) {
    double y = vy[javert[iv]];
    double x = (icount < nvert) ? vx[javert[iv + 1]] : vx[javert[i0]];
    area = area - (x - x1) * (y - y1);
    icount++;
  }
  return fabs(area) * 0.5;
}

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* Connections.f90:702-796 disvconnections with vertexconnect (:1272-1361) on
 * a full grid (no IDOMAIN): node n = j + k*ncpl (GeomUtil.f90 get_node), the
 * cell's vertex list closed as Disv.f90:548-585 define_cellverts closes it
 * (0-based vertex numbers; iavert ncpl+1).  Each row: the diagonal, the cell
 * above and below, then every cell of the same layer that shares an edge,
 * collected over the vertices as vertexconnect does; the off-diagonals sorted
 * ascending (Sparse.f90:217-239).  Then fillisym/filljas and cprops
 * (DisvGeom.f90:136-202) for every n < m.  cap bounds nja; returns nja, or
 * -1 if cap is too small. */
int or_disv_connect(int nlay, int ncpl, const double *vx, const double *vy, const int *iavert,
                    const int *javert, const double *xc, const double *yc, const double *top,
                    const double *bot, const int *nodereduced, int cap, int *ia, int *ja,
                    int *isym, int *jas, int *ihc, double *cl1, double *cl2, double *hwva,
                    double *area) {
  /* nodereduced (the reference's convention, user node -> 1-based reduced
   * number, 0 removed, -1 pass-through) or NULL for a full grid; top/bot per
   * user node */
  const int nodesuser = nlay * ncpl;
  int nodes = nodesuser;
  if (nodereduced) {
    nodes = 0;
    for (int u = 0; u < nodesuser; ++u)
      if (nodereduced[u] > 0) nodes++;
  }
  int *nodeuser = (int *)malloc(sizeof(int) * (nodes + 1));
  for (int u = 0, r = 0; u < nodesuser; ++u)
    if (!nodereduced || nodereduced[u] > 0) nodeuser[r++] = u;
#define RED(u) (nodereduced ? nodereduced[u] : (u) + 1) /* 1-based, 0 removed, -1 pass */
  int nvert = 0;
  for (int q = 0; q < iavert[ncpl]; ++q)
    if (javert[q] + 1 > nvert) nvert = javert[q] + 1;
  /* cells of each vertex (vertcellspm), in cell order */
  int *vcnt = (int *)calloc(nvert + 1, sizeof(int));
  for (int j = 0; j < ncpl; ++j)
    for (int q = iavert[j]; q < iavert[j + 1]; ++q) vcnt[javert[q] + 1]++;
  for (int v = 0; v < nvert; ++v) vcnt[v + 1] += vcnt[v];
  int *vcell = (int *)malloc(sizeof(int) * (vcnt[nvert] + 1));
  int *vfill = (int *)malloc(sizeof(int) * (nvert + 1));
  memcpy(vfill, vcnt, sizeof(int) * (nvert + 1));
  for (int j = 0; j < ncpl; ++j)
    for (int q = iavert[j]; q < iavert[j + 1]; ++q) vcell[vfill[javert[q]]++] = j;
  /* rows as growing lists without duplicates */
  int rowcap = 64;
  int *rows = (int *)malloc(sizeof(int) * (size_t)nodes * rowcap);
  int *rn = (int *)calloc(nodes, sizeof(int));
  int overflow = 0;
#define DISV_ADD(r, c)                                              \
  do {                                                              \
    int dup_ = 0;                                                   \
    for (int t_ = 0; t_ < rn[r]; ++t_)                              \
      if (rows[(size_t)(r) * rowcap + t_] == (c)) dup_ = 1;         \
    if (!dup_) {                                                    \
      if (rn[r] < rowcap) rows[(size_t)(r) * rowcap + rn[r]++] = (c); \
      else overflow = 1;                                            \
    }                                                               \
  } while (0)
  /* vertexconnect (Connections.f90:1272-1361): the diagonal and the
   * vertical neighbours, passing through cells with nodereduced -1 */
  for (int k = 0; k < nlay; ++k)
    for (int j = 0; j < ncpl; ++j) {
      int nr = RED(j + k * ncpl);
      if (nr <= 0) continue;
      nr -= 1;
      DISV_ADD(nr, nr);
      if (k > 0) {
        int mr = 0;
        for (int kk = k - 1; kk >= 0; --kk) {
          mr = RED(j + kk * ncpl);
          if (mr >= 0) break;
        }
        if (mr > 0) DISV_ADD(nr, mr - 1);
      }
      if (k < nlay - 1) {
        int mr = 0;
        for (int kk = k + 1; kk < nlay; ++kk) {
          mr = RED(j + kk * ncpl);
          if (mr >= 0) break;
        }
        if (mr > 0) DISV_ADD(nr, mr - 1);
      }
    }
  for (int v = 0; v < nvert; ++v)
    for (int c1 = vcnt[v]; c1 < vcnt[v + 1]; ++c1) {
      int j1 = vcell[c1];
      for (int k = 0; k < nlay; ++k) {
        int nr = RED(j1 + k * ncpl) - 1;
        if (nr < 0) continue;
        for (int c2 = vcnt[v]; c2 < vcnt[v + 1]; ++c2) {
          int j2 = vcell[c2];
          if (j1 == j2) continue;
          int mr = RED(j2 + k * ncpl) - 1;
          if (mr < 0) continue;
          int a, b;
          disv_shared_edge(javert + iavert[j1], iavert[j1 + 1] - iavert[j1], javert + iavert[j2],
                           iavert[j2 + 1] - iavert[j2], &a, &b);
          if (a >= 0 && b >= 0) DISV_ADD(nr, mr);
        }
      }
    }
#undef DISV_ADD
  int nja = 0;
  for (int n = 0; n < nodes; ++n) nja += rn[n];
  if (overflow || nja > cap) {
    free(vcnt); free(vcell); free(vfill); free(rows); free(rn); free(nodeuser);
    return -1;
  }
  ia[0] = 0;
  for (int n = 0; n < nodes; ++n) {
    int *r = rows + (size_t)n * rowcap;
    qsort(r + 1, rn[n] - 1, sizeof(int), cmp_int); /* diagonal stays in front */
    for (int t = 0; t < rn[n]; ++t) ja[ia[n] + t] = r[t];
    ia[n + 1] = ia[n] + rn[n];
  }
  /* fillisym / filljas (Connections.f90:1205-1268) */
  for (int n = 0; n < nodes; ++n)
    for (int ii = ia[n]; ii < ia[n + 1]; ++ii) {
      int m = ja[ii];
      isym[ii] = (m == n) ? ii : -1;
      if (m != n)
        for (int jj = ia[m]; jj < ia[m + 1]; ++jj)
          if (ja[jj] == n) {
            isym[ii] = jj;
            break;
          }
    }
  int ipos = 0;
  for (int n = 0; n < nodes; ++n) {
    jas[ia[n]] = -1;
    for (int ii = ia[n] + 1; ii < ia[n + 1]; ++ii)
      if (ja[ii] > n) jas[ii] = ipos++;
  }
  for (int n = 0; n < nodes; ++n)
    for (int ii = ia[n]; ii < ia[n + 1]; ++ii)
      if (ja[ii] < n) jas[ii] = jas[isym[ii]];
  for (int j = 0; j < ncpl; ++j) area[j] = disv_area(j, iavert, javert, vx, vy);
  /* cprops for n < m (DisvGeom.f90:136-202) */
  for (int n = 0; n < nodes; ++n) {
    const int un = nodeuser[n], jn = un % ncpl;
    for (int ii = ia[n] + 1; ii < ia[n + 1]; ++ii) {
      const int m = ja[ii];
      if (m < n) continue;
      const int um = nodeuser[m], jm = um % ncpl, s = jas[ii];
      if (jn == jm) {
        ihc[s] = 0;
        hwva[s] = area[jn];
        cl1[s] = 0.5 * (top[un] - bot[un]);
        cl2[s] = 0.5 * (top[um] - bot[um]);
      } else {
        ihc[s] = 1;
        int a, b;
        disv_shared_edge(javert + iavert[jn], iavert[jn + 1] - iavert[jn], javert + iavert[jm],
                         iavert[jm + 1] - iavert[jm], &a, &b);
        if (a < 0 || b < 0) {
          hwva[s] = 0.0;
          cl1[s] = 1.0;
          cl2[s] = 1.0;
        } else {
          hwva[s] = disv_distance(vx[a], vy[a], vx[b], vy[b]);
          cl1[s] = disv_distance_normal(xc[jn], yc[jn], vx[a], vy[a], vx[b], vy[b]);
          cl2[s] = disv_distance_normal(xc[jm], yc[jm], vx[a], vy[a], vx[b], vy[b]);
        }
      }
    }
  }
  free(vcnt); free(vcell); free(vfill); free(rows); free(rn); free(nodeuser);
#undef RED
  return nja;
}

/* ------------------------------------------------------------------------ */
/* STO and boundary packages                                                 */
/* ------------------------------------------------------------------------ */

/* gwf-sto.f90:226-345 (sto_fc) with GwfStorageUtils.f90 SsTerms/SyTerms/
 * SsCapacity/SyCapacity; istor_coef=0, iorig_ss=0, iconf_ss=0, no TVS. */
void or_sto_fc(const or_gwf_model *m, const int *ibound, double delt, const double *hold,
               const double *hnew, double *amat, double *rhs) {
  double tled = 1.0 / delt;
  for (int n = 0; n < m->nodes; ++n) {
    int idiag = SIA(m)[n];
    if (ibound[n] < 1) continue;
    double tp = m->top[n], bt = m->bot[n];
    int iconvert = m->iconvert[n];
    double snold, snnew;
    if (iconvert == 0) {
      snold = 1.0;
      snnew = 1.0;
    } else {
      snold = or_squadratic_sat(tp, bt, hold[n], m->satomega);
      snnew = or_squadratic_sat(tp, bt, hnew[n], m->satomega);
    }
    double sc1 = m->ss[n] * (tp - bt) * m->area[n];
    double rho1 = sc1 * tled;
    double rho1old = rho1;
    /* SsTerms */
    double aterm = -rho1 * snnew;
    double rhsterm;
    if (iconvert != 0) {
      double tthk = tp - bt;
      double zold = bt + 0.5 * tthk * snold;
      double znew = bt + 0.5 * tthk * snnew;
      rhsterm = -rho1old * snold * (hold[n] - zold) - rho1 * snnew * znew;
    } else {
      rhsterm = -rho1old * snold * hold[n];
    }
    amat[idiag] = amat[idiag] + aterm;
    rhs[n] = rhs[n] + rhsterm;
    if (iconvert != 0) {
      double sc2 = m->sy[n] * m->area[n];
      double rho2 = sc2 * tled;
      double rho2old = rho2;
      double tthk = tp - bt;
      aterm = 0.0;
      if (snnew < 1.0) {
        if (snnew > 0.0) {
          aterm = -rho2;
          rhsterm = -rho2old * tthk * snold - rho2 * bt;
        } else {
          rhsterm = tthk * (0.0 - rho2old * snold);
        }
      } else {
        rhsterm = tthk * (rho2 * snnew - rho2old * snold);
      }
      amat[idiag] = amat[idiag] + aterm;
      rhs[n] = rhs[n] + rhsterm;
    }
  }
}

/* gwf-sto.f90:353-439, sto_fn (the saturation here uses the default omega
 * of the smoothing function, as in the Fortran call without eps). */
void or_sto_fn(const or_gwf_model *m, const int *ibound, double delt, const double *hnew,
               double *amat, double *rhs) {
  double tled = 1.0 / delt;
  for (int n = 0; n < m->nodes; ++n) {
    int idiag = SIA(m)[n];
    if (ibound[n] <= 0) continue;
    double tp = m->top[n], bt = m->bot[n];
    double tthk = tp - bt;
    double h = hnew[n];
    double snnew = or_squadratic_sat(tp, bt, h, DEM6);
    double sc1 = m->ss[n] * (tp - bt) * m->area[n];
    double sc2 = m->sy[n] * m->area[n];
    double rho1 = sc1 * tled;
    double rho2 = sc2 * tled;
    if (m->iconvert[n] != 0) {
      double derv = or_squadratic_sat_derv(tp, bt, h, DEM6);
      double drterm = -rho1 * derv * (h - bt) + rho1 * tthk * snnew * derv;
      amat[idiag] = amat[idiag] + drterm;
      rhs[n] = rhs[n] + drterm * h;
      if (snnew < 1.0) {
        if (snnew > 0.0) {
          double rterm = -rho2 * tthk * snnew;
          drterm = -rho2 * tthk * derv;
          amat[idiag] = amat[idiag] + (drterm + rho2);
          rhs[n] = rhs[n] - rterm + drterm * h + rho2 * bt;
        }
      }
    }
  }
}

/* gwf-wel.f90:296-332 (wel_cf without AUTO_FLOW_REDUCE) and
 * gwf-rch.f90:303-353 (rch_cf, recharge on the listed cell), each followed by
 * BoundaryPackage.f90:453-472 (bnd_fc: rhs += rhs_i, diag += hcof_i = 0). */
void or_bnd_fc(const or_gwf_model *m, const int *ibound, double *amat, double *rhs) {
  for (int i = 0; i < m->nwel; ++i) {
    int node = m->wel_node[i];
    double r = (ibound[node] <= 0) ? 0.0 : -m->wel_q[i];
    rhs[node] = rhs[node] + r;
    amat[SIA(m)[node]] = amat[SIA(m)[node]] + 0.0;
  }
  for (int i = 0; i < m->nrch; ++i) {
    int node = m->rch_node[i];
    double r = -m->rch_rate[i] * m->area[node];
    if (ibound[node] <= 0) r = 0.0;
    rhs[node] = rhs[node] + r;
    amat[SIA(m)[node]] = amat[SIA(m)[node]] + 0.0;
  }
}

/* gwf.f90:741-830 (gwf_cq, then gwf_bd's csr_diagsum and CHD rates) and the
 * model budget entries, in package order STO-SS, STO-SY, CHD, WEL, RCH:
 *  - npf_cq, gwf-npf.f90:745-770 (qcalc :800-865, no perched option);
 *  - sto_cq, gwf-sto.f90:447-564 (SsTerms/SyTerms rates,
 *    GwfStorageUtils.f90:32-134);
 *  - bnd_cq_simrate, BoundaryPackage.f90:583-619 (WEL, then RCH);
 *  - csr_diagsum, Sparse.f90:262-281;
 *  - calc_chd_rate, gwf-chd.f90:264-320;
 *  - rate_accumulator, Budget.f90:631-648.
 * terms[2k], terms[2k+1]: rate in and out of entry k.  flowja: nja values. */
void or_gwf_budget(const or_gwf_model *m, const int *ibound, const double *condsat,
                   const double *sat, double delt, int transient, const double *hold,
                   const double *hnew, double *flowja, double *terms) {
  for (int k = 0; k < 10; ++k) terms[k] = 0.0;
  for (int k = 0; k < m->nja; ++k) flowja[k] = 0.0;
  /* npf_cq (with XT3D: xt3d_flowja, gwf-npf.f90:756-757) */
  if (m->ixt3d) or_xt3d_flowja(m, ibound, sat, hnew, flowja);
  for (int n = 0; n < m->nodes && !m->ixt3d; ++n) {
    for (int ii = m->ia[n] + 1; ii < m->ia[n + 1]; ++ii) {
      int mm = m->ja[ii];
      if (mm < n) continue;
      int jj = m->jas[ii];
      double cond;
      if (m->ihc[jj] == 0) {
        cond = vcond(ibound[n], ibound[mm], m->icelltype[n], m->icelltype[mm], m->ivarcv,
                     m->idewatcv, condsat[jj], hnew[n], hnew[mm], HYN(m, jj, n, 1), HYM(m, jj, mm, 1), sat[n],
                     sat[mm], m->top[n], m->top[mm], m->bot[n], m->bot[mm], m->hwva[jj]);
      } else {
        cond = hcond(ibound[n], ibound[mm], m->icelltype[n], m->icelltype[mm], m->inewton,
                     m->ihc[jj], m->icellavg, condsat[jj], hnew[n], hnew[mm], sat[n], sat[mm], HYN(m, jj, n, 0),
                     HYM(m, jj, mm, 0), m->top[n], m->top[mm], m->bot[n], m->bot[mm], m->cl1[jj],
                     m->cl2[jj], m->hwva[jj]);
      }
      double qnm = cond * (hnew[mm] - hnew[n]);
      flowja[ii] = qnm;
      flowja[m->isym[ii]] = -qnm;
    }
  }
  /* sto_cq */
  if (transient) {
    double tled = 1.0 / delt;
    for (int n = 0; n < m->nodes; ++n) {
      if (ibound[n] <= 0) continue;
      double tp = m->top[n], bt = m->bot[n];
      int iconvert = m->iconvert[n];
      double snold = 1.0, snnew = 1.0;
      if (iconvert != 0) {
        snold = or_squadratic_sat(tp, bt, hold[n], m->satomega);
        snnew = or_squadratic_sat(tp, bt, hnew[n], m->satomega);
      }
      double sc1 = m->ss[n] * (tp - bt) * m->area[n];
      double rho1 = sc1 * tled;
      double rho1old = rho1;
      double aterm = -rho1 * snnew;
      double rhsterm;
      if (iconvert != 0) {
        double tthk = tp - bt;
        double zold = bt + 0.5 * tthk * snold;
        double znew = bt + 0.5 * tthk * snnew;
        rhsterm = -rho1old * snold * (hold[n] - zold) - rho1 * snnew * znew;
      } else {
        rhsterm = -rho1old * snold * hold[n];
      }
      double rate = aterm * hnew[n] - rhsterm;
      int idiag = m->ia[n];
      flowja[idiag] = flowja[idiag] + rate;
      if (rate < 0.0) terms[1] = terms[1] - rate;
      else terms[0] = terms[0] + rate;
      rate = 0.0;
      if (iconvert != 0) {
        double rho2 = m->sy[n] * m->area[n] * tled;
        double rho2old = rho2;
        double tthk = tp - bt;
        rate = rho2old * tthk * snold - rho2 * tthk * snnew;
      }
      flowja[idiag] = flowja[idiag] + rate;
      if (rate < 0.0) terms[3] = terms[3] - rate;
      else terms[2] = terms[2] + rate;
    }
  }
  /* bnd_cq: WEL, RCH (hcof = 0, rhs as in or_bnd_fc) */
  for (int i = 0; i < m->nwel; ++i) {
    int node = m->wel_node[i];
    double rrate = 0.0;
    if (ibound[node] > 0) rrate = 0.0 * hnew[node] - (-m->wel_q[i]);
    flowja[m->ia[node]] = flowja[m->ia[node]] + rrate;
    if (rrate < 0.0) terms[7] = terms[7] - rrate;
    else terms[6] = terms[6] + rrate;
  }
  for (int i = 0; i < m->nrch; ++i) {
    int node = m->rch_node[i];
    double rrate = 0.0;
    if (ibound[node] > 0) rrate = 0.0 * hnew[node] - (-m->rch_rate[i] * m->area[node]);
    flowja[m->ia[node]] = flowja[m->ia[node]] + rrate;
    if (rrate < 0.0) terms[9] = terms[9] - rrate;
    else terms[8] = terms[8] + rrate;
  }
  /* csr_diagsum */
  for (int n = 0; n < m->nodes; ++n)
    for (int ii = m->ia[n] + 1; ii < m->ia[n + 1]; ++ii)
      flowja[m->ia[n]] = flowja[m->ia[n]] + flowja[ii];
  /* calc_chd_rate */
  for (int i = 0; i < m->nchd; ++i) {
    int node = m->chd_node[i];
    int idiag = m->ia[node];
    double rate = 0.0, ratein = 0.0, rateout = 0.0;
    for (int ii = m->ia[node] + 1; ii < m->ia[node + 1]; ++ii) {
      double q = flowja[ii];
      rate = rate - q;
      if (ibound[m->ja[ii]] > 0) {
        if (q < 0.0) ratein = ratein - q;
        else rateout = rateout + q;
      }
    }
    flowja[idiag] = flowja[idiag] + rate;
    terms[4] = terms[4] + ratein;
    terms[5] = terms[5] + rateout;
  }
}

/* gwf.f90:466-555, gwf_fc order for the packages restated here:
 * NPF fc, STO fc, BND fc, then NPF fn, STO fn.  amat and rhs must be zero on
 * entry (NumericalSolution sln_reset). */
static void gwf_fc_flag(const or_gwf_model *m, const int *ibound, const double *condsat,
                        double *sat, double delt, int transient, const double *hold,
                        const double *hnew, double *amat, double *rhs, int inwtflag) {
  or_npf_cf(m, ibound, hnew, sat);
  double *qsat = NULL;
  if (m->ixt3d) {
    /* npf_fc with XT3D (gwf-npf.f90:492-493) */
    qsat = (double *)calloc(m->nja, sizeof(double));
    or_xt3d_fc(m, ibound, sat, hnew, amat, rhs, qsat);
  } else {
    or_npf_fc(m, ibound, condsat, sat, hnew, amat, rhs);
  }
  if (transient) or_sto_fc(m, ibound, delt, hold, hnew, amat, rhs);
  or_bnd_fc(m, ibound, amat, rhs);
  if (inwtflag && m->inewton) {
    if (m->ixt3d) or_xt3d_fn(m, ibound, hnew, qsat, amat, rhs);
    else or_npf_fn(m, ibound, condsat, hnew, amat, rhs);
    if (transient) or_sto_fn(m, ibound, delt, hnew, amat, rhs);
  }
  free(qsat);
}

void or_gwf_fc(const or_gwf_model *m, const int *ibound, const double *condsat,
               double *sat, double delt, int transient, const double *hold,
               const double *hnew, double *amat, double *rhs) {
  gwf_fc_flag(m, ibound, condsat, sat, delt, transient, hold, hnew, amat, rhs, 1);
}

/* ------------------------------------------------------------------------ */
/* NumericalSolution pieces                                                  */
/* ------------------------------------------------------------------------ */

/* NumericalSolution.f90:2434-2478, sln_ls loose ends: small-diagonal fix,
 * identity rows for CHD / inactive cells, and (CG) the symmetric column
 * elimination of CHD cells. */
void or_sln_ls_fixups(int neq, const int *ia, const int *ja, const int *active,
                      int isymmetric, double *amat, double *rhs, const double *x,
                      double *xtemp) {
  for (int ieq = 0; ieq < neq; ++ieq) {
    xtemp[ieq] = x[ieq];
    if (active[ieq] > 0) {
      double diagval = -1.0;
      double adiag = fabs(amat[ia[ieq]]);
      if (adiag < DEM15) {
        amat[ia[ieq]] = diagval;
        rhs[ieq] = rhs[ieq] + diagval * x[ieq];
      }
    } else {
      amat[ia[ieq]] = 1.0;
      for (int ipos = ia[ieq] + 1; ipos < ia[ieq + 1]; ++ipos) amat[ipos] = 0.0;
      rhs[ieq] = x[ieq];
    }
  }
  if (isymmetric) {
    for (int ieq = 0; ieq < neq; ++ieq) {
      if (active[ieq] > 0) {
        for (int ipos = ia[ieq]; ipos < ia[ieq + 1]; ++ipos) {
          int jcol = ja[ipos];
          if (jcol == ieq) continue;
          if (active[jcol] < 0) {
            rhs[ieq] = rhs[ieq] - (amat[ipos] * x[jcol]);
            amat[ipos] = 0.0;
          }
        }
      }
    }
  }
}

/* NumericalSolution.f90:3122-3153, sln_get_dxmax. */
double or_sln_get_dxmax(int neq, const int *active, const double *x, const double *xtemp,
                        int *lrch) {
  int nb = -1;
  double bigch = 0.0, abigch = 0.0;
  for (int n = 0; n < neq; ++n) {
    if (active[n] < 1) continue;
    double hdif = x[n] - xtemp[n];
    double ahdif = fabs(hdif);
    if (ahdif > abigch) {
      bigch = hdif;
      abigch = ahdif;
      nb = n;
    }
  }
  if (lrch) *lrch = nb;
  return bigch;
}

/* NumericalSolution.f90:2989-3114, sln_underrelax (nonmeth 1, 2, 3). */
void or_sln_underrelax(or_nonlinear *nl, int kiter, double bigch, int neq,
                       const int *active, double *x, const double *xtemp) {
  if (nl->nonmeth == 1) {
    for (int n = 0; n < neq; ++n) {
      if (active[n] < 1) continue;
      double delx = x[n] - xtemp[n];
      nl->dxold[n] = delx;
      x[n] = xtemp[n] + nl->gamma * delx;
    }
  } else if (nl->nonmeth == 2) {
    double relax;
    nl->bigch = bigch;
    if (kiter == 1) {
      relax = 1.0;
      nl->relaxold = 1.0;
      nl->bigchold = bigch;
    } else {
      double es = nl->bigch / (nl->bigchold * nl->relaxold);
      double aes = fabs(es);
      if (es < -1.0) relax = 0.5 / aes;
      else relax = (3.0 + es) / (3.0 + aes);
    }
    nl->relaxold = relax;
    nl->bigchold = (1.0 - nl->gamma) * nl->bigch + nl->gamma * nl->bigchold;
    if (relax < 1.0) {
      for (int n = 0; n < neq; ++n) {
        if (active[n] < 1) continue;
        double delx = x[n] - xtemp[n];
        nl->dxold[n] = delx;
        x[n] = xtemp[n] + relax * delx;
      }
    }
  } else if (nl->nonmeth == 3) {
    for (int n = 0; n < neq; ++n) {
      if (active[n] < 1) continue;
      double delx = x[n] - xtemp[n];
      if (kiter == 1) {
        nl->wsave[n] = 1.0;
        nl->hchold[n] = DEM20;
        nl->deold[n] = 0.0;
      }
      double ww = nl->wsave[n];
      if (nl->deold[n] * delx < 0.0) ww = nl->theta * nl->wsave[n];
      else ww = nl->wsave[n] + nl->akappa;
      if (ww > 1.0) ww = 1.0;
      nl->wsave[n] = ww;
      if (kiter == 1) nl->hchold[n] = delx;
      else nl->hchold[n] = (1.0 - nl->gamma) * delx + nl->gamma * nl->hchold[n];
      nl->deold[n] = delx;
      nl->dxold[n] = delx;
      double amom = 0.0;
      if (kiter > 4) amom = nl->amomentum;
      delx = delx * ww + amom * nl->hchold[n];
      x[n] = xtemp[n] + delx;
    }
  }
}

/* NumericalSolution.f90:2878-2905, sln_maxval. */
static double sln_maxval(int nsize, const double *v) {
  double vmax = v[0];
  for (int n = 1; n < nsize; ++n) {
    double d = v[n];
    double denom = fabs(vmax);
    if (denom == 0.0) denom = DPREC;
    double dnorm = fabs(d) / denom;
    if (dnorm > 1.0) vmax = d;
  }
  return vmax;
}

/* NumericalSolution.f90:2966-2982 + SeqVector.f90:152-164: L2 norm of the
 * residual A*x - b with inactive rows zeroed. */
static double sln_l2norm(int neq, const int *ia, const int *ja, const double *amat,
                         const double *x, const double *rhs, const int *active,
                         double *work) {
  or_amux(neq, x, work, amat, ja, ia);
  double n2 = 0.0;
  for (int n = 0; n < neq; ++n) {
    double r = work[n] - rhs[n];
    if (active[n] < 1) r = 0.0;
    work[n] = r;
    n2 = n2 + r * r;
  }
  return sqrt(n2);
}

/* One time step of NumericalSolution for a single GWF model:
 * prepareSolve (gwf_ad, chd_ad) then the Picard/Newton outer loop of
 * sln_ca/solve (NumericalSolution.f90:1287-1322, 1482-1837) with sln_ls
 * (:2404-2615) including pseudo-transient continuation for steady-state
 * Newton models (gwf.f90:625-687).  Backtracking is not restated
 * (numtrack must be 0).  Returns 0 on success. */
int or_gwf_timestep(const or_gwf_model *m, or_ims *ims, or_nonlinear *nl,
                    const double *condsat, int *ibound, int kper, int kstp, double delt,
                    int transient, double *x, double *xold, or_timestep_stats *st) {
  int neq = m->nodes, nja = SNJA(m);
  double *amat = (double *)calloc(nja, sizeof(double));
  double *rhs = (double *)calloc(neq, sizeof(double));
  double *sat = (double *)calloc(neq, sizeof(double));
  double *xtemp = (double *)calloc(neq, sizeof(double));
  double *work = (double *)calloc(neq, sizeof(double));
  /* npf_ar's initial saturation (gwf-npf.f90:1853-1884): 1 in every cell;
   * npf_cf updates the convertible ones */
  for (int n = 0; n < neq; ++n) sat[n] = 1.0;
  /* gwf_ad: xold = x ; chd_ad: x = xold = chd head */
  for (int n = 0; n < neq; ++n) xold[n] = x[n];
  for (int i = 0; i < m->nchd; ++i) {
    x[m->chd_node[i]] = m->chd_head[i];
    xold[m->chd_node[i]] = m->chd_head[i];
  }
  int isymmetric = (ims_ilinmeth(ims) == 1);
  int steady = !transient;
  memset(st, 0, sizeof(*st));
  int converged = 0;
  double l2norm0_ptc = 0.0, ptcdel = 0.0;
  for (int kiter = 1; kiter <= nl->mxiter; ++kiter) {
    if (nl->numtrack > 0) {
      /* sln_backtracking (NumericalSolution.f90:2680-2760): the system
       * without Newton terms (sln_buildsystem with inewton = 0) and its
       * residual L2 norm; from the second outer iteration on, while the
       * norm exceeds BTOL x the previous one, the last change is cut by
       * BREDUC (get_backtracking_flag :2795-2817, apply_backtracking
       * :2823-2838) */
      memset(amat, 0, sizeof(double) * nja);
      memset(rhs, 0, sizeof(double) * neq);
      gwf_fc_flag(m, ibound, condsat, sat, delt, transient, xold, x, amat, rhs, 0);
      double l2 = sln_l2norm(neq, SIA(m), SJA(m), amat, x, rhs, ibound, work);
      if (kiter == 1) {
        nl->res_prev = l2;
      } else {
        nl->res_new = l2;
        if (nl->res_new > nl->res_prev * nl->btol) {
          for (int nb = 1; nb <= nl->numtrack; ++nb) {
            double dx_abs_max = 0.0;
            for (int n = 0; n < neq; ++n) {
              if (ibound[n] < 1) continue;
              double dx_abs = fabs(x[n] - xtemp[n]);
              if (dx_abs > dx_abs_max) dx_abs_max = dx_abs;
            }
            if (!(nl->breduc * dx_abs_max >= nl->dvclose)) break;
            for (int n = 0; n < neq; ++n) {
              if (ibound[n] < 1) continue;
              double delx = nl->breduc * (x[n] - xtemp[n]);
              x[n] = xtemp[n] + delx;
            }
            st->backtracks += 1;
            memset(amat, 0, sizeof(double) * nja);
            memset(rhs, 0, sizeof(double) * neq);
            gwf_fc_flag(m, ibound, condsat, sat, delt, transient, xold, x, amat, rhs, 0);
            nl->res_new = sln_l2norm(neq, SIA(m), SJA(m), amat, x, rhs, ibound, work);
            if (nb == nl->numtrack) break;
            if (nl->res_new < nl->res_prev * nl->btol) break;
            if (nl->res_new < nl->res_lim) break;
          }
        }
        nl->res_prev = nl->res_new;
      }
    }
    memset(amat, 0, sizeof(double) * nja);
    memset(rhs, 0, sizeof(double) * neq);
    or_gwf_fc(m, ibound, condsat, sat, delt, transient, xold, x, amat, rhs);
    /* sln_calc_ptc -> gwf_ptc */
    int iptc = 0;
    double ptcf = 0.0;
    int iptct = (steady && m->inewton > 0) ? 1 : 0;
    if (iptct > 0) {
      or_amux(neq, x, work, amat, SJA(m), SIA(m));
      for (int n = 0; n < neq; ++n) {
        work[n] = work[n] - rhs[n];
        if (ibound[n] < 1) work[n] = 0.0;
      }
      for (int n = 0; n < neq; ++n) {
        if (ibound[n] < 1) continue;
        double v = m->area[n] * (m->top[n] - m->bot[n]);
        double ptcdelem1 = fabs(work[n]) / v;
        if (ptcdelem1 > ptcf) ptcf = ptcdelem1;
      }
      if (ptcf == 0.0) ptcf = 1.0 / (delt * 10.0);
      iptc = 1;
    }
    /* sln_ls */
    or_sln_ls_fixups(neq, SIA(m), SJA(m), ibound, isymmetric, amat, rhs, x, xtemp);
    int iallowptc = nl->iallowptc;
    if (iallowptc < 0) iallowptc = (kper > 1) ? 1 : 0;
    iptct = iptc * iallowptc;
    if (iptct != 0) {
      double l2norm = sln_l2norm(neq, SIA(m), SJA(m), amat, x, rhs, ibound, work);
      if (kiter == 1) {
        if (kper > 1 || kstp > 1) {
          if (l2norm <= l2norm0_ptc) iptc = 0;
        }
      } else {
        if (or_is_close(l2norm, l2norm0_ptc)) iptc = 0;
      }
      iptct = iptc * iallowptc;
      if (iptct != 0) {
        if (kiter == 1) {
          ptcdel = 1.0 / ptcf; /* iptcopt = 0, ptcdel0 = 0 */
        } else {
          if (l2norm > 0.0) ptcdel = ptcdel * (l2norm0_ptc / l2norm); /* ptcexp = 1 */
          else ptcdel = 0.0;
        }
        double ptcval = (ptcdel > 0.0) ? 1.0 / ptcdel : 1.0;
        for (int ieq = 0; ieq < neq; ++ieq) {
          if (ibound[ieq] > 0) {
            amat[SIA(m)[ieq]] = amat[SIA(m)[ieq]] + (-ptcval);
            rhs[ieq] = rhs[ieq] - ptcval * x[ieq];
          }
        }
        l2norm0_ptc = l2norm;
      }
    }
    int icnvg = 0, in_iter = 0;
    int rc = or_ims_apply(ims, amat, rhs, x, kstp, kiter, &icnvg, &in_iter, NULL, 0);
    if (rc != 0) {
      free(amat); free(rhs); free(sat); free(xtemp); free(work);
      return rc;
    }
    st->inner_total += in_iter;
    st->outer = kiter;
    st->pivot_retries += or_ims_pivot_retries(ims);
    int lrch;
    double hncg = or_sln_get_dxmax(neq, ibound, x, xtemp, &lrch);
    st->last_dxmax = hncg;
    int cnvg = fabs(hncg) <= nl->dvclose;
    if (!cnvg) {
      if (nl->nonmeth > 0) or_sln_underrelax(nl, kiter, hncg, neq, ibound, x, xtemp);
      else
        for (int n = 0; n < neq; ++n) nl->dxold[n] = (ibound[n] < 1) ? 0.0 : x[n] - xtemp[n];
      if (m->inewton && m->inewtonur) { /* gwf_nur, gwf.f90:717 */
        int inewtonur = 0, locmax = -1;
        double dxmax_nur = 0.0;
        or_npf_nur(m, ibound, x, xtemp, nl->dxold, &inewtonur, &dxmax_nur, &locmax);
        if (inewtonur != 0) {
          double dxold_max = sln_maxval(neq, nl->dxold);
          if (fabs(dxold_max) <= nl->dvclose && fabs(hncg) <= nl->dvclose) {
            cnvg = 1;
            hncg = or_sln_get_dxmax(neq, ibound, x, xtemp, &lrch);
          }
        }
      }
    }
    if (cnvg) {
      converged = 1;
      break;
    }
  }
  st->converged = converged;
  free(amat); free(rhs); free(sat); free(xtemp); free(work);
  return 0;
}
