/*
 * xt3d_oracle.c -- CPU restatement of XT3D, the NPF formulation with the
 * full conductivity tensor and the extended stencil (Xt3dInterface.f90,
 * Xt3dAlgorithm.f90), matrix form (XT3D without RHS), on DIS, DISV and
 * DISU grids.
 * TEST INFRASTRUCTURE ONLY (the oracle); the product never includes this.
 *
 * Loops, branches and the order of every sum follow the Fortran.  Arrays are
 * 0-based; a neighbour slot holds its cell number or -1 where the Fortran
 * holds 0 (an inactive neighbour).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "gwf_oracle.h"

#define NBRMX 32

/* xt3d_fillrmatck (Xt3dInterface.f90:1577-1613) and the tensor of xt3d_load
 * (:1230-1237): ck = R diag(k11, k22, k33) R^T, row-major, angles in
 * radians; nozee drops angle2 and angle3. */
void or_xt3d_ck(int nodes, const double *k11, const double *k22, const double *k33,
                const double *angle1, const double *angle2, const double *angle3, int nozee,
                double *ck) {
  for (int n = 0; n < nodes; ++n) {
    double ang1 = angle1[n], ang2 = 0.0, ang3 = 0.0;
    if (!nozee) {
      ang2 = angle2[n];
      ang3 = angle3[n];
    }
    double s1 = sin(ang1), c1 = cos(ang1), s2 = sin(ang2), c2 = cos(ang2), s3 = sin(ang3),
           c3 = cos(ang3);
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
    double d[3][3] = {{k11[n], 0.0, 0.0}, {0.0, k22[n], 0.0}, {0.0, 0.0, k33[n]}};
    double t[3][3], c[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s = s + r[i][k] * d[k][j];
        t[i][j] = s;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s = s + t[i][k] * r[j][k];
        c[i][j] = s;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) ck[9 * (size_t)n + 3 * i + j] = c[i][j];
  }
}

/* The solution's pattern with XT3D (xt3d_ac, Xt3dInterface.f90:124-189):
 * each row holds the model's connections and every neighbour of a
 * neighbour, the diagonal first and the rest ascending (Sparse.f90:217-239).
 * idxglo maps each model position to its solution position.  Returns the
 * solution's nja, or -1 if cap is too small. */
int or_xt3d_pattern(int nodes, const int *ia, const int *ja, int cap, int *sia, int *sja,
                    int *idxglo) {
  int nja = 0;
  sia[0] = 0;
  for (int n = 0; n < nodes; ++n) {
    int start = nja;
    if (nja >= cap) return -1;
    sja[nja++] = n;
    for (int pass = 0; pass < 2; ++pass)
      for (int ii = ia[n] + 1; ii < ia[n + 1]; ++ii) {
        int j = ja[ii];
        int lo = (pass == 0) ? ii : ia[j] + 1, hi = (pass == 0) ? ii + 1 : ia[j + 1];
        for (int kk = lo; kk < hi; ++kk) {
          int k = (pass == 0) ? j : ja[kk];
          int dup = 0;
          for (int t = start; t < nja; ++t)
            if (sja[t] == k) dup = 1;
          if (dup) continue;
          if (nja >= cap) return -1;
          sja[nja++] = k;
        }
      }
    /* sort the off-diagonals */
    for (int a = start + 2; a < nja; ++a) {
      int v = sja[a], b = a - 1;
      while (b > start && sja[b] > v) {
        sja[b + 1] = sja[b];
        --b;
      }
      sja[b + 1] = v;
    }
    sia[n + 1] = nja;
  }
  for (int n = 0; n < nodes; ++n)
    for (int ii = ia[n]; ii < ia[n + 1]; ++ii)
      for (int p = sia[n]; p < sia[n + 1]; ++p)
        if (sja[p] == ja[ii]) {
          idxglo[ii] = p;
          break;
        }
  return nja;
}

/* ---- XT3D state of one formulate -------------------------------------- */

typedef struct {
  const or_gwf_model *m;
  const int *ibound;
  const double *sat;
  int nbrmax;
  /* extended neighbours: ext[n] = the neighbours of n's neighbours */
  int *ext_ia, *ext_ja;
  /* iallpc (Xt3dInterface.f90:1109-1179) and lamatsaved */
  int *iallpc;
  int lamatsaved;
} xt3d_t;

static int pos_in(const int *ia, const int *ja, int n, int col) {
  for (int p = ia[n]; p < ia[n + 1]; ++p)
    if (ja[p] == col) return p;
  return -1;
}

/* get_ijk (GeomUtil.f90:99-123), 0-based */
static void ijk(const or_gwf_model *m, int node, int *i, int *j, int *k) {
  int nrc = m->nrow * m->ncol;
  *k = node / nrc;
  int ij = node - *k * nrc;
  *i = ij / m->ncol;
  *j = ij - *i * m->ncol;
}

/* connection_normal (Dis.f90:1039-1087) */
static void dis_normal(const or_gwf_model *m, int n, int nm, int ihc, double *v) {
  v[0] = 0.0;
  v[1] = 0.0;
  v[2] = 0.0;
  if (ihc == 0) {
    v[2] = (nm < n) ? 1.0 : -1.0;
  } else {
    int i1, j1, k1, i2, j2, k2;
    ijk(m, n, &i1, &j1, &k1);
    ijk(m, nm, &i2, &j2, &k2);
    if (i2 < i1) v[1] = 1.0;
    else if (j2 < j1) v[0] = -1.0;
    else if (j2 > j1) v[0] = 1.0;
    else v[1] = -1.0;
  }
}

/* connection_vector (Dis.f90:1094-1160) with line_unit_vector
 * (DisvGeom.f90:473-496) */
static void dis_vector(const or_gwf_model *m, int n, int nm, int nozee, double satn,
                       double satm, int ihc, double *v, double *conlen) {
  if (ihc == 0) {
    v[0] = 0.0;
    v[1] = 0.0;
    v[2] = (nm < n) ? 1.0 : -1.0;
    double z1 = m->bot[n] + 0.5 * (m->top[n] - m->bot[n]);
    double z2 = m->bot[nm] + 0.5 * (m->top[nm] - m->bot[nm]);
    *conlen = fabs(z2 - z1);
  } else {
    double z1, z2;
    if (nozee) {
      z1 = 0.0;
      z2 = 0.0;
    } else {
      z1 = m->bot[n] + 0.5 * satn * (m->top[n] - m->bot[n]);
      z2 = m->bot[nm] + 0.5 * satm * (m->top[nm] - m->bot[nm]);
    }
    int ipos = pos_in(m->ia, m->ja, n, nm);
    int s = m->jas[ipos];
    double ds = m->cl1[s] + m->cl2[s];
    int i1, j1, k1, i2, j2, k2;
    ijk(m, n, &i1, &j1, &k1);
    ijk(m, nm, &i2, &j2, &k2);
    double x1 = 0.0, x2 = 0.0, y1 = 0.0, y2 = 0.0;
    if (i2 < i1) y2 = ds;
    else if (j2 < j1) x2 = -ds;
    else if (j2 > j1) x2 = ds;
    else y2 = -ds;
    double dx = x2 - x1, dy = y2 - y1, dz = z2 - z1;
    double vmag = sqrt(dx * dx + dy * dy + dz * dz);
    v[0] = dx / vmag;
    v[1] = dy / vmag;
    v[2] = dz / vmag;
    *conlen = vmag;
  }
}

/* line_unit_vector (DisvGeom.f90:473-496) */
static void unit_vector(double x0, double y0, double z0, double x1, double y1, double z1,
                        double *v, double *vmag) {
  double dx = x1 - x0, dy = y1 - y0, dz = z1 - z0;
  *vmag = sqrt(dx * dx + dy * dy + dz * dz);
  v[0] = dx / *vmag;
  v[1] = dy / *vmag;
  v[2] = dz / *vmag;
}

/* connection_normal: DIS (Dis.f90:1039-1087); DISV and DISU from anglex
 * (Disv.f90:979-1018, Disu.f90:1062-1102) */
static void conn_normal(const or_gwf_model *m, int n, int nm, int ihc, int ipos, double *v) {
  if (m->xt_grid == 0) {
    dis_normal(m, n, nm, ihc, v);
    return;
  }
  if (ihc == 0) {
    v[0] = 0.0;
    v[1] = 0.0;
    v[2] = (nm < n) ? 1.0 : -1.0;
  } else {
    double angle = m->anglex[m->jas[ipos]];
    double dmult = (nm < n) ? -1.0 : 1.0;
    v[0] = cos(angle) * dmult;
    v[1] = sin(angle) * dmult;
    v[2] = 0.0;
  }
}

/* connection_vector: DIS (Dis.f90:1094-1160), DISV (Disv.f90:1024-1080:
 * vertical as DIS, horizontal between the cell centres) and DISU
 * (Disu.f90:1108-1164: between the cell centres, vertical ones included) */
static void conn_vector(const or_gwf_model *m, int n, int nm, int nozee, double satn,
                        double satm, int ihc, double *v, double *conlen) {
  if (m->xt_grid == 0 || (m->xt_grid == 1 && ihc == 0)) {
    dis_vector(m, n, nm, nozee, satn, satm, ihc, v, conlen);
    return;
  }
  double zn, zm;
  if (ihc == 0) {
    zn = m->bot[n] + 0.5 * (m->top[n] - m->bot[n]);
    zm = m->bot[nm] + 0.5 * (m->top[nm] - m->bot[nm]);
  } else if (nozee) {
    zn = 0.0;
    zm = 0.0;
  } else {
    zn = m->bot[n] + 0.5 * satn * (m->top[n] - m->bot[n]);
    zm = m->bot[nm] + 0.5 * satm * (m->top[nm] - m->bot[nm]);
  }
  unit_vector(m->xc[n], m->yc[n], zn, m->xc[nm], m->yc[nm], zm, v, conlen);
}

/* xt3d_load (Xt3dInterface.f90:1211-1275) */
static void xt3d_load(const xt3d_t *x, int n, int nnbr, int *inbr, double vc[][3],
                      double vn[][3], double *dl, double *dln, int *allhc) {
  const or_gwf_model *m = x->m;
  *allhc = 1;
  for (int il = 0; il < nnbr; ++il) {
    int ii = il + 1 + m->ia[n];
    int jj = m->ja[ii];
    int jjs = m->jas[ii];
    if (x->ibound[jj] != 0) {
      inbr[il] = jj;
      double satn = x->sat[n], satjj = x->sat[jj];
      int ihc = m->ihc[jjs];
      double dltot;
      conn_normal(m, n, jj, ihc, ii, vn[il]);
      conn_vector(m, n, jj, m->nozee, satn, satjj, ihc, vc[il], &dltot);
      double cl1njj, cl2njj;
      if (jj > n) {
        cl1njj = m->cl1[jjs];
        cl2njj = m->cl2[jjs];
      } else {
        cl1njj = m->cl2[jjs];
        cl2njj = m->cl1[jjs];
      }
      double ooclsum = 1.0 / (cl1njj + cl2njj);
      dl[il] = dltot * cl1njj * ooclsum;
      dln[il] = dltot * cl2njj * ooclsum;
      if (m->ihc[jjs] == 0) *allhc = 0;
    } else {
      inbr[il] = -1;
    }
  }
}

/* getrot (Xt3dAlgorithm.f90:283-357) */
static void getrot(int nnbr, const int *inbr, double vc[][3], int il01, double rmat[3][3],
                   int *iml0) {
  double vcc[3] = {vc[il01][0], vc[il01][1], vc[il01][2]};
  double acmpmn = 1.0 - 1e-10, cmpmn = 0.0;
  *iml0 = -1;
  for (int il = 0; il < nnbr; ++il) {
    if (il == il01 || inbr[il] < 0) continue;
    double cmp = vc[il][0] * vcc[0] + vc[il][1] * vcc[1] + vc[il][2] * vcc[2];
    double acmp = fabs(cmp);
    if (acmp < acmpmn) {
      cmpmn = cmp;
      acmpmn = acmp;
      *iml0 = il;
    }
  }
  if (*iml0 < 0) {
    for (int i = 0; i < 3; ++i) rmat[i][0] = vcc[i];
    return;
  }
  double vcd[3], vce[3];
  for (int i = 0; i < 3; ++i) vcd[i] = vc[*iml0][i] - cmpmn * vcc[i];
  double s = sqrt(1.0 - cmpmn * cmpmn);
  for (int i = 0; i < 3; ++i) vcd[i] = vcd[i] / s;
  vce[0] = vcc[1] * vcd[2] - vcc[2] * vcd[1];
  vce[1] = vcc[2] * vcd[0] - vcc[0] * vcd[2];
  vce[2] = vcc[0] * vcd[1] - vcc[1] * vcd[0];
  for (int i = 0; i < 3; ++i) {
    rmat[i][0] = vcc[i];
    rmat[i][1] = vcd[i];
    rmat[i][2] = vce[i];
  }
}

/* abwts (Xt3dAlgorithm.f90:389-490); nde1 is 1 (d) or 2 (e), 0-based */
static void abwts(int nnbr, const int *inbr, int il01, int nde1, double vccde[][3],
                  double vcthresh, const double *dl0, const double *dln, double *acd,
                  double *add, double *aed, double *bd) {
  int nde2 = 3 - nde1;
  double omwt[NBRMX];
  double dsum = 0.0, vcmx = 0.0;
  for (int il = 0; il < nnbr; ++il) omwt[il] = 0.0;
  for (int il = 0; il < nnbr; ++il) {
    if (il == il01 || inbr[il] < 0) continue;
    double a = fabs(vccde[il][nde1]);
    vcmx = (a > vcmx) ? a : vcmx;
    double dlm = 0.5 * (dl0[il] + dln[il]);
    double cosang = vccde[il][0];
    double dl4wt = sqrt(dlm * dlm + dl0[il01] * dl0[il01] - 2.0 * dlm * dl0[il01] * cosang);
    omwt[il] = fabs(vccde[il][nde1]) * dl4wt;
    dsum = dsum + omwt[il];
  }
  dsum = dsum + 1e-10 * dsum;
  for (int il = 0; il < nnbr; ++il) {
    if (il == il01 || inbr[il] < 0) continue;
    double fact = dsum - omwt[il];
    omwt[il] = fact * fabs(vccde[il][nde1]);
  }
  for (int il = 0; il < nnbr; ++il) bd[il] = 0.0;
  dsum = 0.0;
  for (int il = 0; il < nnbr; ++il) {
    if (il == il01 || inbr[il] < 0) continue;
    bd[il] = omwt[il] * copysign(1.0, vccde[il][nde1]);
    dsum = dsum + omwt[il] * fabs(vccde[il][nde1]);
  }
  double oodsum = 1.0 / dsum;
  for (int il = 0; il < nnbr; ++il) {
    if (il == il01 || inbr[il] < 0) continue;
    bd[il] = bd[il] * oodsum;
  }
  *add = 1.0;
  *acd = 0.0;
  *aed = 0.0;
  for (int il = 0; il < nnbr; ++il) {
    if (il == il01 || inbr[il] < 0) continue;
    *acd = *acd + bd[il] * vccde[il][0];
    *aed = *aed + bd[il] * vccde[il][nde2];
  }
  if (vcmx < vcthresh) {
    double fatten = vcmx / vcthresh;
    *acd = *acd * fatten;
    *aed = *aed * fatten;
    for (int il = 0; il < nnbr; ++il) bd[il] = bd[il] * fatten;
  }
}

/* abhats (Xt3dAlgorithm.f90:127-272) */
static void abhats(int nnbr, const int *inbr, int il01, double vc[][3], double vn[][3],
                   const double *dl0, const double *dln, const double *ck, double vcthresh,
                   int allhc, double ar01, double *ahat, double *bhat) {
  double rmat[3][3];
  int iml0;
  getrot(nnbr, inbr, vc, il01, rmat, &iml0);
  if (iml0 < 0) {
    double w[3];
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s = s + ck[3 * i + k] * rmat[k][0];
      w[i] = s;
    }
    double sigma1 = 0.0;
    for (int i = 0; i < 3; ++i) sigma1 = sigma1 + vn[il01][i] * w[i];
    *ahat = sigma1 / dl0[il01];
    for (int il = 0; il < nnbr; ++il) bhat[il] = 0.0;
  } else {
    double vccde[NBRMX][3];
    for (int il = 0; il < nnbr; ++il)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int i = 0; i < 3; ++i) s = s + rmat[i][j] * vc[il][i];
        vccde[il][j] = s;
      }
    double acd, add, aed, bd[NBRMX];
    abwts(nnbr, inbr, il01, 1, vccde, vcthresh, dl0, dln, &acd, &add, &aed, bd);
    double ace, aee, ade, be[NBRMX];
    int zero_e = 1;
    if (!allhc) {
      int iscomp = 0;
      for (int il = 0; il < nnbr; ++il) {
        if (il == il01 || inbr[il] < 0) continue;
        if (fabs(vccde[il][2]) > 1e-10) {
          iscomp = 1;
          break;
        }
      }
      if (iscomp) {
        abwts(nnbr, inbr, il01, 2, vccde, vcthresh, dl0, dln, &ace, &aee, &ade, be);
        zero_e = 0;
      }
    }
    if (zero_e) {
      ace = 0.0;
      aee = 1.0;
      ade = 0.0;
      for (int il = 0; il < nnbr; ++il) be[il] = 0.0;
    }
    double determ = add * aee - ade * aed;
    double oodet = 1.0 / determ;
    double alphad = (acd * aee - ace * aed) * oodet;
    double alphae = (ace * add - acd * ade) * oodet;
    double betad[NBRMX], betae[NBRMX];
    for (int il = 0; il < nnbr; ++il) {
      betad[il] = 0.0;
      betae[il] = 0.0;
    }
    for (int il = 0; il < nnbr; ++il) {
      if (il == il01 || inbr[il] < 0) continue;
      betad[il] = (bd[il] * aee - be[il] * aed) * oodet;
      betae[il] = (be[il] * add - bd[il] * ade) * oodet;
    }
    /* sigma = matmul(vn(il01,:), matmul(ck, rmat)) */
    double cr[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s = s + ck[3 * i + k] * rmat[k][j];
        cr[i][j] = s;
      }
    double sigma[3];
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int i = 0; i < 3; ++i) s = s + vn[il01][i] * cr[i][j];
      sigma[j] = s;
    }
    *ahat = (sigma[0] - sigma[1] * alphad - sigma[2] * alphae) / dl0[il01];
    for (int il = 0; il < nnbr; ++il) bhat[il] = 0.0;
    for (int il = 0; il < nnbr; ++il) {
      if (il == il01 || inbr[il] < 0) continue;
      double dl0il = dl0[il] + dln[il];
      bhat[il] = (sigma[1] * betad[il] + sigma[2] * betae[il]) / dl0il;
    }
    bhat[il01] = 0.0;
  }
  *ahat = *ahat * ar01;
  for (int il = 0; il < nnbr; ++il) bhat[il] = bhat[il] * ar01;
}

/* qconds (Xt3dAlgorithm.f90:47-121); the chat arrays have nbrmax entries */
static void qconds(int nbrmax, int nnbr0, const int *inbr0, int il01, double vc0[][3],
                   double vn0[][3], const double *dl0, const double *dl0n, const double *ck0,
                   int nnbr1, const int *inbr1, int il10, double vc1[][3], double vn1[][3],
                   const double *dl1, const double *dl1n, const double *ck1, double ar01,
                   double ar10, double vcthresh, int allhc0, int allhc1, double *chat01,
                   double *chati0, double *chat1j) {
  if (ar01 == 0.0) {
    *chat01 = 0.0;
    for (int i = 0; i < nbrmax; ++i) {
      chati0[i] = 0.0;
      chat1j[i] = 0.0;
    }
    return;
  }
  double ahat0, ahat1, bhat0[NBRMX], bhat1[NBRMX];
  for (int i = 0; i < NBRMX; ++i) {
    bhat0[i] = 0.0;
    bhat1[i] = 0.0;
  }
  abhats(nnbr0, inbr0, il01, vc0, vn0, dl0, dl0n, ck0, vcthresh, allhc0, ar01, &ahat0, bhat0);
  abhats(nnbr1, inbr1, il10, vc1, vn1, dl1, dl1n, ck1, vcthresh, allhc1, ar10, &ahat1, bhat1);
  double denom = ahat0 + ahat1;
  double wght1 = (fabs(denom) > 2.220446049250313e-16) ? ahat0 / (ahat0 + ahat1) : 1.0;
  double wght0 = 1.0 - wght1;
  *chat01 = wght1 * ahat1;
  for (int i = 0; i < nbrmax; ++i) {
    chati0[i] = wght0 * bhat0[i];
    chat1j[i] = wght1 * bhat1[i];
  }
}

/* xt3d_areas (Xt3dInterface.f90:1300-1379) */
static void xt3d_areas(const xt3d_t *x, int n, int mm, int jjs01, int lsat, double *ar01,
                       double *ar10, const double *hnew) {
  const or_gwf_model *m = x->m;
  if (m->ihc[jjs01] == 0) {
    *ar01 = m->hwva[jjs01];
    *ar10 = *ar01;
  } else if (m->inewton != 0) {
    if (lsat) {
      double topn = m->top[n], botn = m->bot[n], topm = m->top[mm], botm = m->bot[mm];
      double thksatn = topn - botn, thksatm = topm - botm;
      if (m->ihc[jjs01] == 2) {
        double sill_top = (topn < topm) ? topn : topm;
        double sill_bot = (botn > botm) ? botn : botm;
        double tpn = botn + thksatn, tpm = botm + thksatm;
        double a = ((tpn < sill_top) ? tpn : sill_top) - sill_bot;
        double b = ((tpm < sill_top) ? tpm : sill_top) - sill_bot;
        thksatn = (a > 0.0) ? a : 0.0;
        thksatm = (b > 0.0) ? b : 0.0;
      }
      *ar01 = m->hwva[jjs01] * 0.5 * (thksatn + thksatm);
    } else {
      double satups = (hnew[mm] < hnew[n]) ? x->sat[n] : x->sat[mm];
      *ar01 = *ar01 * satups;
    }
    *ar10 = *ar01;
  } else {
    double topn = m->top[n], botn = m->bot[n], topm = m->top[mm], botm = m->bot[mm];
    double thksatn = topn - botn, thksatm = topm - botm;
    if (!lsat) {
      thksatn = x->sat[n] * thksatn;
      thksatm = x->sat[mm] * thksatm;
    }
    if (m->ihc[jjs01] == 2) {
      double sill_top = (topn < topm) ? topn : topm;
      double sill_bot = (botn > botm) ? botn : botm;
      double tpn = botn + thksatn, tpm = botm + thksatm;
      double a = ((tpn < sill_top) ? tpn : sill_top) - sill_bot;
      double b = ((tpm < sill_top) ? tpm : sill_top) - sill_bot;
      thksatn = (a > 0.0) ? a : 0.0;
      thksatm = (b > 0.0) ? b : 0.0;
    }
    *ar01 = m->hwva[jjs01] * thksatn;
    *ar10 = m->hwva[jjs01] * thksatm;
  }
}

/* position of (n, col) among n's extended neighbours, in solution-row
 * order (jax, xt3d_mc :191-271), or -1; ext_base[n] is the first index */
static int ext_index(const xt3d_t *x, int n, int col, const int *ext_base) {
  const or_gwf_model *m = x->m;
  int k = ext_base[n];
  for (int p = m->sia[n]; p < m->sia[n + 1]; ++p) {
    int c = m->sja[p];
    if (pos_in(x->ext_ia, x->ext_ja, n, c) >= 0) {
      if (c == col) return k;
      ++k;
    }
  }
  return -1;
}

static int xt3d_setup(xt3d_t *x, const or_gwf_model *m, const int *ibound, const double *sat) {
  x->m = m;
  x->ibound = ibound;
  x->sat = sat;
  int nodes = m->nodes;
  x->nbrmax = 0;
  for (int n = 0; n < nodes; ++n) {
    int nn = m->ia[n + 1] - m->ia[n] - 1;
    if (nn > x->nbrmax) x->nbrmax = nn;
  }
  if (x->nbrmax > NBRMX) return -1;
  /* neighbours of neighbours (xt3d_ac) */
  x->ext_ia = (int *)malloc(sizeof(int) * (nodes + 1));
  int cap = 0;
  for (int n = 0; n < nodes; ++n)
    for (int ii = m->ia[n] + 1; ii < m->ia[n + 1]; ++ii) cap += m->ia[m->ja[ii] + 1] - m->ia[m->ja[ii]];
  x->ext_ja = (int *)malloc(sizeof(int) * (cap + 1));
  int e = 0;
  x->ext_ia[0] = 0;
  for (int i = 0; i < nodes; ++i) {
    int start = e;
    for (int jj = m->ia[i] + 1; jj < m->ia[i + 1]; ++jj) {
      int j = m->ja[jj];
      for (int kk = m->ia[j] + 1; kk < m->ia[j + 1]; ++kk) {
        int k = m->ja[kk];
        int dup = 0;
        for (int t = start; t < e; ++t)
          if (x->ext_ja[t] == k) dup = 1;
        if (!dup) x->ext_ja[e++] = k;
      }
    }
    x->ext_ia[i + 1] = e;
  }
  /* iallpc */
  x->iallpc = (int *)malloc(sizeof(int) * nodes);
  for (int n = 0; n < nodes; ++n) x->iallpc[n] = 1;
  for (int n = 0; n < nodes; ++n) {
    if (m->icelltype[n] != 0) {
      x->iallpc[n] = 0;
      continue;
    }
    for (int ii = m->ia[n] + 1; ii < m->ia[n + 1]; ++ii) {
      int mm = ibound[m->ja[ii]] != 0 ? m->ja[ii] : -1;
      if (mm < n) continue;
      if (m->icelltype[mm] != 0) {
        x->iallpc[n] = 0;
        x->iallpc[mm] = 0;
        continue;
      }
      for (int kk = m->ia[mm] + 1; kk < m->ia[mm + 1]; ++kk) {
        int q = ibound[m->ja[kk]] != 0 ? m->ja[kk] : -1;
        /* an inactive neighbour reads icelltype(0) in the Fortran, which is
         * outside the array; it is taken as confined here */
        if (q >= 0 && m->icelltype[q] != 0) {
          x->iallpc[n] = 0;
          x->iallpc[mm] = 0;
          x->iallpc[q] = 0;
        }
      }
    }
  }
  x->lamatsaved = 0;
  for (int n = 0; n < nodes; ++n)
    if (x->iallpc[n] == 1) x->lamatsaved = 1;
  if (m->ixt3d == 2) x->lamatsaved = 0; /* the RHS form saves nothing */
  return 0;
}

static void xt3d_free(xt3d_t *x) {
  free(x->ext_ia);
  free(x->ext_ja);
  free(x->iallpc);
}

/* The coefficients of connection (n, mm) (the body of xt3d_fc's loop,
 * :416-465, and of xt3d_fcpc's, :529-561).  mode 0: xt3d_fc; mode 1:
 * xt3d_fcpc (lsat areas, no Newton scaling).  Fills chat01, chati0,
 * chat1j; qsat gets the saturated flow under Newton. */
static void pair_coefs(const xt3d_t *x, int n, int il0, int mode, const double *hnew,
                       double *chat01, double *chati0, double *chat1j, double *qsat,
                       int *inbr0, int *inbr1, int *nnbr0_out, int *nnbr1_out, int *il10_out) {
  const or_gwf_model *m = x->m;
  int nnbr0 = m->ia[n + 1] - m->ia[n] - 1;
  double vc0[NBRMX][3], vn0[NBRMX][3], dl0[NBRMX], dl0n[NBRMX];
  double vc1[NBRMX][3], vn1[NBRMX][3], dl1[NBRMX], dl1n[NBRMX];
  int allhc0, allhc1;
  xt3d_load(x, n, nnbr0, inbr0, vc0, vn0, dl0, dl0n, &allhc0);
  int mm = inbr0[il0];
  int nnbr1 = m->ia[mm + 1] - m->ia[mm] - 1;
  xt3d_load(x, mm, nnbr1, inbr1, vc1, vn1, dl1, dl1n, &allhc1);
  int ii01 = m->ia[n] + 1 + il0;
  int jjs01 = m->jas[ii01];
  int iinm = pos_in(m->ia, m->ja, mm, n);
  int il10 = iinm - m->ia[mm] - 1;
  const double *ck0 = m->ck + 9 * (size_t)n, *ck1 = m->ck + 9 * (size_t)mm;
  double ar01, ar10;
  if (mode == 1) {
    xt3d_areas(x, n, mm, jjs01, 1, &ar01, &ar10, hnew);
  } else if (m->inewton != 0) {
    ar01 = 1.0;
    ar10 = 1.0;
  } else {
    xt3d_areas(x, n, mm, jjs01, 0, &ar01, &ar10, hnew);
  }
  qconds(x->nbrmax, nnbr0, inbr0, il0, vc0, vn0, dl0, dl0n, ck0, nnbr1, inbr1, il10, vc1, vn1,
         dl1, dl1n, ck1, ar01, ar10, 1e-10, allhc0, allhc1, chat01, chati0, chat1j);
  if (mode == 0 && m->inewton != 0) {
    double qnm = *chat01 * (hnew[mm] - hnew[n]);
    double qnbrs = 0.0;
    for (int iil = 0; iil < nnbr0; ++iil)
      if (inbr0[iil] >= 0) {
        int jjj = m->ja[m->ia[n] + 1 + iil];
        qnbrs = qnbrs + chati0[iil] * (hnew[jjj] - hnew[n]);
      }
    qnm = qnm + qnbrs;
    qnbrs = 0.0;
    for (int iil = 0; iil < nnbr1; ++iil)
      if (inbr1[iil] >= 0) {
        int jjj = m->ja[m->ia[mm] + 1 + iil];
        qnbrs = qnbrs + chat1j[iil] * (hnew[jjj] - hnew[mm]);
      }
    qnm = qnm - qnbrs;
    xt3d_areas(x, n, mm, jjs01, 1, &ar01, &ar10, hnew);
    *qsat = qnm * ar01;
    xt3d_areas(x, n, mm, jjs01, 0, &ar01, &ar10, hnew);
    *chat01 = *chat01 * ar01;
    for (int i = 0; i < x->nbrmax; ++i) {
      chati0[i] = chati0[i] * ar01;
      chat1j[i] = chat1j[i] * ar01;
    }
  }
  *nnbr0_out = nnbr0;
  *nnbr1_out = nnbr1;
  *il10_out = il10;
}

/* xt3d_fc (Xt3dInterface.f90:371-497) with xt3d_fcpc (:499-571) for the
 * permanently confined cells, whose coefficients are made with every
 * saturation 1 (npf_ar's initial sat), as the reference makes them once at
 * allocation.  amat is in the solution pattern; qsat (model nja) gets the
 * saturated flows under Newton. */
int or_xt3d_fc(const or_gwf_model *m, const int *ibound, const double *sat,
               const double *hnew, double *amat, double *rhs, double *qsat) {
  xt3d_t x;
  double *one = (double *)malloc(sizeof(double) * m->nodes);
  for (int n = 0; n < m->nodes; ++n) one[n] = 1.0;
  if (xt3d_setup(&x, m, ibound, one) != 0) {
    free(one);
    return -1;
  }
  int nodes = m->nodes;
  int *ext_base = (int *)malloc(sizeof(int) * (nodes + 1));
  ext_base[0] = 0;
  for (int n = 0; n < nodes; ++n) ext_base[n + 1] = ext_base[n] + (x.ext_ia[n + 1] - x.ext_ia[n]);
  double chat01, chati0[NBRMX], chat1j[NBRMX], qs = 0.0;
  int inbr0[NBRMX], inbr1[NBRMX], nnbr0, nnbr1, il10;
  if (x.lamatsaved) {
    double *amatpc = (double *)calloc(m->nja, sizeof(double));
    double *amatpcx = (double *)calloc(ext_base[nodes] + 1, sizeof(double));
    for (int n = 0; n < nodes; ++n) {
      if (x.iallpc[n] == 0) continue;
      if (ibound[n] == 0) continue;
      int nn0 = m->ia[n + 1] - m->ia[n] - 1;
      for (int il0 = 0; il0 < nn0; ++il0) {
        int mm = (ibound[m->ja[m->ia[n] + 1 + il0]] != 0) ? m->ja[m->ia[n] + 1 + il0] : -1;
        if (mm < n) continue;
        pair_coefs(&x, n, il0, 1, hnew, &chat01, chati0, chat1j, &qs, inbr0, inbr1, &nnbr0,
                   &nnbr1, &il10);
        int ii00 = m->ia[n], ii01 = ii00 + 1 + il0, ii11 = m->ia[mm], ii10 = ii11 + 1 + il10;
        amatpc[ii00] = amatpc[ii00] - chat01;
        amatpc[ii01] = amatpc[ii01] + chat01;
        amatpc[ii11] = amatpc[ii11] - chat01;
        amatpc[ii10] = amatpc[ii10] + chat01;
        /* xt3d_amatpc_nbrs and xt3d_amatpcx_nbrnbrs (:1437-1481), for every
         * neighbour slot */
        for (int side = 0; side < 4; ++side) {
          int a = (side < 2) ? n : mm, b = (side < 2) ? mm : n;
          int nnb = (side == 0 || side == 3) ? nnbr0 : nnbr1;
          const double *ch = (side == 0 || side == 3) ? chati0 : chat1j;
          if (side == 0 || side == 2) {
            int idiag = m->ia[a];
            for (int iil = 0; iil < nnb; ++iil) {
              int iii = m->ia[a] + 1 + iil;
              amatpc[idiag] = amatpc[idiag] - ch[iil];
              amatpc[iii] = amatpc[iii] + ch[iil];
            }
          } else {
            int iiab = (side == 1) ? ii01 : ii10;
            for (int iil = 0; iil < nnb; ++iil) {
              amatpc[iiab] = amatpc[iiab] + ch[iil];
              int jjj = m->ja[m->ia[b] + 1 + iil];
              int ix = ext_index(&x, a, jjj, ext_base);
              if (ix >= 0) amatpcx[ix] = amatpcx[ix] - ch[iil];
              else {
                int p = pos_in(m->ia, m->ja, a, jjj);
                amatpc[p] = amatpc[p] - ch[iil];
              }
            }
          }
        }
      }
    }
    /* xt3d_fc: amatpc into the model positions, then amatpcx into the
     * extended ones */
    for (int i = 0; i < m->nja; ++i) amat[m->idxglo[i]] = amat[m->idxglo[i]] + amatpc[i];
    for (int n = 0; n < nodes; ++n)
      for (int p = m->sia[n]; p < m->sia[n + 1]; ++p) {
        int ix = ext_index(&x, n, m->sja[p], ext_base);
        if (ix >= 0) amat[p] = amat[p] + amatpcx[ix];
      }
    free(amatpc);
    free(amatpcx);
  }
  /* the loop of xt3d_fc over the other cells, with the current saturation */
  x.sat = sat;
  for (int n = 0; n < nodes; ++n) {
    if (ibound[n] == 0) continue;
    if (x.lamatsaved && x.iallpc[n] == 1) continue;
    int nn0 = m->ia[n + 1] - m->ia[n] - 1;
    for (int il0 = 0; il0 < nn0; ++il0) {
      int jm = m->ja[m->ia[n] + 1 + il0];
      int mm = (ibound[jm] != 0) ? jm : -1;
      if (mm < 0 || mm < n) continue;
      pair_coefs(&x, n, il0, 0, hnew, &chat01, chati0, chat1j, &qs, inbr0, inbr1, &nnbr0,
                 &nnbr1, &il10);
      int ii00 = m->ia[n], ii01 = ii00 + 1 + il0, ii11 = m->ia[mm], ii10 = ii11 + 1 + il10;
      if (m->inewton != 0) qsat[ii01] = qs;
      const int *G = m->idxglo;
      amat[G[ii00]] = amat[G[ii00]] + (-chat01);
      amat[G[ii01]] = amat[G[ii01]] + chat01;
      amat[G[ii11]] = amat[G[ii11]] + (-chat01);
      amat[G[ii10]] = amat[G[ii10]] + chat01;
      if (m->ixt3d == 2) {
        /* the RHS form: xt3d_rhs (:1522-1546) for both cells */
        for (int side = 0; side < 2; ++side) {
          int a = side ? mm : n, b = side ? n : mm;
          int nnb = side ? nnbr1 : nnbr0;
          const int *inb = side ? inbr1 : inbr0;
          const double *ch = side ? chat1j : chati0;
          for (int iil = 0; iil < nnb; ++iil) {
            if (inb[iil] < 0) continue;
            int jjj = m->ja[m->ia[a] + 1 + iil];
            double term = ch[iil] * (hnew[jjj] - hnew[a]);
            rhs[a] = rhs[a] - term;
            rhs[b] = rhs[b] + term;
          }
        }
        continue;
      }
      /* xt3d_amat_nbrs and xt3d_amat_nbrnbrs (:1382-1435), active slots */
      for (int side = 0; side < 4; ++side) {
        int a = (side < 2) ? n : mm, b = (side < 2) ? mm : n;
        int nnb = (side == 0 || side == 3) ? nnbr0 : nnbr1;
        const int *inb = (side == 0 || side == 3) ? inbr0 : inbr1;
        const double *ch = (side == 0 || side == 3) ? chati0 : chat1j;
        if (side == 0 || side == 2) {
          int idiag = G[m->ia[a]];
          for (int iil = 0; iil < nnb; ++iil) {
            if (inb[iil] < 0) continue;
            int iii = G[m->ia[a] + 1 + iil];
            amat[idiag] = amat[idiag] + (-ch[iil]);
            amat[iii] = amat[iii] + ch[iil];
          }
        } else {
          int iiab = G[(side == 1) ? ii01 : ii10];
          for (int iil = 0; iil < nnb; ++iil) {
            if (inb[iil] < 0) continue;
            amat[iiab] = amat[iiab] + ch[iil];
            int jjj = m->ja[m->ia[b] + 1 + iil];
            int p = pos_in(m->sia, m->sja, a, jjj);
            amat[p] = amat[p] + (-ch[iil]);
          }
        }
      }
    }
  }
  free(ext_base);
  free(one);
  xt3d_free(&x);
  return 0;
}

/* xt3d_fn (Xt3dInterface.f90:693-795) */
void or_xt3d_fn(const or_gwf_model *m, const int *ibound, const double *hnew,
                const double *qsat, double *amat, double *rhs) {
  xt3d_t x;
  if (xt3d_setup(&x, m, ibound, hnew) != 0) return;
  const int *G = m->idxglo;
  for (int n = 0; n < m->nodes; ++n) {
    if (ibound[n] == 0) continue;
    if (x.lamatsaved && x.iallpc[n] == 1) continue;
    int nn0 = m->ia[n + 1] - m->ia[n] - 1;
    for (int il0 = 0; il0 < nn0; ++il0) {
      int jm = m->ja[m->ia[n] + 1 + il0];
      if (ibound[jm] == 0 || jm < n) continue;
      int mm = jm;
      int ii00 = m->ia[n], ii01 = ii00 + 1 + il0;
      int jjs01 = m->jas[ii01];
      int ii11 = m->ia[mm];
      int ii10 = pos_in(m->ia, m->ja, mm, n);
      int iups = (hnew[mm] < hnew[n]) ? n : mm;
      if (m->icelltype[iups] == 0 && m->ixt3d == 1) continue;
      double topup = m->top[iups], botup = m->bot[iups];
      if (m->ihc[jjs01] == 2) {
        topup = (m->top[n] < m->top[mm]) ? m->top[n] : m->top[mm];
        botup = (m->bot[n] > m->bot[mm]) ? m->bot[n] : m->bot[mm];
      }
      double derv = or_squadratic_sat_derv(topup, botup, hnew[iups], 1.0e-6);
      double term = qsat[ii01] * derv;
      if (iups == n) {
        amat[G[ii00]] = amat[G[ii00]] + term;
        rhs[n] = rhs[n] + term * hnew[n];
        amat[G[ii10]] = amat[G[ii10]] + (-term);
        rhs[mm] = rhs[mm] - term * hnew[n];
      } else {
        amat[G[ii01]] = amat[G[ii01]] + term;
        rhs[n] = rhs[n] + term * hnew[mm];
        amat[G[ii11]] = amat[G[ii11]] + (-term);
        rhs[mm] = rhs[mm] - term * hnew[mm];
      }
    }
  }
  xt3d_free(&x);
}

/* xt3d_flowja (Xt3dInterface.f90:797-875): the flow through every
 * connection of two active cells, from the coefficients with the current
 * saturation (and, under Newton, the saturated area scaled by the upstream
 * saturation); flowja must hold zeros on the connections. */
void or_xt3d_flowja(const or_gwf_model *m, const int *ibound, const double *sat,
                    const double *hnew, double *flowja) {
  xt3d_t x;
  if (xt3d_setup(&x, m, ibound, sat) != 0) return;
  double chat01, chati0[NBRMX], chat1j[NBRMX];
  int inbr0[NBRMX], inbr1[NBRMX];
  for (int n = 0; n < m->nodes; ++n) {
    if (ibound[n] == 0) continue;
    int nnbr0 = m->ia[n + 1] - m->ia[n] - 1;
    double vc0[NBRMX][3], vn0[NBRMX][3], dl0[NBRMX], dl0n[NBRMX];
    int allhc0;
    xt3d_load(&x, n, nnbr0, inbr0, vc0, vn0, dl0, dl0n, &allhc0);
    for (int il0 = 0; il0 < nnbr0; ++il0) {
      int mm = inbr0[il0];
      if (mm < 0 || mm < n) continue;
      int nnbr1 = m->ia[mm + 1] - m->ia[mm] - 1;
      double vc1[NBRMX][3], vn1[NBRMX][3], dl1[NBRMX], dl1n[NBRMX];
      int allhc1;
      xt3d_load(&x, mm, nnbr1, inbr1, vc1, vn1, dl1, dl1n, &allhc1);
      int ii01 = m->ia[n] + 1 + il0;
      int jjs01 = m->jas[ii01];
      int il10 = pos_in(m->ia, m->ja, mm, n) - m->ia[mm] - 1;
      double ar01 = 0.0, ar10 = 0.0;
      if (m->inewton != 0) xt3d_areas(&x, n, mm, jjs01, 1, &ar01, &ar10, hnew);
      xt3d_areas(&x, n, mm, jjs01, 0, &ar01, &ar10, hnew);
      qconds(x.nbrmax, nnbr0, inbr0, il0, vc0, vn0, dl0, dl0n, m->ck + 9 * (size_t)n, nnbr1,
             inbr1, il10, vc1, vn1, dl1, dl1n, m->ck + 9 * (size_t)mm, ar01, ar10, 1e-10, allhc0,
             allhc1, &chat01, chati0, chat1j);
      double qnm = chat01 * (hnew[mm] - hnew[n]);
      double qnbrs = 0.0;
      for (int iil = 0; iil < nnbr0; ++iil)
        if (inbr0[iil] >= 0) {
          int jjj = m->ja[m->ia[n] + 1 + iil];
          qnbrs = qnbrs + chati0[iil] * (hnew[jjj] - hnew[n]);
        }
      qnm = qnm + qnbrs;
      qnbrs = 0.0;
      for (int iil = 0; iil < nnbr1; ++iil)
        if (inbr1[iil] >= 0) {
          int jjj = m->ja[m->ia[mm] + 1 + iil];
          qnbrs = qnbrs + chat1j[iil] * (hnew[jjj] - hnew[mm]);
        }
      qnm = qnm - qnbrs;
      flowja[ii01] = flowja[ii01] + qnm;
      flowja[m->isym[ii01]] = flowja[m->isym[ii01]] - qnm;
    }
  }
  xt3d_free(&x);
}

/* hyeff (HGeoUtil.f90:29-108) */
static double hyeff(double k11, double k22, double k33, double ang1, double ang2, double ang3,
                    double vg1, double vg2, double vg3, int iavgmeth) {
  double s1 = sin(ang1), c1 = cos(ang1), s2 = sin(ang2), c2 = cos(ang2), s3 = sin(ang3),
         c3 = cos(ang3);
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
  double ve1 = r[0][0] * vg1 + r[1][0] * vg2 + r[2][0] * vg3;
  double ve2 = r[0][1] * vg1 + r[1][1] * vg2 + r[2][1] * vg3;
  double ve3 = r[0][2] * vg1 + r[1][2] * vg2 + r[2][2] * vg3;
  double k = 0.0;
  if (iavgmeth == 0) {
    double dnum = 1.0, d1 = ve1 * ve1, d2 = ve2 * ve2, d3 = ve3 * ve3;
    if (ve1 != 0.0) {
      dnum = dnum * k11;
      d2 = d2 * k11;
      d3 = d3 * k11;
    }
    if (ve2 != 0.0) {
      dnum = dnum * k22;
      d1 = d1 * k22;
      d3 = d3 * k22;
    }
    if (ve3 != 0.0) {
      dnum = dnum * k33;
      d1 = d1 * k33;
      d2 = d2 * k33;
    }
    double denom = d1 + d2 + d3;
    if (denom > 0.0) k = dnum / denom;
  } else if (iavgmeth == 1) {
    k = ve1 * ve1 * k11 + ve2 * ve2 * k22 + ve3 * ve3 * k33;
  }
  return k;
}

/* hy_eff (gwf-npf.f90:2280-2357) of cell a toward cell b; ipos is the
 * position of the connection in the lower-numbered cell's row */
static double hy_eff(const or_gwf_model *m, const double *k22, const double *angle1,
                     const double *angle2, const double *angle3, int iavgkeff, int a, int b,
                     int ihc, int ipos) {
  double hy11 = m->k11[a], hy22 = k22 ? k22[a] : m->k11[a], hy33 = m->k33[a];
  double v[3];
  if (ihc == 0) {
    if (!angle2) return hy33;
    conn_normal(m, a, b, ihc, ipos, v);
    double ang1 = angle1[a], ang2 = angle2[a], ang3 = angle3 ? angle3[a] : 0.0;
    return hyeff(hy11, hy22, hy33, ang1, ang2, ang3, v[0], v[1], v[2], iavgkeff);
  }
  if (!k22) return hy11;
  conn_normal(m, a, b, ihc, ipos, v);
  double ang1 = 0.0, ang2 = 0.0, ang3 = 0.0;
  if (angle1) {
    ang1 = angle1[a];
    if (angle2) {
      ang2 = angle2[a];
      if (angle3) ang3 = angle3[a];
    }
  }
  return hyeff(hy11, hy22, hy33, ang1, ang2, ang3, v[0], v[1], v[2], iavgkeff);
}

void or_npf_hy(const or_gwf_model *m, const double *k22, const double *angle1,
               const double *angle2, const double *angle3, int iavgkeff, double *hy) {
  for (int n = 0; n < m->nodes; ++n)
    for (int ii = m->ia[n] + 1; ii < m->ia[n + 1]; ++ii) {
      int mm = m->ja[ii];
      if (mm < n) continue;
      int s = m->jas[ii], ihc = m->ihc[s];
      hy[2 * s] = hy_eff(m, k22, angle1, angle2, angle3, iavgkeff, n, mm, ihc, ii);
      hy[2 * s + 1] = hy_eff(m, k22, angle1, angle2, angle3, iavgkeff, mm, n, ihc, ii);
    }
}
