/*
 * ims_oracle.c -- CPU restatement of the MODFLOW 6 IMS linear path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library is
 * checked against; nothing in the product links or calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py (its cpu_baseline / reference arm)
 * load the shared library built from it.
 *
 * Each routine follows the cited Fortran routine of MODFLOW 6 (6.7.0.dev1)
 * loop for loop, with 0-based indices in place of the Fortran 1-based ones.
 * Summation order is kept, so with the same floating-point contraction
 * setting the results are bit-for-bit those of the Fortran code.  The oracle
 * is compiled with -ffp-contract=off (no fused multiply-add), which is what
 * gfortran does on x86-64 without -march flags.
 *
 * Parity pins: the known answers of autotest/test_gwf_chd01.py:118-127 and
 * autotest/test_gwf_newton01.py:95-103 (see tests/test_oracle_known_answers.py).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#include "ims_oracle.h"

/* src/Utilities/Constants.f90:120-122 */
#define DPREC DBL_EPSILON
#define DSAME (100.0 * DBL_EPSILON)
#define DEM3 1.0e-3
#define DEM4 1.0e-4
#define DEM6 1.0e-6

/* Fortran SIGN(a, b): |a| with the sign of b (signed zeros honoured). */
static inline double f_sign(double a, double b) { return copysign(fabs(a), b); }

/* src/Utilities/MathUtil.f90:45-86, is_close with default rtol=DSAME, atol=0,
 * symmetric test. */
int or_is_close(double a, double b) {
  if (a == b) return 1;
  double m = fmax(fabs(a), fabs(b));
  double tol = DSAME * m;
  if (tol < 0.0) tol = 0.0;
  return fabs(a - b) <= tol;
}

/* src/Utilities/Libraries/sparsekit/sparsekit.f90:1-59, amux: y = A*x, row
 * dot product in CSR order. */
void or_amux(int n, const double *x, double *y, const double *a, const int *ja,
             const int *ia) {
  for (int i = 0; i < n; ++i) {
    double t = 0.0;
    for (int k = ia[i]; k < ia[i + 1]; ++k) t = t + a[k] * x[ja[k]];
    y[i] = t;
  }
}

/* src/Utilities/Libraries/blas/blas1_d.f90:295-386, ddot = dot_product,
 * summed sequentially from the first element. */
double or_ddot(int n, const double *x, const double *y) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s = s + x[i] * y[i];
  return s;
}

/* src/Utilities/Libraries/blas/blas1_d.f90:387-470, dnrm2 with the scaled sum
 * of squares. */
double or_dnrm2(int n, const double *x) {
  if (n < 1) return 0.0;
  if (n == 1) return fabs(x[0]);
  double scale = 0.0, ssq = 1.0;
  for (int i = 0; i < n; ++i) {
    if (x[i] != 0.0) {
      double absxi = fabs(x[i]);
      if (scale < absxi) {
        double r = scale / absxi;
        ssq = 1.0 + ssq * (r * r);
        scale = absxi;
      } else {
        double r = absxi / scale;
        ssq = ssq + r * r;
      }
    }
  }
  return scale * sqrt(ssq);
}

/* ImsLinearBase.f90:1291-1312, ims_base_residual: d = b - A*x. */
void or_residual(int neq, const double *x, const double *b, double *d,
                 const double *a, const int *ia, const int *ja) {
  or_amux(neq, x, d, a, ja, ia);
  for (int n = 0; n < neq; ++n) d[n] = b[n] - d[n];
}

/* ImsLinearBase.f90:1316-1333, ims_base_epfact.  The 0.01 and 0.10 literals
 * are default (single-precision) reals in the Fortran source, so they are
 * converted from float here to give the same double values. */
double or_epfact(int icnvgopt, int kstp) {
  if (icnvgopt == 2) return (kstp == 1) ? (double)0.01f : (double)0.10f;
  if (icnvgopt == 4) return DEM4;
  return 1.0;
}

/* ImsLinearBase.f90:1101-1146, ims_base_testcnvg. */
void or_testcnvg(int icnvgopt, int *icnvg, int iiter, double dvmax, double rmax,
                 double rmax0, double epfact, double dvclose, double rclose) {
  if (icnvgopt == 0) {
    if (fabs(dvmax) <= dvclose && fabs(rmax) <= rclose) *icnvg = 1;
  } else if (icnvgopt == 1) {
    if (fabs(dvmax) <= dvclose && fabs(rmax) <= rclose) *icnvg = (iiter == 1) ? 1 : -1;
  } else if (icnvgopt == 2) {
    if (fabs(dvmax) <= dvclose || rmax <= rclose) *icnvg = 1;
    else if (rmax <= rmax0 * epfact) *icnvg = -1;
  } else if (icnvgopt == 3) {
    if (fabs(dvmax) <= dvclose) *icnvg = 1;
    else if (rmax <= rmax0 * rclose) *icnvg = -1;
  } else if (icnvgopt == 4) {
    if (fabs(dvmax) <= dvclose && rmax <= rclose) *icnvg = 1;
    else if (rmax <= rmax0 * epfact) *icnvg = -1;
  }
}

/* ImsLinearBase.f90:1207-1261, ims_base_pccrs: builds IAPC/JAPC.  japc[0:neq]
 * holds, per row, the position of the first upper entry; japc[neq:nja] the
 * sorted off-diagonal columns.  Positions and columns are 0-based. */
void or_pccrs(int neq, int nja, const int *ia, const int *ja, int *iapc, int *japc) {
  int ip = neq;
  int *iarr = (int *)malloc(sizeof(int) * 64);
  int cap = 64;
  for (int n = 0; n < neq; ++n) {
    int i0 = ia[n], i1 = ia[n + 1];
    int nlen = i1 - i0 - 1;
    if (nlen + 1 > cap) {
      cap = nlen + 1;
      iarr = (int *)realloc(iarr, sizeof(int) * cap);
    }
    int ic = 0;
    for (int j = i0; j < i1; ++j) {
      int jcol = ja[j];
      if (jcol == n) continue;
      iarr[ic++] = jcol;
    }
    /* ims_base_isort (ImsLinearBase.f90:1268-1284): exchange sort */
    for (int a = 0; a < nlen - 1; ++a)
      for (int b = a + 1; b < nlen; ++b)
        if (iarr[a] > iarr[b]) {
          int t = iarr[b];
          iarr[b] = iarr[a];
          iarr[a] = t;
        }
    iapc[n] = ip;
    for (int j = 0; j < nlen; ++j) japc[ip++] = iarr[j];
  }
  iapc[neq] = nja;
  free(iarr);
  for (int n = 0; n < neq; ++n) {
    int i0 = iapc[n], i1 = iapc[n + 1];
    japc[n] = iapc[n + 1];
    for (int j = i0; j < i1; ++j) {
      if (japc[j] > n) {
        japc[n] = j;
        break;
      }
    }
  }
}

/* ImsLinearBase.f90:928-1042, ims_base_pcilu0: ILU0 (relax = 0) or MILU0
 * (relax > 0) into APC.  iw/w are work vectors of length neq that must be
 * zero on entry (they are left zero on normal exit). */
void or_pcilu0(int nja, int neq, const double *amat, const int *ia, const int *ja,
               double *apc, const int *iapc, const int *japc, int *iw, double *w,
               double relax, int *ipcflag, double delta) {
  double drelax = relax;
  for (int n = 0; n < neq; ++n) {
    iw[n] = 0;
    w[n] = 0.0;
  }
  for (int n = 0; n < neq; ++n) {
    for (int j = ia[n]; j < ia[n + 1]; ++j) {
      int jcol = ja[j];
      iw[jcol] = 1;
      w[jcol] = w[jcol] + amat[j];
    }
    int ic0 = iapc[n], ic1 = iapc[n + 1];
    int iu = japc[n];
    double rs = 0.0;
    for (int j = ic0; j < iu; ++j) {
      int jcol = japc[j];
      int iic1 = iapc[jcol + 1];
      int iiu = japc[jcol];
      double tl = w[jcol] * apc[jcol];
      w[jcol] = tl;
      for (int jj = iiu; jj < iic1; ++jj) {
        int jjcol = japc[jj];
        if (iw[jjcol] != 0) w[jjcol] = w[jjcol] - tl * apc[jj];
        else rs = rs + tl * apc[jj];
      }
    }
    double d = w[n];
    double tl = (1.0 + delta) * d - (drelax * rs);
    double sd1 = f_sign(d, tl);
    if (sd1 != d) {
      if (*ipcflag > 1) {
        tl = f_sign(DEM6, d);
      } else {
        *ipcflag = 1;
        goto cleanup_exit; /* EXIT MAIN */
      }
    }
    if (fabs(tl) == 0.0) {
      if (*ipcflag > 1) {
        tl = f_sign(DEM6, d);
      } else {
        *ipcflag = 1;
        goto cleanup_exit;
      }
    }
    apc[n] = 1.0 / tl;
    iw[n] = 0;
    w[n] = 0.0;
    for (int j = ic0; j < ic1; ++j) {
      int jcol = japc[j];
      apc[j] = w[jcol];
      iw[jcol] = 0;
      w[jcol] = 0.0;
    }
  }
  *ipcflag = 0;
  return;
cleanup_exit:
  /* The Fortran leaves IW/W dirty after EXIT MAIN; the next call re-zeroes
   * them at its start, exactly as done at the top of this routine. */
  return;
}

/* ImsLinearBase.f90:761-864, ims_base_pcu for IPC 1/2: retry with a growing
 * diagonal increment.  Returns the number of retries (icount). */
int or_pcu(int nja, int neq, int ipc, double relax, const double *amat,
           const int *ia, const int *ja, double *apc, const int *iapc,
           const int *japc, int *iw, double *w) {
  int ipcflag = 0, icount = 0;
  double delta = 0.0;
  for (;;) {
    if (ipc == 1 || ipc == 2) {
      or_pcilu0(nja, neq, amat, ia, ja, apc, iapc, japc, iw, w, relax, &ipcflag, delta);
    } else {
      ipcflag = 0;
    }
    if (ipcflag < 1) break;
    delta = 1.5 * delta + DEM3;
    ipcflag = 0;
    if (delta > 0.5) {
      delta = 0.5;
      ipcflag = 2;
    }
    icount = icount + 1;
    if (icount > 10) break;
  }
  return icount;
}

/* sparskit2/ilut.f90:519-581, qsplit: partial quick-sort of a[0..n) by
 * decreasing magnitude so that the ncut-th entry (1-based, as in the
 * reference) splits larger from smaller ones; ind moves with a. */
static void or_qsplit(int n, double *a, int *ind, int ncut) {
  int first = 0, last = n - 1, cut = ncut - 1;
  if (cut < first || cut > last) return;
  for (;;) {
    int mid = first;
    double abskey = fabs(a[mid]);
    for (int j = first + 1; j <= last; ++j) {
      if (fabs(a[j]) > abskey) {
        ++mid;
        double t = a[mid]; a[mid] = a[j]; a[j] = t;
        int it = ind[mid]; ind[mid] = ind[j]; ind[j] = it;
      }
    }
    double t = a[mid]; a[mid] = a[first]; a[first] = t;
    int it = ind[mid]; ind[mid] = ind[first]; ind[first] = it;
    if (mid == cut) return;
    if (mid > cut) last = mid - 1;
    else first = mid + 1;
  }
}

/* sparskit2/ilut.f90:48-462, ilut: dual-threshold incomplete LU with the
 * MODFLOW changes (relaxation of the dropped sum, MILUT; pivot guard through
 * izero and delta).  Row ii keeps at most lfil L entries (|multiplier| above
 * droptol) and lfil - 1 U entries (|u| above droptol x the row's mean |a|),
 * the largest by qsplit, in qsplit's order.
 *
 * Layout: sparskit's modified sparse row storage with its row pointers moved
 * out of jlu, so that the factor has the IAPC/JAPC/APC shape the ILU0
 * application reads: alu[0..n) the inverse pivots; row ii's L entries at
 * [iapc[ii], japc[ii]) and its U entries at [japc[ii], iapc[ii+1]), columns
 * in japc and values in alu from position n + 1 on (sparskit's jlu(1) = n+2).
 * iwk is the reference's storage length (ims_calc_pcdims,
 * ImsLinearBase.f90:1148-1197); the arrays hold max(iwk, n + 1) entries.
 * Work arrays: w (n), jw (n), jr (n).  Returns ierr: 0, -1 (row longer than
 * n), -2/-3 (L/U storage), -4 (lfil < 0), -5 (zero row). */
int or_ilut(int n, const double *a, const int *ja, const int *ia, int lfil, double droptol,
            double *alu, int *iapc, int *japc, int iwk, double *w, int *jw, int *jr,
            double relax, int *izero, double delta) {
  if (lfil < 0) return -4;
  int ju0 = n + 1; /* next free storage position */
  iapc[0] = ju0;
  for (int j = 0; j < n; ++j) jr[j] = -1;
  for (int ii = 0; ii < n; ++ii) {
    const int j1 = ia[ii], j2 = ia[ii + 1];
    double dropsum = 0.0, tnorm = 0.0;
    for (int k = j1; k < j2; ++k) tnorm = tnorm + fabs(a[k]);
    if (tnorm == 0.0) return -5;
    tnorm = tnorm / (double)(j2 - j1);
    /* unpack: L part at [0, lenl), the diagonal at ii, U part at ii+1.. */
    int lenu = 1, lenl = 0;
    jw[ii] = ii;
    w[ii] = 0.0;
    jr[ii] = ii;
    for (int j = j1; j < j2; ++j) {
      const int k = ja[j];
      const double t = a[j];
      if (k < ii) {
        jw[lenl] = k;
        w[lenl] = t;
        jr[k] = lenl;
        ++lenl;
      } else if (k == ii) {
        w[ii] = t;
      } else {
        const int jpos = ii + lenu;
        ++lenu;
        jw[jpos] = k;
        w[jpos] = t;
        jr[k] = jpos;
      }
    }
    /* eliminate the earlier rows, smallest column first */
    int ilen = 0;
    for (int jj = 0; jj < lenl; ++jj) {
      int jrow = jw[jj], k = jj;
      for (int j = jj + 1; j < lenl; ++j)
        if (jw[j] < jrow) {
          jrow = jw[j];
          k = j;
        }
      if (k != jj) {
        const int j = jw[jj];
        jw[jj] = jw[k];
        jw[k] = j;
        jr[jrow] = jj;
        jr[j] = k;
        const double s = w[jj];
        w[jj] = w[k];
        w[k] = s;
      }
      jr[jrow] = -1;
      const double fact = w[jj] * alu[jrow];
      if (fabs(fact) <= droptol) {
        dropsum = dropsum + w[jj];
        continue;
      }
      for (int kk = japc[jrow]; kk < iapc[jrow + 1]; ++kk) {
        const double s = fact * alu[kk];
        const int j = japc[kk];
        const int jpos = jr[j];
        if (j >= ii) {
          if (jpos < 0) {
            if (lenu + 1 > n) return -1;
            const int i = ii + lenu;
            ++lenu;
            jw[i] = j;
            jr[j] = i;
            w[i] = -s;
          } else {
            w[jpos] = w[jpos] - s;
          }
        } else {
          if (jpos < 0) {
            if (lenl + 1 > n) return -1;
            jw[lenl] = j;
            jr[j] = lenl;
            w[lenl] = -s;
            ++lenl;
          } else {
            w[jpos] = w[jpos] - s;
          }
        }
      }
      w[ilen] = fact;
      jw[ilen] = jrow;
      ++ilen;
    }
    for (int k = 0; k < lenu; ++k) jr[jw[ii + k]] = -1;
    /* L: the lfil largest multipliers */
    lenl = ilen;
    ilen = lenl < lfil ? lenl : lfil;
    or_qsplit(lenl, w, jw, ilen);
    for (int k = 0; k < ilen; ++k) {
      if (ju0 + 1 > iwk) return -2;
      alu[ju0] = w[k];
      japc[ju0] = jw[k];
      ++ju0;
    }
    japc[ii] = ju0;
    /* U: drop below droptol x tnorm, then the lfil - 1 largest */
    ilen = 0;
    for (int k = 1; k < lenu; ++k) {
      if (fabs(w[ii + k]) > droptol * tnorm) {
        ++ilen;
        w[ii + ilen] = w[ii + k];
        jw[ii + ilen] = jw[ii + k];
      } else {
        dropsum = dropsum + w[ii + k];
      }
    }
    lenu = ilen + 1;
    ilen = lenu < lfil ? lenu : lfil;
    or_qsplit(lenu - 1, w + ii + 1, jw + ii + 1, ilen);
    if (ilen + ju0 + 1 > iwk) return -3;
    for (int k = ii + 1; k < ii + ilen; ++k) {
      japc[ju0] = jw[k];
      alu[ju0] = w[k];
      ++ju0;
    }
    /* the pivot, guarded against a sign change or zero */
    const double diag = w[ii];
    double dw = (1.0 + delta) * diag + (relax * dropsum);
    const double sc = f_sign(diag, dw);
    if (sc != diag) {
      if (*izero > 1) {
        dw = f_sign(1.0, diag) * (1.0e-4 + droptol) * tnorm;
      } else {
        *izero = 1;
        return 0; /* EXIT MAIN */
      }
    }
    if (fabs(dw) == 0.0) {
      if (*izero > 1) {
        dw = f_sign(1.0, diag) * (1.0e-4 + droptol) * tnorm;
      } else {
        *izero = 1;
        return 0;
      }
    }
    w[ii] = dw;
    alu[ii] = 1.0 / w[ii];
    iapc[ii + 1] = ju0;
  }
  return 0;
}

/* ImsLinearBase.f90:761-864, ims_base_pcu for IPC 3/4.  ilut leaves izero
 * as it found it on success, so once the retries reach delta = 0.5
 * (ipcflag 2) the loop refactors until icount exceeds 10, as the reference
 * does.  Returns icount, or ierr (< 0) from ilut. */
int or_pcu_ilut(int neq, int lfil, double droptol, double relax, const double *amat,
                const int *ia, const int *ja, double *alu, int *iapc, int *japc, int iwk,
                double *w, int *jw, int *jr) {
  int ipcflag = 0, icount = 0;
  double delta = 0.0;
  for (;;) {
    int ierr = or_ilut(neq, amat, ja, ia, lfil, droptol, alu, iapc, japc, iwk, w, jw, jr,
                       relax, &ipcflag, delta);
    if (ierr != 0) return ierr;
    if (ipcflag < 1) break;
    delta = 1.5 * delta + DEM3;
    ipcflag = 0;
    if (delta > 0.5) {
      delta = 0.5;
      ipcflag = 2;
    }
    icount = icount + 1;
    if (icount > 10) break;
  }
  return icount;
}

/* ---- REORDERING_METHOD RCM: rcm/rcm.f90 (George & Liu's GENRCM as
 * vendored in the reference).  The routines below keep the reference's
 * 1-based node numbers internally (arrays of n + 1, index 0 unused) so each
 * loop bound reads as in the source; the caller converts at the edges.
 * A separate visited array stands in for degree's sign flips of adj_row. */

/* rcm.f90:853-1001, degree: component of root among mask != 0 and each
 * node's count of neighbours with mask != 0 (its own diagonal included). */
static void rcm_degree(int root, const int *ia, const int *ja, const int *mask, int *deg,
                       int *iccsze, int *ls, char *vis) {
  ls[1] = root;
  vis[root] = 1;
  int lvlend = 0, cc = 1;
  for (;;) {
    const int lbegin = lvlend + 1;
    lvlend = cc;
    for (int i = lbegin; i <= lvlend; ++i) {
      const int node = ls[i];
      int ideg = 0;
      for (int j = ia[node]; j <= ia[node + 1] - 1; ++j) {
        const int nbr = ja[j];
        if (mask[nbr] != 0) {
          ++ideg;
          if (!vis[nbr]) {
            vis[nbr] = 1;
            ++cc;
            ls[cc] = nbr;
          }
        }
      }
      deg[node] = ideg;
    }
    if (cc - lvlend == 0) break;
  }
  for (int i = 1; i <= cc; ++i) vis[ls[i]] = 0;
  *iccsze = cc;
}

/* rcm.f90:2188-2330, level_set: the rooted level structure of root's
 * component; mask is restored to 1 on the component on exit. */
static void rcm_level_set(int root, const int *ia, const int *ja, int *mask, int *level_num,
                          int *level_row, int *level) {
  mask[root] = 0;
  level[1] = root;
  int nl = 0, lvlend = 0, cc = 1;
  for (;;) {
    const int lbegin = lvlend + 1;
    lvlend = cc;
    ++nl;
    level_row[nl] = lbegin;
    for (int i = lbegin; i <= lvlend; ++i) {
      const int node = level[i];
      for (int j = ia[node]; j <= ia[node + 1] - 1; ++j) {
        const int nbr = ja[j];
        if (mask[nbr] != 0) {
          ++cc;
          level[cc] = nbr;
          mask[nbr] = 0;
        }
      }
    }
    if (cc - lvlend <= 0) break;
  }
  level_row[nl + 1] = lvlend + 1;
  for (int i = 1; i <= cc; ++i) mask[level[i]] = 1;
  *level_num = nl;
}

/* rcm.f90:3121-3316, root_find: a pseudo-peripheral node of root's
 * component (the minimum-degree node of the last level, while the level
 * structure keeps growing). */
static void rcm_root_find(int *root, const int *ia, const int *ja, int *mask, int *level_row,
                          int *level) {
  int level_num, level_num2;
  rcm_level_set(*root, ia, ja, mask, &level_num, level_row, level);
  const int iccsze = level_row[level_num + 1] - 1;
  if (level_num == 1 || level_num == iccsze) return;
  for (;;) {
    int mindeg = iccsze;
    const int jstrt = level_row[level_num];
    *root = level[jstrt];
    if (jstrt < iccsze) {
      for (int j = jstrt; j <= iccsze; ++j) {
        const int node = level[j];
        int ndeg = 0;
        for (int k = ia[node]; k <= ia[node + 1] - 1; ++k)
          if (0 < mask[ja[k]]) ++ndeg;
        if (ndeg < mindeg) {
          *root = node;
          mindeg = ndeg;
        }
      }
    }
    rcm_level_set(*root, ia, ja, mask, &level_num2, level_row, level);
    if (level_num2 <= level_num) break;
    level_num = level_num2;
    if (iccsze <= level_num) break;
  }
}

/* rcm.f90:2899-3120, rcm: breadth-first numbering of root's component,
 * each node's new neighbours ordered by increasing degree with the
 * insertion sort of the vendored source (its inner loop stops above the
 * first new neighbour), then reversed. */
static void rcm_number(int root, const int *ia, const int *ja, int *mask, int *perm,
                       int *iccsze, int *deg, char *vis) {
  rcm_degree(root, ia, ja, mask, deg, iccsze, perm, vis);
  mask[root] = 0;
  const int cc = *iccsze;
  if (cc == 1) return;
  int lvlend = 0, lnbr = 1;
  while (lvlend < lnbr) {
    const int lbegin = lvlend + 1;
    lvlend = lnbr;
    for (int i = lbegin; i <= lvlend; ++i) {
      const int node = perm[i];
      const int fnbr = lnbr + 1;
      for (int j = ia[node]; j <= ia[node + 1] - 1; ++j) {
        const int nbr = ja[j];
        if (mask[nbr] != 0) {
          ++lnbr;
          mask[nbr] = 0;
          perm[lnbr] = nbr;
        }
      }
      if (lnbr <= fnbr) continue;
      int k = fnbr;
      while (k < lnbr) {
        int l = k;
        ++k;
        const int nbr = perm[k];
        while (fnbr < l) {
          const int lperm = perm[l];
          if (deg[lperm] <= deg[nbr]) break;
          perm[l + 1] = lperm;
          --l;
        }
        perm[l + 1] = nbr;
      }
    }
  }
  for (int i = 1; i <= cc / 2; ++i) {
    const int t = perm[i];
    perm[i] = perm[cc + 1 - i];
    perm[cc + 1 - i] = t;
  }
}

/* rcm.f90:1003-1107, genrcm, on a 0-based CSR pattern (the diagonal
 * included, as IMS passes it): lorder[i] (0-based) is the i-th node of the
 * RCM numbering. */
void or_genrcm(int n, const int *ia0, const int *ja0, int *lorder) {
  if (n <= 0) return;
  const int nja = ia0[n];
  if (nja <= 0) return;
  int *ia = (int *)malloc(sizeof(int) * ((size_t)n + 2));
  int *ja = (int *)malloc(sizeof(int) * ((size_t)nja + 1));
  for (int i = 0; i <= n; ++i) ia[i + 1] = ia0[i] + 1;
  for (int k = 0; k < nja; ++k) ja[k + 1] = ja0[k] + 1;
  int *mask = (int *)malloc(sizeof(int) * (n + 1));
  int *perm = (int *)calloc(n + 2, sizeof(int));
  int *level_row = (int *)calloc(n + 2, sizeof(int));
  int *level = (int *)calloc(n + 2, sizeof(int));
  int *deg = (int *)calloc(n + 1, sizeof(int));
  char *vis = (char *)calloc(n + 1, 1);
  for (int i = 1; i <= n; ++i) mask[i] = 1;
  int num = 1;
  for (int i = 1; i <= n; ++i) {
    if (mask[i] != 0) {
      int root = i, iccsze = 0;
      rcm_root_find(&root, ia, ja, mask, level_row, level);
      rcm_number(root, ia, ja, mask, perm + num - 1, &iccsze, deg, vis);
      num += iccsze;
      if (n < num) break;
    }
  }
  for (int i = 1; i <= n; ++i) lorder[i - 1] = perm[i] - 1;
  free(ia); free(ja); free(mask); free(perm); free(level_row); free(level); free(deg); free(vis);
}

/* ---- REORDERING_METHOD MD: ImsReordering.f90 (the Yale sparse matrix
 * package's minimum-degree ordering: odrv, md, mdi, mdm, mdp, mdu).  Arrays
 * are 1-based as in the source; v doubles as mark (odrv passes isp(v) for
 * both: mark lives in v(1:n), the list nodes from n + 1 on); vk and ek are
 * one variable, as are vs and es.  The labels of the source are kept. */

/* :359-461, mdi: element/vertex lists of the symmetric pattern and the
 * degree lists. */
static int md_init(int n, const int *ia, const int *ja, int mmax, int *v, int *l, int *head,
                   int *last, int *next, int tag) {
  int *mark = v;
  for (int vi = 1; vi <= n; ++vi) {
    mark[vi] = 1;
    l[vi] = 0;
    head[vi] = 0;
  }
  int sfs = n + 1;
  for (int vi = 1; vi <= n; ++vi) {
    const int jmin = ia[vi], jmax = ia[vi + 1] - 1;
    for (int j = jmin; j <= jmax; ++j) {
      const int vj = ja[j];
      const int ieval = vj - vi;
      if (ieval == 0) continue;
      if (ieval < 0) {
        int lvk = vi, found = 0;
        const int kmax = mark[vi] - 1;
        for (int k = 1; k <= kmax; ++k) {
          lvk = l[lvk];
          if (v[lvk] == vj) { found = 1; break; }
        }
        if (found) continue;
      }
      if (sfs >= mmax) return 9 * n + vi;
      mark[vi] = mark[vi] + 1;
      v[sfs] = vj;
      l[sfs] = l[vi];
      l[vi] = sfs;
      sfs = sfs + 1;
      mark[vj] = mark[vj] + 1;
      v[sfs] = vi;
      l[sfs] = l[vj];
      l[vj] = sfs;
      sfs = sfs + 1;
    }
  }
  for (int vi = 1; vi <= n; ++vi) {
    const int dvi = mark[vi];
    next[vi] = head[dvi];
    head[dvi] = vi;
    last[vi] = -dvi;
    const int nextvi = next[vi];
    if (nextvi > 0) last[nextvi] = vi;
    mark[vi] = tag;
  }
  return 0;
}

/* :463-540, mdm: the list of uneliminated vertices reachable from vk. */
static void md_merge(int vk, int *tail, int *v, int *l, const int *last, const int *next) {
  int *mark = v;
  const int tag = mark[vk];
  *tail = vk;
  int ls = l[vk];
  for (;;) {
    const int s = ls;
    if (s == 0) break;
    ls = l[s];
    const int vs = v[s];
    if (next[vs] >= 0) {
      mark[vs] = tag;
      l[*tail] = s;
      *tail = s;
      continue;
    }
    const int es = vs;
    int lb = l[es];
    const int blpmax = last[es];
    for (int blp = 1; blp <= blpmax; ++blp) {
      const int b = lb;
      lb = l[b];
      const int vb = v[b];
      if (mark[vb] >= tag) continue;
      mark[vb] = tag;
      l[*tail] = b;
      *tail = b;
    }
    mark[es] = tag;
  }
  l[*tail] = 0;
}

/* :542-657, mdp: purges the reachable vertices' lists of the elements
 * absorbed by ek and eliminates the vertices left with no other element. */
static void md_purge(int *k, int ek, int tail, int *v, int *l, int *head, int *last, int *next) {
  int *mark = v;
  const int tag = mark[ek];
  int li = ek, free_ = 0;
  const int ilpmax = last[ek];
  if (ilpmax <= 0) goto L12;
  for (int ilp = 1; ilp <= ilpmax; ++ilp) {
    int i = li, ls, s, lvi, evi;
    li = l[i];
    const int vi = v[li];
    if (last[vi] == 0) goto L3;
    if (last[vi] > 0) goto L1;
    head[-last[vi]] = next[vi];
    goto L2;
  L1:
    next[last[vi]] = next[vi];
  L2:
    if (next[vi] > 0) last[next[vi]] = last[vi];
  L3:
    ls = vi;
  L4:
    s = ls;
    ls = l[s];
    if (ls == 0) goto L6;
    {
      const int es = v[ls];
      if (mark[es] < tag) goto L4;
    }
    free_ = ls;
    l[s] = l[ls];
    ls = s;
    goto L4;
  L6:
    lvi = l[vi];
    if (lvi != 0) goto L7;
    l[i] = l[li];
    li = i;
    *k = *k + 1;
    next[vi] = -*k;
    last[ek] = last[ek] - 1;
    continue;
  L7:
    if (l[lvi] != 0) goto L9;
    evi = v[lvi];
    if (next[evi] >= 0) goto L9;
    if (mark[evi] < 0) goto L8;
    last[vi] = evi;
    mark[evi] = -1;
    l[tail] = li;
    tail = li;
    l[i] = l[li];
    li = i;
    goto L10;
  L8:
    last[vi] = 0;
    mark[evi] = mark[evi] - 1;
    goto L10;
  L9:
    last[vi] = -ek;
  L10:
    v[free_] = ek;
    l[free_] = l[vi];
    l[vi] = free_;
  }
L12:
  l[tail] = 0;
}

/* :659-772, mdu: new degrees of the vertices reachable from ek. */
static void md_update(int ek, int *dmin, int *v, int *l, int *head, int *last, int *next) {
  int *mark = v;
  int tag = mark[ek] - last[ek];
  int i = ek;
  const int ilpmax = last[ek];
  if (ilpmax <= 0) return;
  for (int ilp = 1; ilp <= ilpmax; ++ilp) {
    int vi, dvi, s, es, evi;
    i = l[i];
    vi = v[i];
    if (last[vi] == 0) continue;
    if (last[vi] > 0) goto L8;
    tag = tag + 1;
    dvi = last[ek];
    s = l[vi];
  L2:
    s = l[s];
    if (s == 0) goto L9;
    es = v[s];
    if (next[es] < 0) goto L3;
    mark[es] = tag;
    dvi = dvi + 1;
    goto L2;
  L3:
    if (mark[es] < 0) goto L6;
    {
      int b = es;
      const int blpmax = last[es];
      for (int blp = 1; blp <= blpmax; ++blp) {
        b = l[b];
        const int vb = v[b];
        if (mark[vb] >= tag) continue;
        mark[vb] = tag;
        dvi = dvi + 1;
      }
    }
    goto L2;
  L6:
    last[vi] = 0;
    mark[es] = mark[es] - 1;
  L7:
    s = l[s];
    if (s == 0) continue;
    es = v[s];
    if (mark[es] < 0) mark[es] = mark[es] - 1;
    goto L7;
  L8:
    evi = last[vi];
    dvi = last[ek] + last[evi] + mark[evi];
    mark[evi] = 0;
  L9:
    next[vi] = head[dvi];
    head[dvi] = vi;
    last[vi] = -dvi;
    if (next[vi] > 0) last[next[vi]] = vi;
    if (dvi < *dmin) *dmin = dvi;
  }
}

/* :7-196 (odrv, path 1) and :198-357 (md) with the work length IMS gives
 * (nsp = 3 NEQ + 4 NJA, ImsLinearBase.f90:585): lorder[i] (0-based) is the
 * i-th eliminated node.  Returns odrv's flag (0 on success). */
int or_genmd(int n, const int *ia0, const int *ja0, int *lorder) {
  if (n <= 0) return 0;
  const int nja = ia0[n];
  const long long nsp = 3LL * n + 4LL * nja;
  const int mmax = (int)((nsp - n) / 2);
  if (mmax < n) return 10 * n + 1;
  int *ia = (int *)malloc(sizeof(int) * ((size_t)n + 2));
  int *ja = (int *)malloc(sizeof(int) * ((size_t)nja + 1));
  for (int i = 0; i <= n; ++i) ia[i + 1] = ia0[i] + 1;
  for (int k = 0; k < nja; ++k) ja[k + 1] = ja0[k] + 1;
  int *v = (int *)calloc((size_t)mmax + 1, sizeof(int));
  int *l = (int *)calloc((size_t)mmax + 1, sizeof(int));
  int *head = (int *)calloc(2 * (size_t)n + 2, sizeof(int));
  int *last = (int *)calloc((size_t)n + 1, sizeof(int));
  int *next = (int *)calloc((size_t)n + 1, sizeof(int));
  int tag = 0;
  int flag = md_init(n, ia, ja, mmax, v, l, head, last, next, tag);
  if (flag == 0) {
    int k = 0, dmin = 1, tail = 0;
    while (k < n) {
      while (head[dmin] <= 0) dmin = dmin + 1;
      const int vk = head[dmin];
      head[dmin] = next[vk];
      if (head[dmin] > 0) last[head[dmin]] = -dmin;
      k = k + 1;
      next[vk] = -k;
      last[vk] = dmin - 1;
      tag = tag + last[vk];
      v[vk] = tag;
      md_merge(vk, &tail, v, l, last, next);
      md_purge(&k, vk, tail, v, l, head, last, next);
      md_update(vk, &dmin, v, l, head, last, next);
    }
    for (int kk = 1; kk <= n; ++kk) {
      next[kk] = -next[kk];
      last[next[kk]] = kk;
    }
    for (int i = 1; i <= n; ++i) lorder[i - 1] = last[i] - 1;
  }
  free(ia); free(ja); free(v); free(l); free(head); free(last); free(next);
  return flag;
}

/* sparsekit.f90:353-447 (dperm with job 1: rperm then cperm with the same
 * permutation) -- row j of A becomes row perm[j] of B, its entries in the
 * same order, columns relabelled by perm -- and :61-161 (dvperm):
 * y[perm[j]] = x[j].  perm is IMS's LORDER as passed (ImsLinear.f90:653-658). */
void or_dperm(int n, const double *a, const int *ja, const int *ia, double *ao, int *jao,
              int *iao, const int *perm) {
  for (int j = 0; j < n; ++j) iao[perm[j] + 1] = ia[j + 1] - ia[j];
  iao[0] = 0;
  for (int j = 0; j < n; ++j) iao[j + 1] += iao[j];
  for (int ii = 0; ii < n; ++ii) {
    int ko = iao[perm[ii]];
    for (int k = ia[ii]; k < ia[ii + 1]; ++k) {
      jao[ko] = perm[ja[k]];
      if (a) ao[ko] = a[k];
      ++ko;
    }
  }
}

static void or_dvperm(int n, double *x, const int *perm, double *tmp) {
  for (int j = 0; j < n; ++j) tmp[perm[j]] = x[j];
  memcpy(x, tmp, sizeof(double) * n);
}

/* ImsLinearBase.f90:1148-1197, ims_calc_pcdims: the ILUT storage length. */
int or_ilut_iwk(int neq, const int *ia, int level) {
  if (level > 0) return neq * (level * 2 + 1);
  int iwk = 0;
  for (int n = 0; n < neq; ++n) {
    int i = ia[n + 1] - ia[n];
    if (i > iwk) iwk = i;
  }
  return neq * iwk;
}

/* ImsLinearBase.f90:1049-1092, ims_base_ilu0a: forward then backward solve.
 * sparskit2/ilut.f90:465-516 (lusol, the ILUT application) is the same
 * pair of sweeps over the ILUT storage. */
void or_ilu0a(int nja, int neq, const double *apc, const int *iapc, const int *japc,
              const double *r, double *d) {
  (void)nja;
  for (int n = 0; n < neq; ++n) {
    double tv = r[n];
    int ic0 = iapc[n];
    int iu = japc[n];
    for (int j = ic0; j < iu; ++j) tv = tv - apc[j] * d[japc[j]];
    d[n] = tv;
  }
  for (int n = neq - 1; n >= 0; --n) {
    int ic1 = iapc[n + 1];
    int iu = japc[n];
    double tv = d[n];
    for (int j = iu; j < ic1; ++j) tv = tv - apc[j] * d[japc[j]];
    d[n] = tv * apc[n];
  }
}

/* ImsLinearBase.f90:619-754, ims_base_scale: iopt 0 scales, 1 unscales. */
void or_scale(int iopt, int iscl, int neq, int nja, const int *ia, const int *ja,
              double *amat, double *x, double *b, double *dscale, double *dscale2) {
  (void)nja;
  if (iopt == 0) {
    if (iscl == 1) {
      for (int n = 0; n < neq; ++n) {
        double v = amat[ia[n]];
        double c1 = 1.0 / sqrt(fabs(v));
        dscale[n] = c1;
        dscale2[n] = c1;
      }
      for (int n = 0; n < neq; ++n) {
        double c1 = dscale[n];
        for (int i = ia[n]; i < ia[n + 1]; ++i) {
          double c2 = dscale2[ja[i]];
          amat[i] = c1 * amat[i] * c2;
        }
      }
    } else if (iscl == 2) {
      for (int n = 0; n < neq; ++n) {
        double c1 = 0.0;
        for (int i = ia[n]; i < ia[n + 1]; ++i) c1 = c1 + amat[i] * amat[i];
        c1 = sqrt(c1);
        c1 = (c1 == 0.0) ? 1.0 : 1.0 / c1;
        dscale[n] = c1;
        for (int i = ia[n]; i < ia[n + 1]; ++i) amat[i] = c1 * amat[i];
      }
      for (int n = 0; n < neq; ++n) dscale2[n] = 0.0;
      for (int n = 0; n < neq; ++n)
        for (int i = ia[n]; i < ia[n + 1]; ++i) {
          double c2 = amat[i];
          dscale2[ja[i]] = dscale2[ja[i]] + c2 * c2;
        }
      for (int n = 0; n < neq; ++n) {
        double c2 = dscale2[n];
        c2 = (c2 == 0.0) ? 1.0 : 1.0 / sqrt(c2);
        dscale2[n] = c2;
      }
      for (int n = 0; n < neq; ++n)
        for (int i = ia[n]; i < ia[n + 1]; ++i) amat[i] = dscale2[ja[i]] * amat[i];
    }
    for (int n = 0; n < neq; ++n) {
      x[n] = x[n] / dscale2[n];
      b[n] = b[n] * dscale[n];
    }
  } else {
    for (int n = 0; n < neq; ++n) {
      double c1 = dscale[n];
      for (int i = ia[n]; i < ia[n + 1]; ++i) {
        double c2 = dscale2[ja[i]];
        amat[i] = (1.0 / c1) * amat[i] * (1.0 / c2);
      }
      double c2 = dscale2[n];
      x[n] = x[n] * c2;
      b[n] = b[n] / c1;
    }
  }
}

/* ImsLinearBase.f90:30-240, ims_base_cg (single model).  The preconditioner
 * is applied by or_ilu0a for every IPC: ilu0a for ILU0/MILU0 and lusol for
 * ILUT/MILUT are the same sweeps over the IAPC/JAPC/APC storage. */
static void or_cg(int *icnvg, int itmax, int *innerit, int neq, int nja, int icnvgopt,
                  int north, double dvclose, double rclose, double l2norm0,
                  double epfact, const int *ia0, const int *ja0, const double *a0,
                  const int *iapc, const int *japc, const double *apc, double *x,
                  double *b, double *d, double *p, double *q, double *z,
                  or_cnvg_record *rec, int nrec, const or_models *mods) {
  double rho0 = 0.0, rho = 0.0;
  *innerit = 0;
  for (int iiter = 1; iiter <= itmax; ++iiter) {
    *innerit = *innerit + 1;
    or_ilu0a(nja, neq, apc, iapc, japc, d, z);
    rho = or_ddot(neq, d, z);
    if (iiter == 1) {
      for (int n = 0; n < neq; ++n) p[n] = z[n];
    } else {
      double beta = rho / rho0;
      for (int n = 0; n < neq; ++n) p[n] = z[n] + beta * p[n];
    }
    or_amux(neq, p, q, a0, ja0, ia0);
    double denominator = or_ddot(neq, p, q);
    denominator = denominator + f_sign(DPREC, denominator);
    double alpha = rho / denominator;
    double deltax = 0.0, rmax = 0.0, l2norm = 0.0;
    int xloc = -1, rloc = -1;
    /* per-model maxima (ImsLinearBase.f90:141-182): reset every iteration */
    const int nm = mods ? mods->nmod : 0;
    double mdv[64], mrm[64];
    for (int im = 0; im < nm; ++im) {
      mods->loc[2 * im] = -1;
      mods->loc[2 * im + 1] = -1;
      mdv[im] = 0.0;
      mrm[im] = 0.0;
    }
    int im = 0;
    for (int n = 0; n < neq; ++n) {
      while (nm > 0 && n == mods->modstart[im + 1]) ++im;
      double tv = alpha * p[n];
      x[n] = x[n] + tv;
      if (fabs(tv) > fabs(deltax)) {
        deltax = tv;
        xloc = n;
      }
      if (nm > 0 && fabs(tv) > fabs(mdv[im])) {
        mdv[im] = tv;
        mods->loc[2 * im] = n;
      }
      tv = d[n];
      tv = tv - alpha * q[n];
      d[n] = tv;
      if (fabs(tv) > fabs(rmax)) {
        rmax = tv;
        rloc = n;
      }
      if (nm > 0 && fabs(tv) > fabs(mrm[im])) {
        mrm[im] = tv;
        mods->loc[2 * im + 1] = n;
      }
      l2norm = l2norm + tv * tv;
    }
    l2norm = sqrt(l2norm);
    if (rec && iiter <= nrec) {
      or_cnvg_record *r = &rec[iiter - 1];
      r->dvmax = deltax; r->rmax = rmax; r->locdv = xloc; r->locr = rloc;
      r->l2norm = l2norm; r->alpha = alpha; r->beta = (iiter == 1) ? 0.0 : rho / rho0;
      r->rho = rho; r->omega = 0.0;
      for (int k = 0; k < nm; ++k) {
        const int o = (iiter - 1) * nm + k;
        mods->dvmax[o] = mdv[k]; mods->locdv[o] = mods->loc[2 * k];
        mods->rmax[o] = mrm[k]; mods->locr[o] = mods->loc[2 * k + 1];
      }
    }
    double rcnvg = (icnvgopt == 2 || icnvgopt == 3 || icnvgopt == 4) ? l2norm : rmax;
    or_testcnvg(icnvgopt, icnvg, *innerit, deltax, rcnvg, l2norm0, epfact, dvclose, rclose);
    if (rcnvg == 0.0) *icnvg = 1;
    if (*icnvg != 0) break;
    if (or_is_close(rho, rho0)) break;
    if (north > 0) {
      if ((iiter + 1) % north == 0) or_residual(neq, x, b, d, a0, ia0, ja0);
    }
    if (rho == 0.0) break;
    rho0 = rho;
  }
  if (*icnvg < 0) *icnvg = 0;
}

/* ImsLinearBase.f90:249-549, ims_base_bcgs (single model, every IPC). */
static void or_bcgs(int *icnvg, int itmax, int *innerit, int neq, int nja, int icnvgopt,
                    int north, int iscl, const double *dscale, double dvclose,
                    double rclose, double l2norm0, double epfact, const int *ia0,
                    const int *ja0, const double *a0, const int *iapc, const int *japc,
                    const double *apc, double *x, double *b, double *d, double *p,
                    double *q, double *t, double *v, double *dhat, double *phat,
                    double *qhat, or_cnvg_record *rec, int nrec, const or_models *mods) {
  *innerit = 0;
  double alpha = 0.0, alpha0 = 0.0, beta = 0.0, rho = 0.0, rho0 = 0.0;
  double omega = 0.0, omega0 = 0.0;
  for (int n = 0; n < neq; ++n) dhat[n] = d[n];
  for (int iiter = 1; iiter <= itmax; ++iiter) {
    *innerit = *innerit + 1;
    rho = or_ddot(neq, dhat, d);
    if (iiter == 1) {
      for (int n = 0; n < neq; ++n) p[n] = d[n];
    } else {
      beta = (rho / rho0) * (alpha0 / omega0);
      for (int n = 0; n < neq; ++n) p[n] = d[n] + beta * (p[n] - omega0 * v[n]);
    }
    or_ilu0a(nja, neq, apc, iapc, japc, p, phat);
    or_amux(neq, phat, v, a0, ja0, ia0);
    double denominator = or_ddot(neq, dhat, v);
    denominator = denominator + f_sign(DPREC, denominator);
    alpha = rho / denominator;
    for (int n = 0; n < neq; ++n) q[n] = d[n] - alpha * v[n];
    or_ilu0a(nja, neq, apc, iapc, japc, q, qhat);
    or_amux(neq, qhat, t, a0, ja0, ia0);
    double numerator = or_ddot(neq, t, q);
    denominator = or_ddot(neq, t, t);
    denominator = denominator + f_sign(DPREC, denominator);
    omega = numerator / denominator;
    double deltax = 0.0, rmax = 0.0, l2norm = 0.0;
    int xloc = -1, rloc = -1;
    /* per-model maxima (ImsLinearBase.f90:431-480): the values are reset
     * every iteration, the locations are not */
    const int nm = mods ? mods->nmod : 0;
    double mdv[64], mrm[64];
    for (int im = 0; im < nm; ++im) {
      mdv[im] = 0.0;
      mrm[im] = 0.0;
    }
    int im = 0;
    for (int n = 0; n < neq; ++n) {
      while (nm > 0 && n == mods->modstart[im + 1]) ++im;
      double tv = alpha * phat[n] + omega * qhat[n];
      x[n] = x[n] + tv;
      if (iscl != 0) tv = tv * dscale[n];
      if (fabs(tv) > fabs(deltax)) {
        deltax = tv;
        xloc = n;
      }
      if (nm > 0 && fabs(tv) > fabs(mdv[im])) {
        mdv[im] = tv;
        mods->loc[2 * im] = n;
      }
      tv = q[n] - omega * t[n];
      d[n] = tv;
      if (iscl != 0) tv = tv / dscale[n];
      if (fabs(tv) > fabs(rmax)) {
        rmax = tv;
        rloc = n;
      }
      if (nm > 0 && fabs(tv) > fabs(mrm[im])) {
        mrm[im] = tv;
        mods->loc[2 * im + 1] = n;
      }
      l2norm = l2norm + tv * tv;
    }
    l2norm = sqrt(l2norm);
    if (rec && iiter <= nrec) {
      or_cnvg_record *r = &rec[iiter - 1];
      r->dvmax = deltax; r->rmax = rmax; r->locdv = xloc; r->locr = rloc;
      r->l2norm = l2norm; r->alpha = alpha; r->beta = beta; r->rho = rho; r->omega = omega;
      for (int k = 0; k < nm; ++k) {
        const int o = (iiter - 1) * nm + k;
        mods->dvmax[o] = mdv[k]; mods->locdv[o] = mods->loc[2 * k];
        mods->rmax[o] = mrm[k]; mods->locr[o] = mods->loc[2 * k + 1];
      }
    }
    double rcnvg = (icnvgopt == 2 || icnvgopt == 3 || icnvgopt == 4) ? l2norm : rmax;
    or_testcnvg(icnvgopt, icnvg, *innerit, deltax, rcnvg, l2norm0, epfact, dvclose, rclose);
    if (rcnvg == 0.0) *icnvg = 1;
    if (*icnvg != 0) break;
    if (or_is_close(rho, rho0)) break;
    if (or_is_close(alpha, alpha0)) break;
    if (or_is_close(omega, omega0)) break;
    if (north > 0) {
      if ((iiter + 1) % north == 0) or_residual(neq, x, b, d, a0, ia0, ja0);
    }
    if (rho * omega == 0.0) break;
    rho0 = rho;
    alpha0 = alpha;
    omega0 = omega;
  }
  if (*icnvg < 0) *icnvg = 0;
}

/* ImsLinear.f90:111-339 (imslinear_ar, the parts that do not read files):
 * choose IPC (:178-185), build IAPC/JAPC for ILU0/MILU0 (:244-248) or size
 * the ILUT storage (ims_calc_pcdims, :227-228). */
struct or_ims {
  or_ims_settings s;
  int neq, nja, ipc;
  int *ia, *ja; /* 0-based copies */
  int *iapc, *japc;
  double *apc, *w;
  int *iw;
  int njapc, iwk;  /* storage of IAPC/JAPC/APC; ILUT: the reference's iwk */
  int *jw, *jr;    /* ILUT work arrays */
  int ilut_ierr;
  int *lorder, *iorder;  /* REORDERING_METHOD RCM: LORDER/IORDER */
  int *iaro, *jaro;      /* the permuted pattern */
  int md_flag;           /* odrv's flag (MD) */
  double *aro, *tmp;
  double *d, *p, *q, *z, *t, *v, *dhat, *phat, *qhat;
  double *dscale, *dscale2;
  double l2norm0, epfact;
  int npivot_retries;
  const or_models *mods; /* per-model records, or NULL */
};

void or_ims_set_models(or_ims *h, const or_models *m) { h->mods = (m && m->nmod > 0 && m->nmod <= 64) ? m : NULL; }

or_ims *or_ims_create(const or_ims_settings *s, int neq, int nja, const int *ia,
                      const int *ja) {
  or_ims *h = (or_ims *)calloc(1, sizeof(or_ims));
  h->s = *s;
  h->neq = neq;
  h->nja = nja;
  if (s->level > 0 || s->droptol > 0.0) h->ipc = 3;
  else h->ipc = 1;
  if (s->relax > 0.0) h->ipc += 1;
  h->ia = (int *)malloc(sizeof(int) * (neq + 1));
  h->ja = (int *)malloc(sizeof(int) * nja);
  memcpy(h->ia, ia, sizeof(int) * (neq + 1));
  memcpy(h->ja, ja, sizeof(int) * nja);
  h->njapc = nja;
  if (h->ipc == 3 || h->ipc == 4) {
    h->iwk = or_ilut_iwk(neq, ia, s->level);
    h->njapc = h->iwk > neq + 1 ? h->iwk : neq + 1;
    h->jw = (int *)calloc(neq, sizeof(int));
    h->jr = (int *)calloc(neq, sizeof(int));
  }
  h->iapc = (int *)calloc(neq + 1, sizeof(int));
  h->japc = (int *)calloc(h->njapc, sizeof(int));
  h->apc = (double *)calloc(h->njapc, sizeof(double));
  h->iw = (int *)calloc(neq, sizeof(int));
  h->w = (double *)calloc(neq, sizeof(double));
  double **vecs[] = {&h->d, &h->p, &h->q, &h->z, &h->t, &h->v, &h->dhat, &h->phat,
                     &h->qhat, &h->dscale, &h->dscale2};
  for (size_t i = 0; i < sizeof(vecs) / sizeof(vecs[0]); ++i)
    *vecs[i] = (double *)calloc(neq, sizeof(double));
  for (int n = 0; n < neq; ++n) {
    h->dscale[n] = 1.0;
    h->dscale2[n] = 1.0;
  }
  if (h->ipc == 1 || h->ipc == 2) or_pccrs(neq, nja, h->ia, h->ja, h->iapc, h->japc);
  /* ims_base_calc_order (ImsLinearBase.f90:556-610), after the IAPC/JAPC
   * above were built from the unpermuted pattern (ImsLinear.f90:244-248,
   * 333-336) */
  if (s->iord == 1 || s->iord == 2) {
    h->lorder = (int *)malloc(sizeof(int) * neq);
    h->iorder = (int *)malloc(sizeof(int) * neq);
    if (s->iord == 1) or_genrcm(neq, h->ia, h->ja, h->lorder);
    else h->md_flag = or_genmd(neq, h->ia, h->ja, h->lorder);
    for (int n = 0; n < neq; ++n) h->iorder[h->lorder[n]] = n;
    h->iaro = (int *)calloc(neq + 1, sizeof(int));
    h->jaro = (int *)calloc(nja, sizeof(int));
    h->aro = (double *)calloc(nja, sizeof(double));
    h->tmp = (double *)calloc(neq, sizeof(double));
  }
  return h;
}

const int *or_ims_lorder(const or_ims *h) { return h->lorder; }

void or_ims_destroy(or_ims *h) {
  if (!h) return;
  free(h->ia); free(h->ja); free(h->iapc); free(h->japc); free(h->apc);
  free(h->iw); free(h->w); free(h->d); free(h->p); free(h->q); free(h->z);
  free(h->t); free(h->v); free(h->dhat); free(h->phat); free(h->qhat);
  free(h->dscale); free(h->dscale2);
  free(h->jw); free(h->jr);
  free(h->lorder); free(h->iorder); free(h->iaro); free(h->jaro); free(h->aro); free(h->tmp);
  free(h);
}

int or_ims_ipc(const or_ims *h) { return h->ipc; }
int or_ims_njapc(const or_ims *h) { return h->njapc; }
int or_ims_ilut_ierr(const or_ims *h) { return h->ilut_ierr; }
const int *or_ims_iapc(const or_ims *h) { return h->iapc; }
const int *or_ims_japc(const or_ims *h) { return h->japc; }
const double *or_ims_apc(const or_ims *h) { return h->apc; }
double or_ims_l2norm0(const or_ims *h) { return h->l2norm0; }
int or_ims_pivot_retries(const or_ims *h) { return h->npivot_retries; }

/* ImsLinear.f90:617-750, imslinear_ap (IORD 0 or 1). */
int or_ims_apply(or_ims *h, double *amat, double *rhs, double *x, int kstp, int kiter,
                 int *icnvg, int *in_iter, or_cnvg_record *rec, int nrec) {
  const or_ims_settings *s = &h->s;
  int neq = h->neq, nja = h->nja;
  /* ImsLinearBase.f90:590-595: an MD failure is fatal in the reference */
  if (s->iord == 2 && h->md_flag != 0) return -2;
  h->epfact = or_epfact(s->icnvgopt, kstp);
  if (s->iscl != 0)
    or_scale(0, s->iscl, neq, nja, h->ia, h->ja, amat, x, rhs, h->dscale, h->dscale2);
  /* PERMUTE ROWS, COLUMNS, AND RHS (:652-666): the solve works on
   * A0/IA0/JA0; IAPC/JAPC stay those of the unpermuted pattern */
  const int *ia0 = h->ia, *ja0 = h->ja;
  const double *a0 = amat;
  if (s->iord != 0) {
    or_dperm(neq, amat, h->ja, h->ia, h->aro, h->jaro, h->iaro, h->lorder);
    or_dvperm(neq, x, h->lorder, h->tmp);
    or_dvperm(neq, rhs, h->lorder, h->tmp);
    ia0 = h->iaro;
    ja0 = h->jaro;
    a0 = h->aro;
  }
  if (h->ipc == 1 || h->ipc == 2) {
    h->npivot_retries = or_pcu(nja, neq, h->ipc, s->relax, a0, ia0, ja0, h->apc,
                               h->iapc, h->japc, h->iw, h->w);
  } else {
    int rc = or_pcu_ilut(neq, s->level, s->droptol, s->relax, a0, ia0, ja0, h->apc,
                         h->iapc, h->japc, h->iwk, h->w, h->jw, h->jr);
    /* ImsLinearBase.f90:822-834: an ilut error is fatal in the reference */
    h->ilut_ierr = rc < 0 ? rc : 0;
    if (rc < 0) return -4;
    h->npivot_retries = rc;
  }
  (void)kiter;
  *icnvg = 0;
  for (int n = 0; n < neq; ++n) {
    h->d[n] = 0.0; h->p[n] = 0.0; h->q[n] = 0.0; h->z[n] = 0.0;
  }
  or_residual(neq, x, rhs, h->d, a0, ia0, ja0);
  h->l2norm0 = or_dnrm2(neq, h->d);
  int itmax = s->iter1;
  if (h->l2norm0 == 0.0) {
    itmax = 0;
    *icnvg = 1;
  }
  int innerit = 0;
  if (s->ilinmeth == 1) {
    or_cg(icnvg, itmax, &innerit, neq, nja, s->icnvgopt, s->north, s->dvclose,
          s->rclose, h->l2norm0, h->epfact, ia0, ja0, a0, h->iapc, h->japc,
          h->apc, x, rhs, h->d, h->p, h->q, h->z, rec, nrec, h->mods);
  } else {
    /* DSCALE keeps the unpermuted numbering, as in the reference */
    or_bcgs(icnvg, itmax, &innerit, neq, nja, s->icnvgopt, s->north, s->iscl,
            h->dscale, s->dvclose, s->rclose, h->l2norm0, h->epfact, ia0, ja0,
            a0, h->iapc, h->japc, h->apc, x, rhs, h->d, h->p, h->q, h->t, h->v,
            h->dhat, h->phat, h->qhat, rec, nrec, h->mods);
  }
  /* BACK PERMUTE (:730-737); AMAT itself was not permuted in place */
  if (s->iord != 0) {
    or_dvperm(neq, x, h->iorder, h->tmp);
    or_dvperm(neq, rhs, h->iorder, h->tmp);
  }
  if (s->iscl != 0)
    or_scale(1, s->iscl, neq, nja, h->ia, h->ja, amat, x, rhs, h->dscale, h->dscale2);
  *in_iter = innerit;
  return 0;
}

int ims_ilinmeth(const or_ims *h) { return h->s.ilinmeth; }

/* FMA-contracted variants of amux and ilu0a: the same loops with a*b+c
 * evaluated as one fused operation, which is what gfortran emits on aarch64
 * (GNU -ffp-contract=fast default) and what the GPU kernels compute. */
void or_amux_fma(int n, const double *x, double *y, const double *a, const int *ja,
                 const int *ia) {
  for (int i = 0; i < n; ++i) {
    double t = 0.0;
    for (int k = ia[i]; k < ia[i + 1]; ++k) t = fma(a[k], x[ja[k]], t);
    y[i] = t;
  }
}

void or_ilu0a_fma(int neq, const double *apc, const int *iapc, const int *japc,
                  const double *r, double *d) {
  for (int n = 0; n < neq; ++n) {
    double tv = r[n];
    for (int j = iapc[n]; j < japc[n]; ++j) tv = fma(-apc[j], d[japc[j]], tv);
    d[n] = tv;
  }
  for (int n = neq - 1; n >= 0; --n) {
    double tv = d[n];
    for (int j = japc[n]; j < iapc[n + 1]; ++j) tv = fma(-apc[j], d[japc[j]], tv);
    d[n] = tv * apc[n];
  }
}
