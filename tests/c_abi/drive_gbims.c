/* A C caller of libgbims.so: the allocate / apply / deallocate sequence a
 * host makes in place of imslinear_allocate, imslinear_apply and
 * imslinear_da (ImsLinear.f90:111-339, 617-750, 495-552), with Fortran
 * (1-based) CSR arrays as NumericalSolution holds them.
 *
 * The system is a 2-D 5-point grid with the diagonal first in every row and
 * the rest ascending (SparseMatrix.f90:16), constant heads on the first and
 * last columns (rows with only a diagonal), and a source everywhere else.
 * The program solves it with PCG + ILU0 and with BiCGSTAB + ILU0, checks
 * ICNVG, the residual of the returned heads on the host, the per-iteration
 * records, and the status of a call with a bad argument.  It prints
 * "drive_gbims ok" and exits 0 on success. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbims.h"

#define NX 61
#define NY 47

/* conductance of the connection n-m, the same from either side */
static double cond(int n, int m) {
  const int lo = n < m ? n : m, hi = n < m ? m : n;
  return 1.0 + 0.5 * ((lo * 7 + hi * 13) % 5);
}

static int fail(const char *what, int rc) {
  printf("drive_gbims FAILED: %s (status %d: %s)\n", what, rc, gbims_status_string(rc));
  return 1;
}

int main(void) {
  const int neq = NX * NY;
  int *ia = malloc(sizeof(int) * (neq + 1));
  int *ja = malloc(sizeof(int) * 5 * neq);
  double *amat = malloc(sizeof(double) * 5 * neq);
  double *rhs = malloc(sizeof(double) * neq);
  double *x = malloc(sizeof(double) * neq);
  int nja = 0;
  for (int n = 0; n < neq; ++n) {
    const int i = n / NX, j = n % NX;
    ia[n] = nja + 1;
    const int fixed = (j == 0 || j == NX - 1);
    ja[nja] = n + 1;
    amat[nja++] = fixed ? 1.0 : 0.0;
    if (fixed) {
      rhs[n] = (j == 0) ? 10.0 : 0.0;
      continue;
    }
    double diag = 0.0;
    const int nb[4] = {i > 0 ? n - NX : -1, n - 1, n + 1, i < NY - 1 ? n + NX : -1};
    for (int k = 0; k < 4; ++k) {
      if (nb[k] < 0) continue;
      const int jn = nb[k] % NX;
      const double c = cond(n, nb[k]);
      diag -= c;
      if (jn == 0 || jn == NX - 1) continue; /* constant head moved to the rhs below */
      ja[nja] = nb[k] + 1;
      amat[nja++] = c;
    }
    amat[ia[n] - 1] = diag;
    rhs[n] = -0.01;
    for (int k = 0; k < 4; ++k) {
      if (nb[k] < 0) continue;
      const int jn = nb[k] % NX;
      if (jn == 0) rhs[n] -= cond(n, nb[k]) * 10.0;
    }
  }
  ia[neq] = nja + 1;
  for (int ilinmeth = 1; ilinmeth <= 2; ++ilinmeth) {
    gbims_settings s;
    memset(&s, 0, sizeof(s));
    s.dvclose = 1e-9;
    s.rclose = 1e-8;
    s.iter1 = 1000;
    s.ilinmeth = ilinmeth;
    s.precision = GBIMS_FP64;
    s.index_base = 1;
    gbims_handle *h = NULL;
    int rc = gbims_create(&s, neq, nja, ia, ja, &h);
    if (rc < 0) return fail(gbims_last_error(h), rc);
    const int modstart[3] = {1, 1 + neq / 2, neq + 1};
    rc = gbims_set_inner_records(h, 2000, 2, modstart);
    if (rc < 0) return fail("gbims_set_inner_records", rc);
    for (int n = 0; n < neq; ++n) x[n] = 5.0;
    int icnvg = 0, in_iter = 0;
    gbims_summary sm;
    rc = gbims_apply(h, amat, rhs, x, 1, 1, &icnvg, &in_iter, &sm);
    if (rc < 0) return fail(gbims_last_error(h), rc);
    if (icnvg != 1 || in_iter < 1) return fail("no closure", icnvg);
    /* residual of the returned heads, on the host */
    double rmax = 0.0;
    for (int n = 0; n < neq; ++n) {
      double r = rhs[n];
      for (int q = ia[n] - 1; q < ia[n + 1] - 1; ++q) r -= amat[q] * x[ja[q] - 1];
      if (fabs(r) > rmax) rmax = fabs(r);
    }
    if (!(rmax <= 1e-6)) return fail("residual of the returned heads", (int)(rmax * 1e6));
    int nrec = 0;
    int *it = malloc(sizeof(int) * in_iter), *ldv = malloc(sizeof(int) * 2 * in_iter),
        *lr = malloc(sizeof(int) * 2 * in_iter);
    double *al = malloc(sizeof(double) * in_iter), *om = malloc(sizeof(double) * in_iter),
           *dv = malloc(sizeof(double) * 2 * in_iter), *rm = malloc(sizeof(double) * 2 * in_iter);
    rc = gbims_get_inner_records(h, in_iter, &nrec, it, al, om, ldv, dv, lr, rm);
    if (rc < 0 || nrec != in_iter) return fail("gbims_get_inner_records", rc);
    for (int k = 0; k < nrec; ++k) {
      if (it[k] != k + 1) return fail("ITINNER", it[k]);
      for (int im = 0; im < 2; ++im) {
        const int l = ldv[2 * k + im];
        if (l != 0 && (l < modstart[im] || l >= modstart[im + 1])) return fail("locdv outside its model", l);
      }
      if ((ilinmeth == 1) != (om[k] == 0.0)) return fail("CACCEL omega", k);
    }
    free(it); free(ldv); free(lr); free(al); free(om); free(dv); free(rm);
    /* an argument error comes back as a status, not an exit */
    if (gbims_apply(h, NULL, rhs, x, 1, 1, &icnvg, &in_iter, &sm) != GBIMS_ERR_ARG)
      return fail("NULL amat was accepted", 0);
    printf("  %s: %d inner iterations, max |b - Ax| %.3e, structured %d\n",
           ilinmeth == 1 ? "PCG" : "BiCGSTAB", in_iter, rmax, sm.structured);
    gbims_destroy(h);
  }
  free(ia); free(ja); free(amat); free(rhs); free(x);
  printf("drive_gbims ok\n");
  return 0;
}
