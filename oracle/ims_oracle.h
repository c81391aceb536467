/*
 * ims_oracle.h -- CPU restatement of MODFLOW 6 IMS and GWF hot-path routines.
 * TEST INFRASTRUCTURE ONLY (the oracle); the product never includes this.
 */
#ifndef IMS_ORACLE_H
#define IMS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double dvclose, rclose;
  int icnvgopt, iter1, ilinmeth, iscl, iord, north;
  double relax;
  int level;
  double droptol;
} or_ims_settings;

/* one record per inner iteration (ConvergenceSummary.f90 fields, one model) */
typedef struct {
  double dvmax, rmax, l2norm, alpha, beta, rho, omega;
  int locdv, locr;
} or_cnvg_record;

typedef struct or_ims or_ims;

/* Per-model rows of the convergence records (CONVNMOD, CONVMODSTART and the
 * ConvergenceSummary arrays convdvmax, convlocdv, convrmax, convlocr; layout
 * [nrec][nmod], model fastest).  modstart: first row of each model, 0-based,
 * nmod + 1 entries ending at neq.  loc holds the per-model locations that the
 * reference keeps in summary%locdv/locr between iterations (2*nmod, -1 at
 * the start). */
typedef struct {
  int nmod;
  const int *modstart;
  double *dvmax, *rmax;
  int *locdv, *locr;
  int *loc;
} or_models;

int or_is_close(double a, double b);
void or_amux(int n, const double *x, double *y, const double *a, const int *ja, const int *ia);
double or_ddot(int n, const double *x, const double *y);
double or_dnrm2(int n, const double *x);
void or_residual(int neq, const double *x, const double *b, double *d, const double *a,
                 const int *ia, const int *ja);
double or_epfact(int icnvgopt, int kstp);
void or_testcnvg(int icnvgopt, int *icnvg, int iiter, double dvmax, double rmax,
                 double rmax0, double epfact, double dvclose, double rclose);
void or_pccrs(int neq, int nja, const int *ia, const int *ja, int *iapc, int *japc);
void or_pcilu0(int nja, int neq, const double *amat, const int *ia, const int *ja,
               double *apc, const int *iapc, const int *japc, int *iw, double *w,
               double relax, int *ipcflag, double delta);
int or_pcu(int nja, int neq, int ipc, double relax, const double *amat, const int *ia,
           const int *ja, double *apc, const int *iapc, const int *japc, int *iw, double *w);
void or_ilu0a(int nja, int neq, const double *apc, const int *iapc, const int *japc,
              const double *r, double *d);
void or_scale(int iopt, int iscl, int neq, int nja, const int *ia, const int *ja,
              double *amat, double *x, double *b, double *dscale, double *dscale2);

void or_amux_fma(int n, const double *x, double *y, const double *a, const int *ja, const int *ia);
void or_ilu0a_fma(int neq, const double *apc, const int *iapc, const int *japc, const double *r,
                  double *d);

or_ims *or_ims_create(const or_ims_settings *s, int neq, int nja, const int *ia, const int *ja);
void or_ims_destroy(or_ims *h);
int or_ims_apply(or_ims *h, double *amat, double *rhs, double *x, int kstp, int kiter,
                 int *icnvg, int *in_iter, or_cnvg_record *rec, int nrec);
int or_ims_ipc(const or_ims *h);
/* Per-model records for the next applies (NULL: none). */
void or_ims_set_models(or_ims *h, const or_models *m);
int or_ims_njapc(const or_ims *h);
int or_ims_ilut_ierr(const or_ims *h);
int or_ilut(int n, const double *a, const int *ja, const int *ia, int lfil, double droptol,
            double *alu, int *iapc, int *japc, int iwk, double *w, int *jw, int *jr,
            double relax, int *izero, double delta);
int or_pcu_ilut(int neq, int lfil, double droptol, double relax, const double *amat,
                const int *ia, const int *ja, double *alu, int *iapc, int *japc, int iwk,
                double *w, int *jw, int *jr);
int or_ilut_iwk(int neq, const int *ia, int level);
void or_genrcm(int n, const int *ia0, const int *ja0, int *lorder);
int or_genmd(int n, const int *ia0, const int *ja0, int *lorder);
void or_dperm(int n, const double *a, const int *ja, const int *ia, double *ao, int *jao,
              int *iao, const int *perm);
const int *or_ims_lorder(const or_ims *h);
const int *or_ims_iapc(const or_ims *h);
const int *or_ims_japc(const or_ims *h);
const double *or_ims_apc(const or_ims *h);
double or_ims_l2norm0(const or_ims *h);
int or_ims_pivot_retries(const or_ims *h);

#ifdef __cplusplus
}
#endif
#endif
