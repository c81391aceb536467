/*
 * gwf_oracle.h -- CPU restatement of GWF assembly and the outer loop.
 * TEST INFRASTRUCTURE ONLY (the oracle); the product never includes this.
 */
#ifndef GWF_ORACLE_H
#define GWF_ORACLE_H

#include "ims_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A single DIS model with NPF/STO/CHD/WEL/RCH.  All indices 0-based.  The
 * struct only borrows the arrays; the caller keeps them alive. */
typedef struct {
  int nlay, nrow, ncol, nodes, nja, njas;
  const int *ia, *ja, *isym, *jas, *ihc;
  const double *cl1, *cl2, *hwva;
  const double *top, *bot, *area;
  const double *k11, *k33;
  const int *icelltype;
  int inewton, ivarcv, idewatcv, icellavg;
  double satomega;
  /* NEWTON UNDER_RELAXATION (gwf.f90:181): npf_nur runs only when it is set
   * together with inewton (gwf_nur, gwf.f90:717) */
  int inewtonur;
  /* storage */
  const double *ss, *sy;
  const int *iconvert;
  /* boundaries */
  int nwel;
  const int *wel_node;
  const double *wel_q;
  int nrch;
  const int *rch_node;
  const double *rch_rate;
  int nchd;
  const int *chd_node;
  const double *chd_head;
  /* XT3D (NPF option XT3D): 0 off, 1 the matrix form, 2 XT3D RHS.  ck: the
   * conductivity tensor per cell (9, row-major, or_xt3d_ck); nozee when
   * ANGLE2 is not given.  With XT3D amat is indexed by the solution pattern
   * sia/sja (nja_sln entries: the connections and the neighbours of
   * neighbours), idxglo maps each model position into it. */
  int ixt3d, nozee, nja_sln;
  const double *ck;
  const int *sia, *sja, *idxglo;
  /* the grid's connection geometry for XT3D: 0 DIS (from the cell's row
   * and column), 1 DISV, 2 DISU (cell centres xc/yc per node, anglex per
   * connection n < m in radians) */
  int xt_grid;
  const double *xc, *yc, *anglex;
  /* hy_eff per connection n < m (2 each: from n toward m, from m toward
   * n) when K22 or the angles are given (or_npf_hy), else NULL */
  const double *hy;
} or_gwf_model;

/* NONLINEAR block state (NumericalSolution.f90 members). */
typedef struct {
  double dvclose;
  int mxiter, nonmeth, iallowptc;
  double theta, akappa, gamma, amomentum;
  double bigch, bigchold, relaxold;
  double *wsave, *hchold, *deold, *dxold; /* length neq, caller-owned */
  /* backtracking (BACKTRACKING_NUMBER, _TOLERANCE, _REDUCTION_FACTOR,
   * _RESIDUAL_LIMIT); numtrack 0 switches it off */
  int numtrack;
  double btol, breduc, res_lim;
  double res_prev, res_new; /* state */
} or_nonlinear;

typedef struct {
  int outer, inner_total, converged, pivot_retries;
  double last_dxmax;
  int backtracks; /* backtracking steps taken in the time step */
} or_timestep_stats;

void or_dis_sizes(int nlay, int nrow, int ncol, int *nodes, int *nja, int *njas);
void or_dis_connect(int nlay, int nrow, int ncol, const double *delr, const double *delc,
                    const double *top, const double *bot, int *ia, int *ja, int *isym,
                    int *jas, int *ihc, double *cl1, double *cl2, double *hwva);
int or_disv_connect(int nlay, int ncpl, const double *vx, const double *vy, const int *iavert,
                    const int *javert, const double *xc, const double *yc, const double *top,
                    const double *bot, const int *nodereduced, int cap, int *ia, int *ja,
                    int *isym, int *jas, int *ihc, double *cl1, double *cl2, double *hwva,
                    double *area);
/* DISU: disuconnections + con_finalize (Connections.f90:801-928, 160-316).
 * iainp (nodesuser+1, 0-based offsets from IAC), jainp (1-based, a negative
 * number read as its magnitude), ihcinp/cl12inp/hwvainp per entry;
 * nodereduced (nodesuser, 0-based reduced number or -1) or NULL for a full
 * grid.  Returns nja, or -1 (cap too small), -2 (diagonal not first), -3 (a
 * row not ascending), -4 (no symmetric counterpart), -5 (IHC not
 * symmetric), -6 (HWVA not symmetric), -7 (IHC outside 0..2), -8 (no
 * active cell). */
int or_disu_connect(int nodesuser, const int *iainp, const int *jainp, const int *ihcinp,
                    const double *cl12inp, const double *hwvainp, const double *angldegxinp,
                    const int *nodereduced, int cap, int *nodes, int *ia, int *ja, int *isym,
                    int *jas, int *ihc, double *cl1, double *cl2, double *hwva, double *anglex);
/* DisvGeom.f90:193-199 and :394-412 (cprops' anglex): the angle of the
 * shared edge's normal for each horizontal connection n < m of a DISV grid
 * (nodeuser: reduced -> user cell, or NULL), 0 for vertical ones */
void or_disv_anglex(int nodes, int ncpl, const double *vx, const double *vy, const int *iavert,
                    const int *javert, const int *nodeuser, const int *ia, const int *ja,
                    const int *jas, const int *ihc, double *anglex);
void or_xt3d_ck(int nodes, const double *k11, const double *k22, const double *k33,
                const double *angle1, const double *angle2, const double *angle3, int nozee,
                double *ck);
int or_xt3d_pattern(int nodes, const int *ia, const int *ja, int cap, int *sia, int *sja,
                    int *idxglo);
int or_xt3d_fc(const or_gwf_model *m, const int *ibound, const double *sat,
               const double *hnew, double *amat, double *rhs, double *qsat);
void or_xt3d_flowja(const or_gwf_model *m, const int *ibound, const double *sat,
                    const double *hnew, double *flowja);
void or_xt3d_fn(const or_gwf_model *m, const int *ibound, const double *hnew,
                const double *qsat, double *amat, double *rhs);
/* hy_eff (gwf-npf.f90:2280-2357) with hyeff (HGeoUtil.f90:29-108) for
 * every connection n < m: hy[2s] of cell n toward m, hy[2s+1] of m toward
 * n; k22 NULL for none, angles in radians or NULL. */
void or_npf_hy(const or_gwf_model *m, const double *k22, const double *angle1,
               const double *angle2, const double *angle3, int iavgkeff, double *hy);
double or_squadratic_sat(double top, double bot, double x, double eps);
double or_squadratic_sat_derv(double top, double bot, double x, double eps);
void or_npf_condsat(const or_gwf_model *m, double *condsat);
void or_npf_cf(const or_gwf_model *m, const int *ibound, const double *hnew, double *sat);
void or_npf_fc(const or_gwf_model *m, const int *ibound, const double *condsat,
               const double *sat, const double *hnew, double *amat, double *rhs);
void or_npf_fn(const or_gwf_model *m, const int *ibound, const double *condsat,
               const double *hnew, double *amat, double *rhs);
void or_npf_nur(const or_gwf_model *m, const int *ibound, double *x, const double *xtemp,
                double *dx, int *inewtonur, double *dxmax, int *locmax);
void or_sto_fc(const or_gwf_model *m, const int *ibound, double delt, const double *hold,
               const double *hnew, double *amat, double *rhs);
void or_sto_fn(const or_gwf_model *m, const int *ibound, double delt, const double *hnew,
               double *amat, double *rhs);
void or_bnd_fc(const or_gwf_model *m, const int *ibound, double *amat, double *rhs);
void or_gwf_fc(const or_gwf_model *m, const int *ibound, const double *condsat,
               double *sat, double delt, int transient, const double *hold,
               const double *hnew, double *amat, double *rhs);
void or_sln_ls_fixups(int neq, const int *ia, const int *ja, const int *active,
                      int isymmetric, double *amat, double *rhs, const double *x,
                      double *xtemp);
double or_sln_get_dxmax(int neq, const int *active, const double *x, const double *xtemp,
                        int *lrch);
void or_sln_underrelax(or_nonlinear *nl, int kiter, double bigch, int neq,
                       const int *active, double *x, const double *xtemp);
void or_gwf_budget(const or_gwf_model *m, const int *ibound, const double *condsat,
                   const double *sat, double delt, int transient, const double *hold,
                   const double *hnew, double *flowja, double *terms);
int or_gwf_timestep(const or_gwf_model *m, or_ims *ims, or_nonlinear *nl,
                    const double *condsat, int *ibound, int kper, int kstp, double delt,
                    int transient, double *x, double *xold, or_timestep_stats *st);

int ims_ilinmeth(const or_ims *h);

#ifdef __cplusplus
}
#endif
#endif
