// k_gwf.cuh -- device views and launchers of the GWF assembly kernels (k_gwf.cu).
#pragma once
#include "gbims_internal.cuh"

namespace gb {

// Grid connectivity and NPF properties on the device (Connections.f90:26-35,
// gwf-npf.f90 k11/k33/icelltype and options).  Indices are 0-based.
struct NpfDev {
  const int *ia, *ja, *jas, *isym, *ihc;
  const double *cl1, *cl2, *hwva;
  const double *top, *bot, *k11, *k33;
  const int *icelltype;
  int inewton, ivarcv, idewatcv, icellavg;
  double satomega;
};

// Storage and boundary inputs of one fill.  bnd_ptr/bnd_val list, per node,
// the WEL q then the RCH rate*area values in package and list order.
struct FillDev {
  int transient;
  int fn = 1;   // add the Newton terms (npf_fn, sto_fn) when the model uses Newton
  double tled;  // 1/delt
  const double *ss, *sy, *area;
  const int *bnd_ptr;
  const double *bnd_val;
};

void gwf_condsat(int nodes, const NpfDev &g, double *condsat, cudaStream_t st);
void gwf_npf_cf(int nodes, const NpfDev &g, const int *ibound, const double *h, double *sat,
                cudaStream_t st);
void gwf_fill(int nodes, const NpfDev &g, const FillDev &f, const int *ibound, const double *h,
              const double *hold, const double *sat, const double *condsat, double *amat,
              double *rhs, cudaStream_t st);
void gwf_ptc_resid(int nodes, const int *ia, const int *ja, const double *amat, const double *x,
                   const double *rhs, const int *ibound, const double *vol, double *part, int G,
                   cudaStream_t st);
void gwf_l2_resid(int nodes, const int *ia, const int *ja, const double *amat, const double *x,
                  const double *rhs, const int *ibound, double *part, int G, cudaStream_t st);
void gwf_fixups(int nodes, const int *ia, const int *ja, const int *active, int isymmetric,
                double *amat, double *rhs, const double *x, double *xtemp, cudaStream_t st);
void gwf_ptc_apply(int nodes, const int *ia, const int *ibound, double ptcval, double *amat,
                   double *rhs, const double *x, cudaStream_t st);
void gwf_dxmax(int nodes, const int *active, const double *x, const double *xtemp, double *part,
               int G, cudaStream_t st);
void gwf_underrelax(int nodes, int nonmeth, int kiter, double theta, double akappa, double gamma,
                    double amomentum, const int *active, double *x, const double *xtemp,
                    double *wsave, double *hchold, double *deold, double *dxold, cudaStream_t st);
void gwf_relax_scale(int nodes, double relax, const int *active, double *x, const double *xtemp,
                     double *dxold, cudaStream_t st);
void gwf_calcdx(int nodes, const int *active, const double *x, const double *xtemp, double *dx,
                cudaStream_t st);
void gwf_npf_nur(int nodes, const int *ibotnode, const NpfDev &g, const int *ibound, double *x,
                 const double *xtemp, double *dx, int *flag, cudaStream_t st);
// apply_backtracking: x = xtemp + breduc * (x - xtemp) on active cells
void gwf_backtrack(int nodes, double breduc, const int *active, double *x, const double *xtemp,
                   cudaStream_t st);
// Flows and model budget terms; part holds kGwfBudgetSlots doubles per block
// (in/out of STO-SS, STO-SY, CHD, WEL, RCH; max |flowja diagonal|, its row).
constexpr int kGwfBudgetSlots = 12;
void gwf_budget(int nodes, const NpfDev &g, const FillDev &f, const int *bnd_kind,
                const int *ibound, const double *h, const double *hold, const double *sat,
                const double *condsat, double *flowja, double *part, int G, cudaStream_t st);

}  // namespace gb
