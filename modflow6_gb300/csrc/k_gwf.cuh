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
  // hy_eff per connection n < m (2 each: from n toward m, from m toward n)
  // when K22 or the angles are given; nullptr: K11 horizontal, K33 vertical
  const double *hy = nullptr;
};

// XT3D (Xt3dInterface.f90, Xt3dAlgorithm.f90), the NPF formulation with the
// full conductivity tensor on the neighbours-of-neighbours stencil, matrix
// form, on DIS grids.  With XT3D on, amat is indexed by the solution pattern
// sia/sja (each row: the connections and the neighbours of the neighbours,
// diagonal first, ascending); idxglo maps a model position into it.
constexpr int kXtNb = 8;                    // neighbours per cell at most
constexpr int kXtRow = 48;                  // solution-row length at most
constexpr int kXtStride = 2 + 2 * kXtNb;    // chat01, chati0[kXtNb], chat1j[kXtNb], qsat
struct Xt3dDev {
  int on = 0;
  int lamatsaved = 0;    // some cells have all their connections permanently confined
  int nozee = 0;         // no ANGLE2: horizontal connections have no z component
  int vcentre = 0;       // vertical connections run between the cell centres (DISU)
  int rhsform = 0;       // XT3D RHS: the neighbours' terms go to the right-hand side
  const int *sia = nullptr, *sja = nullptr, *idxglo = nullptr;
  const unsigned char *sflag = nullptr;  // per solution position: 1 connection, 2 extended
  const int *iallpc = nullptr;           // per cell (xt3d_iallpc)
  const double *ck = nullptr;            // per cell, 9 (row-major tensor)
  const double *geo = nullptr;           // per connection n < m: dx, dy, nx, ny from n to m,
                                         // then from m to n (8)
  const int *pair_n = nullptr, *pair_il0 = nullptr, *pair_il10 = nullptr;  // per connection
  double *coef = nullptr;                // per connection, kXtStride
  const double *pcval = nullptr;         // per solution position (lamatsaved)
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
  Xt3dDev xt{};
};

// XT3D coefficients of every connection n < m (xt3d_fc's loop body,
// Xt3dInterface.f90:416-465): mode 0 for the fill (the permanently confined
// cells skipped when lamatsaved), mode 1 for those cells alone with
// saturated areas (xt3d_fcpc, :499-571), mode 2 the flow of every connection
// into coef[0] (xt3d_flowja, :797-875)
void xt3d_pairs(int njas, const NpfDev &g, const Xt3dDev &x, const int *ibound, const double *sat,
                const double *h, int mode, cudaStream_t st);
// The permanently confined part of every solution position (amatpc, then
// amatpcx, added to a zero matrix as xt3d_fc does first)
void xt3d_pcrows(int nodes, const NpfDev &g, const Xt3dDev &x, const int *ibound, double *pcval,
                 cudaStream_t st);

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
// cells (or nullptr): the per-cell rates STO-SS [0, n), STO-SY [n, 2n), CHD
// [2n, 3n), then each boundary entry's rate in bnd_ptr order.
constexpr int kGwfBudgetSlots = 12;
void gwf_budget(int nodes, const NpfDev &g, const FillDev &f, const int *bnd_kind, double *cells,
                const int *ibound, const double *h, const double *hold, const double *sat,
                const double *condsat, double *flowja, double *part, int G, cudaStream_t st);

}  // namespace gb
