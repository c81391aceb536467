// gbims_internal.cuh -- shared declarations of the GB300 IMS library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/gbims.h"

namespace gb {

constexpr int kNumSM = 152;       // GB300: 2 dies x 76 SMs
constexpr int kRedBlock = 256;    // threads per reduction block
constexpr int kMaxRedBlocks = 8 * kNumSM;  // grid of reduction kernels: 8 x 256 threads per SM
constexpr int kSell = 32;         // SELL slice height (one warp)
constexpr int kMaxRowLen = 64;    // ILU0 factor: longest supported CSR row

// Exit reasons reported in gbims_summary.exit_reason.
enum ExitReason { kExitNone = 0, kExitClosure = 1, kExitStagnation = 2, kExitItmax = 3,
                  kExitExact = 4, kExitZeroRho = 5 };

// Device control block of one Krylov solve: inputs, scalars and the loop
// state.  Written by the single-thread control kernels, read by all others.
struct Ctl {
  // inputs
  int itmax, icnvgopt, north, iscl;
  double dvclose, rclose, l2norm0, epfact;
  // loop state
  int iter;        // current inner iteration (1-based, INNERIT)
  int done;        // 1 = stop: every kernel of the loop returns at once
  int icnvg;
  int exit_reason;
  int north_due;   // recompute the residual after this iteration
  int first;       // 1 in the first iteration (P = Z)
  double rho, rho0, alpha, alpha0, beta, omega, omega0;
  double deltax, rmax, l2norm;
  long long xloc, rloc;
  double scratch[4];
  int pivot_fail;  // factorization: first row whose pivot failed (or INT_MAX)
  int nonfinite;
  int bodies;         // loop bodies executed in this solve
  int guard_tripped;  // the body limit ended the loop
  int restart_due;    // mixed form: the pending true-residual check restarts the recurrence
  // Per-inner-iteration records (gbims_set_inner_records; rec == nullptr:
  // off).  Row r of rec (stride 3 + 4*rec_nmod): iteration, alpha, omega,
  // then per model dvmax, locdv, rmax, locr.  rec_part holds the per-model
  // block partials of k_rec_models (rec_nmod > 1); rec_loc the per-model
  // locations carried from one iteration to the next (2*rec_nmod).
  double *rec;
  const double *rec_part;
  long long *rec_loc;
  int rec_cap, rec_nmod, rec_G, rec_count;
};

// A batched ensemble on the device: members concatenated into one
// block-diagonal system; rows cut into chunks that never straddle members.
struct BatchDev {
  int nm = 0, nchunks = 0;
  const int *cm = nullptr;  // chunk -> member (nchunks)
  const int *cr = nullptr;  // chunk -> first row (nchunks + 1)
  const int *mc = nullptr;  // member -> first chunk (nm + 1)
  const int *mr = nullptr;  // member -> first row (nm + 1)
  Ctl *ctls = nullptr;      // one control block per member
};
constexpr int kChunkRows = 2048;  // rows per chunk (8 per thread of a 256-thread block)

// Reduction partial layout: value slots per block.
struct MaxLoc {
  double val;      // signed value
  long long idx;   // row (-1 = none)
};

__device__ __forceinline__ bool absgt(double a, double b) {
  // |a| > |b| on the integer image of |a|, |b|: for finite doubles the order
  // of the bit patterns of the magnitudes is the order of the magnitudes,
  // and it keeps the comparison off the FP64 pipe.  NaN magnitudes compare
  // greater than every finite value here; the reference's strict > never
  // selects a NaN, so NaN input is detected separately (Ctl::nonfinite).
  unsigned long long ua = __double_as_longlong(a) & 0x7fffffffffffffffULL;
  unsigned long long ub = __double_as_longlong(b) & 0x7fffffffffffffffULL;
  return ua > ub;
}

__device__ __forceinline__ void maxloc_merge(MaxLoc &a, const MaxLoc &b) {
  unsigned long long ua = __double_as_longlong(a.val) & 0x7fffffffffffffffULL;
  unsigned long long ub = __double_as_longlong(b.val) & 0x7fffffffffffffffULL;
  if (ub > ua || (ub == ua && ub != 0 && b.idx >= 0 && (a.idx < 0 || b.idx < a.idx))) a = b;
}

// ---------------------------------------------------------------------------
// Sparse formats
// ---------------------------------------------------------------------------

// SELL-32: slices of 32 consecutive rows, entries stored column-major inside
// the slice (entry k of row r at slice_ptr[s] + k*32 + r%32), padded to the
// longest row of the slice.  Entry k of a row is its k-th CSR entry, so the
// per-row summation order is the CSR (JA) order of amux.
struct Sell {
  int n = 0, nslices = 0;
  long long nstored = 0;
  int *d_ptr = nullptr;   // nslices+1 element offsets
  int *d_col = nullptr;   // nstored, padded entries point at the row itself
  int *d_src = nullptr;   // nstored, CSR position or -1 for padding
  double *d_val = nullptr;
  float *d_val32 = nullptr;
  // batched ensembles: the products skip the rows of members that are done
  int *d_slm = nullptr;         // per slice: its member, or -1 if it straddles two
  const int *d_mrow = nullptr;  // member -> first row (nm + 1)
  const Ctl *mctl = nullptr;    // member control blocks (null: single system)
  int nm = 0;
};

// Level schedule of a triangular sweep: rows grouped by level.
struct Levels {
  int nlev = 0;
  std::vector<int> ptr;   // nlev+1
  int *d_rows = nullptr;  // n
  int maxwidth = 0;
};

// The level-scheduled sweeps' form: mode 0 launches one kernel per level;
// mode 1 runs each sweep as one sync-free launch over result words tagged
// with the launch's epoch (fwd, bwd: n words each, 16 bytes in FP64, 8 in
// FP32, zeroed once; ticket: two counters, 128 bytes apart, zeroed once).
struct LevelWords {
  int mode = 1;
  int sf_mult = 8;  // sync-free sweeps: threads per row of the widest level (tuned)
  void *fwd = nullptr, *bwd = nullptr;
  unsigned long long *ticket = nullptr;
  int *err = nullptr;
};

// ILUT / MILUT factorisation (k_ilut.cu).  kIlutCap bounds the working row
// of one row (its L and its U candidates before dropping, each): ILUT with
// PRECONDITIONER_LEVELS 5 and DROP_TOLERANCE 1e-4 on a 7-point grid reaches
// about 125 L and 65 U candidates; PRECONDITIONER_LEVELS 10 about 230 and 165.
constexpr int kIlutCap = 256;
enum IlutError { kIlutOk = 0, kIlutErrWait = 1, kIlutErrCap = 2, kIlutErrZeroRow = 3 };

struct IlutStatus {
  unsigned long long next;  // next row to claim
  int pivot_fail;           // lowest row whose pivot changed sign or vanished (INT_MAX: none)
  int err;                  // IlutError
  int err_row;
  int pad;
};

// Per-row results in padded slots (sl = lfil L entries, su = lfil - 1 U
// entries per row) and the completion word of each row (equal to epoch once
// the row of the current attempt is stored).
struct IlutDev {
  int n = 0, lfil = 0, sl = 0, su = 0;
  int *lcol = nullptr, *ucol = nullptr, *nl = nullptr, *nu = nullptr;
  double *lval = nullptr, *uval = nullptr, *dinv = nullptr;
  unsigned *rdone = nullptr;
  IlutStatus *stat = nullptr;
  unsigned epoch = 0;
};

// One full DIS grid ("member") of the wavefront layout.  A single model is
// one member; a batched ensemble has one per model, laid end to end.
struct Dia7Geo {
  int nlay, nrow, ncol;
  int nb, G;          // blocks of W lines per layer, padded steps per block
  int ticket0;        // first CTA ticket (local ticket = b * nlay + k)
  long long slot0;    // first slot of the member's skewed tiles
  long long row0;     // first row of the member in the natural-order vectors
};

// Structured 7-point DIS layout of the ILU0 factors for the wavefront sweeps:
// per block of lines, G x W tiles (row = wavefront step, column = lane).
struct Dia7 {
  int nlay = 0, nrow = 0, ncol = 0;  // single model: its shape (index-free SpMV)
  int nb = 0, G = 0;       // single model: blocks per layer, padded steps per block
  long long slots = 0;     // total elements per skewed array (all members)
  int nm = 0;              // members
  std::vector<Dia7Geo> geo;
  Dia7Geo *d_geo = nullptr;
  const Ctl *mctl = nullptr;  // batched ensembles: members that are done are skipped
  int ntickets = 0;
  int cfg = 0;  // sweep configuration (chunk, ring, prefetch): an index of dia7_cfg
  int cfg_b = -1;  // the backward sweep's configuration (-1: cfg)
  int only = 0;    // timing: 1 forward sweep only, -1 backward sweep only, 0 both
  // FP64 handles: 1 while the tiles hold df64 pairs (the factor lies in the
  // float exponent range), 0 for native FP64 tiles; ext_allowed 0 keeps the
  // native sweeps (GBIMS_SWEEP_NATIVE)
  int ext = 0, ext_allowed = 1;
  // forward tiles: lower coefficients (unit diagonal) z (layer above),
  // y (row behind), x (column left); backward tiles: dinv*U for z, y, x and
  // dinv; zero where the neighbour or the cell does not exist
  double *d_lz = nullptr, *d_ly = nullptr, *d_lx = nullptr;
  double *d_ux = nullptr, *d_uy = nullptr, *d_uz = nullptr, *d_dinv = nullptr;
  float *f_lz = nullptr, *f_ly = nullptr, *f_lx = nullptr;
  float *f_ux = nullptr, *f_uy = nullptr, *f_uz = nullptr, *f_dinv = nullptr;
  // forward and backward results, skewed, as words that carry the epoch of
  // the sweep that wrote them (16 bytes per element in FP64, 8 in FP32)
  void *ll_y = nullptr, *ll_z = nullptr;
  // matrix values for the index-free SpMV: 7 slots of n (FP64; FP32 copy in
  // the mixed form), slot order = CSR order of a row
  double *d_sv = nullptr;
  float *f_sv = nullptr;
  int *d_flags = nullptr;  // the sweeps' ticket counters (forward, backward), one 128-byte line each
  int nflags = 0;
  int *d_err = nullptr;    // wait-limit error flag
  // a DIS grid reduced by IDOMAIN (gbims_set_dis_nodes): the sweeps run on
  // the full grid, inactive cells decoupled with zero factors; r is spread
  // onto it and z gathered back (nodeuser: reduced -> user cell, userred:
  // user cell -> reduced node or -1)
  bool mapped = false;
  long long nuser = 0;
  int *d_nodeuser = nullptr, *d_userred = nullptr;
  double *d_rfull = nullptr, *d_zfull = nullptr;
  float *f_rfull = nullptr, *f_zfull = nullptr;
};

// Elements of slack after every n-vector, so that a kernel may read or
// write whole 16-byte aligned segments past the last cell.
constexpr int kVecPad = 256;
void dia7_geometry(int nlay, int nrow, int ncol, bool fp32, int *nb, int *G, long long *slots);
// The wavefront sweep configurations: chunk C, ring depth NS, prefetch PF,
// occupancy cap OCC (0: as many CTAs per SM as fit, 2: at most two).
int dia7_num_cfgs();
void dia7_cfg(int i, int *C, int *NS, int *PF, int *OCC);
// Members (nlay, nrow, ncol) and their first rows -> D.geo, D.slots,
// D.ntickets (host side; the caller uploads D.geo to D.d_geo).
void dia7_layout(Dia7 &D, const std::vector<int> &shapes, const std::vector<long long> &row0,
                 bool fp32);

// ---------------------------------------------------------------------------
// kernel launchers (implemented in the .cu files)
// ---------------------------------------------------------------------------
void sell_build_host(int n, const std::vector<int> &ia, const std::vector<int> &ja,
                     std::vector<int> &ptr, std::vector<int> &col, std::vector<int> &src);
void launch_sell_fill(const Sell &S, const double *d_amat, cudaStream_t st);
void launch_spmv64(const Sell &S, const double *x, double *y, const Ctl *ctl, cudaStream_t st);
void launch_residual64(const Sell &S, const double *x, const double *b, double *d,
                       const Ctl *ctl, int only_if_north_due, cudaStream_t st);
// The mixed form's inner loop: FP32 matrix values, vectors and factors.
void launch_spmv32(const Sell &S, const float *x, float *y, const Ctl *ctl, cudaStream_t st);
void launch_dia7_spmv32(const Dia7 &D, const float *x, float *y, const Ctl *ctl,
                        cudaStream_t st);
void launch_dia7_apply32(const Dia7 &D, const float *r, float *z, const Ctl *ctl,
                         cudaStream_t st);

void levels_build_host(int n, const std::vector<int> &iapc, const std::vector<int> &japc,
                       bool forward, Levels &L);
// REORDERING_METHOD RCM (h_rcm.cu): lorder[i] is the i-th node (0-based) of
// the numbering genrcm gives for the 0-based CSR pattern ia/ja.
void rcm_order(int n, const std::vector<int> &ia, const std::vector<int> &ja,
               std::vector<int> &lorder);
// REORDERING_METHOD MD (h_md.cu): lorder[i] is the i-th node eliminated by
// the Yale minimum-degree ordering; returns odrv's flag (0 on success).
int md_order(int n, const std::vector<int> &ia, const std::vector<int> &ja,
             std::vector<int> &lorder);
void launch_ilu_factor(int n, const int *d_ia, const int *d_ja, const double *d_amat,
                       const int *d_iapc, const int *d_japc, double *d_apc,
                       const Levels &L, double relax, double delta, int ipcflag,
                       Ctl *ctl, cudaStream_t st);
void launch_ilut_factor(const IlutDev &I, const int *d_ia, const int *d_ja, const double *d_amat,
                        double droptol, double relax, double delta, int izero, cudaStream_t st);
void launch_ilut_scatter(const IlutDev &I, const int *d_iapc, const int *d_japc, double *d_apc,
                         cudaStream_t st);
void launch_ilu_apply_levels(int n, const int *d_iapc, const int *d_japc,
                             const double *d_apc, const Levels &F, const Levels &B,
                             const LevelWords &Wd, const double *r, double *d, const Ctl *ctl,
                             cudaStream_t st);
void launch_ilu_apply_levels32(int n, const int *d_iapc, const int *d_japc,
                               const float *d_apc32, const Levels &F, const Levels &B,
                               const LevelWords &Wd, const float *r, float *d, const Ctl *ctl,
                               cudaStream_t st);

bool dia7_matches(int nlay, int nrow, int ncol, int n, const std::vector<int> &ia,
                  const std::vector<int> &ja);
// The DIS shape of a 0-based CSR pattern that is a full 7-point grid in
// natural order (false if it is not one).
bool dia7_matches_reduced(int nlay, int nrow, int ncol, int n, const std::vector<int> &ia,
                          const std::vector<int> &ja, const int *nodeuser);
void launch_dia7_spread(const Dia7 &D, int n, const double *r, double *rfull, cudaStream_t st);
void launch_dia7_spread32(const Dia7 &D, int n, const float *r, float *rfull, cudaStream_t st);
void launch_dia7_collect(const Dia7 &D, int n, const double *zfull, double *z, cudaStream_t st);
void launch_dia7_collect32(const Dia7 &D, int n, const float *zfull, float *z, cudaStream_t st);
bool dia7_detect(int n, const std::vector<int> &ia, const std::vector<int> &ja, int *nlay,
                 int *nrow, int *ncol);
// Factor -> skewed tiles; FP64 handles choose df64 or native tiles here (D.ext).
// Returns 0, or -1 on a CUDA error.
int launch_dia7_extract(Dia7 &D, int n, const int *d_iapc, const int *d_japc,
                        const double *d_apc, bool mixed, cudaStream_t st);
void launch_dia7_apply64(const Dia7 &D, const double *r, double *z, const Ctl *ctl,
                         cudaStream_t st);
void launch_dia7_vfill(const Dia7 &D, const int *d_ia, const double *d_amat, cudaStream_t st);
void launch_dia7_spmv64(const Dia7 &D, const double *x, double *y, const Ctl *ctl,
                        cudaStream_t st);
void launch_dia7_residual64(const Dia7 &D, const double *x, const double *b, double *d,
                            const Ctl *ctl, int only_if_north_due, cudaStream_t st);

// ims_base_scale (k_scale.cu): the column-major position map used by the
// L2-norm column sums, the scaling before a solve (returns its kernel count)
// and the unscaling of x after it.
void scale_colmap_host(int n, const std::vector<int> &ia, const std::vector<int> &ja,
                       std::vector<int> &cptr, std::vector<int> &cpos);
int launch_scale(int iscl, int n, const int *ia, const int *ja, const int *cptr, const int *cpos,
                 double *amat, double *x, double *b, double *dscale, double *dscale2,
                 cudaStream_t st);
void launch_unscale_x(int n, double *x, const double *dscale2, cudaStream_t st);

// Device state of a time-step handle that the warm start reads: the heads of
// the last step (x), those of the step before (xold), IBOUND and the stream.
struct SlnView {
  int n = 0;
  const double *x = nullptr, *xold = nullptr;
  const int *ibound = nullptr;
  cudaStream_t st = nullptr;
};
int sln_view(gbsln_handle *h, SlnView *v);

// IMS handle internals shared with the device-resident solution.
void ims_buffers(gbims_handle *h, double **amat, double **rhs, double **x);
cudaStream_t ims_stream(gbims_handle *h);
int ims_apply_inplace(gbims_handle *h, int kstp, int kiter, int *icnvg, int *in_iter,
                      gbims_summary *summary);
const char *ims_error(gbims_handle *h);

}  // namespace gb
