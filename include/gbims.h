/*
 * gbims.h -- C ABI of the GB300-native Iterative Model Solution (IMS) hot path
 * for MODFLOW 6.
 *
 * The library replaces, behind the same calling contract, the IMS linear
 * accelerator of MODFLOW 6 (src/Solution/LinearMethods/ImsLinear.f90) and the
 * NPF conductance fill (src/Model/GroundWaterFlow/gwf-npf.f90).  All entry
 * points take plain pointers and sizes, never abort, and return an int status:
 *   0  success
 *  >0  warning (e.g. GBIMS_WARN_PIVOT: the ILU0 pivot guard added a diagonal
 *      increment, ImsLinearBase.f90:812-863)
 *  <0  error (see gbims_status_string)
 *
 * Index arrays (ia, ja, node lists) are 0-based unless index_base is 1 in the
 * settings (Fortran callers pass 1).  The diagonal entry must be the first
 * entry of each CSR row, as in MODFLOW 6 (src/Utilities/Matrix/SparseMatrix.f90:16).
 */
#ifndef GBIMS_H
#define GBIMS_H

#ifdef __cplusplus
extern "C" {
#endif

#define GBIMS_OK 0
#define GBIMS_WARN_PIVOT 1
#define GBIMS_WARN_FALLBACK 2 /* gbsln_timestep_warm dropped its guess */
#define GBIMS_ERR_ARG (-1)
#define GBIMS_ERR_CUDA (-2)
#define GBIMS_ERR_UNSUPPORTED (-3)
#define GBIMS_ERR_NONFINITE (-4)
#define GBIMS_ERR_NOMEM (-5)
#define GBIMS_ERR_STATE (-6)

/* precision modes */
#define GBIMS_FP64 0  /* FP64 everywhere: the plain drop-in */
#define GBIMS_MIXED 1 /* FP32 matrix and ILU0 factors (FP32 triangular
                         sweeps); FP64 Krylov vectors and scalars, FP64 true
                         residual, head update and closure, with iterative
                         refinement between the two */

/* IMS LINEAR block options, with the meaning of
 * src/Solution/LinearMethods/ImsLinearSettings.f90:10-253 and
 * ImsLinear.f90:178-185 (IPC derived from relax/level/droptol). */
typedef struct gbims_settings {
  double dvclose;   /* INNER_DVCLOSE */
  double rclose;    /* INNER_RCLOSE */
  int icnvgopt;     /* RCLOSE option 0..4 (ImsLinearBase.f90:1101-1146) */
  int iter1;        /* INNER_MAXIMUM */
  int ilinmeth;     /* LINEAR_ACCELERATION: 1 CG, 2 BICGSTAB */
  int iscl;         /* SCALING_METHOD: 0 none, 1 diagonal, 2 L2 norm */
  int iord;         /* REORDERING_METHOD: 0 none, 1 RCM, 2 MD (with
                       ILUT/MILUT; with ILU0/MILU0: GBIMS_ERR_UNSUPPORTED) */
  int north;        /* NUMBER_ORTHOGONALIZATIONS */
  double relax;     /* RELAXATION_FACTOR (> 0 selects MILU0 / MILUT) */
  int level;        /* PRECONDITIONER_LEVELS (> 0: ILUT with lfil = level) */
  double droptol;   /* PRECONDITIONER_DROP_TOLERANCE (> 0: ILUT).  ILUT works
                       on the general pattern (no wavefront sweeps) and on up
                       to 256 candidates per row and triangle before dropping
                       (GBIMS_ERR_UNSUPPORTED beyond) */
  int precision;    /* GBIMS_FP64 or GBIMS_MIXED */
  int index_base;   /* 0 (C) or 1 (Fortran) for ia/ja */
  int nlay, nrow, ncol; /* DIS shape for the structured (7-point) wavefront
                           sweeps and the index-free product, used when the
                           CSR pattern is that of a full DIS grid in natural
                           order.  All three 0: the shape is found from the
                           pattern (row 0's neighbour offsets 1, ncol,
                           nrow*ncol, then every row checked), so a caller
                           that passes only IA/JA, as imslinear_ar does,
                           reaches the structured path.  nlay < 0: never (the
                           level-scheduled sweeps on the general pattern). */
} gbims_settings;

/* Convergence summary of the last apply (ConvergenceSummary.f90 fields for a
 * solution with one model). */
typedef struct gbims_summary {
  int iter_cnt;        /* inner iterations of the last apply */
  int icnvg;           /* 1 converged, 0 not */
  int pivot_retries;   /* ims_base_pcu retries (0 = none) */
  int exit_reason;     /* 0 none, 1 closure, 2 stagnation, 3 itmax, 4 exact, 5 zero rho */
  double dvmax;        /* signed max head change of the last inner iteration */
  int locdv;           /* its 0-based row */
  double rmax;         /* signed max residual of the last inner iteration */
  int locr;            /* its 0-based row */
  double l2norm0;      /* initial residual L2 norm */
  double l2norm;       /* last residual L2 norm */
  double solve_ms;     /* device time of the apply (CUDA events) */
  int refinements;     /* mixed precision: FP64 refinement steps */
  int structured;      /* 1 if the structured 7-point sweeps were used */
} gbims_summary;

typedef struct gbims_handle gbims_handle;

/* Replaces ImsLinearDataType%imslinear_allocate (ImsLinear.f90:111-339):
 * validates options, derives IPC, builds IAPC/JAPC (ims_base_pccrs,
 * ImsLinearBase.f90:1207-1261), the ILU0 level schedule and the device
 * layouts.  neq/nja are the solution's NEQ and NJA. */
int gbims_create(const gbims_settings *settings, int neq, int nja, const int *ia,
                 const int *ja, gbims_handle **out);

/* Replaces ImsLinearDataType%imslinear_apply (ImsLinear.f90:617-750) with host
 * arrays: amat (nja), rhs (neq) and x (neq) are read, x is overwritten with
 * the solution (x on entry is the initial guess).  amat and rhs are left as
 * passed (the reference restores them after scaling).  icnvg and in_iter have
 * the meaning of ICNVG and IN_ITER.  summary may be NULL. */
int gbims_apply(gbims_handle *h, double *amat, double *rhs, double *x, int kstp,
                int kiter, int *icnvg, int *in_iter, gbims_summary *summary);

/* Same as gbims_apply with device pointers (the device-resident assembly
 * path); amat, rhs and x live in HBM and stay there. */
int gbims_apply_device(gbims_handle *h, double *d_amat, double *d_rhs, double *d_x,
                       int kstp, int kiter, int *icnvg, int *in_iter,
                       gbims_summary *summary);

/* Replaces ImsLinearDataType%imslinear_da. */
int gbims_destroy(gbims_handle *h);

/* Per-inner-iteration convergence records, the NCONV, CONVNMOD, CONVMODSTART
 * and CACCEL arguments of imslinear_ap (ImsLinear.f90:617-633) and the rows
 * ims_base_cg / ims_base_bcgs write into the solution's ConvergenceSummary
 * (ImsLinearBase.f90:141-197, 431-493), which feed CSV_INNER_OUTPUT
 * (NumericalSolution.f90:2060-2200).
 *
 * gbims_set_inner_records: from the next apply on, keep up to nconv records
 * per apply (nconv = 0 switches them off).  convmodstart (convnmod + 1
 * entries, in the handle's index_base) gives the first row of each model and
 * ends at neq + index_base, as CONVMODSTART does.  FP64 PCG and BiCGSTAB on a
 * single system (GBIMS_ERR_UNSUPPORTED for the mixed form and batches).
 *
 * gbims_get_inner_records: the records of the last apply, at most cap of
 * them (*nrec gets the count): itinner (ITINNER, the inner iteration),
 * alpha and omega (CACCEL: PCG alpha, omega 0; BiCGSTAB alpha and omega),
 * and per model (arrays [nrec][convnmod], model fastest, the layout of the
 * reference's convdvmax(im, n)): the signed largest head change dvmax with
 * its row locdv and the signed largest residual rmax with its row locr, rows
 * in the handle's index_base (index_base - 1 when no row of the model
 * changed).  Rows are those of the system the solver iterates on (the
 * permuted one under REORDERING_METHOD), as in the reference. */
int gbims_set_inner_records(gbims_handle *h, int nconv, int convnmod, const int *convmodstart);
int gbims_get_inner_records(gbims_handle *h, int cap, int *nrec, int *itinner, double *alpha,
                            double *omega, int *locdv, double *dvmax, int *locr, double *rmax);

/* Batched ensembles (no counterpart in the reference, which solves one
 * simulation at a time): nmembers independent systems concatenated into one
 * block-diagonal system.  member_rows (nmembers+1, index_base) gives each
 * member's first row; ia/ja are the concatenated CSR with global column
 * numbers, which must stay inside the member's own rows.  One apply solves
 * every member to its own closure with its own PCG iteration
 * (ImsLinearBase.f90:30-240): per-member Krylov scalars, convergence test and
 * exit, all members advanced by the same kernel launches.  icnvg, in_iter and
 * summaries (may be NULL) have nmembers entries; locdv/locr are member-local
 * rows.  shapes (3 * nmembers: nlay, nrow, ncol per member) may be NULL;
 * when given, every member must be a full DIS grid of that shape and the
 * preconditioner runs as one wavefront launch over all members (otherwise the
 * level schedule of the whole batch).  FP64 PCG only (GBIMS_ERR_UNSUPPORTED
 * otherwise); the handle is released with gbims_destroy. */
int gbims_batch_create(const gbims_settings *settings, int nmembers, const int *member_rows,
                       int neq, int nja, const int *ia, const int *ja, const int *shapes,
                       gbims_handle **out);
int gbims_batch_apply(gbims_handle *h, double *amat, double *rhs, double *x, int kstp,
                      int kiter, int *icnvg, int *in_iter, gbims_summary *summaries);
int gbims_batch_apply_device(gbims_handle *h, double *d_amat, double *d_rhs, double *d_x,
                             int kstp, int kiter, int *icnvg, int *in_iter,
                             gbims_summary *summaries);

/* Building blocks of apply, exposed for callers that drive their own loop
 * and for kernel-level checks (host arrays):
 *  gbims_factor       preconditioner update, ims_base_pcu + ims_base_pcilu0
 *                     (ImsLinearBase.f90:761-864, 928-1042) or, for IPC 3/4,
 *                     ilut (sparskit2/ilut.f90:48-462), from amat (nja);
 *  gbims_get_apc      copies APC (nja, the reference's layout: APC(1:NEQ) the
 *                     inverse pivots, then the L\U entries in JAPC order);
 *                     ILU0/MILU0 only;
 *  gbims_get_factor   copies the preconditioner as IAPC (neq+1), JAPC and APC
 *                     (njapc each; 0-based).  Row i's L entries are at
 *                     [IAPC(i), JAPC(i)), its U entries at [JAPC(i), IAPC(i+1)),
 *                     APC(0:neq) the inverse pivots.  For ILUT this is
 *                     sparskit's MSR storage (ALU/JLU/JU of ImsLinear.f90)
 *                     with JLU's row pointers in IAPC and JU in JAPC(0:neq).
 *                     Null arrays: *njapc only;
 *  gbims_matvec       y = A*x, amux (sparsekit.f90:1-59), with the matrix of
 *                     the last gbims_factor or apply;
 *  gbims_precondition z = M^-1 r, ims_base_ilu0a (ImsLinearBase.f90:1049-1092),
 *                     with the last factor (FP32 factors in GBIMS_MIXED). */
/* Per-kernel device times (ms per launch, CUDA events on the library's
 * stream, averaged over reps launches after one warm-up) of the last factor:
 * the SpMV, the preconditioner (forward+backward sweeps), a dot product and
 * the x/residual update, in the handle's precision. */
typedef struct gbims_kernel_times {
  double spmv_ms, precond_ms, dot_ms, update_ms;
  double spmv_bytes, precond_bytes; /* algorithmic bytes per launch */
} gbims_kernel_times;
int gbims_time_kernels(gbims_handle *h, int reps, gbims_kernel_times *t);

/* Autotuner (no counterpart in the reference, which has no tunable kernels):
 * on the handle's own factored system it times every wavefront tiling of
 * the structured sweeps (chunk of steps per ring buffer, ring depth,
 * neighbour-word prefetch depth, CTAs per SM), the form of the level-
 * scheduled sweeps of other patterns, and the thread-block count of the
 * dot/update reductions, and keeps the fastest for the following applies.
 * The tiling does not change any cell's arithmetic; the reduction grid only
 * changes the order in which the partial sums are added.  Batched handles
 * tune the tiling only.  reps: timed applications per candidate. */
typedef struct gbims_tuning {
  int sweep_config;                 /* chosen tiling, -1 when the handle has no wavefront sweeps */
  int sweep_chunk, sweep_ring, sweep_prefetch;
  int sweep_occupancy;              /* 0: as many sweep CTAs per SM as fit; 2: at most two */
  int reduction_blocks;             /* chosen reduction grid (0: batched handle) */
  int level_mode;                   /* level-scheduled sweeps (handles without wavefront
                                       sweeps): 0 one launch per level, 1 one sync-free
                                       launch per sweep; -1 not applicable */
  double level_ms[2];               /* one ILU0 application in each level mode */
  int ncandidates;                  /* tilings timed (level-scheduled handles: the
                                       sync-free form at 1, 2, 4, 8, 16 threads per
                                       row of the widest level) */
  double candidate_ms[16];          /* one ILU0 application per candidate */
  double precond_ms;                /* of the chosen tilings */
  double vector_ms;                 /* dot + update at the chosen grid */
  int sweep_config_backward;        /* the backward sweep's tiling (sweep_config: the
                                       forward sweep's); candidate_ms sums both sweeps */
} gbims_tuning;
int gbims_autotune(gbims_handle *h, int reps, gbims_tuning *out);
/* A DIS grid reduced by IDOMAIN (no counterpart call in the reference; it
 * holds the same map as DisType%nodeuser, Dis.f90): nodeuser[n] is the user
 * cell (k*nrow*ncol + i*ncol + j, plus index_base) of node n, strictly
 * increasing, and the pattern must be the full grid's (settings nlay, nrow,
 * ncol) with the inactive cells removed.  The ILU0 factor is still that of
 * the reduced matrix; its triangular sweeps then run as wavefront sweeps on
 * the full grid, the inactive cells decoupled with zero factors, r spread
 * onto it and z gathered back.  Call after gbims_create and before the
 * first factorisation; single models, ILU0/MILU0, no reordering. */
int gbims_set_dis_nodes(gbims_handle *h, const int *nodeuser);
/* Applies a tuning found earlier (sweep_config < 0, reduction_blocks <= 0 or
 * level_mode < 0 leave that part unchanged); sweep_config sets the tiling of
 * both sweeps. */
int gbims_set_tuning(gbims_handle *h, int sweep_config, int reduction_blocks, int level_mode);

int gbims_factor(gbims_handle *h, const double *amat, int *pivot_retries);
int gbims_get_apc(gbims_handle *h, double *apc);
int gbims_get_factor(gbims_handle *h, int *iapc, int *japc, double *apc, int capacity,
                     int *njapc);

/* ims_base_calc_order (ImsLinearBase.f90:556-610) on a CSR pattern: IORD 1
 * RCM (genrcm of rcm/rcm.f90), IORD 2 minimum degree (ims_odrv of
 * ImsReordering.f90).  LORDER(i) is the i-th node of the numbering and
 * IORDER its inverse, in index_base.  Host only (no device work).  A handle
 * created with iord 1 or 2 applies LORDER as imslinear_ap does (dperm/dvperm,
 * ImsLinear.f90:652-666 and 730-737); its gbims_matvec, gbims_precondition
 * and gbims_get_factor then work in that permuted numbering. */
int gbims_calc_order(int iord, int neq, int nja, const int *ia, const int *ja, int index_base,
                     int *lorder, int *iorder);
int gbims_matvec(gbims_handle *h, const double *x, double *y);
int gbims_precondition(gbims_handle *h, const double *r, double *z);

/* Kernels this handle has launched so far (loop bodies of the inner-loop
 * graph counted once per executed body). */
long long gbims_kernel_launches(const gbims_handle *h);

/* Message of the last error on this handle (never NULL). */
const char *gbims_last_error(const gbims_handle *h);
const char *gbims_status_string(int status);

/* No counterpart in the reference: an entry point that allocates nothing,
 * for callers that cannot call cudaMalloc themselves or through this library:
 * a host whose device memory is owned by its own memory manager (an
 * application that reserves the GPU's memory up front and hands out pieces of
 * it, so that any further cudaMalloc would fail or fragment its pool).
 *
 * d = b - A x (the initial residual of an IMS solve, ims_base_residual,
 * ImsLinearBase.f90:1291-1312), its L2 norm (L2NORM0) and its signed max|d|
 * with the 0-based row, from CSR arrays in device memory (ia, ja with
 * index_base 0 or 1; diagonal first in each row).  d_resid may be NULL.  The
 * L2 norm equals, bit for bit, the l2norm0 that gbims_apply reports for the
 * same system and initial x; the residual equals b - gbims_matvec(x).
 *
 * Limit: neq <= 155,648 rows (608 reduction blocks of 256 rows, held in a
 * static device array); larger systems get GBIMS_ERR_ARG.  Runs on `stream`
 * (a cudaStream_t, NULL = the legacy default stream); it copies its three
 * results to the host and synchronizes `stream` before it returns, so it
 * must not be called while `stream` is capturing.  The first call on a
 * device looks up the static array and loads the library's device code:
 * make it before any stream capture.  The static array is shared
 * by all callers on a device: calls that overlap in time (two host threads,
 * or work on two streams in flight) race on it. */
int gbims_residual_noalloc(int neq, int nja, const int *d_ia, const int *d_ja,
                           const double *d_amat, const double *d_x, const double *d_rhs,
                           double *d_resid, int index_base, void *stream, double *l2norm,
                           double *rmax, int *locr);

/* ---- GWF NPF conductance fill (gwf-npf.f90:474-698) ---------------------- */

/* NPF options with the meaning of the NPF OPTIONS block. */
typedef struct gbnpf_options {
  int inewton;      /* NEWTON formulation */
  int ivarcv;       /* VARIABLECV */
  int idewatcv;     /* DEWATERED */
  int icellavg;     /* ALTERNATIVE_CELL_AVERAGING: 0 harmonic, 1 log, 2 AMT-LMK, 3 AMT-HMK */
  double satomega;  /* Newton saturation smoothing (default 1e-6) */
  int index_base;   /* 0 or 1 for the index arrays */
  int inewtonur;    /* NEWTON UNDER_RELAXATION (gwf.f90:181, gwf_nur :717): heads
                       that fall below the bottom of their column are pulled back
                       (npf_nur) by gbsln_timestep; needs inewton */
} gbnpf_options;

typedef struct gbnpf_handle gbnpf_handle;

/* Uploads the grid connectivity (Connections.f90:26-35: ia, ja, jas, isym,
 * ihc, cl1, cl2, hwva), cell geometry and K, and computes the saturated
 * conductance (calc_condsat, gwf-npf.f90:1950-2044) on the device. */
int gbnpf_create(const gbnpf_options *opt, int nodes, int nja, int njas, const int *ia,
                 const int *ja, const int *jas, const int *isym, const int *ihc,
                 const double *cl1, const double *cl2, const double *hwva,
                 const double *top, const double *bot, const double *k11,
                 const double *k33, const int *icelltype, gbnpf_handle **out);

/* npf_cf + npf_fc (+ npf_fn when inewton) on device arrays: adds the
 * conductance terms to d_amat (nja) and d_rhs (nodes) in the reference's
 * per-row summation order.  d_ibound (nodes, int) and d_hnew are device
 * pointers. */
int gbnpf_fill(gbnpf_handle *h, const int *d_ibound, const double *d_hnew,
               double *d_amat, double *d_rhs);

/* Copies the saturated conductance (njas) to the host. */
int gbnpf_get_condsat(gbnpf_handle *h, double *condsat);

int gbnpf_destroy(gbnpf_handle *h);

/* ---- Device-resident single-model solution ------------------------------ */

/* A GWF DIS model whose whole outer Picard/Newton loop (NumericalSolution
 * solve, NumericalSolution.f90:1482-1837) runs with x, amat and rhs in HBM:
 * NPF/STO/CHD/WEL/RCH fill, sln_ls fixups, IMS apply, dxmax, under-relaxation. */
typedef struct gbsln_model {
  int nlay, nrow, ncol;
  const double *delr, *delc;  /* ncol, nrow */
  const double *top;          /* nrow*ncol (model top) */
  const double *botm;         /* nlay*nrow*ncol */
  const double *k11, *k33;    /* nodes */
  const int *icelltype;       /* nodes */
  const double *ss, *sy;      /* nodes, or NULL for steady state only */
  int nchd;
  const int *chd_node;        /* 0-based node numbers */
  const double *chd_head;
  int nwel;
  const int *wel_node;
  const double *wel_q;
  int nrch;
  const int *rch_node;
  const double *rch_rate;
} gbsln_model;

/* NONLINEAR block (NumericalSolution.f90:567-866, sln_setouter :2623-2671). */
typedef struct gbsln_nonlinear {
  double dvclose;  /* OUTER_DVCLOSE */
  int mxiter;      /* OUTER_MAXIMUM */
  int nonmeth;     /* UNDER_RELAXATION: 0 none, 1 simple, 2 cooley, 3 dbd */
  double theta, akappa, gamma, amomentum;
  int iallowptc;   /* 1 = pseudo-transient continuation allowed (default) */
  /* backtracking (sln_backtracking, NumericalSolution.f90:2680-2838):
   * BACKTRACKING_NUMBER (0 = off), _TOLERANCE, _REDUCTION_FACTOR,
   * _RESIDUAL_LIMIT */
  int numtrack;
  double btol, breduc, res_lim;
} gbsln_nonlinear;

typedef struct gbsln_handle gbsln_handle;

typedef struct gbsln_stats {
  int outer;          /* outer iterations of the last time step */
  int inner_total;    /* inner iterations summed over them */
  int converged;
  int pivot_retries;
  double dxmax;       /* last outer max head change */
  double fill_ms, solve_ms, total_ms; /* device time of the step */
  int backtracks;     /* backtracking reductions taken in the step */
  /* the step's first iterate on its active cells was
   * xold + prev_alpha*(last step's change) + guess_alpha*(guess - xold):
   * guess_alpha 1 for gbsln_timestep_guess, both projection factors for
   * gbsln_timestep_warm, both 0 for a step from the previous heads */
  double guess_alpha;
  double prev_alpha;
} gbsln_stats;

int gbsln_create(const gbsln_model *model, const gbnpf_options *npf,
                 const gbims_settings *ims, const gbsln_nonlinear *nl,
                 const double *strt, gbsln_handle **out);

/* The hydraulic conductivity tensor of NPF (K22, ANGLE1..3) and its
 * formulation.  k22: K22 per cell, or NULL (K22 = K11); angle1..3: ANGLE1..3
 * per cell in degrees, or NULL (ANGLE2 needs ANGLE1; ANGLE2 and ANGLE3 both
 * or neither).  xt3d 0: the standard two-point conductances with the
 * effective K of each connection's direction (hy_eff, gwf-npf.f90:2280-2357;
 * hyeff, HGeoUtil.f90:29-108; iavgkeff 0 harmonic, 1 arithmetic
 * weighting); 1: XT3D, the full tensor on the neighbours-of-neighbours
 * stencil (Xt3dInterface.f90, Xt3dAlgorithm.f90; without ANGLE2 the
 * horizontal connections have no z component, as in the reference), whose
 * matrix has the wider pattern (each row: the cell, its neighbours and
 * theirs) and is solved on the level-scheduled path; 2: XT3D RHS, the
 * neighbours' terms on the right-hand side at the current heads and the
 * model's own pattern (:478-490). */
typedef struct gbsln_ktensor {
  const double *k22;
  const double *angle1, *angle2, *angle3;
  int xt3d;
  int iavgkeff;
} gbsln_ktensor;

/* gbsln_create with the conductivity tensor on a DIS model.  With XT3D,
 * ALTERNATIVE_CELL_AVERAGING (icellavg > 0) is refused as the reference
 * refuses it (GBIMS_ERR_ARG), and gbsln_budget takes the flows from
 * xt3d_flowja (Xt3dInterface.f90:797-875). */
int gbsln_create_tensor(const gbsln_model *model, const gbsln_ktensor *kt,
                        const gbnpf_options *npf, const gbims_settings *ims,
                        const gbsln_nonlinear *nl, const double *strt, gbsln_handle **out);

/* A grid given by its connectivity: a DISV or DISU grid (or DIS written out
 * this way), in the form Connections.f90 keeps it (con_finalize, :160-316),
 * all 0-based.  ia/ja is the symmetric CSR pattern with each row's diagonal
 * first and the off-diagonals ascending; ihc, cl1, cl2 and hwva hold one
 * value per connection n < m, numbered in row order of the upper triangle
 * (the reference's JAS numbering): ihc 0 vertical, 1 horizontal, 2
 * horizontal between vertically staggered cells; cl1 the distance from n,
 * cl2 from m, to the shared face; hwva the face area (ihc 0) or width. */
typedef struct gbsln_grid {
  int nodes, nja;
  const int *ia, *ja;               /* nodes+1, nja */
  const int *ihc;                   /* (nja - nodes)/2 */
  const double *cl1, *cl2, *hwva;   /* (nja - nodes)/2 */
  const double *top, *bot, *area;   /* nodes */
} gbsln_grid;

/* gbsln_create on a grid given by its connectivity.  The model's K,
 * ICELLTYPE, storage and boundaries are read from `model` (its nlay, nrow,
 * ncol, delr, delc, top and botm are not read).  The solve takes the
 * general-pattern path (SELL-32 product, level-scheduled ILU0) unless the
 * pattern is that of a full DIS grid, which is found from IA/JA.  The checks
 * of con_finalize are made (diagonal first, ascending rows, every
 * connection with its counterpart, ihc in 0..2): GBIMS_ERR_ARG with the
 * reason in gbsln_last_error. */
int gbsln_create_grid(const gbsln_grid *grid, const gbsln_model *model,
                      const gbnpf_options *npf, const gbims_settings *ims,
                      const gbsln_nonlinear *nl, const double *strt, gbsln_handle **out);

/* The connection geometry the tensor needs on a grid given by its connectivity
 * (connection_normal and connection_vector of Disv.f90:979-1080 and
 * Disu.f90:1062-1164): xc, yc the cell centres (nodes; CELL2D); anglex per
 * connection n < m in JAS order, the angle in radians between the x axis
 * and the normal of the shared face, pointing from n to m (DISV: from the
 * shared edge, DisvGeom.f90:394-412; DISU: ANGLDEGX); centre_vertical 1
 * when vertical connections also run between the cell centres (DISU), 0 when
 * they are vertical lines (DISV). */
typedef struct gbsln_geometry {
  const double *xc, *yc;
  const double *anglex;
  int centre_vertical;
} gbsln_geometry;

/* gbsln_create_grid with the conductivity tensor (gbsln_ktensor) on a DISV
 * or DISU grid. */
int gbsln_create_grid_tensor(const gbsln_grid *grid, const gbsln_model *model,
                             const gbsln_ktensor *kt, const gbsln_geometry *geometry,
                             const gbnpf_options *npf, const gbims_settings *ims,
                             const gbsln_nonlinear *nl, const double *strt,
                             gbsln_handle **out);
/* One time step (prepareSolve + outer loop).  The step is transient when the
 * model has ss/sy and delt > 0, steady state otherwise; delt is also the
 * step length used by the pseudo-transient continuation default
 * (gwf.f90:625-687). */
int gbsln_timestep(gbsln_handle *h, int kper, int kstp, double delt, gbsln_stats *st);
/* The same time step started from a guess (d_guess: device array, nodes):
 * the first outer iterate of every active cell is the guess instead of the
 * previous heads, which stay the storage reference (xold).  The closure is
 * unchanged, so a guess only changes how many iterations it takes. */
int gbsln_timestep_guess(gbsln_handle *h, int kper, int kstp, double delt, const double *d_guess,
                         gbsln_stats *st);
/* The warm start with its fallback (no counterpart in the reference, whose
 * steps always start from the previous heads).  The first iterate of the
 * active cells is xold + a1*d1 + a2*d2 with d1 the head change of the last
 * step (when the last step closed; none after create, restart or
 * set_heads), d2 = d_guess - xold (none when d_guess is NULL), and
 * (a1, a2) = (D'AD)^-1 D'r for A, r the step's first system and its
 * residual at the previous heads: for the symmetric GWF matrix the point of
 * that plane closest to the solution in the energy norm, never farther from
 * it than the previous heads (a single direction when the two are nearly
 * parallel; the previous heads when a factor is not finite or beyond +-4).
 * A step with neither direction starts from the previous heads.  When the
 * step has spent inner_cap inner iterations without closing, the projected
 * start is dropped and the step is solved again from the previous heads;
 * then the status is GBIMS_WARN_FALLBACK and
 * *st counts the iterations and device time of both attempts.  Give
 * inner_cap the inner iterations the plain solver took on the previous step:
 * a guess then never costs more than one step's worth of iterations. */
int gbsln_timestep_warm(gbsln_handle *h, int kper, int kstp, double delt, const double *d_guess,
                        int inner_cap, gbsln_stats *st);
/* sln_buildsystem at the current heads (hold: previous-step heads, needed for
 * a transient step): the assembled amat (nja, CSR order of the DIS grid) and
 * rhs before the sln_ls fix-ups, copied to the host.  The reference writes
 * the same system with its itestmat switch (NumericalSolution.f90:2581-2599). */
int gbsln_formulate(gbsln_handle *h, double delt, const double *hold, double *amat, double *rhs);
const char *gbsln_last_error(const gbsln_handle *h);

/* Model budget of the last time step (or formulate): gwf_cq then gwf_bd
 * (gwf.f90:741-830).  Rates in L^3/T, entries in the order STO-SS, STO-SY,
 * CHD, WEL, RCH (sto_bd, then the packages, gwf-sto.f90:572-595,
 * gwf-chd.f90:324-346, BoundaryPackage bnd_bd); the percent difference is
 * that of Budget.f90:258-266. */
typedef struct gbsln_budget_table {
  double rate_in[5];
  double rate_out[5];
  double total_in, total_out;
  double percent_discrepancy;  /* 100 (in - out) / ((in + out) / 2), 0 when in + out = 0 */
  double max_cell_imbalance;   /* max over active cells of |FLOW-JA-FACE diagonal|, the
                                  net of a cell's storage, boundary and face flows */
  int max_cell;                /* 0-based node of that cell, -1 if none */
} gbsln_budget_table;
/* Cell-by-cell flows (npf_cq, gwf-npf.f90:745-770; sto_cq :447-564 of
 * gwf-sto.f90; bnd_cq; csr_diagsum, Sparse.f90:262-281; calc_chd_rate,
 * gwf-chd.f90:264-320) and the model budget at the current heads, with the
 * saturation of the last formulate, as the reference computes them after
 * a converged time step.  flowja: host array of nja values (FLOW-JA-FACE,
 * CSR order; the diagonal holds the cell's net flow) or NULL. */
int gbsln_budget(gbsln_handle *h, double *flowja, gbsln_budget_table *out);
/* The per-cell and per-entry rates behind the budget, as the packages save
 * them to the budget file (sto_cq strgss/strgsy per cell; the CHD, WEL and
 * RCH rates per list entry in list order; bnd_cq, gwf-chd.f90:264-346).  Any
 * pointer may be NULL. */
int gbsln_budget_cells(gbsln_handle *h, double *sto_ss, double *sto_sy, double *chd_rate,
                       double *wel_rate, double *rch_rate);
/* Restores the initial heads (IC STRT) on the device: the state at the start
 * of the simulation, for repeated runs of the same model. */
int gbsln_restart(gbsln_handle *h);
int gbsln_get_heads(gbsln_handle *h, double *x);
int gbsln_set_heads(gbsln_handle *h, const double *x);
gbims_handle *gbsln_ims(gbsln_handle *h);
int gbsln_destroy(gbsln_handle *h);

/* ---- Learned warm start (no counterpart in the reference) ----------------
 * A message-passing network over the graph of the IMS matrix (hidden width
 * 64, 8 layers, 16 input features per cell) that predicts a time step's head
 * change; trained and evaluated on the GPU (BF16 tensor-core GEMMs, FP32
 * accumulation, FP32 Adam).  Device arrays: features nodes x 16 (row-major
 * FP32), targets, masks and outputs nodes (FP32).  The loss is
 * inv_count * sum(((y - target) * mask)^2), or the energy loss that
 * gbmpnn_set_loss selects. */
typedef struct gbmpnn_handle gbmpnn_handle;
long long gbmpnn_param_count(void);
int gbmpnn_create(int nodes, int nja, const int *ia, const int *ja, unsigned long long seed,
                  gbmpnn_handle **out);
/* Edge weights from an assembled matrix (device amat, nja, the CSR of create). */
int gbmpnn_set_graph(gbmpnn_handle *h, const double *d_amat);
int gbmpnn_forward(gbmpnn_handle *h, const float *d_x, float *d_y);
/* Loss and (grad != NULL) the gradient, both to the host, without an update. */
int gbmpnn_gradients(gbmpnn_handle *h, const float *d_x, const float *d_target,
                     const float *d_mask, float inv_count, float *loss, float *grad);
/* One Adam step (learning rate lr) on one sample; the loss before the step. */
int gbmpnn_train_step(gbmpnn_handle *h, const float *d_x, const float *d_target,
                      const float *d_mask, float inv_count, float lr, float *loss);
int gbmpnn_get_params(gbmpnn_handle *h, float *params);
int gbmpnn_set_params(gbmpnn_handle *h, const float *params);
const char *gbmpnn_last_error(const gbmpnn_handle *h);
int gbmpnn_destroy(gbmpnn_handle *h);

/* The scalings between heads and the network's units. */
typedef struct gbmpnn_scaling {
  double head_ref, head_scale; /* feature 1: (previous head - head_ref) / head_scale */
  double dh_soft, dh_scale;    /* a head change dh in network units: asinh(dh / dh_soft) / dh_scale */
  double unit_max;             /* bound on |output| in network units (0: none) */
} gbmpnn_scaling;

/* The training loss.  mode 0: the masked squared error in network units
 * (the default).  mode 1: the relative energy error of the predicted head
 * change, e'We / t'Wt with W = -A over the active (mask) cells, A the matrix
 * of the last gbmpnn_set_graph (copied there), e = dh(y) - dh(target),
 * t = dh(target), dh(u) = dh_soft * sinh(u * dh_scale) -- the error that a
 * conjugate-gradient solve started from the guess has to remove, relative
 * to the one it has from the previous heads -- plus mse_weight times the
 * squared error of mode 0.  A sample whose t'Wt is not positive adds
 * nothing. */
int gbmpnn_set_loss(gbmpnn_handle *h, int mode, const gbmpnn_scaling *sc, float mse_weight);

/* The guess for the next time step of a solution, on the device and on the
 * solution's own stream (no host synchronisation): the features are built
 * from d_static (nodes x 16 FP32: the static columns; columns 1 and 6 are
 * replaced by the last step's heads and head change, the change taken as 0
 * when first_step), the network runs, and d_guess (nodes, FP64) = heads +
 * predicted change on active cells.  Pass d_guess to gbsln_timestep_warm or
 * gbsln_timestep_guess.  device_ms (may be NULL) gets the device time of the
 * guess; asking for it synchronises. */
int gbsln_warm_guess(gbsln_handle *sln, gbmpnn_handle *net, const float *d_static,
                     const gbmpnn_scaling *sc, int first_step, double *d_guess, float *device_ms);

#ifdef __cplusplus
}
#endif
#endif
