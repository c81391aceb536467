// gbims_api.cu -- C ABI of the IMS linear accelerator (include/gbims.h).
//
// gbims_create mirrors ImsLinearDataType%imslinear_allocate
// (src/Solution/LinearMethods/ImsLinear.f90:111-339) and gbims_apply mirrors
// %imslinear_apply (:617-750): preconditioner update with the pivot retry of
// ims_base_pcu (ImsLinearBase.f90:761-864), zeroed work vectors, the initial
// residual and L2NORM0, then PCG or BiCGSTAB.
//
// The inner Krylov loop is one CUDA graph: a WHILE conditional node whose body
// is one iteration; the device control kernels clear the condition when the
// reference would EXIT INNER.  One graph launch per linear solve, no host
// round trip per iteration.
#include "gbims_internal.cuh"
#include "k_krylov.cuh"
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <new>

using namespace gb;

struct gbims_handle {
  gbims_settings s{};
  int n = 0, nja = 0, ipc = 1;
  bool mixed = false, bcgs = false;
  std::vector<int> ia, ja, iapc, japc;
  int *d_ia = nullptr, *d_ja = nullptr, *d_iapc = nullptr, *d_japc = nullptr;
  double *d_apc = nullptr;
  float *d_apc32 = nullptr;
  Sell S;
  Levels F, B;
  Dia7 D;
  bool structured = false;  // wavefront sweeps (one or more full DIS grids)
  bool dia_spmv = false;    // index-free SpMV (a single full DIS grid)
  // owned FP64 buffers
  double *d_amat = nullptr, *d_rhs = nullptr, *d_x = nullptr;
  double *v_d = nullptr, *v_p = nullptr, *v_q = nullptr, *v_z = nullptr, *v_t = nullptr,
         *v_v = nullptr, *v_dhat = nullptr, *v_phat = nullptr, *v_qhat = nullptr;
  // FP32 inner vectors (mixed)
  float *f_d = nullptr, *f_p = nullptr, *f_q = nullptr, *f_z = nullptr, *f_t = nullptr,
        *f_v = nullptr, *f_dhat = nullptr, *f_phat = nullptr, *f_qhat = nullptr;
  // SCALING_METHOD: DSCALE, DSCALE2 and the column position map (L2NORM)
  double *d_dscale = nullptr, *d_dscale2 = nullptr;
  int *d_cptr = nullptr, *d_cpos = nullptr;
  double *d_part = nullptr;
  int G = 1;
  // per-inner-iteration records (gbims_set_inner_records): capacity per
  // apply, models, their first rows (0-based, nmod+1), the record rows, the
  // per-model partials and the locations carried between iterations
  int rec_cap = 0, rec_nmod = 0, rec_G = 0;
  int *d_modstart = nullptr;
  double *d_rec = nullptr, *d_rec_part = nullptr;
  long long *d_rec_loc = nullptr;
  Ctl *d_ctl = nullptr, *h_ctl = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_tried = false, graph_ok = false;
  bool no_graph = false;   // GBIMS_GRAPH=0: the host drives the loop
  LevelWords LW;           // the level-scheduled sweeps' result words (unstructured handles)
  int G_alloc = 0;         // reduction blocks the partials were sized for
  double refine_factor = 1.0e-5;  // 1e-4 saves 3 % of the iterations but loses accuracy with BiCGSTAB
  bool factored = false;
  // ILUT / MILUT (IPC 3/4): padded per-row factor, the reference's storage
  // length iwk (ims_calc_pcdims) and the positions of IAPC/JAPC/APC in use
  IlutDev I;
  IlutStatus *h_ilut = nullptr;
  long long ilut_iwk = 0;
  int njapc = 0;
  // REORDERING_METHOD RCM/MD: the solve runs on the permuted system (A0, IA0,
  // JA0 of imslinear_ap); callers' arrays, the scaling and the unscaling
  // stay in the model's numbering (u_*), gathered in and out at each apply
  bool reorder = false;
  std::vector<int> lorder, ia_u, ja_u, asrc;
  int *d_lorder = nullptr, *d_iorder = nullptr, *d_asrc = nullptr;
  int *d_ia_u = nullptr, *d_ja_u = nullptr;
  double *u_amat = nullptr, *u_rhs = nullptr, *u_x = nullptr;
  // batched ensemble (nm > 0): members concatenated into one block-diagonal
  // system, one control block per member, the handle's Ctl = all done
  int nm = 0;
  std::vector<int> mrow;  // member -> first row (nm + 1)
  int *d_bcm = nullptr, *d_bcr = nullptr, *d_bmc = nullptr, *d_bmr = nullptr;
  Ctl *d_ctls = nullptr, *h_ctls = nullptr;
  BatchDev bd;
  long long launches = 0;  // kernels launched by this handle (graph bodies counted per body)
  int body_kernels = 0;    // kernel nodes in one inner-loop body
  std::string err;
};

#define GB_CUDA(h, call)                                                            \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      if (h) (h)->err = std::string(#call) + ": " + cudaGetErrorString(e_);         \
      return GBIMS_ERR_CUDA;                                                        \
    }                                                                               \
  } while (0)

template <typename T>
static cudaError_t dalloc(T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)p, sizeof(T) * count);
}

static int fail(gbims_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

// ---------------------------------------------------------------------------
// graph body: one inner iteration
// ---------------------------------------------------------------------------
// The sync-free level sweeps' words, allocated (zeroed) before their first
// use; a handle with wavefront sweeps never needs them.
static int ensure_level_words(gbims_handle *h) {
  if (h->structured || h->LW.fwd) return GBIMS_OK;
  const size_t wb = (size_t)h->n * (h->mixed ? 8 : 16);
  GB_CUDA(h, cudaMalloc(&h->LW.fwd, wb));
  GB_CUDA(h, cudaMalloc(&h->LW.bwd, wb));
  GB_CUDA(h, cudaMalloc((void **)&h->LW.ticket, 256));
  GB_CUDA(h, cudaMalloc((void **)&h->LW.err, sizeof(int)));
  GB_CUDA(h, cudaMemset(h->LW.fwd, 0, wb));
  GB_CUDA(h, cudaMemset(h->LW.bwd, 0, wb));
  GB_CUDA(h, cudaMemset(h->LW.ticket, 0, 256));
  GB_CUDA(h, cudaMemset(h->LW.err, 0, sizeof(int)));
  return GBIMS_OK;
}

// A level sweep whose wait ran out (reported by the kernels' error word).
static int level_words_error(gbims_handle *h) {
  if (h->structured || !h->LW.err) return GBIMS_OK;
  int e = 0;
  GB_CUDA(h, cudaMemcpy(&e, h->LW.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return fail(h, GBIMS_ERR_CUDA, "level sweep wait limit reached");
  return GBIMS_OK;
}

static void precond64(gbims_handle *h, const double *r, double *z) {
  if (h->structured && h->D.mapped) {
    // an IDOMAIN-reduced grid: the sweeps on the full grid
    launch_dia7_spread(h->D, h->n, r, h->D.d_rfull, h->st);
    launch_dia7_apply64(h->D, h->D.d_rfull, h->D.d_zfull, h->d_ctl, h->st);
    launch_dia7_collect(h->D, h->n, h->D.d_zfull, z, h->st);
  } else if (h->structured) launch_dia7_apply64(h->D, r, z, h->d_ctl, h->st);
  else launch_ilu_apply_levels(h->n, h->d_iapc, h->d_japc, h->d_apc, h->F, h->B, h->LW, r, z, h->d_ctl, h->st);
}

// The mixed form's preconditioner: FP32 factors, vectors and sweeps.
static void precond32(gbims_handle *h, const float *r, float *z) {
  if (h->structured && h->D.mapped) {
    launch_dia7_spread32(h->D, h->n, r, h->D.f_rfull, h->st);
    launch_dia7_apply32(h->D, h->D.f_rfull, h->D.f_zfull, h->d_ctl, h->st);
    launch_dia7_collect32(h->D, h->n, h->D.f_zfull, z, h->st);
  } else if (h->structured) launch_dia7_apply32(h->D, r, z, h->d_ctl, h->st);
  else launch_ilu_apply_levels32(h->n, h->d_iapc, h->d_japc, h->d_apc32, h->F, h->B, h->LW, r, z, h->d_ctl, h->st);
}

// A*x and b - A*x: index-free on full DIS grids, SELL-32 otherwise.
static void spmv64(gbims_handle *h, const double *x, double *y, const Ctl *c) {
  if (h->dia_spmv) launch_dia7_spmv64(h->D, x, y, c, h->st);
  else launch_spmv64(h->S, x, y, c, h->st);
}

// The mixed form's product: FP32 matrix values and vectors.
static void spmv32(gbims_handle *h, const float *x, float *y, const Ctl *c) {
  if (h->dia_spmv) launch_dia7_spmv32(h->D, x, y, c, h->st);
  else launch_spmv32(h->S, x, y, c, h->st);
}

static void residual64(gbims_handle *h, const Ctl *c, int only_if_north_due) {
  if (h->dia_spmv) launch_dia7_residual64(h->D, h->d_x, h->d_rhs, h->v_d, c, only_if_north_due, h->st);
  else launch_residual64(h->S, h->d_x, h->d_rhs, h->v_d, c, only_if_north_due, h->st);
}

static void enqueue_iteration(gbims_handle *h, unsigned long long cond, int use_cond) {
  const int n = h->n, G = h->G;
  Ctl *c = h->d_ctl;
  cudaStream_t st = h->st;
  double *part = h->d_part;
  if (h->nm > 0 && h->mixed) {
    // batched ensemble, mixed form: every member's FP32 PCG iteration and,
    // where due, its FP64 refinement, in the same launches
    const BatchDev &B = h->bd;
    precond32(h, h->f_d, h->f_z);
    kb_dot32(B, h->f_d, h->f_z, part, st);
    kb_ctl_cg_rho(B, part, st);
    kb_cg_pupdate32(B, h->f_z, h->f_p, st);
    spmv32(h, h->f_p, h->f_q, c);
    kb_dot32(B, h->f_p, h->f_q, part, st);
    kb_ctl_alpha(B, part, st);
    kb_cg_update_mixed(B, h->d_x, h->f_d, h->f_p, h->f_q, part, st);
    kb_ctl_mixed_inner(B, part, h->refine_factor, st);
    kb_any_due(B, c, st);
    residual64(h, c, 1);
    kb_true_resid_stats(B, h->v_d, h->f_d, part, st);
    kb_ctl_refine(B, part, st);
    kb_all_done(B, c, cond, use_cond, 1, st);
    return;
  }
  if (h->nm > 0) {
    // batched ensemble, PCG: every member's iteration in the same launches
    const BatchDev &B = h->bd;
    precond64(h, h->v_d, h->v_z);
    kb_dot64(B, h->v_d, h->v_z, part, st);
    kb_ctl_cg_rho(B, part, st);
    kb_cg_pupdate64(B, h->v_z, h->v_p, st);
    spmv64(h, h->v_p, h->v_q, c);
    kb_dot64(B, h->v_p, h->v_q, part, st);
    kb_ctl_alpha(B, part, st);
    kb_cg_update64(B, h->d_x, h->v_d, h->v_p, h->v_q, part, st);
    kb_ctl_cg_cnvg(B, part, st);
    kb_all_done(B, c, cond, use_cond, 1, st);
    return;
  }
  if (!h->mixed && !h->bcgs) {
    // ims_base_cg, ImsLinearBase.f90:100-236
    precond64(h, h->v_d, h->v_z);
    kr_dot64(n, h->v_d, h->v_z, part, G, c, st);
    kr_ctl_cg_rho(c, part, G, st);
    kr_cg_pupdate64(n, h->v_z, h->v_p, c, st);
    spmv64(h, h->v_p, h->v_q, c);
    kr_dot64(n, h->v_p, h->v_q, part, G, c, st);
    kr_ctl_alpha(c, part, G, st);
    kr_cg_update64(n, h->d_x, h->v_d, h->v_p, h->v_q, part, G, c, st, h->s.icnvgopt >= 2);
    if (h->rec_cap > 0 && h->rec_nmod > 1)
      kr_rec_models(false, h->rec_nmod, h->d_modstart, h->v_p, nullptr, h->v_d, nullptr,
                    h->d_rec_part, h->rec_G, c, st);
    kr_ctl_cg_cnvg(c, part, G, cond, use_cond, st);
    if (h->s.north > 0) residual64(h, c, 1);  // the NORTH residual refresh
  } else if (!h->mixed && h->bcgs) {
    // ims_base_bcgs, ImsLinearBase.f90:338-545
    kr_dot64(n, h->v_dhat, h->v_d, part, G, c, st);
    kr_ctl_bcgs_rho(c, part, G, st);
    kr_bcgs_p64(n, h->v_d, h->v_p, h->v_v, c, st);
    precond64(h, h->v_p, h->v_phat);
    spmv64(h, h->v_phat, h->v_v, c);
    kr_dot64(n, h->v_dhat, h->v_v, part, G, c, st);
    kr_ctl_alpha(c, part, G, st);
    kr_bcgs_q64(n, h->v_d, h->v_v, h->v_q, c, st);
    precond64(h, h->v_q, h->v_qhat);
    spmv64(h, h->v_qhat, h->v_t, c);
    kr_dot_tq_tt64(n, h->v_t, h->v_q, part, G, c, st);
    kr_ctl_omega(c, part, G, st);
    kr_bcgs_update64(n, h->d_x, h->v_d, h->v_phat, h->v_qhat, h->v_q, h->v_t, h->d_dscale, part, G, c, st,
                     h->s.icnvgopt >= 2);
    if (h->rec_cap > 0 && h->rec_nmod > 1)
      kr_rec_models(true, h->rec_nmod, h->d_modstart, h->v_phat, h->v_qhat, h->v_d, h->d_dscale,
                    h->d_rec_part, h->rec_G, c, st);
    kr_ctl_bcgs_cnvg(c, part, G, cond, use_cond, st);
    if (h->s.north > 0) residual64(h, c, 1);  // the NORTH residual refresh
  } else if (h->mixed && !h->bcgs) {
    // PCG on the FP32 matrix with FP32 vectors and preconditioner, FP64
    // scalars and heads; the FP64 true residual restarts the recurrence at
    // each refinement
    precond32(h, h->f_d, h->f_z);
    kr_dot32(n, h->f_d, h->f_z, part, G, c, st);
    kr_ctl_cg_rho(c, part, G, st);
    kr_cg_pupdate32(n, h->f_z, h->f_p, c, st);
    spmv32(h, h->f_p, h->f_q, c);
    kr_dot32(n, h->f_p, h->f_q, part, G, c, st);
    kr_ctl_alpha(c, part, G, st);
    kr_cg_update_mixed(n, h->d_x, h->f_d, h->f_p, h->f_q, part, G, c, st);
    kr_ctl_mixed_inner(c, part, G, 0, h->refine_factor, st);
    residual64(h, c, 1);
    kr_true_resid_stats(n, h->v_d, h->f_d, nullptr, nullptr, nullptr, part, G, c, st);
    kr_ctl_refine(c, part, G, cond, use_cond, st);
  } else {
    // BiCGSTAB, same precision split
    kr_dot32(n, h->f_dhat, h->f_d, part, G, c, st);
    kr_ctl_bcgs_rho(c, part, G, st);
    kr_bcgs_p32(n, h->f_d, h->f_p, h->f_v, c, st);
    precond32(h, h->f_p, h->f_phat);
    spmv32(h, h->f_phat, h->f_v, c);
    kr_dot32(n, h->f_dhat, h->f_v, part, G, c, st);
    kr_ctl_alpha(c, part, G, st);
    kr_bcgs_q32(n, h->f_d, h->f_v, h->f_q, c, st);
    precond32(h, h->f_q, h->f_qhat);
    spmv32(h, h->f_qhat, h->f_t, c);
    kr_dot_tq_tt32(n, h->f_t, h->f_q, part, G, c, st);
    kr_ctl_omega(c, part, G, st);
    kr_bcgs_update32(n, h->d_x, h->f_d, h->f_phat, h->f_qhat, h->f_q, h->f_t, h->d_dscale, part, G, c, st);
    kr_ctl_mixed_inner(c, part, G, 1, h->refine_factor, st);
    residual64(h, c, 1);
    kr_true_resid_stats(n, h->v_d, h->f_d, h->f_dhat, nullptr, h->d_dscale, part, G, c, st);
    kr_ctl_refine(c, part, G, cond, use_cond, st);
  }
}

static bool build_graph(gbims_handle *h) {
  h->graph_tried = true;
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
  cudaGraphConditionalHandle cond;
  if (cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    return false;
  }
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  cp.conditional.handle = cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    return false;
  }
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  if (cudaStreamBeginCaptureToGraph(h->st, body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    return false;
  }
  enqueue_iteration(h, (unsigned long long)cond, 1);
  cudaGraph_t captured = nullptr;
  cudaError_t e = cudaStreamEndCapture(h->st, &captured);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    return false;
  }
  // kernel nodes per loop body, for the launch count
  size_t nn = 0;
  cudaGraphGetNodes(body, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn) cudaGraphGetNodes(body, nodes.data(), &nn);
  h->body_kernels = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType ty;
    if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) h->body_kernels++;
  }
  cudaGraphExec_t exec = nullptr;
  if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    return false;
  }
  h->graph = g;
  h->exec = exec;
  h->graph_ok = true;
  return true;
}

// ---------------------------------------------------------------------------
// create
// ---------------------------------------------------------------------------
// Wavefront-sweep buffers for members of the given DIS shapes (nlay, nrow,
// ncol per member) whose rows start at row0.
static int setup_structured(gbims_handle *h, const std::vector<int> &shapes,
                            const std::vector<long long> &row0) {
  dia7_layout(h->D, shapes, row0, h->mixed);
  const size_t nn = (size_t)h->D.slots;
  if (!h->mixed) {
    double **a[] = {&h->D.d_lz, &h->D.d_ly, &h->D.d_lx, &h->D.d_ux, &h->D.d_uy, &h->D.d_uz,
                    &h->D.d_dinv};
    for (double **p : a) GB_CUDA(h, dalloc(p, nn));
  } else {
    float **a[] = {&h->D.f_lz, &h->D.f_ly, &h->D.f_lx, &h->D.f_ux, &h->D.f_uy, &h->D.f_uz,
                   &h->D.f_dinv};
    for (float **p : a) GB_CUDA(h, dalloc(p, nn));
  }
  // result words: zero, so that no word carries the epoch of a sweep yet
  const size_t llb = nn * (h->mixed ? 8 : 16);
  for (void **p : {&h->D.ll_y, &h->D.ll_z}) {
    GB_CUDA(h, dalloc((unsigned char **)p, llb));
    GB_CUDA(h, cudaMemset(*p, 0, llb));
  }
  GB_CUDA(h, dalloc(&h->D.d_geo, h->D.geo.size()));
  GB_CUDA(h, cudaMemcpy(h->D.d_geo, h->D.geo.data(), sizeof(Dia7Geo) * h->D.geo.size(),
                        cudaMemcpyHostToDevice));
  // the forward and backward ticket counters, one 128-byte line each
  h->D.nflags = 2 * 32;
  GB_CUDA(h, dalloc(&h->D.d_flags, h->D.nflags));
  GB_CUDA(h, cudaMemset(h->D.d_flags, 0, sizeof(int) * h->D.nflags));
  GB_CUDA(h, dalloc(&h->D.d_err, 4));
  GB_CUDA(h, cudaMemset(h->D.d_err, 0, sizeof(int) * 4));
  // default tiling: the fastest on the 10M-cell case in both precisions
  // (chunk 8, ring 4, prefetch 2, two CTAs per SM); gbims_autotune picks
  // per system
  h->D.cfg = 7;
  if (const char *nv = std::getenv("GBIMS_SWEEP_NATIVE")) h->D.ext_allowed = (nv[0] == '0');
  h->structured = true;
  return GBIMS_OK;
}

extern "C" int gbims_create(const gbims_settings *s, int neq, int nja, const int *ia,
                            const int *ja, gbims_handle **out) {
  if (!out) return GBIMS_ERR_ARG;
  *out = nullptr;
  if (!s || !ia || !ja || neq <= 0 || nja < neq) return GBIMS_ERR_ARG;
  gbims_handle *h = new (std::nothrow) gbims_handle();
  if (!h) return GBIMS_ERR_NOMEM;
  h->s = *s;
  h->n = neq;
  h->nja = nja;
  // ImsLinear.f90:178-185: IPC from level/droptol/relax
  h->ipc = (s->level > 0 || s->droptol > 0.0) ? 3 : 1;
  if (s->relax > 0.0) h->ipc += 1;
  // option checks (ImsLinear.f90:187-215)
  if (s->ilinmeth != 1 && s->ilinmeth != 2) { *out = h; return fail(h, GBIMS_ERR_ARG, "ilinmeth must be 1 (CG) or 2 (BICGSTAB)"); }
  if (s->iscl < 0 || s->iscl > 2) { *out = h; return fail(h, GBIMS_ERR_ARG, "IMSLINEAR7AR ISCL MUST BE <= 2"); }
  if (s->iord < 0 || s->iord > 2) { *out = h; return fail(h, GBIMS_ERR_ARG, "IMSLINEAR7AR IORD MUST BE <= 2"); }
  if (s->north < 0) { *out = h; return fail(h, GBIMS_ERR_ARG, "IMSLINEAR7AR NORTH MUST >= 0"); }
  if (s->rclose == 0.0 && s->icnvgopt != 3) { *out = h; return fail(h, GBIMS_ERR_ARG, "IMSLINEAR7AR RCLOSE MUST > 0.0"); }
  if (s->relax < 0.0) { *out = h; return fail(h, GBIMS_ERR_ARG, "IMSLINEAR7AR RELAX MUST BE >= 0.0"); }
  if (s->relax > 1.0) { *out = h; return fail(h, GBIMS_ERR_ARG, "IMSLINEAR7AR RELAX MUST BE <= 1.0"); }
  if (s->level < 0) { *out = h; return fail(h, GBIMS_ERR_ARG, "ILUT: PRECONDITIONER_LEVELS must be >= 0"); }
  // With ILU0/MILU0 the reference factors the permuted matrix against the
  // IAPC/JAPC of the unpermuted pattern (built at ImsLinear.f90:244-248,
  // before the ordering at :333-336), carrying work-vector entries from row
  // to row; that combination is declined rather than changed.
  if (s->iord != 0 && h->ipc < 3) { *out = h; return fail(h, GBIMS_ERR_UNSUPPORTED, "REORDERING_METHOD RCM/MD is supported with ILUT/MILUT only (PRECONDITIONER_LEVELS or DROP_TOLERANCE > 0)"); }
  if (s->precision != GBIMS_FP64 && s->precision != GBIMS_MIXED) { *out = h; return fail(h, GBIMS_ERR_ARG, "precision must be GBIMS_FP64 or GBIMS_MIXED"); }
  h->mixed = (s->precision == GBIMS_MIXED);
  h->bcgs = (s->ilinmeth == 2);
  // GBIMS_GRAPH=0: the inner loop is driven from the host (the same kernels,
  // launched one by one), for profilers that do not see kernel nodes inside
  // conditional graphs
  if (const char *g = std::getenv("GBIMS_GRAPH")) h->no_graph = (g[0] == '0');
  h->graph_tried = h->no_graph;
  // GBIMS_REFINE: the mixed form's relative L2 reduction per refinement
  if (const char *r = std::getenv("GBIMS_REFINE")) {
    const double v = std::atof(r);
    if (v > 0.0 && v < 1.0) h->refine_factor = v;
  }
  // 0-based copies and checks: diagonal first in every row
  if (s->index_base != 0 && s->index_base != 1) { *out = h; return fail(h, GBIMS_ERR_ARG, "index_base must be 0 or 1"); }
  int base = s->index_base;
  h->ia.resize(neq + 1);
  h->ja.resize(nja);
  for (int i = 0; i <= neq; ++i) h->ia[i] = ia[i] - base;
  for (int k = 0; k < nja; ++k) h->ja[k] = ja[k] - base;
  if (h->ia[0] != 0 || h->ia[neq] != nja) { *out = h; return fail(h, GBIMS_ERR_ARG, "ia must start at index_base and end at nja+index_base"); }
  for (int r = 0; r < neq; ++r) {
    if (h->ia[r + 1] <= h->ia[r]) { *out = h; return fail(h, GBIMS_ERR_ARG, "empty CSR row (the diagonal must be present)"); }
    if (h->ja[h->ia[r]] != r) { *out = h; return fail(h, GBIMS_ERR_ARG, "the diagonal must be the first entry of each row"); }
    if (h->ia[r + 1] - h->ia[r] > kMaxRowLen) { *out = h; return fail(h, GBIMS_ERR_UNSUPPORTED, "CSR row longer than 64 entries"); }
    for (int k = h->ia[r]; k < h->ia[r + 1]; ++k)
      if (h->ja[k] < 0 || h->ja[k] >= neq) { *out = h; return fail(h, GBIMS_ERR_ARG, "column index out of range"); }
  }
  // REORDERING_METHOD RCM/MD: LORDER (ims_base_calc_order) and the permuted
  // pattern of dperm with job 1 (sparsekit.f90:163-447): row j becomes row
  // LORDER(j), its entries kept in order, columns relabelled by LORDER --
  // LORDER is the numbering's list of nodes, used as a new-index map, as
  // imslinear_ap passes it (ImsLinear.f90:653-658)
  if (s->iord != 0) {
    h->reorder = true;
    if (s->iord == 1) {
      rcm_order(neq, h->ia, h->ja, h->lorder);
    } else if (int flag = md_order(neq, h->ia, h->ja, h->lorder)) {
      // ImsLinearBase.f90:590-595: fatal in the reference
      *out = h;
      return fail(h, GBIMS_ERR_ARG, "IMSLINEARSUB_CALC_ORDER error creating minimum degree order permutation (flag " + std::to_string(flag) + ")");
    }
    h->ia_u = h->ia;
    h->ja_u = h->ja;
    std::vector<int> iaro(neq + 1, 0), jaro(nja);
    h->asrc.assign(nja, 0);
    for (int j = 0; j < neq; ++j) iaro[h->lorder[j] + 1] = h->ia_u[j + 1] - h->ia_u[j];
    for (int j = 0; j < neq; ++j) iaro[j + 1] += iaro[j];
    for (int r = 0; r < neq; ++r) {
      int ko = iaro[h->lorder[r]];
      for (int k = h->ia_u[r]; k < h->ia_u[r + 1]; ++k) {
        jaro[ko] = h->lorder[h->ja_u[k]];
        h->asrc[ko] = k;
        ++ko;
      }
    }
    h->ia = iaro;
    h->ja = jaro;
  }
  // ims_base_pccrs (ImsLinearBase.f90:1207-1261)
  h->iapc.assign(neq + 1, 0);
  h->japc.assign(nja, 0);
  {
    int ip = neq;
    std::vector<int> iarr;
    for (int r = 0; r < neq; ++r) {
      iarr.clear();
      for (int k = h->ia[r]; k < h->ia[r + 1]; ++k)
        if (h->ja[k] != r) iarr.push_back(h->ja[k]);
      std::stable_sort(iarr.begin(), iarr.end());
      h->iapc[r] = ip;
      for (int c : iarr) h->japc[ip++] = c;
    }
    h->iapc[neq] = nja;
    if (ip != nja) { *out = h; return fail(h, GBIMS_ERR_ARG, "nja is inconsistent with ia (one diagonal per row expected)"); }
    for (int r = 0; r < neq; ++r) {
      h->japc[r] = h->iapc[r + 1];
      for (int j = h->iapc[r]; j < h->iapc[r + 1]; ++j)
        if (h->japc[j] > r) { h->japc[r] = j; break; }
    }
  }
  h->njapc = nja;
  long long ilut_cap = 0;
  if (h->ipc >= 3) {
    // ILUT keeps at most lfil L and lfil - 1 U entries per row; its storage
    // starts after the n inverse pivots and one unused slot (sparskit's MSR)
    const long long sl = s->level, su = std::max(0, s->level - 1);
    ilut_cap = (long long)neq + 1 + (long long)neq * (sl + su);
    if (ilut_cap > INT_MAX) { *out = h; return fail(h, GBIMS_ERR_UNSUPPORTED, "ILUT storage exceeds 32-bit positions"); }
    int maxrow = 0;
    for (int r = 0; r < neq; ++r) maxrow = std::max(maxrow, h->ia[r + 1] - h->ia[r]);
    h->ilut_iwk = s->level > 0 ? (long long)neq * (2LL * s->level + 1) : (long long)neq * maxrow;
    // until the first factorisation: no L or U entries in any row
    h->japc.assign((size_t)ilut_cap, 0);
    h->iapc.assign(neq + 1, neq + 1);
    for (int r = 0; r < neq; ++r) h->japc[r] = neq + 1;
    h->njapc = neq + 1;
    h->I.n = neq;
    h->I.lfil = s->level;
    h->I.sl = (int)sl;
    h->I.su = (int)su;
  }
  const size_t npc = h->ipc >= 3 ? (size_t)ilut_cap : (size_t)nja;
  // device state
  *out = h;
  GB_CUDA(h, cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  GB_CUDA(h, cudaEventCreate(&h->ev0));
  GB_CUDA(h, cudaEventCreate(&h->ev1));
  GB_CUDA(h, dalloc(&h->d_ia, neq + 1));
  GB_CUDA(h, dalloc(&h->d_ja, nja));
  GB_CUDA(h, dalloc(&h->d_iapc, neq + 1));
  GB_CUDA(h, dalloc(&h->d_japc, npc));
  GB_CUDA(h, dalloc(&h->d_apc, npc));
  GB_CUDA(h, cudaMemcpy(h->d_ia, h->ia.data(), sizeof(int) * (neq + 1), cudaMemcpyHostToDevice));
  GB_CUDA(h, cudaMemcpy(h->d_ja, h->ja.data(), sizeof(int) * nja, cudaMemcpyHostToDevice));
  if (h->reorder) {
    std::vector<int> iorder(neq);
    for (int j = 0; j < neq; ++j) iorder[h->lorder[j]] = j;
    GB_CUDA(h, dalloc(&h->d_lorder, neq));
    GB_CUDA(h, dalloc(&h->d_iorder, neq));
    GB_CUDA(h, dalloc(&h->d_asrc, nja));
    GB_CUDA(h, dalloc(&h->d_ia_u, neq + 1));
    GB_CUDA(h, dalloc(&h->d_ja_u, nja));
    GB_CUDA(h, cudaMemcpy(h->d_lorder, h->lorder.data(), sizeof(int) * neq, cudaMemcpyHostToDevice));
    GB_CUDA(h, cudaMemcpy(h->d_iorder, iorder.data(), sizeof(int) * neq, cudaMemcpyHostToDevice));
    GB_CUDA(h, cudaMemcpy(h->d_asrc, h->asrc.data(), sizeof(int) * nja, cudaMemcpyHostToDevice));
    GB_CUDA(h, cudaMemcpy(h->d_ia_u, h->ia_u.data(), sizeof(int) * (neq + 1), cudaMemcpyHostToDevice));
    GB_CUDA(h, cudaMemcpy(h->d_ja_u, h->ja_u.data(), sizeof(int) * nja, cudaMemcpyHostToDevice));
    GB_CUDA(h, dalloc(&h->u_amat, nja));
    GB_CUDA(h, dalloc(&h->u_rhs, (size_t)neq + kVecPad));
    GB_CUDA(h, dalloc(&h->u_x, (size_t)neq + kVecPad));
  }
  GB_CUDA(h, cudaMemcpy(h->d_iapc, h->iapc.data(), sizeof(int) * (neq + 1), cudaMemcpyHostToDevice));
  GB_CUDA(h, cudaMemcpy(h->d_japc, h->japc.data(), sizeof(int) * h->njapc, cudaMemcpyHostToDevice));
  GB_CUDA(h, cudaMemset(h->d_apc, 0, sizeof(double) * npc));
  if (h->ipc >= 3) {
    IlutDev &I = h->I;
    const size_t nsl = std::max<size_t>(1, (size_t)neq * I.sl);
    const size_t nsu = std::max<size_t>(1, (size_t)neq * I.su);
    GB_CUDA(h, dalloc(&I.lcol, nsl));
    GB_CUDA(h, dalloc(&I.lval, nsl));
    GB_CUDA(h, dalloc(&I.ucol, nsu));
    GB_CUDA(h, dalloc(&I.uval, nsu));
    GB_CUDA(h, dalloc(&I.nl, neq));
    GB_CUDA(h, dalloc(&I.nu, neq));
    GB_CUDA(h, dalloc(&I.dinv, neq));
    GB_CUDA(h, dalloc(&I.rdone, neq));
    GB_CUDA(h, dalloc(&I.stat, 1));
    GB_CUDA(h, cudaMemset(I.rdone, 0, sizeof(unsigned) * neq));
    GB_CUDA(h, cudaMemset(I.nl, 0, sizeof(int) * neq));
    GB_CUDA(h, cudaMemset(I.nu, 0, sizeof(int) * neq));
    GB_CUDA(h, cudaMemset(I.dinv, 0, sizeof(double) * neq));
    GB_CUDA(h, cudaMallocHost((void **)&h->h_ilut, sizeof(IlutStatus)));
  }
  // optional structured 7-point sweeps (and the index-free SpMV); the
  // wavefront sweeps carry the ILU0 pattern only
  int dl = s->nlay, dr = s->nrow, dc = s->ncol;
  bool dis = false;
  if (h->ipc < 3 && dl >= 0) {
    if (dl == 0 && dr == 0 && dc == 0) dis = dia7_detect(neq, h->ia, h->ja, &dl, &dr, &dc);
    else dis = dl > 0 && dr > 0 && dc > 0 && dia7_matches(dl, dr, dc, neq, h->ia, h->ja);
  }
  if (dis) {
    std::vector<int> shape = {dl, dr, dc};
    int rc = setup_structured(h, shape, std::vector<long long>{0});
    if (rc != GBIMS_OK) return rc;
    GB_CUDA(h, dalloc(&h->D.d_sv, (size_t)7 * neq));
    if (h->mixed) GB_CUDA(h, dalloc(&h->D.f_sv, (size_t)7 * neq));
    h->dia_spmv = true;
  }
  // SELL-32 layout of A (unstructured patterns; a single full DIS grid uses
  // the index-free product)
  if (!h->dia_spmv) {
    std::vector<int> ptr, col, src;
    sell_build_host(neq, h->ia, h->ja, ptr, col, src);
    if ((long long)col.size() > INT_MAX) return fail(h, GBIMS_ERR_UNSUPPORTED, "matrix too large for 32-bit SELL offsets");
    h->S.n = neq;
    h->S.nslices = (int)ptr.size() - 1;
    h->S.nstored = (long long)col.size();
    GB_CUDA(h, dalloc(&h->S.d_ptr, ptr.size()));
    GB_CUDA(h, dalloc(&h->S.d_col, col.size()));
    GB_CUDA(h, dalloc(&h->S.d_src, src.size()));
    GB_CUDA(h, dalloc(&h->S.d_val, col.size()));
    GB_CUDA(h, cudaMemcpy(h->S.d_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice));
    GB_CUDA(h, cudaMemcpy(h->S.d_col, col.data(), sizeof(int) * col.size(), cudaMemcpyHostToDevice));
    GB_CUDA(h, cudaMemcpy(h->S.d_src, src.data(), sizeof(int) * src.size(), cudaMemcpyHostToDevice));
    if (h->mixed) GB_CUDA(h, dalloc(&h->S.d_val32, col.size()));
  }
  // level schedules of the triangular sweeps and the factorisation
  levels_build_host(neq, h->iapc, h->japc, true, h->F);
  levels_build_host(neq, h->iapc, h->japc, false, h->B);
  // vectors (with slack after the last cell for the sweeps' aligned copies)
  size_t nn = (size_t)neq + kVecPad;
  GB_CUDA(h, dalloc(&h->d_amat, nja));
  GB_CUDA(h, dalloc(&h->d_rhs, nn));
  GB_CUDA(h, dalloc(&h->d_x, nn));
  GB_CUDA(h, dalloc(&h->v_d, nn));
  if (!h->mixed) {
    GB_CUDA(h, dalloc(&h->v_p, nn));
    GB_CUDA(h, dalloc(&h->v_q, nn));
    GB_CUDA(h, dalloc(&h->v_z, nn));
    if (h->bcgs) {
      GB_CUDA(h, dalloc(&h->v_t, nn)); GB_CUDA(h, dalloc(&h->v_v, nn));
      GB_CUDA(h, dalloc(&h->v_dhat, nn)); GB_CUDA(h, dalloc(&h->v_phat, nn));
      GB_CUDA(h, dalloc(&h->v_qhat, nn));
    }
  } else {
    // FP32 factors and inner vectors; FP64 heads and true residual
    GB_CUDA(h, dalloc(&h->d_apc32, npc));
    GB_CUDA(h, dalloc(&h->f_d, nn)); GB_CUDA(h, dalloc(&h->f_p, nn));
    GB_CUDA(h, dalloc(&h->f_q, nn)); GB_CUDA(h, dalloc(&h->f_z, nn));
    if (h->bcgs) {
      GB_CUDA(h, dalloc(&h->f_t, nn)); GB_CUDA(h, dalloc(&h->f_v, nn));
      GB_CUDA(h, dalloc(&h->f_dhat, nn)); GB_CUDA(h, dalloc(&h->f_phat, nn));
      GB_CUDA(h, dalloc(&h->f_qhat, nn));
    }
  }
  // SCALING_METHOD (ImsLinear.f90:222-224): DSCALE/DSCALE2 only when scaling;
  // BiCGSTAB reads DSCALE in its convergence maxima (null without scaling)
  if (s->iscl != 0) {
    GB_CUDA(h, dalloc(&h->d_dscale, nn));
    GB_CUDA(h, dalloc(&h->d_dscale2, nn));
    if (s->iscl == 2) {
      std::vector<int> cptr, cpos;
      // the scaling works in the model's numbering
      scale_colmap_host(neq, h->reorder ? h->ia_u : h->ia, h->reorder ? h->ja_u : h->ja, cptr,
                        cpos);
      GB_CUDA(h, dalloc(&h->d_cptr, cptr.size()));
      GB_CUDA(h, dalloc(&h->d_cpos, cpos.size()));
      GB_CUDA(h, cudaMemcpy(h->d_cptr, cptr.data(), sizeof(int) * cptr.size(), cudaMemcpyHostToDevice));
      GB_CUDA(h, cudaMemcpy(h->d_cpos, cpos.data(), sizeof(int) * cpos.size(), cudaMemcpyHostToDevice));
    }
  }
  h->G = std::max(1, std::min(kMaxRedBlocks, (neq + kRedBlock - 1) / kRedBlock));
  h->G_alloc = h->G;
  GB_CUDA(h, dalloc(&h->d_part, (size_t)h->G * 8));
  GB_CUDA(h, dalloc(&h->d_ctl, 1));
  GB_CUDA(h, cudaMallocHost((void **)&h->h_ctl, sizeof(Ctl)));
  memset(h->h_ctl, 0, sizeof(Ctl));
  return GBIMS_OK;
}

// ---------------------------------------------------------------------------
// apply
// ---------------------------------------------------------------------------
static double epfact_of(int icnvgopt, int kstp) {
  // ims_base_epfact (ImsLinearBase.f90:1316-1333); 0.01/0.10 are default
  // (single-precision) real literals in the Fortran source
  if (icnvgopt == 2) return (kstp == 1) ? (double)0.01f : (double)0.10f;
  if (icnvgopt == 4) return 1.0e-4;
  return 1.0;
}

// dst[i] = src[idx[i]]: the permutations of REORDERING_METHOD RCM/MD (dperm and
// dvperm of sparsekit, as gathers)
__global__ void k_gather(int n, const int *__restrict__ idx, const double *__restrict__ src,
                         double *__restrict__ dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dst[i] = src[idx[i]];
}

static void gather(gbims_handle *h, int n, const int *idx, const double *src, double *dst) {
  const int g = std::max(1, std::min(8 * kNumSM, (n + 255) / 256));
  k_gather<<<g, 256, 0, h->st>>>(n, idx, src, dst);
  h->launches += 1;
}

// The arrays a caller fills and reads back: the model's numbering.
static double *in_amat(gbims_handle *h) { return h->reorder ? h->u_amat : h->d_amat; }
static double *in_rhs(gbims_handle *h) { return h->reorder ? h->u_rhs : h->d_rhs; }
static double *in_x(gbims_handle *h) { return h->reorder ? h->u_x : h->d_x; }

// PERMUTE ROWS, COLUMNS, AND RHS (ImsLinear.f90:652-666): AMAT by dperm,
// X and RHS by dvperm with LORDER (x0[LORDER(j)] = x[j]).
static void permute_in(gbims_handle *h) {
  gather(h, h->nja, h->d_asrc, h->u_amat, h->d_amat);
  gather(h, h->n, h->d_iorder, h->u_x, h->d_x);
  gather(h, h->n, h->d_iorder, h->u_rhs, h->d_rhs);
}

__global__ void k_zero_vec(int n, double *a, double *b, double *c, double *d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (a) a[i] = 0.0;
    if (b) b[i] = 0.0;
    if (c) c[i] = 0.0;
    if (d) d[i] = 0.0;
  }
}

static void drop_graph(gbims_handle *h);

// ILUT / MILUT update (ims_base_pcu, IPC 3/4: ImsLinearBase.f90:812-864
// around sparskit2/ilut.f90:48-462).  The pivot guard's retry loop is the
// reference's; ilut leaves izero unchanged on success, so a factorisation
// with izero 2 (delta 0.5) makes the reference repeat the same factorisation
// until icount exceeds 10: that count is taken without the repeats.  The
// pattern the factor kept is turned into IAPC/JAPC here, with the storage
// checks of ilut (ierr -2/-3) at the reference's positions, and the level
// schedules of the sweeps are rebuilt for it.
static int ilut_factor_core(gbims_handle *h) {
  const int n = h->n;
  cudaStream_t st = h->st;
  IlutDev &I = h->I;
  int ipcflag = 0, icount = 0;
  double delta = 0.0;
  for (;;) {
    I.epoch += 1;
    if (I.epoch == 0) {  // completion words wrapped: clear them
      GB_CUDA(h, cudaMemsetAsync(I.rdone, 0, sizeof(unsigned) * n, st));
      I.epoch = 1;
    }
    IlutStatus init{0ULL, INT_MAX, kIlutOk, -1, 0};
    *h->h_ilut = init;
    GB_CUDA(h, cudaMemcpyAsync(I.stat, h->h_ilut, sizeof(IlutStatus), cudaMemcpyHostToDevice, st));
    launch_ilut_factor(I, h->d_ia, h->d_ja, h->d_amat, h->s.droptol, h->s.relax, delta, ipcflag,
                       st);
    h->launches += 1;
    GB_CUDA(h, cudaMemcpyAsync(h->h_ilut, I.stat, sizeof(IlutStatus), cudaMemcpyDeviceToHost, st));
    GB_CUDA(h, cudaStreamSynchronize(st));
    GB_CUDA(h, cudaGetLastError());
    const IlutStatus r = *h->h_ilut;
    if (r.err == kIlutErrCap)
      return fail(h, GBIMS_ERR_UNSUPPORTED,
                  "ILUT: the working row of row " + std::to_string(r.err_row) + " exceeds " +
                      std::to_string(kIlutCap) +
                      " candidates (lower PRECONDITIONER_LEVELS or raise DROP_TOLERANCE)");
    if (r.err == kIlutErrZeroRow)
      return fail(h, GBIMS_ERR_ARG, "ILUT: zero row encountered (ilut ierr -5)");
    if (r.err != kIlutOk) return fail(h, GBIMS_ERR_CUDA, "ILUT factorisation wait limit reached");
    if (r.pivot_fail != INT_MAX) ipcflag = 1;
    if (ipcflag < 1) break;
    if (ipcflag == 2) {  // the repeats of an identical factorisation
      icount = std::max(icount, 11);
      break;
    }
    delta = 1.5 * delta + 1.0e-3;
    ipcflag = 0;
    if (delta > 0.5) {
      delta = 0.5;
      ipcflag = 2;
    }
    icount += 1;
    if (icount > 10) break;
  }
  // the kept pattern as IAPC/JAPC, with ilut's storage checks
  std::vector<int> nl(n), nu(n), lc((size_t)n * I.sl), uc((size_t)n * I.su);
  GB_CUDA(h, cudaMemcpyAsync(nl.data(), I.nl, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  GB_CUDA(h, cudaMemcpyAsync(nu.data(), I.nu, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  if (!lc.empty())
    GB_CUDA(h, cudaMemcpyAsync(lc.data(), I.lcol, sizeof(int) * lc.size(), cudaMemcpyDeviceToHost, st));
  if (!uc.empty())
    GB_CUDA(h, cudaMemcpyAsync(uc.data(), I.ucol, sizeof(int) * uc.size(), cudaMemcpyDeviceToHost, st));
  GB_CUDA(h, cudaStreamSynchronize(st));
  long long ju0 = (long long)n + 1;
  h->iapc[0] = (int)ju0;
  for (int r = 0; r < n; ++r) {
    if (nl[r] < 0 || nl[r] > I.sl || nu[r] < 0 || nu[r] > I.su)
      return fail(h, GBIMS_ERR_STATE, "ILUT: row counts out of range");
    for (int k = 0; k < nl[r]; ++k) {
      if (ju0 + 1 > h->ilut_iwk) return fail(h, GBIMS_ERR_ARG, "ILUT: L storage exceeded (ilut ierr -2)");
      h->japc[ju0++] = lc[(size_t)r * I.sl + k];
    }
    h->japc[r] = (int)ju0;
    const long long ilen = I.lfil > 0 ? nu[r] + 1 : 0;
    if (ilen + ju0 + 1 > h->ilut_iwk) return fail(h, GBIMS_ERR_ARG, "ILUT: U storage exceeded (ilut ierr -3)");
    for (int k = 0; k < nu[r]; ++k) h->japc[ju0++] = uc[(size_t)r * I.su + k];
    h->iapc[r + 1] = (int)ju0;
  }
  h->njapc = (int)ju0;
  GB_CUDA(h, cudaMemcpyAsync(h->d_iapc, h->iapc.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
  GB_CUDA(h, cudaMemcpyAsync(h->d_japc, h->japc.data(), sizeof(int) * h->njapc, cudaMemcpyHostToDevice, st));
  launch_ilut_scatter(I, h->d_iapc, h->d_japc, h->d_apc, st);
  h->launches += 1;
  levels_build_host(n, h->iapc, h->japc, true, h->F);
  levels_build_host(n, h->iapc, h->japc, false, h->B);
  drop_graph(h);  // the sweeps' level schedule is part of the captured loop
  GB_CUDA(h, cudaStreamSynchronize(st));
  return icount;
}

// Preconditioner update from h->d_amat: ims_base_pcu with its retry loop
// (ImsLinearBase.f90:761-864).  Returns the retry count or a negative status.
static int factor_core(gbims_handle *h) {
  const int n = h->n;
  cudaStream_t st = h->st;
  if (h->dia_spmv) launch_dia7_vfill(h->D, h->d_ia, h->d_amat, st);
  else launch_sell_fill(h->S, h->d_amat, st);
  h->launches += 1;
  if (h->ipc >= 3) {
    int icount = ilut_factor_core(h);
    if (icount < 0) return icount;
    if (h->mixed) {
      kr_f64_to_f32(h->njapc, h->d_apc, h->d_apc32, st);
      h->launches += 1;
    }
    GB_CUDA(h, cudaGetLastError());
    h->factored = true;
    return icount;
  }
  int ipcflag = 0, icount = 0;
  double delta = 0.0;
  for (;;) {
    Ctl init;
    memset(&init, 0, sizeof(init));
    init.pivot_fail = INT_MAX;
    *h->h_ctl = init;
    GB_CUDA(h, cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
    launch_ilu_factor(n, h->d_ia, h->d_ja, h->d_amat, h->d_iapc, h->d_japc, h->d_apc, h->F,
                      h->s.relax, delta, ipcflag, h->d_ctl, st);
    h->launches += h->F.nlev;
    GB_CUDA(h, cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    GB_CUDA(h, cudaStreamSynchronize(st));
    GB_CUDA(h, cudaGetLastError());
    ipcflag = (h->h_ctl->pivot_fail != INT_MAX) ? 1 : 0;
    if (ipcflag < 1) break;
    delta = 1.5 * delta + 1.0e-3;
    ipcflag = 0;
    if (delta > 0.5) {
      delta = 0.5;
      ipcflag = 2;
    }
    icount += 1;
    if (icount > 10) break;
  }
  if (h->mixed) kr_f64_to_f32(h->nja, h->d_apc, h->d_apc32, st);
  if (h->structured) {
    const int was = h->D.ext;
    if (launch_dia7_extract(h->D, n, h->d_iapc, h->d_japc, h->d_apc, h->mixed, st) < 0)
      return fail(h, GBIMS_ERR_CUDA, "wavefront tile extraction failed");
    // the captured inner loop holds the sweep kernels of the arithmetic
    if (h->D.ext != was) drop_graph(h);
    // the range check, and the seven in-place df64 conversions
    h->launches += ((!h->mixed && h->D.ext_allowed) ? 1 : 0) + (h->D.ext ? 7 : 0);
  }
  h->launches += (h->mixed ? 1 : 0) + (h->structured ? 1 : 0);
  GB_CUDA(h, cudaGetLastError());
  h->factored = true;
  return icount;
}

static int apply_core(gbims_handle *h, int kstp, int kiter, int *icnvg, int *in_iter,
                      gbims_summary *summary) {
  if (int rc = ensure_level_words(h)) return rc;
  const int n = h->n;
  cudaStream_t st = h->st;
  (void)kiter;
  GB_CUDA(h, cudaEventRecord(h->ev0, st));
  // SCALE PROBLEM (ImsLinear.f90:644-650), in the model's numbering
  if (h->s.iscl != 0)
    h->launches += launch_scale(h->s.iscl, n, h->reorder ? h->d_ia_u : h->d_ia,
                                h->reorder ? h->d_ja_u : h->d_ja, h->d_cptr, h->d_cpos,
                                in_amat(h), in_x(h), in_rhs(h), h->d_dscale, h->d_dscale2, st);
  // PERMUTE (:652-666); BiCGSTAB reads DSCALE in the model's numbering at
  // the permuted row index, as the reference does
  if (h->reorder) permute_in(h);
  int icount = factor_core(h);
  if (icount < 0) return icount;
  // control block
  Ctl c;
  memset(&c, 0, sizeof(c));
  c.itmax = h->s.iter1;
  c.icnvgopt = h->s.icnvgopt;
  c.north = h->mixed ? 0 : h->s.north;
  c.iscl = h->s.iscl;
  c.dvclose = h->s.dvclose;
  c.rclose = h->s.rclose;
  c.epfact = epfact_of(h->s.icnvgopt, kstp);
  c.iter = 1;
  c.first = 1;
  c.pivot_fail = INT_MAX;
  if (h->rec_cap > 0 && !h->mixed && h->nm == 0) {
    c.rec = h->d_rec;
    c.rec_part = h->d_rec_part;
    c.rec_loc = h->d_rec_loc;
    c.rec_cap = h->rec_cap;
    c.rec_nmod = h->rec_nmod;
    c.rec_G = h->rec_G;
  }
  *h->h_ctl = c;
  GB_CUDA(h, cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
  // D, P, Q, Z = 0 ; D = B - A X ; L2NORM0 (ImsLinear.f90:686-703)
  int eg = std::min(4 * kNumSM, (n + 255) / 256);
  k_zero_vec<<<eg, 256, 0, st>>>(n, h->v_p, h->v_q, h->v_z, nullptr);
  residual64(h, nullptr, 0);
  kr_sumsq64(n, h->v_d, h->d_part, h->G, st);
  kr_ctl_set_l2norm0(h->d_ctl, h->d_part, h->G, st);
  if (h->bcgs && !h->mixed) GB_CUDA(h, cudaMemcpyAsync(h->v_dhat, h->v_d, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  if (h->mixed) {
    kr_f64_to_f32(n, h->v_d, h->f_d, st);
    GB_CUDA(h, cudaMemsetAsync(h->f_p, 0, sizeof(float) * n, st));
    if (h->bcgs) {
      GB_CUDA(h, cudaMemcpyAsync(h->f_dhat, h->f_d, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
      GB_CUDA(h, cudaMemsetAsync(h->f_v, 0, sizeof(float) * n, st));
    }
  }
  GB_CUDA(h, cudaGetLastError());
  // inner loop
  if (!h->graph_tried) build_graph(h);
  if (h->graph_ok) {
    GB_CUDA(h, cudaGraphLaunch(h->exec, st));
  } else {
    // fallback: host-driven loop in growing batches of iterations
    int batch = 1, total = 0;
    for (;;) {
      for (int b = 0; b < batch; ++b) enqueue_iteration(h, 0ULL, 0);
      total += batch;
      GB_CUDA(h, cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
      GB_CUDA(h, cudaStreamSynchronize(st));
      if (h->h_ctl->done || total > 4 * (h->s.iter1 + 2)) break;
      batch = std::min(batch * 2, 32);
    }
  }
  // the L2 norm of the final residual when the loop's updates did not take it
  // (infinity-norm closure tests): for the summary
  const bool l2_after = !h->mixed && h->nm == 0 && h->s.icnvgopt < 2;
  if (l2_after) {
    kr_sumsq64(n, h->v_d, h->d_part, h->G, st);
    kr_ctl_set_l2norm(h->d_ctl, h->d_part, h->G, st);
  }
  // BACK PERMUTE the solution (ImsLinear.f90:730-737: dvperm with IORDER,
  // x[j] = x0[LORDER(j)]); amat and rhs are the handle's own copies and are
  // refilled by the next apply
  if (h->reorder) gather(h, n, h->d_lorder, h->d_x, h->u_x);
  // UNSCALE the solution (ImsLinear.f90:739-745)
  if (h->s.iscl != 0) {
    launch_unscale_x(n, in_x(h), h->d_dscale2, st);
    h->launches += 1;
  }
  GB_CUDA(h, cudaEventRecord(h->ev1, st));
  GB_CUDA(h, cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
  GB_CUDA(h, cudaStreamSynchronize(st));
  GB_CUDA(h, cudaGetLastError());
  const Ctl &r = *h->h_ctl;
  // zero, residual, sum of squares, L2NORM0 control (+ FP32 copy), then the loop bodies
  h->launches += 4 + (h->mixed ? 1 : 0) + (l2_after ? 2 : 0) + (long long)h->body_kernels * r.bodies;
  int iters = (r.l2norm0 == 0.0 || h->s.iter1 <= 0) ? 0 : r.iter;
  *icnvg = r.icnvg;
  *in_iter = iters;
  if (summary) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    summary->iter_cnt = iters;
    summary->icnvg = r.icnvg;
    summary->pivot_retries = icount;
    summary->exit_reason = r.exit_reason;
    summary->dvmax = r.deltax;
    summary->locdv = (int)r.xloc;
    summary->rmax = r.rmax;
    summary->locr = (int)r.rloc;
    summary->l2norm0 = r.l2norm0;
    summary->l2norm = r.l2norm;
    summary->solve_ms = ms;
    summary->refinements = (int)r.scratch[3];
    summary->structured = h->structured ? 1 : 0;
  }
  if (r.nonfinite) return fail(h, GBIMS_ERR_NONFINITE, "non-finite values in the residual or head change");
  if (r.guard_tripped) return fail(h, GBIMS_ERR_STATE, "inner loop cut by the body limit");
  if (h->structured) {
    int derr = 0;
    GB_CUDA(h, cudaMemcpy(&derr, h->D.d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (derr) return fail(h, GBIMS_ERR_CUDA, "structured sweep wait limit reached");
  }
  if (int rc = level_words_error(h)) return rc;
  return icount > 0 ? GBIMS_WARN_PIVOT : GBIMS_OK;
}

extern "C" int gbims_apply(gbims_handle *h, double *amat, double *rhs, double *x, int kstp,
                           int kiter, int *icnvg, int *in_iter, gbims_summary *summary) {
  if (!h || !amat || !rhs || !x || !icnvg || !in_iter) return GBIMS_ERR_ARG;
  if (!h->d_ctl) return fail(h, GBIMS_ERR_STATE, "handle was not created successfully");
  if (h->nm > 0) return fail(h, GBIMS_ERR_STATE, "batch handle: use gbims_batch_apply");
  GB_CUDA(h, cudaMemcpyAsync(in_amat(h), amat, sizeof(double) * h->nja, cudaMemcpyHostToDevice, h->st));
  GB_CUDA(h, cudaMemcpyAsync(in_rhs(h), rhs, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  GB_CUDA(h, cudaMemcpyAsync(in_x(h), x, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  int rc = apply_core(h, kstp, kiter, icnvg, in_iter, summary);
  if (rc < 0 && rc != GBIMS_ERR_NONFINITE) return rc;
  cudaError_t e = cudaMemcpy(x, in_x(h), sizeof(double) * h->n, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(h, GBIMS_ERR_CUDA, cudaGetErrorString(e));
  return rc;
}

extern "C" int gbims_apply_device(gbims_handle *h, double *d_amat, double *d_rhs, double *d_x,
                                  int kstp, int kiter, int *icnvg, int *in_iter,
                                  gbims_summary *summary) {
  if (!h || !d_amat || !d_rhs || !d_x || !icnvg || !in_iter) return GBIMS_ERR_ARG;
  if (!h->d_ctl) return fail(h, GBIMS_ERR_STATE, "handle was not created successfully");
  if (h->nm > 0) return fail(h, GBIMS_ERR_STATE, "batch handle: use gbims_batch_apply_device");
  GB_CUDA(h, cudaMemcpyAsync(in_amat(h), d_amat, sizeof(double) * h->nja, cudaMemcpyDeviceToDevice, h->st));
  GB_CUDA(h, cudaMemcpyAsync(in_rhs(h), d_rhs, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st));
  GB_CUDA(h, cudaMemcpyAsync(in_x(h), d_x, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st));
  int rc = apply_core(h, kstp, kiter, icnvg, in_iter, summary);
  if (rc < 0 && rc != GBIMS_ERR_NONFINITE) return rc;
  cudaError_t e = cudaMemcpyAsync(d_x, in_x(h), sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) return fail(h, GBIMS_ERR_CUDA, cudaGetErrorString(e));
  return rc;
}

extern "C" int gbims_factor(gbims_handle *h, const double *amat, int *pivot_retries) {
  if (!h || !amat) return GBIMS_ERR_ARG;
  if (!h->d_ctl) return fail(h, GBIMS_ERR_STATE, "handle was not created successfully");
  GB_CUDA(h, cudaMemcpyAsync(in_amat(h), amat, sizeof(double) * h->nja, cudaMemcpyHostToDevice, h->st));
  if (h->reorder) gather(h, h->nja, h->d_asrc, h->u_amat, h->d_amat);  // factor the permuted matrix
  int icount = factor_core(h);
  if (icount < 0) return icount;
  GB_CUDA(h, cudaStreamSynchronize(h->st));
  if (pivot_retries) *pivot_retries = icount;
  return icount > 0 ? GBIMS_WARN_PIVOT : GBIMS_OK;
}

extern "C" int gbims_get_apc(gbims_handle *h, double *apc) {
  if (!h || !apc) return GBIMS_ERR_ARG;
  if (!h->factored) return fail(h, GBIMS_ERR_STATE, "no factor: call gbims_factor or gbims_apply first");
  GB_CUDA(h, cudaStreamSynchronize(h->st));
  if (h->ipc >= 3) return fail(h, GBIMS_ERR_STATE, "ILUT: the factor's pattern varies; use gbims_get_factor");
  GB_CUDA(h, cudaMemcpy(apc, h->d_apc, sizeof(double) * h->nja, cudaMemcpyDeviceToHost));
  return GBIMS_OK;
}

extern "C" int gbims_calc_order(int iord, int neq, int nja, const int *ia, const int *ja,
                                int index_base, int *lorder, int *iorder) {
  if (neq <= 0 || nja < neq || !ia || !ja || !lorder || !iorder) return GBIMS_ERR_ARG;
  if (iord != 1 && iord != 2) return GBIMS_ERR_ARG;
  if (index_base != 0 && index_base != 1) return GBIMS_ERR_ARG;
  const int base = index_base;
  std::vector<int> a(neq + 1), c(nja), lo;
  for (int i = 0; i <= neq; ++i) a[i] = ia[i] - base;
  if (a[0] != 0 || a[neq] != nja) return GBIMS_ERR_ARG;
  for (int r = 0; r < neq; ++r)
    if (a[r + 1] < a[r]) return GBIMS_ERR_ARG;
  for (int k = 0; k < nja; ++k) {
    c[k] = ja[k] - base;
    if (c[k] < 0 || c[k] >= neq) return GBIMS_ERR_ARG;
  }
  if (iord == 1) rcm_order(neq, a, c, lo);
  else if (md_order(neq, a, c, lo) != 0) return GBIMS_ERR_ARG;
  for (int i = 0; i < neq; ++i) {
    lorder[i] = lo[i] + base;
    iorder[lo[i]] = i + base;
  }
  return GBIMS_OK;
}

extern "C" int gbims_get_factor(gbims_handle *h, int *iapc, int *japc, double *apc,
                                int capacity, int *njapc) {
  if (!h || !njapc) return GBIMS_ERR_ARG;
  if (!h->factored) return fail(h, GBIMS_ERR_STATE, "no factor: call gbims_factor or gbims_apply first");
  *njapc = h->njapc;
  if (!iapc || !japc || !apc) return GBIMS_OK;  // size query
  if (capacity < h->njapc) return fail(h, GBIMS_ERR_ARG, "capacity below the factor's storage");
  GB_CUDA(h, cudaStreamSynchronize(h->st));
  GB_CUDA(h, cudaMemcpy(iapc, h->d_iapc, sizeof(int) * (h->n + 1), cudaMemcpyDeviceToHost));
  GB_CUDA(h, cudaMemcpy(japc, h->d_japc, sizeof(int) * h->njapc, cudaMemcpyDeviceToHost));
  GB_CUDA(h, cudaMemcpy(apc, h->d_apc, sizeof(double) * h->njapc, cudaMemcpyDeviceToHost));
  return GBIMS_OK;
}

extern "C" int gbims_matvec(gbims_handle *h, const double *x, double *y) {
  if (!h || !x || !y) return GBIMS_ERR_ARG;
  if (!h->factored) return fail(h, GBIMS_ERR_STATE, "no matrix: call gbims_factor or gbims_apply first");
  GB_CUDA(h, cudaMemcpyAsync(h->v_d, x, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  spmv64(h, h->v_d, h->d_rhs, nullptr);
  GB_CUDA(h, cudaGetLastError());
  GB_CUDA(h, cudaMemcpyAsync(y, h->d_rhs, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->st));
  GB_CUDA(h, cudaStreamSynchronize(h->st));
  return GBIMS_OK;
}

extern "C" int gbims_precondition(gbims_handle *h, const double *r, double *z) {
  if (!h || !r || !z) return GBIMS_ERR_ARG;
  if (int rc = ensure_level_words(h)) return rc;
  if (!h->factored) return fail(h, GBIMS_ERR_STATE, "no factor: call gbims_factor or gbims_apply first");
  GB_CUDA(h, cudaMemcpyAsync(h->v_d, r, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  // a control block with done = 0 lets the gated sweep kernels run
  Ctl c;
  memset(&c, 0, sizeof(c));
  c.pivot_fail = INT_MAX;
  *h->h_ctl = c;
  GB_CUDA(h, cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->st));
  if (!h->mixed) {
    precond64(h, h->v_d, h->d_rhs);
  } else {
    kr_f64_to_f32(h->n, h->v_d, h->f_d, h->st);
    precond32(h, h->f_d, h->f_z);
    kr_f32_to_f64(h->n, h->f_z, h->d_rhs, h->st);
  }
  GB_CUDA(h, cudaGetLastError());
  GB_CUDA(h, cudaMemcpyAsync(z, h->d_rhs, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->st));
  GB_CUDA(h, cudaStreamSynchronize(h->st));
  return GBIMS_OK;
}

// The inner-loop graph holds launch parameters (reduction blocks, sweep
// tiling): after a change it is captured again at the next apply.
static void drop_graph(gbims_handle *h) {
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  h->exec = nullptr;
  h->graph = nullptr;
  h->graph_ok = false;
  h->graph_tried = h->no_graph;
}

// Times the wavefront tilings and the reduction grid on the handle's own
// (factored) system and keeps the fastest.  Neither choice changes the
// arithmetic of a cell: the sweeps compute every cell in the same order
// whatever the tiling; the reduction grid changes only the order in which
// dot-product partials are summed.
extern "C" int gbims_autotune(gbims_handle *h, int reps, gbims_tuning *out) {
  if (!h || !out || reps <= 0) return GBIMS_ERR_ARG;
  if (int rc = ensure_level_words(h)) return rc;
  if (!h->factored) return fail(h, GBIMS_ERR_STATE, "no factor: call gbims_factor or an apply first");
  memset(out, 0, sizeof(*out));
  out->sweep_config = -1;
  const int n = h->n;
  cudaStream_t st = h->st;
  // control blocks that let every kernel run (batch members included)
  Ctl c;
  memset(&c, 0, sizeof(c));
  c.pivot_fail = INT_MAX;
  c.alpha = 1.0e-30;  // keeps x unchanged to rounding in the update timing
  *h->h_ctl = c;
  GB_CUDA(h, cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
  if (h->nm > 0) GB_CUDA(h, cudaMemsetAsync(h->d_ctls, 0, sizeof(Ctl) * h->nm, st));
  const int eg = std::min(4 * kNumSM, (n + 255) / 256);
  if (!h->mixed) {
    k_zero_vec<<<eg, 256, 0, st>>>(n, h->v_p, h->v_q, h->v_z, nullptr);
    GB_CUDA(h, cudaMemcpyAsync(h->v_p, h->d_x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  } else {
    kr_f64_to_f32(n, h->d_x, h->f_p, st);
    GB_CUDA(h, cudaMemsetAsync(h->f_q, 0, sizeof(float) * n, st));
    GB_CUDA(h, cudaMemsetAsync(h->f_d, 0, sizeof(float) * n, st));
  }
  auto time_it = [&](auto &&fn) -> double {
    fn();
    cudaEventRecord(h->ev0, st);
    for (int r = 0; r < reps; ++r) fn();
    cudaEventRecord(h->ev1, st);
    cudaEventSynchronize(h->ev1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    return ms / reps;
  };
  if (h->structured) {
    // each tiling timed on each sweep alone (the backward sweep reads the
    // forward words of the last forward launch), the fastest kept for each
    const int nc = std::min(dia7_num_cfgs(), (int)(sizeof(out->candidate_ms) / sizeof(double)));
    int best = 0, best_b = 0;
    double bt = 1e300, btf = 1e300, btb = 1e300;
    auto pre = [&] {
      if (!h->mixed) precond64(h, h->v_p, h->v_z);
      else precond32(h, h->f_p, h->f_z);
    };
    h->D.cfg_b = -1;
    for (int i = 0; i < nc; ++i) {
      h->D.cfg = i;
      h->D.only = 1;
      const double tf = time_it(pre);
      h->D.only = -1;
      const double tb = time_it(pre);
      h->D.only = 0;
      out->candidate_ms[i] = tf + tb;
      if (tf + tb < bt) bt = tf + tb;
      if (tf < btf) {
        btf = tf;
        best = i;
      }
      if (tb < btb) {
        btb = tb;
        best_b = i;
      }
    }
    h->D.cfg = best;
    h->D.cfg_b = best_b;
    bt = time_it(pre);
    int err = 0;
    GB_CUDA(h, cudaMemcpy(&err, h->D.d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
      cudaMemset(h->D.d_err, 0, sizeof(int));
      return fail(h, GBIMS_ERR_CUDA, "structured sweep wait limit reached while tuning");
    }
    out->ncandidates = nc;
    out->sweep_config = best;
    out->sweep_config_backward = best_b;
    dia7_cfg(best, &out->sweep_chunk, &out->sweep_ring, &out->sweep_prefetch, &out->sweep_occupancy);
    out->precond_ms = bt;
  }
  out->level_mode = -1;
  if (!h->structured) {
    // level-scheduled sweeps: one launch per level, or one sync-free launch
    // per sweep (the sync-free form also with 1 to 16 threads per row of
    // the widest level, as far as the resident grid goes; level_ms[1] is its
    // best, candidate_ms[0..4] its time at each)
    double bt = 1e300;
    int best = 1, best_mult = 1;
    auto pre = [&] {
      if (!h->mixed) precond64(h, h->v_p, h->v_z);
      else precond32(h, h->f_p, h->f_z);
    };
    h->LW.mode = 0;
    out->level_ms[0] = time_it(pre);
    bt = out->level_ms[0];
    best = 0;
    out->level_ms[1] = 1e300;
    for (int mult : {1, 2, 4, 8, 16}) {
      h->LW.mode = 1;
      h->LW.sf_mult = mult;
      const double ms = time_it(pre);
      out->candidate_ms[out->ncandidates++] = ms;
      out->level_ms[1] = std::min(out->level_ms[1], ms);
      if (ms < bt) {
        bt = ms;
        best = 1;
        best_mult = mult;
      }
    }
    if (int rc = level_words_error(h)) return rc;
    h->LW.mode = best;
    h->LW.sf_mult = best_mult;
    out->level_mode = best;
    out->precond_ms = bt;
  }
  if (h->nm == 0) {
    // reduction blocks: multiples of the SM count up to the allocated grid
    int best = h->G;
    double bt = 1e300;
    std::vector<int> cand;
    for (int g = kNumSM; g < h->G_alloc; g *= 2) cand.push_back(g);
    cand.push_back(h->G_alloc);
    for (int g : cand) {
      const double ms = time_it([&] {
        if (!h->mixed) {
          kr_dot64(n, h->v_p, h->v_q, h->d_part, g, h->d_ctl, st);
          kr_cg_update64(n, h->v_z, h->v_d, h->v_p, h->v_q, h->d_part, g, h->d_ctl, st, h->s.icnvgopt >= 2);
        } else {
          kr_dot32(n, h->f_p, h->f_q, h->d_part, g, h->d_ctl, st);
          kr_cg_update_mixed(n, h->v_d, h->f_d, h->f_p, h->f_q, h->d_part, g, h->d_ctl, st);
        }
      });
      if (ms < bt) {
        bt = ms;
        best = g;
      }
    }
    h->G = best;
    out->reduction_blocks = best;
    out->vector_ms = bt;
  }
  GB_CUDA(h, cudaGetLastError());
  drop_graph(h);
  return GBIMS_OK;
}

extern "C" int gbims_set_dis_nodes(gbims_handle *h, const int *nodeuser) {
  if (!h || !nodeuser) return GBIMS_ERR_ARG;
  if (h->structured) return fail(h, GBIMS_ERR_ARG, "the handle already has the wavefront sweeps");
  if (h->factored) return fail(h, GBIMS_ERR_ARG, "set the DIS node map before the first factorisation");
  if (h->nm > 0 || h->reorder || h->ipc >= 3)
    return fail(h, GBIMS_ERR_UNSUPPORTED,
                "a node map needs a single model, no reordering and ILU0/MILU0");
  const int dl = h->s.nlay, dr = h->s.nrow, dc = h->s.ncol;
  if (dl <= 0 || dr <= 0 || dc <= 0)
    return fail(h, GBIMS_ERR_ARG, "a node map needs the grid shape (settings nlay, nrow, ncol)");
  const int n = h->n;
  const int base = h->s.index_base;
  std::vector<int> nu(n);
  for (int r = 0; r < n; ++r) nu[r] = nodeuser[r] - base;
  if (!dia7_matches_reduced(dl, dr, dc, n, h->ia, h->ja, nu.data()))
    return fail(h, GBIMS_ERR_ARG, "the pattern is not the DIS grid reduced by the node map");
  std::vector<int> shape = {dl, dr, dc};
  if (int rc = setup_structured(h, shape, std::vector<long long>{0})) return rc;
  const long long nuser = (long long)dl * dr * dc;
  std::vector<int> ur((size_t)nuser, -1);
  for (int r = 0; r < n; ++r) ur[(size_t)nu[r]] = r;
  Dia7 &D = h->D;
  D.nuser = nuser;
  GB_CUDA(h, dalloc(&D.d_nodeuser, (size_t)n));
  GB_CUDA(h, dalloc(&D.d_userred, (size_t)nuser));
  GB_CUDA(h, cudaMemcpy(D.d_nodeuser, nu.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  GB_CUDA(h, cudaMemcpy(D.d_userred, ur.data(), sizeof(int) * nuser, cudaMemcpyHostToDevice));
  // full-grid vectors, with the sweeps' slack after the last cell
  if (!h->mixed) {
    GB_CUDA(h, dalloc(&D.d_rfull, (size_t)nuser + kVecPad));
    GB_CUDA(h, dalloc(&D.d_zfull, (size_t)nuser + kVecPad));
    GB_CUDA(h, cudaMemset(D.d_rfull, 0, sizeof(double) * ((size_t)nuser + kVecPad)));
  } else {
    GB_CUDA(h, dalloc(&D.f_rfull, (size_t)nuser + kVecPad));
    GB_CUDA(h, dalloc(&D.f_zfull, (size_t)nuser + kVecPad));
    GB_CUDA(h, cudaMemset(D.f_rfull, 0, sizeof(float) * ((size_t)nuser + kVecPad)));
  }
  D.mapped = true;
  drop_graph(h);
  return GBIMS_OK;
}

extern "C" int gbims_set_tuning(gbims_handle *h, int sweep_config, int reduction_blocks,
                                int level_mode) {
  if (!h) return GBIMS_ERR_ARG;
  if (level_mode >= 0) {
    if (h->structured || level_mode > 1)
      return fail(h, GBIMS_ERR_ARG, "level mode out of range (or a structured handle)");
    h->LW.mode = level_mode;
  }
  if (sweep_config >= 0) {
    if (!h->structured || sweep_config >= dia7_num_cfgs())
      return fail(h, GBIMS_ERR_ARG, "sweep configuration out of range (or not a structured handle)");
    h->D.cfg = sweep_config;
    h->D.cfg_b = -1;
  }
  if (reduction_blocks > 0) {
    if (h->nm > 0 || reduction_blocks > h->G_alloc)
      return fail(h, GBIMS_ERR_ARG, "reduction blocks out of range (or a batch handle)");
    h->G = reduction_blocks;
  }
  drop_graph(h);
  return GBIMS_OK;
}

extern "C" int gbims_time_kernels(gbims_handle *h, int reps, gbims_kernel_times *t) {
  if (!h || !t || reps <= 0) return GBIMS_ERR_ARG;
  if (int rc = ensure_level_words(h)) return rc;
  if (!h->factored) return fail(h, GBIMS_ERR_STATE, "no factor: call gbims_factor or gbims_apply first");
  const int n = h->n;
  cudaStream_t st = h->st;
  Ctl c;
  memset(&c, 0, sizeof(c));
  c.pivot_fail = INT_MAX;
  c.alpha = 1.0e-30;  // keeps x unchanged to rounding in the update timing
  *h->h_ctl = c;
  GB_CUDA(h, cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
  int eg = std::min(4 * kNumSM, (n + 255) / 256);
  // deterministic, finite operands
  if (!h->mixed) {
    k_zero_vec<<<eg, 256, 0, st>>>(n, h->v_p, h->v_q, h->v_z, nullptr);
    GB_CUDA(h, cudaMemcpyAsync(h->v_p, h->d_x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  } else {
    kr_f64_to_f32(n, h->d_x, h->f_p, st);
    GB_CUDA(h, cudaMemsetAsync(h->f_q, 0, sizeof(float) * n, st));
    GB_CUDA(h, cudaMemsetAsync(h->f_d, 0, sizeof(float) * n, st));
  }
  auto time_it = [&](auto &&fn) -> double {
    fn();
    cudaEventRecord(h->ev0, st);
    for (int r = 0; r < reps; ++r) fn();
    cudaEventRecord(h->ev1, st);
    cudaEventSynchronize(h->ev1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    return ms / reps;
  };
  if (!h->mixed) {
    t->spmv_ms = time_it([&] { spmv64(h, h->v_p, h->v_q, h->d_ctl); });
    t->precond_ms = time_it([&] { precond64(h, h->v_p, h->v_z); });
    t->dot_ms = time_it([&] { kr_dot64(n, h->v_p, h->v_q, h->d_part, h->G, h->d_ctl, st); });
    t->update_ms = time_it([&] { kr_cg_update64(n, h->v_z, h->v_d, h->v_p, h->v_q, h->d_part, h->G, h->d_ctl, st, h->s.icnvgopt >= 2); });
  } else {
    t->spmv_ms = time_it([&] { spmv32(h, h->f_p, h->f_q, h->d_ctl); });
    t->precond_ms = time_it([&] { precond32(h, h->f_p, h->f_z); });
    t->dot_ms = time_it([&] { kr_dot32(n, h->f_p, h->f_q, h->d_part, h->G, h->d_ctl, st); });
    t->update_ms = time_it([&] { kr_cg_update_mixed(n, h->v_d, h->f_d, h->f_p, h->f_q, h->d_part, h->G, h->d_ctl, st); });
  }
  GB_CUDA(h, cudaGetLastError());
  // algorithmic bytes: CSR values + column indices + row pointers, x read
  // once, y written once (the index-free product of a full DIS grid: values,
  // x and y only); preconditioner: every factor value once, r read
  // and z written once, plus JAPC/IAPC for the unstructured sweeps (the
  // structured sweeps need no indices).  The forward result kept between
  // the two sweeps is not counted.
  double vb = h->mixed ? 4.0 : 8.0;
  t->spmv_bytes = h->dia_spmv ? vb * h->nja + 2.0 * vb * n
                              : (vb + 4.0) * h->nja + 4.0 * (n + 1) + 2.0 * vb * n;
  t->precond_bytes = vb * h->njapc + 2.0 * vb * n;
  if (!h->structured) t->precond_bytes += 4.0 * h->njapc + 4.0 * (n + 1);
  return GBIMS_OK;
}

// ---------------------------------------------------------------------------
// per-inner-iteration records (imslinear_ap's NCONV, CONVNMOD, CONVMODSTART,
// CACCEL and the ConvergenceSummary rows, ImsLinear.f90:617-633,
// ImsLinearBase.f90:141-197 and :431-493)
// ---------------------------------------------------------------------------
extern "C" int gbims_set_inner_records(gbims_handle *h, int nconv, int convnmod,
                                       const int *convmodstart) {
  if (!h) return GBIMS_ERR_ARG;
  if (!h->d_ctl) return fail(h, GBIMS_ERR_STATE, "handle was not created successfully");
  if (nconv < 0) return fail(h, GBIMS_ERR_ARG, "nconv must be >= 0");
  if (nconv > 0 && (h->mixed || h->nm > 0))
    return fail(h, GBIMS_ERR_UNSUPPORTED, "inner records: single FP64 systems only");
  std::vector<int> ms;
  if (nconv > 0) {
    if (convnmod < 1 || !convmodstart) return fail(h, GBIMS_ERR_ARG, "convnmod >= 1 and convmodstart are required");
    const int base = h->s.index_base;
    ms.resize(convnmod + 1);
    for (int m = 0; m <= convnmod; ++m) ms[m] = convmodstart[m] - base;
    if (ms[0] != 0 || ms[convnmod] != h->n)
      return fail(h, GBIMS_ERR_ARG, "convmodstart must run from index_base to neq+index_base");
    for (int m = 0; m < convnmod; ++m)
      if (ms[m + 1] <= ms[m]) return fail(h, GBIMS_ERR_ARG, "convmodstart must increase");
  }
  GB_CUDA(h, cudaStreamSynchronize(h->st));
  for (void *p : {(void *)h->d_modstart, (void *)h->d_rec, (void *)h->d_rec_part, (void *)h->d_rec_loc})
    if (p) cudaFree(p);
  h->d_modstart = nullptr;
  h->d_rec = h->d_rec_part = nullptr;
  h->d_rec_loc = nullptr;
  h->rec_cap = h->rec_nmod = h->rec_G = 0;
  drop_graph(h);  // the loop body gains or loses the record kernel
  if (nconv == 0) return GBIMS_OK;
  h->rec_nmod = convnmod;
  h->rec_G = std::max(1, std::min(h->G, (h->n + kRedBlock - 1) / kRedBlock));
  GB_CUDA(h, dalloc(&h->d_modstart, (size_t)convnmod + 1));
  GB_CUDA(h, dalloc(&h->d_rec, (size_t)nconv * (3 + 4 * convnmod)));
  GB_CUDA(h, dalloc(&h->d_rec_part, (size_t)4 * convnmod * h->rec_G));
  GB_CUDA(h, dalloc(&h->d_rec_loc, (size_t)2 * convnmod));
  GB_CUDA(h, cudaMemcpy(h->d_modstart, ms.data(), sizeof(int) * (convnmod + 1), cudaMemcpyHostToDevice));
  std::vector<long long> none(2 * convnmod, -1);
  GB_CUDA(h, cudaMemcpy(h->d_rec_loc, none.data(), sizeof(long long) * 2 * convnmod, cudaMemcpyHostToDevice));
  h->rec_cap = nconv;
  return GBIMS_OK;
}

extern "C" int gbims_get_inner_records(gbims_handle *h, int cap, int *nrec, int *itinner,
                                       double *alpha, double *omega, int *locdv, double *dvmax,
                                       int *locr, double *rmax) {
  if (!h || !nrec || cap < 0) return GBIMS_ERR_ARG;
  *nrec = 0;
  if (h->rec_cap == 0 || !h->h_ctl) return GBIMS_OK;
  const int nm = h->rec_nmod, stride = 3 + 4 * nm;
  const int have = std::min(h->h_ctl->rec_count, h->rec_cap);
  const int k = std::min(have, cap);
  if (k > 0 && (!itinner || !alpha || !omega || !locdv || !dvmax || !locr || !rmax))
    return fail(h, GBIMS_ERR_ARG, "record arrays are required");
  std::vector<double> buf((size_t)k * stride);
  if (k > 0)
    GB_CUDA(h, cudaMemcpy(buf.data(), h->d_rec, sizeof(double) * buf.size(), cudaMemcpyDeviceToHost));
  const int base = h->s.index_base;
  for (int r = 0; r < k; ++r) {
    const double *row = &buf[(size_t)r * stride];
    itinner[r] = (int)row[0];
    alpha[r] = row[1];
    omega[r] = row[2];
    for (int im = 0; im < nm; ++im) {
      dvmax[r * nm + im] = row[3 + 4 * im];
      locdv[r * nm + im] = (int)row[4 + 4 * im] + base;
      rmax[r * nm + im] = row[5 + 4 * im];
      locr[r * nm + im] = (int)row[6 + 4 * im] + base;
    }
  }
  *nrec = k;
  return GBIMS_OK;
}

extern "C" int gbims_destroy(gbims_handle *h) {
  if (!h) return GBIMS_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  void *ptrs[] = {h->d_ia, h->d_ja, h->d_iapc, h->d_japc, h->d_apc, h->d_apc32, h->S.d_ptr,
                  h->S.d_col, h->S.d_src, h->S.d_val, h->S.d_val32, h->F.d_rows, h->B.d_rows,
                  h->D.d_lz, h->D.d_ly, h->D.d_lx, h->D.d_ux, h->D.d_uy, h->D.d_uz, h->D.d_dinv,
                  h->D.f_lz, h->D.f_ly, h->D.f_lx, h->D.f_ux, h->D.f_uy, h->D.f_uz, h->D.f_dinv,
                  h->D.ll_y, h->D.ll_z,
                  h->D.d_flags, h->D.d_err, h->d_amat, h->d_rhs, h->d_x, h->v_d, h->v_p, h->v_q,
                  h->v_z, h->v_t, h->v_v, h->v_dhat, h->v_phat, h->v_qhat, h->f_d, h->f_p,
                  h->f_q, h->f_z, h->f_t, h->f_v, h->f_dhat, h->f_phat, h->f_qhat, h->d_part,
                  h->d_dscale, h->d_dscale2, h->d_cptr, h->d_cpos, h->D.d_sv, h->D.f_sv,
                  h->d_bcm, h->d_bcr, h->d_bmc, h->d_bmr, h->d_ctls, h->D.d_geo, h->S.d_slm,
                  h->LW.fwd, h->LW.bwd, h->LW.ticket, h->LW.err, h->d_ctl, h->I.lcol,
                  h->I.lval, h->I.ucol, h->I.uval, h->I.nl, h->I.nu, h->I.dinv, h->I.rdone,
                  h->I.stat, h->d_lorder, h->d_iorder, h->d_asrc, h->d_ia_u, h->d_ja_u,
                  h->u_amat, h->u_rhs, h->u_x, h->d_modstart, h->d_rec, h->d_rec_part,
                  h->d_rec_loc, h->D.d_nodeuser, h->D.d_userred, h->D.d_rfull, h->D.d_zfull,
                  h->D.f_rfull, h->D.f_zfull};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (h->h_ctl) cudaFreeHost(h->h_ctl);
  if (h->h_ilut) cudaFreeHost(h->h_ilut);
  if (h->h_ctls) cudaFreeHost(h->h_ctls);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return GBIMS_OK;
}

extern "C" long long gbims_kernel_launches(const gbims_handle *h) { return h ? h->launches : 0; }

extern "C" const char *gbims_last_error(const gbims_handle *h) {
  if (!h) return "null handle";
  return h->err.c_str();
}

extern "C" const char *gbims_status_string(int status) {
  switch (status) {
  case GBIMS_OK: return "ok";
  case GBIMS_WARN_PIVOT: return "warning: small value added to ILU0 pivots";
  case GBIMS_ERR_ARG: return "invalid argument";
  case GBIMS_ERR_CUDA: return "CUDA error";
  case GBIMS_ERR_UNSUPPORTED: return "unsupported option";
  case GBIMS_ERR_NONFINITE: return "non-finite values";
  case GBIMS_ERR_NOMEM: return "out of memory";
  case GBIMS_ERR_STATE: return "invalid handle state";
  default: return "unknown status";
  }
}

// ---------------------------------------------------------------------------
// batched ensemble
// ---------------------------------------------------------------------------
extern "C" int gbims_batch_create(const gbims_settings *settings, int nmembers,
                                  const int *member_rows, int neq, int nja, const int *ia,
                                  const int *ja, const int *shapes, gbims_handle **out) {
  if (!out) return GBIMS_ERR_ARG;
  *out = nullptr;
  if (!settings || !member_rows || nmembers <= 0 || neq <= 0) return GBIMS_ERR_ARG;
  if (settings->index_base != 0 && settings->index_base != 1) return GBIMS_ERR_ARG;
  const int base = settings->index_base;
  std::vector<int> mrow(nmembers + 1);
  for (int m = 0; m <= nmembers; ++m) mrow[m] = member_rows[m] - base;
  if (mrow[0] != 0 || mrow[nmembers] != neq) return GBIMS_ERR_ARG;
  for (int m = 0; m < nmembers; ++m)
    if (mrow[m + 1] <= mrow[m]) return GBIMS_ERR_ARG;
  gbims_settings s = *settings;
  s.nlay = -1;  // members are swept by the level schedule of the whole batch
  s.nrow = s.ncol = 0;
  int rc = gbims_create(&s, neq, nja, ia, ja, out);
  gbims_handle *h = *out;
  if (rc != GBIMS_OK) return rc;
  if (h->bcgs || s.north > 0 || (h->mixed && s.iscl != 0) || h->ipc >= 3)
    return fail(h, GBIMS_ERR_UNSUPPORTED,
                "batched ensembles: PCG with ILU0/MILU0 without NORTH (and without scaling in "
                "the mixed form)");
  // block-diagonal: every column of a member's rows lies inside the member
  for (int m = 0; m < nmembers; ++m)
    for (int r = mrow[m]; r < mrow[m + 1]; ++r)
      for (int k = h->ia[r]; k < h->ia[r + 1]; ++k)
        if (h->ja[k] < mrow[m] || h->ja[k] >= mrow[m + 1])
          return fail(h, GBIMS_ERR_ARG, "member rows couple to another member (not block-diagonal)");
  // chunks of kChunkRows rows inside each member
  std::vector<int> cm, cr, mc(nmembers + 1, 0);
  for (int m = 0; m < nmembers; ++m) {
    mc[m] = (int)cm.size();
    for (int r = mrow[m]; r < mrow[m + 1]; r += kChunkRows) {
      cm.push_back(m);
      cr.push_back(r);
    }
  }
  mc[nmembers] = (int)cm.size();
  cr.push_back(neq);
  const int nchunks = (int)cm.size();
  h->nm = nmembers;
  h->mrow = mrow;
  GB_CUDA(h, dalloc(&h->d_bcm, cm.size()));
  GB_CUDA(h, dalloc(&h->d_bcr, cr.size()));
  GB_CUDA(h, dalloc(&h->d_bmc, mc.size()));
  GB_CUDA(h, dalloc(&h->d_bmr, mrow.size()));
  GB_CUDA(h, dalloc(&h->d_ctls, (size_t)nmembers));
  GB_CUDA(h, cudaMallocHost((void **)&h->h_ctls, sizeof(Ctl) * nmembers));
  GB_CUDA(h, cudaMemcpy(h->d_bcm, cm.data(), sizeof(int) * cm.size(), cudaMemcpyHostToDevice));
  GB_CUDA(h, cudaMemcpy(h->d_bcr, cr.data(), sizeof(int) * cr.size(), cudaMemcpyHostToDevice));
  GB_CUDA(h, cudaMemcpy(h->d_bmc, mc.data(), sizeof(int) * mc.size(), cudaMemcpyHostToDevice));
  GB_CUDA(h, cudaMemcpy(h->d_bmr, mrow.data(), sizeof(int) * mrow.size(), cudaMemcpyHostToDevice));
  // partials: 8 slots per chunk
  if ((size_t)nchunks > (size_t)h->G) {
    cudaFree(h->d_part);
    h->d_part = nullptr;
    GB_CUDA(h, dalloc(&h->d_part, (size_t)nchunks * 8));
  }
  h->bd.nm = nmembers;
  h->bd.nchunks = nchunks;
  h->bd.cm = h->d_bcm;
  h->bd.cr = h->d_bcr;
  h->bd.mc = h->d_bmc;
  h->bd.mr = h->d_bmr;
  h->bd.ctls = h->d_ctls;
  // the products skip the rows of members that are done: per SELL slice its
  // member, or -1 where a member boundary falls inside the slice
  if (h->S.nslices > 0) {
    std::vector<int> slm(h->S.nslices);
    for (int sl = 0, m = 0; sl < h->S.nslices; ++sl) {
      const int r0 = sl * kSell, r1 = std::min(neq, r0 + kSell) - 1;
      while (mrow[m + 1] <= r0) ++m;
      slm[sl] = (r1 < mrow[m + 1]) ? m : -1;
    }
    GB_CUDA(h, dalloc(&h->S.d_slm, slm.size()));
    GB_CUDA(h, cudaMemcpy(h->S.d_slm, slm.data(), sizeof(int) * slm.size(), cudaMemcpyHostToDevice));
    h->S.d_mrow = h->d_bmr;
    h->S.nm = nmembers;
    h->S.mctl = h->d_ctls;
  }
  // full DIS grids: the wavefront sweeps run every member's layers and
  // blocks as the CTAs of one launch
  if (shapes) {
    std::vector<int> sh(shapes, shapes + 3 * nmembers);
    std::vector<long long> row0(nmembers);
    std::vector<int> lia, lja;
    for (int m = 0; m < nmembers; ++m) {
      const int r0 = mrow[m], nr = mrow[m + 1] - mrow[m];
      lia.assign(nr + 1, 0);
      lja.clear();
      for (int r = 0; r < nr; ++r) {
        for (int k = h->ia[r0 + r]; k < h->ia[r0 + r + 1]; ++k) lja.push_back(h->ja[k] - r0);
        lia[r + 1] = (int)lja.size();
      }
      if (sh[3 * m] <= 0 || sh[3 * m + 1] <= 0 || sh[3 * m + 2] <= 0 ||
          !dia7_matches(sh[3 * m], sh[3 * m + 1], sh[3 * m + 2], nr, lia, lja))
        return fail(h, GBIMS_ERR_ARG, "member " + std::to_string(m) +
                                          ": pattern is not the full DIS grid of its shape");
      row0[m] = r0;
    }
    int rc2 = setup_structured(h, sh, row0);
    if (rc2 != GBIMS_OK) return rc2;
    h->D.mctl = h->d_ctls;
  }
  return GBIMS_OK;
}

static int batch_apply_core(gbims_handle *h, int kstp, int *icnvg, int *in_iter,
                            gbims_summary *summaries) {
  if (int rc = ensure_level_words(h)) return rc;
  const int n = h->n, nm = h->nm;
  cudaStream_t st = h->st;
  GB_CUDA(h, cudaEventRecord(h->ev0, st));
  if (h->s.iscl != 0)
    h->launches += launch_scale(h->s.iscl, n, h->d_ia, h->d_ja, h->d_cptr, h->d_cpos, h->d_amat,
                                h->d_x, h->d_rhs, h->d_dscale, h->d_dscale2, st);
  int icount = factor_core(h);
  if (icount < 0) return icount;
  Ctl c;
  memset(&c, 0, sizeof(c));
  c.itmax = h->s.iter1;
  c.icnvgopt = h->s.icnvgopt;
  c.iscl = h->s.iscl;
  c.dvclose = h->s.dvclose;
  c.rclose = h->s.rclose;
  c.epfact = epfact_of(h->s.icnvgopt, kstp);
  c.iter = 1;
  c.first = 1;
  c.pivot_fail = INT_MAX;
  for (int m = 0; m < nm; ++m) h->h_ctls[m] = c;
  *h->h_ctl = c;  // the batch's own block: done = every member done
  GB_CUDA(h, cudaMemcpyAsync(h->d_ctls, h->h_ctls, sizeof(Ctl) * nm, cudaMemcpyHostToDevice, st));
  GB_CUDA(h, cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
  int eg = std::min(4 * kNumSM, (n + 255) / 256);
  if (!h->mixed) k_zero_vec<<<eg, 256, 0, st>>>(n, h->v_p, h->v_q, h->v_z, nullptr);
  residual64(h, nullptr, 0);
  kb_sumsq64(h->bd, h->v_d, h->d_part, st);
  kb_ctl_set_l2norm0(h->bd, h->d_part, st);
  kb_all_done(h->bd, h->d_ctl, 0ULL, 0, 0, st);
  if (h->mixed) {
    // the FP32 recurrence starts from the FP64 residual
    kr_f64_to_f32(n, h->v_d, h->f_d, st);
    GB_CUDA(h, cudaMemsetAsync(h->f_p, 0, sizeof(float) * n, st));
  }
  GB_CUDA(h, cudaGetLastError());
  if (!h->graph_tried) build_graph(h);
  if (h->graph_ok) {
    GB_CUDA(h, cudaGraphLaunch(h->exec, st));
  } else {
    int batch = 1, total = 0;
    for (;;) {
      for (int b = 0; b < batch; ++b) enqueue_iteration(h, 0ULL, 0);
      total += batch;
      GB_CUDA(h, cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
      GB_CUDA(h, cudaStreamSynchronize(st));
      if (h->h_ctl->done || total > 4 * (h->s.iter1 + 2)) break;
      batch = std::min(batch * 2, 32);
    }
  }
  if (h->s.iscl != 0) {
    launch_unscale_x(n, h->d_x, h->d_dscale2, st);
    h->launches += 1;
  }
  GB_CUDA(h, cudaEventRecord(h->ev1, st));
  GB_CUDA(h, cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
  GB_CUDA(h, cudaMemcpyAsync(h->h_ctls, h->d_ctls, sizeof(Ctl) * nm, cudaMemcpyDeviceToHost, st));
  GB_CUDA(h, cudaStreamSynchronize(st));
  GB_CUDA(h, cudaGetLastError());
  h->launches += 4 + (h->mixed ? 1 : 0) + (long long)h->body_kernels * h->h_ctl->bodies;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  bool nonfinite = false;
  for (int m = 0; m < nm; ++m) {
    const Ctl &r = h->h_ctls[m];
    const int iters = (r.l2norm0 == 0.0 || h->s.iter1 <= 0) ? 0 : r.iter;
    if (icnvg) icnvg[m] = r.icnvg;
    if (in_iter) in_iter[m] = iters;
    nonfinite = nonfinite || r.nonfinite;
    if (summaries) {
      gbims_summary &sm = summaries[m];
      sm.iter_cnt = iters;
      sm.icnvg = r.icnvg;
      sm.pivot_retries = icount;
      sm.exit_reason = r.exit_reason;
      sm.dvmax = r.deltax;
      sm.locdv = (int)r.xloc;
      sm.rmax = r.rmax;
      sm.locr = (int)r.rloc;
      sm.l2norm0 = r.l2norm0;
      sm.l2norm = r.l2norm;
      sm.solve_ms = ms;
      sm.refinements = h->mixed ? (int)r.scratch[3] : 0;
      sm.structured = h->structured ? 1 : 0;
    }
  }
  if (nonfinite) return fail(h, GBIMS_ERR_NONFINITE, "non-finite values in a member's residual or head change");
  if (h->h_ctl->guard_tripped) return fail(h, GBIMS_ERR_STATE, "inner loop cut by the body limit");
  return icount > 0 ? GBIMS_WARN_PIVOT : GBIMS_OK;
}

extern "C" int gbims_batch_apply(gbims_handle *h, double *amat, double *rhs, double *x, int kstp,
                                 int kiter, int *icnvg, int *in_iter, gbims_summary *summaries) {
  (void)kiter;
  if (!h || !amat || !rhs || !x || !icnvg || !in_iter) return GBIMS_ERR_ARG;
  if (h->nm <= 0) return fail(h, GBIMS_ERR_STATE, "not a batch handle (gbims_batch_create)");
  GB_CUDA(h, cudaMemcpyAsync(h->d_amat, amat, sizeof(double) * h->nja, cudaMemcpyHostToDevice, h->st));
  GB_CUDA(h, cudaMemcpyAsync(h->d_rhs, rhs, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  GB_CUDA(h, cudaMemcpyAsync(h->d_x, x, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->st));
  int rc = batch_apply_core(h, kstp, icnvg, in_iter, summaries);
  if (rc < 0 && rc != GBIMS_ERR_NONFINITE) return rc;
  cudaError_t e = cudaMemcpy(x, h->d_x, sizeof(double) * h->n, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(h, GBIMS_ERR_CUDA, cudaGetErrorString(e));
  return rc;
}

extern "C" int gbims_batch_apply_device(gbims_handle *h, double *d_amat, double *d_rhs,
                                        double *d_x, int kstp, int kiter, int *icnvg,
                                        int *in_iter, gbims_summary *summaries) {
  (void)kiter;
  if (!h || !d_amat || !d_rhs || !d_x || !icnvg || !in_iter) return GBIMS_ERR_ARG;
  if (h->nm <= 0) return fail(h, GBIMS_ERR_STATE, "not a batch handle (gbims_batch_create)");
  GB_CUDA(h, cudaMemcpyAsync(h->d_amat, d_amat, sizeof(double) * h->nja, cudaMemcpyDeviceToDevice, h->st));
  GB_CUDA(h, cudaMemcpyAsync(h->d_rhs, d_rhs, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st));
  GB_CUDA(h, cudaMemcpyAsync(h->d_x, d_x, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st));
  int rc = batch_apply_core(h, kstp, icnvg, in_iter, summaries);
  if (rc < 0 && rc != GBIMS_ERR_NONFINITE) return rc;
  cudaError_t e = cudaMemcpyAsync(d_x, h->d_x, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) return fail(h, GBIMS_ERR_CUDA, cudaGetErrorString(e));
  return rc;
}

// Accessors used by the device-resident solution (gbsln_*): the solution
// assembles straight into the IMS handle's amat/rhs and keeps x there.
namespace gb {
void ims_buffers(gbims_handle *h, double **amat, double **rhs, double **x) {
  *amat = in_amat(h);
  *rhs = in_rhs(h);
  *x = in_x(h);
}
cudaStream_t ims_stream(gbims_handle *h) { return h->st; }
int ims_apply_inplace(gbims_handle *h, int kstp, int kiter, int *icnvg, int *in_iter,
                      gbims_summary *summary) {
  return apply_core(h, kstp, kiter, icnvg, in_iter, summary);
}
const char *ims_error(gbims_handle *h) { return h->err.c_str(); }
}  // namespace gb
