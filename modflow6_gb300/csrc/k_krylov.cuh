// k_krylov.cuh -- launch wrappers of the Krylov kernels (k_krylov.cu).
#pragma once
#include "gbims_internal.cuh"

namespace gb {
void kr_dot64(int n, const double *a, const double *b, double *part, int G, const Ctl *ctl, cudaStream_t st);
void kr_dot_tq_tt64(int n, const double *t, const double *q, double *part, int G, const Ctl *ctl, cudaStream_t st);
void kr_sumsq64(int n, const double *a, double *part, int G, cudaStream_t st);
void kr_ctl_set_l2norm0(Ctl *ctl, const double *part, int G, cudaStream_t st);
// Ctl::l2norm of the residual from sum-of-squares partials (after a loop that skipped it).
void kr_ctl_set_l2norm(Ctl *ctl, const double *part, int G, cudaStream_t st);
void kr_ctl_cg_rho(Ctl *ctl, const double *part, int G, cudaStream_t st);
void kr_ctl_alpha(Ctl *ctl, const double *part, int G, cudaStream_t st);
void kr_cg_pupdate64(int n, const double *z, double *p, const Ctl *ctl, cudaStream_t st);
// l2: take the sum of squares of the new residual (the RCLOSE L2 options)
void kr_cg_update64(int n, double *x, double *d, const double *p, const double *q, double *part, int G, const Ctl *ctl, cudaStream_t st, bool l2);
// Per-model maxima of the inner records (CONVNMOD > 1): PCG p = P, q unused;
// BiCGSTAB p = PHAT, q = QHAT; d the updated residual.
void kr_rec_models(bool bcgs, int nm, const int *modstart, const double *p, const double *q, const double *d, const double *dscale, double *part, int G, const Ctl *ctl, cudaStream_t st);
void kr_ctl_cg_cnvg(Ctl *ctl, const double *part, int G, unsigned long long cond, int use_cond, cudaStream_t st);
void kr_ctl_bcgs_rho(Ctl *ctl, const double *part, int G, cudaStream_t st);
void kr_bcgs_p64(int n, const double *d, double *p, const double *v, const Ctl *ctl, cudaStream_t st);
void kr_bcgs_q64(int n, const double *d, const double *v, double *q, const Ctl *ctl, cudaStream_t st);
void kr_ctl_omega(Ctl *ctl, const double *part, int G, cudaStream_t st);
void kr_bcgs_update64(int n, double *x, double *d, const double *phat, const double *qhat, const double *q, const double *t, const double *dscale, double *part, int G, const Ctl *ctl, cudaStream_t st, bool l2);
void kr_ctl_bcgs_cnvg(Ctl *ctl, const double *part, int G, unsigned long long cond, int use_cond, cudaStream_t st);
void kr_ctl_mixed_inner(Ctl *ctl, const double *part, int G, int bcgs, double refine_factor, cudaStream_t st);
void kr_true_resid_stats(int n, const double *r, float *d32, float *dhat32, double *dhat64, const double *dscale, double *part, int G, const Ctl *ctl, cudaStream_t st);
void kr_ctl_refine(Ctl *ctl, const double *part, int G, unsigned long long cond, int use_cond, cudaStream_t st);
// the mixed form's FP32 inner vectors (FP64 reductions and scalars)
void kr_dot32(int n, const float *a, const float *b, double *part, int G, const Ctl *ctl, cudaStream_t st);
void kr_dot_tq_tt32(int n, const float *t, const float *q, double *part, int G, const Ctl *ctl, cudaStream_t st);
void kr_cg_pupdate32(int n, const float *z, float *p, const Ctl *ctl, cudaStream_t st);
void kr_cg_update_mixed(int n, double *x, float *d, const float *p, const float *q, double *part, int G, const Ctl *ctl, cudaStream_t st);
void kr_bcgs_p32(int n, const float *d, float *p, const float *v, const Ctl *ctl, cudaStream_t st);
void kr_bcgs_q32(int n, const float *d, const float *v, float *q, const Ctl *ctl, cudaStream_t st);
void kr_bcgs_update32(int n, double *x, float *d, const float *phat, const float *qhat, const float *q, const float *t, const double *dscale, double *part, int G, const Ctl *ctl, cudaStream_t st);
void kr_f64_to_f32(int n, const double *s, float *d, cudaStream_t st);
// d = b - A x (CSR, one row per thread; n <= kMaxRedBlocks * kRedBlock) with
// part (3 * ceil(n/256) doubles) and out (3 doubles: L2, signed max, row).
void kr_residual_rows(int n, const int *ia, const int *ja, int base, const double *amat,
                      const double *x, const double *b, double *resid, double *part,
                      double *out, cudaStream_t st);
void kr_f32_to_f64(int n, const float *s, double *d, cudaStream_t st);
// batched ensemble (one block-diagonal system, per-member control blocks)
void kb_dot64(const BatchDev &B, const double *a, const double *b, double *part, cudaStream_t st);
void kb_sumsq64(const BatchDev &B, const double *a, double *part, cudaStream_t st);
void kb_cg_pupdate64(const BatchDev &B, const double *z, double *p, cudaStream_t st);
void kb_cg_update64(const BatchDev &B, double *x, double *d, const double *p, const double *q,
                    double *part, cudaStream_t st);
void kb_ctl_set_l2norm0(const BatchDev &B, const double *part, cudaStream_t st);
void kb_ctl_cg_rho(const BatchDev &B, const double *part, cudaStream_t st);
void kb_ctl_alpha(const BatchDev &B, const double *part, cudaStream_t st);
void kb_ctl_cg_cnvg(const BatchDev &B, const double *part, cudaStream_t st);
void kb_all_done(const BatchDev &B, Ctl *gctl, unsigned long long cond, int use_cond,
                 int count_body, cudaStream_t st);
// batched mixed form (FP32 inner loop, FP64 refinement per member)
void kb_dot32(const BatchDev &B, const float *a, const float *b, double *part, cudaStream_t st);
void kb_cg_pupdate32(const BatchDev &B, const float *z, float *p, cudaStream_t st);
void kb_cg_update_mixed(const BatchDev &B, double *x, float *d, const float *p, const float *q,
                        double *part, cudaStream_t st);
void kb_ctl_mixed_inner(const BatchDev &B, const double *part, double refine_factor,
                        cudaStream_t st);
void kb_any_due(const BatchDev &B, Ctl *gctl, cudaStream_t st);
void kb_true_resid_stats(const BatchDev &B, const double *r, float *d32, double *part,
                         cudaStream_t st);
void kb_ctl_refine(const BatchDev &B, const double *part, cudaStream_t st);
}  // namespace gb
