// gbsln_api.cu -- NPF fill and device-resident solution (C ABI).
#include "gbims_internal.cuh"

extern "C" int gbnpf_create(const gbnpf_options *, int, int, int, const int *, const int *,
                            const int *, const int *, const int *, const double *,
                            const double *, const double *, const double *, const double *,
                            const double *, const double *, const int *, gbnpf_handle **out) {
  if (out) *out = nullptr;
  return GBIMS_ERR_UNSUPPORTED;
}
extern "C" int gbnpf_fill(gbnpf_handle *, const int *, const double *, double *, double *) {
  return GBIMS_ERR_UNSUPPORTED;
}
extern "C" int gbnpf_get_condsat(gbnpf_handle *, double *) { return GBIMS_ERR_UNSUPPORTED; }
extern "C" int gbnpf_destroy(gbnpf_handle *) { return GBIMS_OK; }
extern "C" int gbsln_create(const gbsln_model *, const gbnpf_options *, const gbims_settings *,
                            const gbsln_nonlinear *, const double *, gbsln_handle **out) {
  if (out) *out = nullptr;
  return GBIMS_ERR_UNSUPPORTED;
}
extern "C" int gbsln_timestep(gbsln_handle *, int, int, double, gbsln_stats *) { return GBIMS_ERR_UNSUPPORTED; }
extern "C" int gbsln_get_heads(gbsln_handle *, double *) { return GBIMS_ERR_UNSUPPORTED; }
extern "C" int gbsln_set_heads(gbsln_handle *, const double *) { return GBIMS_ERR_UNSUPPORTED; }
extern "C" gbims_handle *gbsln_ims(gbsln_handle *) { return nullptr; }
extern "C" int gbsln_destroy(gbsln_handle *) { return GBIMS_OK; }
