// k_dia7.cu -- structured 7-point (DIS) ILU0 triangular sweeps.
#include "gbims_internal.cuh"

namespace gb {

bool dia7_matches(int, int, int, int, const std::vector<int> &, const std::vector<int> &) {
  return false;
}
void launch_dia7_extract(const Dia7 &, int, const int *, const int *, const double *, bool,
                         cudaStream_t) {}
void launch_dia7_apply64(const Dia7 &, const double *, double *, const Ctl *, cudaStream_t) {}
void launch_dia7_apply32(const Dia7 &, const float *, float *, const Ctl *, cudaStream_t) {}

}  // namespace gb
