// ephg_tc.cu - 3xTF32 tcgen05 contractions of the rate pipeline (sm_103a).
#include <string>

#include "ephg_tc.cuh"

namespace ephg {
namespace tc {

static std::string g_msg;

const char *last_error() { return g_msg.c_str(); }

void free_split(SplitOperands &s) {
  if (s.G) cudaFree(s.G);
  s.G = nullptr;
}

int split_rates_stage(SplitOperands &, Workspace &, cudaStream_t, const double2 *, int, int,
                      int64_t, int, int, int, int, const int *, int, const double2 *, const int *,
                      const int *, const std::vector<int> &, const int *, const double *,
                      const int *, const double *, const double2 *, const RateParams &,
                      const EpiData &, double *, int, cudaEvent_t, int64_t *) {
  g_msg = "split precision not available in this build";
  return 1;
}

}  // namespace tc
}  // namespace ephg
