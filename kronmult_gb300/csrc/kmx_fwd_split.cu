// Split (double-float) FP64 forward kernels.
#include "kmx_forms.h"
#include "kmx_launch.cuh"

namespace kmx {
cudaError_t launch_f64_split(Problem& p, const LaunchHint& h, cudaStream_t s) {
  return launch_forward<double, FORM_SPLIT>(p, h, s);
}
bool needs_workspace_f64_split(const Problem& p, bool seg, int engine) {
  return needs_workspace<double, FORM_SPLIT>(p, seg, engine);
}
}  // namespace kmx
