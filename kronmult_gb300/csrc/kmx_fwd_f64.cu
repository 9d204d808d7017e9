// Plain FP64 forward kernels (native DFMA).
#include "kmx_forms.h"
#include "kmx_launch.cuh"

namespace kmx {
cudaError_t launch_f64_plain(Problem& p, const LaunchHint& h, cudaStream_t s) {
  return launch_forward<double, FORM_PLAIN>(p, h, s);
}
bool needs_workspace_f64_plain(const Problem& p, bool seg, int engine) {
  return needs_workspace<double, FORM_PLAIN>(p, seg, engine);
}
}  // namespace kmx
