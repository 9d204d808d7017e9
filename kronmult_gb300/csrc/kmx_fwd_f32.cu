// FP32 forward kernels (native FFMA).
#include "kmx_forms.h"
#include "kmx_launch.cuh"

namespace kmx {
cudaError_t launch_f32_plain(Problem& p, const LaunchHint& h, cudaStream_t s) {
  return launch_forward<float, FORM_PLAIN>(p, h, s);
}
}  // namespace kmx
