// FP32 forward kernels with the reference's float semantics: each dot
// product rounded once to FP32, stages applied in the reference's mode order.
#include "kmx_forms.h"
#include "kmx_launch.cuh"

namespace kmx {
cudaError_t launch_f32_ref(Problem& p, const LaunchHint& h, cudaStream_t s) {
  return launch_forward<float, FORM_REF32>(p, h, s);
}
}  // namespace kmx
