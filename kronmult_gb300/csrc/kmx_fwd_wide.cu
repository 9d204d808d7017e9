// Low-precision-storage forward kernels: FP32 or BF16 X and factors, FP32
// arithmetic, FP64 Y accumulation.
#include <cuda_bf16.h>

#include "kmx_forms.h"
#include "kmx_launch.cuh"

namespace kmx {
cudaError_t launch_wide_f32(Problem& p, const LaunchHint& h, cudaStream_t s) {
  return launch_forward<float, FORM_WIDE>(p, h, s);
}
cudaError_t launch_wide_bf16(Problem& p, const LaunchHint& h, cudaStream_t s) {
  return launch_forward<__nv_bfloat16, FORM_WIDE>(p, h, s);
}
}  // namespace kmx
