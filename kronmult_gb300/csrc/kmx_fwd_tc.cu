// Tensor-core (3xTF32) forward kernels for FP32- and BF16-stored data:
// FP32 Y (the FP32 entry points) or FP64 Y (the wide entry point).
#include <cuda_bf16.h>

#include "kmx_forms.h"
#include "kmx_launch.cuh"
#include "kmx_tc.cuh"

namespace kmx {
namespace {

struct TcKernel {
  const void* func;
  int smem;
};

template <typename In, typename Out, bool SEG>
TcKernel pick_tc(int n, int d) {
#define KMX_TC(NN, D)                                                                         \
  if constexpr (!SEG || tc::seg_supported(NN, D)) {                                          \
    if (n == NN && d == D)                                                                    \
      return {(const void*)tc::tc_kernel<NN, D, In, Out, SEG>, tc::smem_bytes(NN, D)};        \
  }
  KMX_TC(4, 4)
  KMX_TC(4, 6)
  KMX_TC(8, 3)
  KMX_TC(8, 4)
  KMX_TC(8, 5)
  KMX_TC(16, 2)
  KMX_TC(16, 3)
#undef KMX_TC
  return {nullptr, 0};
}

template <typename In, typename Out>
cudaError_t launch_tc(Problem& p, cudaStream_t s) {
  // class-filtered segments (deterministic mixed shapes): generic kernels only
  if (!is_square(p) || p.seg_key) return cudaErrorNotSupported;
  const TcKernel k = p.seg_entries ? pick_tc<In, Out, true>(p.n[0], p.d)
                                   : pick_tc<In, Out, false>(p.n[0], p.d);
  if (!k.func) return cudaErrorNotSupported;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const DeviceInfo di = device_info(dev);
  e = ensure_smem(k.func, dev, k.smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.func, tc::THREADS, k.smem);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)di.sms * per_sm;
  if (grid > p.count) grid = p.count;
  if (grid < 1) grid = 1;
  void* args[] = {&p};
  return cudaLaunchKernel(k.func, dim3((unsigned)grid), dim3(tc::THREADS), args, k.smem, s);
}

}  // namespace

cudaError_t launch_tc_f32(Problem& p, cudaStream_t s) { return launch_tc<float, float>(p, s); }
cudaError_t launch_tc_wide_f32(Problem& p, cudaStream_t s) {
  return launch_tc<float, double>(p, s);
}
cudaError_t launch_tc_wide_bf16(Problem& p, cudaStream_t s) {
  return launch_tc<__nv_bfloat16, double>(p, s);
}

}  // namespace kmx
