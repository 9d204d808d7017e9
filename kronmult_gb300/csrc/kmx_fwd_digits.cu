// FP64 forward on the FP16 tensor cores by exact digit products, with the
// double-float kernel as the second pass for the entries the digits kernel
// hands back (see kmx_oz.cuh).
#include "kmx_forms.h"
#include "kmx_launch.cuh"
#include "kmx_oz.cuh"

namespace kmx {
namespace {

struct OzKernel {
  const void* func;
  int smem;
};

OzKernel pick_oz(int n, int d) {
  if (n == 4 && d == 4) return {(const void*)oz::oz_kernel<4, 4>, oz::smem_bytes<4, 4>()};
  if (n == 4 && d == 6) return {(const void*)oz::oz_kernel<4, 6>, oz::smem_bytes<4, 6>()};
  if (n == 16 && d == 2) return {(const void*)oz::oz_kernel<16, 2>, oz::smem_bytes<16, 2>()};
  if (n == 16 && d == 3) return {(const void*)oz::oz_kernel<16, 3>, oz::smem_bytes<16, 3>()};
  return {nullptr, 0};
}

}  // namespace

bool digits_supported(const Problem& p) {
  return is_square(p) && !p.seg_entries && !p.order && !p.count_dev &&
         pick_oz(p.n[0], p.d).func != nullptr;
}

cudaError_t launch_f64_digits(Problem& p, const LaunchHint& h, int* redo, int* redo_count,
                              cudaStream_t s) {
  if (!digits_supported(p)) return cudaErrorNotSupported;
  const OzKernel k = pick_oz(p.n[0], p.d);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const DeviceInfo di = device_info(dev);
  e = ensure_smem(k.func, dev, k.smem);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(redo_count, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.func, oz::THREADS, k.smem);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)di.sms * per_sm;
  if (grid > p.count) grid = p.count;
  if (grid < 1) grid = 1;
  void* args[] = {&p, &redo, &redo_count};
  e = cudaLaunchKernel(k.func, dim3((unsigned)grid), dim3(oz::THREADS), args, k.smem, s);
  if (e != cudaSuccess) return e;
  // second pass: the entries handed back, in double-float (count read on the device)
  Problem q = p;
  q.order = redo;
  q.order_base = nullptr;
  q.count_dev = redo_count;
  q.entry_offset = 0;
  return launch_f64_split(q, h, s);
}

}  // namespace kmx
