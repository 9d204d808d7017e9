// kmx_diag.cu -- live peak probes used as roofline denominators: FP64 and
// FP32 fused multiply-add throughput of the current device, timed with CUDA
// events (no multiply-add instruction count is inferred from vendor tables).
#include <cuda_runtime.h>

#include "../../include/kronmult_gb300.h"

namespace {

template <typename T>
__global__ void fma_loop(T* sink, int iters, T s) {
  T a0 = (T)threadIdx.x * (T)1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  T a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, s, (T)0.5); a1 = fma(a1, s, (T)0.5); a2 = fma(a2, s, (T)0.5); a3 = fma(a3, s, (T)0.5);
    a4 = fma(a4, s, (T)0.5); a5 = fma(a5, s, (T)0.5); a6 = fma(a6, s, (T)0.5); a7 = fma(a7, s, (T)0.5);
  }
  const T r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == (T)12345.678) sink[0] = r;  // never true; keeps the chains live
}

template <typename T>
int probe(int iters, double* fma_per_s) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KMX_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  T* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(T)) != cudaSuccess) return KMX_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256;
  fma_loop<T><<<blocks, threads>>>(sink, iters / 4, (T)0.999);
  cudaEventRecord(e0);
  fma_loop<T><<<blocks, threads>>>(sink, iters, (T)0.999);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess || ms <= 0.f) return KMX_ERR_CUDA;
  *fma_per_s = (double)blocks * threads * iters * 8 / (ms * 1e-3);
  return KMX_OK;
}

}  // namespace

extern "C" int kmx_probe_fma_rate(int fp64, double* fma_per_second) {
  if (!fma_per_second) return KMX_ERR_NULL_POINTER;
  return fp64 ? probe<double>(2048, fma_per_second) : probe<float>(65536, fma_per_second);
}
