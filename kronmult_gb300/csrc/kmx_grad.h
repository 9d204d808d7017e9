// kmx_grad.h -- the launch record of the fused forward + backward kernels,
// shared by kmx_grad.cu (one CTA per entry) and kmx_grad_warp.cu (one warp
// per entry).
#pragma once

#include <cuda_runtime.h>

#include <stddef.h>

namespace kmx {

struct GradProblem {
  int d;
  int N;
  int batch;
  const void* A;   // (n, n, d, batch) column-major
  const void* X;   // (N, batch)
  const void* G;   // (N, batch)
  void* Y;         // (N, batch) or null
  void* dX;        // (N, batch) or null
  void* dA;        // (n, n, d, batch) or null
  void* W;         // global slots for the forward intermediates (or null)
  long long wslot; // elements per slot
  int nslots;
  int f_in_smem;   // forward intermediates in shared memory
  int exp_off;     // split kernel: byte offset of the per-entry exponents in shared memory
  int* status;
};

// Shared memory one warp of the warp-per-entry kernel needs for an FP64 entry
// of n^d elements (factors and d intermediates), or 0 where that kernel does
// not take the shape (d < 3, n outside 2..8, or more than 32 KB per warp).
size_t grad_warp_bytes(int d, int n);

// Launch the warp-per-entry kernel for FP64 data: double-float arithmetic when
// `split`, native FP64 otherwise.  Returns a kmx_status.
int launch_grad_warp(const GradProblem& gp, int n, bool split, cudaStream_t s);

}  // namespace kmx
