// Grouping of mixed-shape instances by class (device side).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#define KMX_MAX_CLASSES 64

namespace kmx {

struct MixedArrays {
  const int* order;    // instance ids sorted by class (stable)
  const int* offsets;  // first position of class c in order[] (device)
  const int* counts;   // instances of class c (device)
};

size_t mixed_workspace_bytes(int count);

// classes: host array of nclasses (d, n) pairs; dims: device array of
// count (d, n) pairs.
cudaError_t mixed_prepare(int count, const int* dims, const int* classes, int nclasses, void* ws,
                          size_t ws_bytes, int* status, cudaStream_t s, MixedArrays* out);

}  // namespace kmx
