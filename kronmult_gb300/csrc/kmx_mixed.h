// Grouping of mixed-shape instances by class (device side).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#define KMX_MAX_CLASSES 64

namespace kmx {

struct MixedArrays {
  const int* keys;     // class of each instance (nclasses: not in the list)
  const int* order;    // instance ids sorted by class (stable)
  const int* offsets;  // first position of class c in order[] (device)
  const int* counts;   // instances of class c (device)
  int* queue;          // work-queue counter of a persistent launch, zeroed on the stream
};

size_t mixed_workspace_bytes(int count);

// Either dims (device array of count (d, n) pairs, matched against classes,
// a host array of nclasses (d, n) pairs) or cls (device array of count class
// ids below nclasses; classes unused) gives each instance its class.
cudaError_t mixed_prepare(int count, const int* dims, const int* cls, const int* classes,
                          int nclasses, void* ws, size_t ws_bytes, int* status, cudaStream_t s,
                          MixedArrays* out);

}  // namespace kmx
