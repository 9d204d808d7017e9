// kmx_mixed.cu -- one call over instances of mixed shapes.
//
// The reference's vbatched takes one shape per call (kronmult_vbatched.hpp:
// 19-248), so a batch mixing (d, n) needs one call per shape class.  Here a
// single call takes per-instance (d, n) and:
//   1. tags each instance with its class (the caller lists the classes);
//   2. sorts instance ids by class on the device (CUB radix sort, stable);
//   3. finds each class's range by binary search (device);
//   4. launches, per class and in the caller's class order, the tuned kernel
//      for that (d, n); each launch reads its count and range start from
//      device memory, so no host synchronisation happens and the whole call
//      can be captured in a CUDA graph.
// Instances whose shape is not in the class list are reported through the
// device status word (DF_BAD_SHAPE) and skipped.  The rectangular form
// (kmx_kronmult_vmixed_*) names each instance's class directly.
#include <cuda_runtime.h>

#include <cub/cub.cuh>
#include <mutex>

#include "../../include/kronmult_gb300.h"
#include "kmx_engine.cuh"
#include "kmx_mixed.h"

namespace kmx {

namespace {

struct ClassList {
  int d[KMX_MAX_CLASSES];
  int n[KMX_MAX_CLASSES];
  int count;
};

__global__ void class_key_kernel(const int* dims, const int* cls, int count, ClassList cl,
                                 int* keys, int* ids, int* status) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    int k = cl.count;
    if (cls != nullptr) {
      const int c = cls[i];
      if (c >= 0 && c < cl.count) k = c;
    } else {
      const int d = dims[2 * i], n = dims[2 * i + 1];
      for (int c = 0; c < cl.count; ++c)
        if (cl.d[c] == d && cl.n[c] == n) {
          k = c;
          break;
        }
    }
    if (k == cl.count) atomicOr(status, DF_BAD_SHAPE);
    keys[i] = k;
    ids[i] = i;
  }
}

// offsets[c] = first position of class c in the sorted keys; counts[c].
__global__ void class_range_kernel(const int* sorted_keys, int count, int nclasses, int* offsets,
                                   int* counts) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > nclasses) return;
  auto lower = [&](int key) {
    int lo = 0, hi = count;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (sorted_keys[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
  };
  if (c < nclasses) {
    const int a = lower(c), b = lower(c + 1);
    offsets[c] = a;
    counts[c] = b - a;
  }
}

inline size_t al256(size_t x) { return (x + 255) / 256 * 256; }

struct MixLayout {
  size_t keys, ids, skeys, order, offsets, counts, queue, temp, temp_bytes, total;
};

MixLayout mix_layout(int count) {
  MixLayout L;
  size_t o = 0;
  auto take = [&](size_t b) {
    const size_t at = o;
    o += al256(b);
    return at;
  };
  const size_t c = (size_t)(count > 0 ? count : 1);
  L.keys = take(c * 4);
  L.ids = take(c * 4);
  L.skeys = take(c * 4);
  L.order = take(c * 4);
  L.offsets = take(KMX_MAX_CLASSES * 4);
  L.counts = take(KMX_MAX_CLASSES * 4);
  L.queue = take(4);
  size_t t = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, t, (int*)nullptr, (int*)nullptr, (int*)nullptr,
                                  (int*)nullptr, (int)c);
  L.temp_bytes = al256(t);
  L.temp = take(L.temp_bytes);
  L.total = o;
  return L;
}

}  // namespace

size_t mixed_workspace_bytes(int count) { return mix_layout(count).total; }

cudaError_t mixed_prepare(int count, const int* dims, const int* cls, const int* classes,
                          int nclasses, void* ws, size_t ws_bytes, int* status, cudaStream_t s,
                          MixedArrays* out) {
  const MixLayout L = mix_layout(count);
  if (ws == nullptr || ws_bytes < L.total) return cudaErrorInvalidValue;
  if (nclasses < 1 || nclasses > KMX_MAX_CLASSES) return cudaErrorInvalidValue;
  unsigned char* w = static_cast<unsigned char*>(ws);
  int* keys = reinterpret_cast<int*>(w + L.keys);
  int* ids = reinterpret_cast<int*>(w + L.ids);
  int* skeys = reinterpret_cast<int*>(w + L.skeys);
  int* order = reinterpret_cast<int*>(w + L.order);
  int* offsets = reinterpret_cast<int*>(w + L.offsets);
  int* counts = reinterpret_cast<int*>(w + L.counts);
  ClassList cl;
  cl.count = nclasses;
  for (int c = 0; c < nclasses; ++c) {
    cl.d[c] = cls ? 0 : classes[2 * c];
    cl.n[c] = cls ? 0 : classes[2 * c + 1];
  }
  const int threads = 256;
  int blocks = (count + threads - 1) / threads;
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  class_key_kernel<<<blocks, threads, 0, s>>>(dims, cls, count, cl, keys, ids, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int bits = 1;
  while (bits < 31 && (1 << bits) <= nclasses) ++bits;
  size_t tb = L.temp_bytes;
  e = cub::DeviceRadixSort::SortPairs(w + L.temp, tb, keys, skeys, ids, order, count, 0, bits, s);
  if (e != cudaSuccess) return e;
  class_range_kernel<<<1, KMX_MAX_CLASSES + 1, 0, s>>>(skeys, count, nclasses, offsets, counts);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int* queue = reinterpret_cast<int*>(w + L.queue);
  e = cudaMemsetAsync(queue, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  out->queue = queue;
  out->keys = keys;
  out->order = order;
  out->offsets = offsets;
  out->counts = counts;
  return cudaSuccess;
}

}  // namespace kmx
