// kmx_segments.cu -- device-side grouping of entries by Y block for the
// deterministic accumulation mode.
//
//   1. key[e] = address of entry e's Y block, value[e] = e
//   2. stable radix sort of (key, value): entries of one Y block become
//      contiguous, in their original order
//   3. run-length encoding: one SEGMENT per distinct Y block (offset, count)
//   4. overlap check: distinct Y blocks must be at least one block apart;
//      partially overlapping blocks cannot be owned by one group, so the
//      call is cancelled (no Y element is written) and DF_OVERLAP is set
//   5. segments ordered longest first (the persistent kernel pops them from a
//      work queue in this order, which bounds the tail)
//
// Everything runs on the stream without a host synchronisation, in
// workspace the caller (or the library's cache) provides.  The sort, the
// encoding and the scan are CUB's device algorithms.
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include "kmx_engine.cuh"
#include "kmx_segments.h"

namespace kmx {

namespace {

__global__ void seg_keys_kernel(void* const* pY, int B, unsigned long long* keys, int* vals) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += gridDim.x * blockDim.x) {
    keys[i] = reinterpret_cast<unsigned long long>(pY[i]);
    vals[i] = i;
  }
}

// Y blocks of consecutive segments must not overlap.  One block; on
// overlap the segment count is zeroed so the compute kernel does nothing.
// With entry classes, a segment's block is as long as the longest block of its
// entries (blocks of different classes may start at one address).
__global__ void seg_check_kernel(const unsigned long long* uniq, int* num, long long ybytes,
                                 const int* entries, const int* offsets, const int* counts,
                                 const int* entry_class, SegClassBytes classes, int* status) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  const int n = *num;
  for (int s = threadIdx.x; s + 1 < n; s += blockDim.x) {
    long long len = ybytes;
    if (entry_class) {
      len = 0;
      for (int j = offsets[s]; j < offsets[s] + counts[s]; ++j) {
        const int c = entry_class[entries[j]];
        if (c >= 0 && c < 64 && classes.bytes[c] > len) len = classes.bytes[c];
      }
    }
    if ((long long)(uniq[s + 1] - uniq[s]) < len) bad = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0 && bad) {
    atomicOr(status, DF_OVERLAP);
    *num = 0;
  }
}

inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }

struct SegLayout {
  size_t keys_in, keys_out, vals_in, entries, uniq, counts, offsets, counts_sorted, order, num,
      queue, temp, temp_bytes, total;
};

SegLayout seg_layout(int B) {
  SegLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += align256(bytes);
    return at;
  };
  const size_t b = (size_t)(B > 0 ? B : 1);
  L.keys_in = take(b * 8);
  L.keys_out = take(b * 8);
  L.vals_in = take(b * 4);
  L.entries = take(b * 4);
  L.uniq = take(b * 8);
  L.counts = take(b * 4);
  L.offsets = take(b * 4);
  L.counts_sorted = take(b * 4);
  L.order = take(b * 4);
  L.num = take(4);
  L.queue = take(4);
  // CUB temporary storage: the largest of the four algorithms
  size_t t1 = 0, t2 = 0, t3 = 0, t4 = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, t1, (unsigned long long*)nullptr,
                                  (unsigned long long*)nullptr, (int*)nullptr, (int*)nullptr, (int)b);
  cub::DeviceRunLengthEncode::Encode(nullptr, t2, (unsigned long long*)nullptr,
                                     (unsigned long long*)nullptr, (int*)nullptr, (int*)nullptr,
                                     (int)b);
  cub::DeviceScan::ExclusiveSum(nullptr, t3, (int*)nullptr, (int*)nullptr, (int)b);
  cub::DeviceRadixSort::SortPairsDescending(nullptr, t4, (int*)nullptr, (int*)nullptr,
                                            (int*)nullptr, (int*)nullptr, (int)b);
  size_t t = t1;
  if (t2 > t) t = t2;
  if (t3 > t) t = t3;
  if (t4 > t) t = t4;
  L.temp_bytes = align256(t);
  L.temp = take(L.temp_bytes);
  L.total = o;
  return L;
}

}  // namespace

size_t seg_workspace_bytes(int B) { return seg_layout(B).total; }

cudaError_t seg_prepare(void* const* pY, int B, long long ybytes, void* ws, size_t ws_bytes,
                        int* status, cudaStream_t s, SegArrays* out, const int* entry_class,
                        const SegClassBytes* classes) {
  const SegLayout L = seg_layout(B);
  if (ws == nullptr || ws_bytes < L.total) return cudaErrorInvalidValue;
  unsigned char* w = static_cast<unsigned char*>(ws);
  auto* keys_in = reinterpret_cast<unsigned long long*>(w + L.keys_in);
  auto* keys_out = reinterpret_cast<unsigned long long*>(w + L.keys_out);
  auto* vals_in = reinterpret_cast<int*>(w + L.vals_in);
  auto* entries = reinterpret_cast<int*>(w + L.entries);
  auto* uniq = reinterpret_cast<unsigned long long*>(w + L.uniq);
  auto* counts = reinterpret_cast<int*>(w + L.counts);
  auto* offsets = reinterpret_cast<int*>(w + L.offsets);
  auto* counts_sorted = reinterpret_cast<int*>(w + L.counts_sorted);
  auto* order = reinterpret_cast<int*>(w + L.order);
  auto* num = reinterpret_cast<int*>(w + L.num);
  auto* queue = reinterpret_cast<int*>(w + L.queue);
  void* temp = w + L.temp;
  size_t tb = L.temp_bytes;

  cudaError_t e;
  const int threads = 256;
  const int blocks = (B + threads - 1) / threads < 4096 ? (B + threads - 1) / threads : 4096;
  seg_keys_kernel<<<blocks > 0 ? blocks : 1, threads, 0, s>>>(pY, B, keys_in, vals_in);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cub::DeviceRadixSort::SortPairs(temp, tb, keys_in, keys_out, vals_in, entries, B, 0, 64,
                                           s)) != cudaSuccess)
    return e;
  if ((e = cudaMemsetAsync(counts, 0, (size_t)B * sizeof(int), s)) != cudaSuccess) return e;
  tb = L.temp_bytes;
  if ((e = cub::DeviceRunLengthEncode::Encode(temp, tb, keys_out, uniq, counts, num, B, s)) !=
      cudaSuccess)
    return e;
  tb = L.temp_bytes;
  if ((e = cub::DeviceScan::ExclusiveSum(temp, tb, counts, offsets, B, s)) != cudaSuccess) return e;
  SegClassBytes cb{};
  if (entry_class && classes) cb = *classes;
  seg_check_kernel<<<1, 1024, 0, s>>>(uniq, num, ybytes, entries, offsets, counts,
                                      classes ? entry_class : nullptr, cb, status);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  int bits = 1;
  while (bits < 31 && (1LL << bits) <= (long long)B) ++bits;
  tb = L.temp_bytes;
  if ((e = cub::DeviceRadixSort::SortPairsDescending(temp, tb, counts, counts_sorted, vals_in, order,
                                                     B, 0, bits, s)) != cudaSuccess)
    return e;
  if ((e = cudaMemsetAsync(queue, 0, sizeof(int), s)) != cudaSuccess) return e;
  out->entries = entries;
  out->offset = offsets;
  out->count = counts;
  out->order = order;
  out->num = num;
  out->queue = queue;
  return cudaSuccess;
}

}  // namespace kmx
