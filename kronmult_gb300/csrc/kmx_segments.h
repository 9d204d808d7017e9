// Device-side grouping of entries by Y block (deterministic mode).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace kmx {

struct SegArrays {
  const int* entries;  // entry ids sorted by Y block (stable)
  const int* offset;   // first position of each segment
  const int* count;    // entries per segment
  const int* order;    // segments, longest first
  int* num;            // number of segments (zeroed when Y blocks partially overlap)
  int* queue;          // work-queue counter, zeroed on the stream
};

// Bytes of workspace seg_prepare needs for B entries.
size_t seg_workspace_bytes(int B);

// Y block sizes per entry class (mixed-shape calls), at most 64 classes.
struct SegClassBytes {
  long long bytes[64];
};

// Build the segments of B entries whose Y blocks are pY[0..B-1] (each ybytes
// long; or, with entry_class, classes->bytes[entry_class[e]] long) in
// workspace ws, asynchronously on stream s.
cudaError_t seg_prepare(void* const* pY, int B, long long ybytes, void* ws, size_t ws_bytes,
                        int* status, cudaStream_t s, SegArrays* out,
                        const int* entry_class = nullptr, const SegClassBytes* classes = nullptr);

}  // namespace kmx
