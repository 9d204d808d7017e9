// kmx_noalloc.cu -- deterministic xbatched for callers that cannot allocate
// device memory.
//
// The deterministic mode needs scratch for its device sort and segment
// tables.  The regular entry points take it from the caller or from a
// cudaMallocAsync'd cache.  Some callers can do neither: code running where a
// device allocation is not allowed or not safe -- inside a larger
// application's memory-pool discipline that forbids foreign allocations, in a
// plug-in loaded into a host that owns all device memory, or in a process
// whose allocator must not be touched between graph launches.  For them this
// file provides kmx_kronmult_xbatched_f64_noalloc, whose scratch is a fixed
// array in the library's own device image.
//
//   - Capacity: KMX_NOALLOC_SCRATCH_BYTES (16 MiB) per GPU, held from module
//     load until process exit; calls whose scratch would exceed it are
//     rejected with KMX_ERR_WORKSPACE before anything is launched.
//   - Shapes: every square shape whose entry fits in on-chip memory; an entry
//     that would need a global workspace for its intermediate (n = 8 with
//     d >= 5, for example) is rejected with KMX_ERR_UNSUPPORTED, also before
//     anything is launched.
//   - Set-up: the first call on a device, with that device current, looks up
//     the array's device address with cudaGetSymbolAddress and caches it for
//     the life of the process.  Make that first call before any stream
//     capture begins.  The cached address belongs to the device's primary
//     context: after cudaDeviceReset it is stale, so do not use the library
//     across a device reset.
//   - Sharing: every call uses the same array and the array keeps the last
//     call's contents; each call zeroes what must start at zero (segment
//     counts, the work-queue counter) on its stream.  Calls that overlap on
//     the GPU (other streams, other host threads) race on the array.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/kronmult_gb300.h"
#include "kmx_forms.h"
#include "kmx_segments.h"

namespace {

constexpr size_t KMX_NOALLOC_SCRATCH_BYTES = size_t(16) << 20;
constexpr int KMX_NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char kmx_noalloc_scratch[KMX_NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[KMX_NOALLOC_MAX_DEVICES];

// Device address of the scratch array on the current device (host code only
// sees a host-side stand-in under the array's name).
int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KMX_ERR_CUDA;
  if (dev < 0 || dev >= KMX_NOALLOC_MAX_DEVICES) return KMX_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, kmx_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) return KMX_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return KMX_OK;
}

}  // namespace

extern "C" int kmx_kronmult_xbatched_f64_noalloc(int d, int n, const double* const* Aarray, int lda,
                                                 double* const* pX, double* const* pY,
                                                 int batchCount, kmx_stream_t stream) {
  if (batchCount < 0) return KMX_ERR_INVALID_ARG;
  // shape and argument checks, then capacity, all before anything is launched
  bool needs_ws = false;
  int rc = kmx::xbatched_f64_plan(d, n, lda, KMX_FORM_AUTO, KMX_ACC_DETERMINISTIC, &needs_ws);
  if (rc != KMX_OK) return rc;
  if (needs_ws) return KMX_ERR_UNSUPPORTED;
  if (batchCount == 0) return KMX_OK;
  if (kmx::seg_workspace_bytes(batchCount) > KMX_NOALLOC_SCRATCH_BYTES) return KMX_ERR_WORKSPACE;
  void* scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc != KMX_OK) return rc;
  kmx_options o = {};  // launch shape and the rest: the defaults
  o.form = KMX_FORM_AUTO;
  o.accumulate = KMX_ACC_DETERMINISTIC;
  o.transpose = 0;
  o.engine = KMX_ENGINE_TUNED;
  o.workspace = scratch;
  o.workspace_bytes = KMX_NOALLOC_SCRATCH_BYTES;
  return kmx_kronmult_xbatched_f64_ex(d, n, Aarray, lda, pX, pY, nullptr, batchCount, 0, &o,
                                      stream);
}
