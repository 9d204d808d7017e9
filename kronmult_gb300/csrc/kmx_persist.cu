// kmx_persist.cu -- one persistent launch over every instance of a mixed-shape
// call (KMX_ENGINE_PERSISTENT), the alternative to one tuned launch per class.
//
// The instances are grouped by class on the device (kmx_mixed.cu); their
// positions in that order are handed out by a device work queue, so the
// classes run in the caller's order (longest first when the caller lists
// them so) and every CTA keeps taking work until the queue is empty.  Each
// instance runs the generic double-float entry (gen_split_entry) with its own
// (d, n): its intermediate in the CTA's shared memory when two buffers fit,
// one buffer (modes updated in place) when only that fits, else in the CTA's
// slot of the caller's workspace.  The cost of one launch for all classes is
// that every class runs the same run-time-shape code with the register and
// shared-memory budget of the largest, where the per-class launches run the
// register-tiled, cluster and small-entry kernels each tuned for its shape.
#include <cuda_runtime.h>

#include "kmx_forms.h"
#include "kmx_launch.cuh"

namespace kmx {
namespace {

constexpr int PT = 256;                 // threads per CTA
constexpr int PSMEM = 96 * 1024;        // shared memory per CTA (two CTAs per SM)

__global__ void __launch_bounds__(PT) persist_kernel(const Problem p, const int* dims, int* queue) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ long long s_pos;
  const int lt = threadIdx.x;
  const long long total = launch_count(p);
  for (;;) {
    if (lt == 0) s_pos = atomicAdd(queue, 1);
    __syncthreads();
    const long long pos = s_pos;
    __syncthreads();  // every thread has its position before the next pop
    if (pos >= total) break;
    const int inst = p.order[pos];
    const int d = dims[2 * inst], n = dims[2 * inst + 1];
    Problem q = p;
    q.d = d;
    long long N = 1;
    for (int l = 0; l < MAXD; ++l) {
      q.m[l] = q.n[l] = q.ld[l] = (l < d) ? n : 1;
      if (l < d) N *= n;
    }
    q.Nx = q.Ny = q.sxw = N;
    EntryPtrs<double> en;
    if (!resolve_entry<double>(q, inst, en)) {
      if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    const size_t fac = ((size_t)d * n * n * 8 + 15) / 16 * 16;
    int* sExp = reinterpret_cast<int*>(smem + fac);
    float* sNrm = reinterpret_cast<float*>(sExp + MAXD + 2);
    unsigned char* braw = smem + fac + GEN_SPLIT_HDR;
    const size_t bb = ((size_t)N * 8 + 15) / 16 * 16;
    double *w0, *w1;
    bool two = true;
    if (fac + GEN_SPLIT_HDR + 2 * bb <= (size_t)PSMEM) {
      w0 = reinterpret_cast<double*>(braw);
      w1 = reinterpret_cast<double*>(braw + bb);
    } else if (fac + GEN_SPLIT_HDR + bb <= (size_t)PSMEM) {
      w0 = reinterpret_cast<double*>(braw);  // one buffer: square modes in place
      w1 = nullptr;
      two = false;
    } else {
      w0 = static_cast<double*>(p.Wbase) + (long long)blockIdx.x * p.w_stride;
      w1 = w0 + N;
    }
    if (N >= 4096) {
      gen_split_entry<4>(q, en, smem, w0, w1, sExp, sNrm, two, lt, PT, 0);
    } else {
      gen_split_entry<2>(q, en, smem, w0, w1, sExp, sNrm, two, lt, PT, 0);
    }
    __syncthreads();
  }
}

}  // namespace

// p: base problem of the call (L_MIXED, order = instances sorted by class,
// count = all instances, Wbase/w_stride/nslots = the caller's workspace in
// slots of 2 * max_elems doubles); queue: a device int, zero at launch.
cudaError_t launch_mixed_persistent(Problem& p, const int* dims, int* queue, long long max_elems,
                                    cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const DeviceInfo di = device_info(dev);
  const void* func = reinterpret_cast<const void*>(&persist_kernel);
  e = ensure_smem(func, dev, PSMEM);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, PT, PSMEM);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  long long grid = (long long)di.sms * per_sm;
  if (grid > p.count) grid = p.count;
  // entries beyond shared memory need a workspace slot per CTA
  const size_t big = (size_t)max_elems * 8 * 2;
  if (big + GEN_SPLIT_HDR + 4096 > (size_t)PSMEM) {
    if (p.Wbase == nullptr || p.nslots < 1) return cudaErrorInvalidValue;
    if (grid > p.nslots) grid = p.nslots;
  }
  if (grid < 1) grid = 1;
  void* args[] = {&p, &dims, &queue};
  return cudaLaunchKernel(func, dim3((unsigned)grid), dim3(PT), args, PSMEM, s);
}

}  // namespace kmx
