// kmx_persist.cu -- one persistent launch over every instance of a mixed-shape
// call (KMX_ENGINE_PERSISTENT), the alternative to one tuned launch per class,
// for square classes (kmx_kronmult_mixed_f64) and rectangular ones
// (kmx_kronmult_vmixed_f64).
//
// The instances are grouped by class on the device (kmx_mixed.cu); their
// positions in that order are handed out by a device work queue, so the
// classes run in the caller's order (longest first when the caller lists
// them so) and every CTA keeps taking work until the queue is empty.  The
// class shapes travel in the kernel's parameters (PersistClasses).  Each
// instance runs the generic double-float entry (gen_split_entry) with its own
// shape: its intermediate in the CTA's shared memory when two buffers fit, one
// buffer (modes updated in place) when only that fits and every mode but the
// last may be applied in place, else in the CTA's slot of the caller's
// workspace.  The cost of one launch for all classes is that every class runs
// the same run-time-shape code with the register and shared-memory budget of
// the largest, where the per-class launches run the register-tiled, cluster
// and small-entry kernels each tuned for its shape.
#include <cuda_runtime.h>

#include "kmx_forms.h"
#include "kmx_launch.cuh"
#include "kmx_mixed.h"

namespace kmx {
static_assert(PERSIST_MAXD == MAXD, "class shapes carry MAXD modes");
static_assert(PERSIST_MAX_CLASSES == KMX_MAX_CLASSES, "one record per class");
namespace {

constexpr int PT = 256;                 // threads per CTA
constexpr int PSMEM = 96 * 1024;        // shared memory per CTA (two CTAs per SM)

__host__ __device__ inline size_t fac_bytes(const PersistClass& c) {
  size_t f = 0;
  for (int l = 0; l < c.d; ++l) f += (size_t)c.m[l] * c.n[l];
  return (f * 8 + 15) / 16 * 16;
}
__host__ __device__ inline size_t buf_bytes(const PersistClass& c) {
  return ((size_t)c.sxw * 8 + 15) / 16 * 16;
}
__host__ __device__ inline bool in_place_ok(const PersistClass& c) {
  for (int k = 0; k + 1 < c.d; ++k)
    if (!gen_split_in_place(c.m[k], c.n[k])) return false;
  return true;
}
// 2: two buffers on chip, 1: one buffer on chip (in place), 0: workspace
__host__ __device__ inline int on_chip_buffers(const PersistClass& c) {
  const size_t head = fac_bytes(c) + GEN_SPLIT_HDR;
  if (head + 2 * buf_bytes(c) <= (size_t)PSMEM) return 2;
  if (in_place_ok(c) && head + buf_bytes(c) <= (size_t)PSMEM) return 1;
  return 0;
}

// pc is a grid constant: indexed in the kernel's parameter space, not copied
// per thread.
__global__ void __launch_bounds__(PT) persist_kernel(const Problem p,
                                                     const __grid_constant__ PersistClasses pc,
                                                     const int* keys, int* queue) {
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
    const int c = keys[inst];
    if (c < 0 || c >= pc.count) continue;  // unknown class: flagged when grouped
    const PersistClass& cs = pc.c[c];
    Problem q = p;
    q.d = cs.d;
    for (int l = 0; l < MAXD; ++l) {
      q.m[l] = cs.m[l];
      q.n[l] = cs.n[l];
      q.ld[l] = cs.ld[l];
    }
    q.Nx = cs.Nx;
    q.Ny = cs.Ny;
    q.sxw = cs.sxw;
    EntryPtrs<double> en;
    if (!resolve_entry<double>(q, inst, en)) {
      if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    const size_t fac = fac_bytes(cs);
    int* sExp = reinterpret_cast<int*>(smem + fac);
    float* sNrm = reinterpret_cast<float*>(sExp + MAXD + 2);
    unsigned char* braw = smem + fac + GEN_SPLIT_HDR;
    double *w0, *w1;
    const int nb = on_chip_buffers(cs);
    if (nb == 2) {
      w0 = reinterpret_cast<double*>(braw);
      w1 = reinterpret_cast<double*>(braw + buf_bytes(cs));
    } else if (nb == 1) {
      w0 = reinterpret_cast<double*>(braw);  // one buffer: modes in place
      w1 = nullptr;
    } else {
      w0 = static_cast<double*>(p.Wbase) + (long long)blockIdx.x * p.w_stride;
      w1 = w0 + cs.sxw;
    }
    if (cs.Nx >= 4096) {
      gen_split_entry<4>(q, en, smem, w0, w1, sExp, sNrm, nb != 1, lt, PT, 0);
    } else {
      gen_split_entry<2>(q, en, smem, w0, w1, sExp, sNrm, nb != 1, lt, PT, 0);
    }
    __syncthreads();
  }
}

}  // namespace

// Whether every class of pc fits the persistent kernel (its factors and 4 KB
// of buffer in the CTA's shared memory), and the largest intermediate
// (elements) of the classes that need the workspace (0: none).
bool persistent_fits(const PersistClasses& pc, long long* ws_elems) {
  long long big = 0;
  for (int c = 0; c < pc.count; ++c) {
    const PersistClass& cs = pc.c[c];
    if (fac_bytes(cs) + GEN_SPLIT_HDR + 4096 > (size_t)PSMEM) return false;
    if (on_chip_buffers(cs) == 0 && cs.sxw > big) big = cs.sxw;
  }
  if (ws_elems) *ws_elems = big;
  return true;
}

// p: base problem of the call (L_MIXED, order = instances sorted by class,
// count = all instances, Wbase/w_stride/nslots = the caller's workspace in
// slots of 2 * the largest intermediate); keys: class of each instance;
// queue: a device int, zero at launch.  cudaErrorNotSupported when a class
// does not fit (persistent_fits), cudaErrorInvalidValue when a class needs
// the workspace and p has none.
cudaError_t launch_mixed_persistent(Problem& p, const PersistClasses& pc, const int* keys,
                                    int* queue, cudaStream_t s) {
  long long ws_elems = 0;
  if (!persistent_fits(pc, &ws_elems)) return cudaErrorNotSupported;
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
  if (ws_elems > 0) {
    if (p.Wbase == nullptr || p.nslots < 1 || p.w_stride < 2 * ws_elems)
      return cudaErrorInvalidValue;
    if (grid > p.nslots) grid = p.nslots;
  }
  if (grid < 1) grid = 1;
  void* args[] = {&p, const_cast<PersistClasses*>(&pc), &keys, &queue};
  return cudaLaunchKernel(func, dim3((unsigned)grid), dim3(PT), args, PSMEM, s);
}

}  // namespace kmx
