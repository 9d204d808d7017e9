// kmx_build.cu -- device-side construction of the xbatched pointer arrays
// from (y, x, a) index triples: the step a caller performs before
// kronmult{d}_xbatched (the reference's tests build these arrays on the host
// and copy them over, test_kronmult6_xbatched.cpp:253-321).
//
// Entry e (0 <= e < count) of the batch refers to
//   Y block  Ypool + y_idx[e] * y_stride,
//   X block  Xpool + x_idx[e] * x_stride,
//   factor l Apool + l * a_level_stride + a_idx[e*d + l] * a_pool_stride,
// all strides in elements.  With sort_by_y the entries are first put in
// increasing y order (stable, CUB radix sort on the device), so that the
// entries of one Y block are adjacent in the batch: their atomic updates
// then meet in L2 while the block is resident.  Indices outside
// [0, n_y) / [0, n_x) / [0, n_pool) produce NULL pointers, which the
// kronmult kernels skip and report; the build flags them too.
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include "../../include/kronmult_gb300.h"
#include "kmx_engine.cuh"
#include "kmx_launch.cuh"

namespace kmx {
namespace {

struct BuildArgs {
  int d, count;
  const char* A;
  const char* X;
  const char* Y;
  long long a_level, a_pool, xs, ys;  // strides in bytes
  int n_pool, n_x, n_y;
  const int* y_idx;
  const int* x_idx;
  const int* a_idx;
  const int* order;  // NULL: identity
  const void** pA;
  const void** pX;
  const void** pY;
  int* status;
};

__global__ void build_kernel(BuildArgs b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < b.count; i += gridDim.x * blockDim.x) {
    const int e = b.order ? b.order[i] : i;
    const int yi = b.y_idx[e], xi = b.x_idx[e];
    bool bad = false;
    if (yi >= 0 && yi < b.n_y) {
      b.pY[i] = b.Y + yi * b.ys;
    } else {
      b.pY[i] = nullptr;
      bad = true;
    }
    if (xi >= 0 && xi < b.n_x) {
      b.pX[i] = b.X + xi * b.xs;
    } else {
      b.pX[i] = nullptr;
      bad = true;
    }
    for (int l = 0; l < b.d; ++l) {
      const int ai = b.a_idx[(long long)e * b.d + l];
      if (ai >= 0 && ai < b.n_pool) {
        b.pA[(long long)i * b.d + l] = b.A + l * b.a_level + ai * b.a_pool;
      } else {
        b.pA[(long long)i * b.d + l] = nullptr;
        bad = true;
      }
    }
    if (bad) atomicOr(b.status, DF_BAD_SHAPE);
  }
}

__global__ void iota_kernel(const int* y_idx, int count, int* keys, int* vals) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    keys[i] = y_idx[i];
    vals[i] = i;
  }
}

inline size_t al256(size_t x) { return (x + 255) / 256 * 256; }

struct SortLayout {
  size_t keys, skeys, vals, order, temp, temp_bytes, total;
};

SortLayout sort_layout(int count) {
  SortLayout L;
  const size_t c = (size_t)(count > 0 ? count : 1);
  size_t o = 0;
  L.keys = o;
  o += al256(c * 4);
  L.skeys = o;
  o += al256(c * 4);
  L.vals = o;
  o += al256(c * 4);
  L.order = o;
  o += al256(c * 4);
  size_t t = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, t, (int*)nullptr, (int*)nullptr, (int*)nullptr,
                                  (int*)nullptr, (int)c);
  L.temp_bytes = al256(t);
  L.temp = o;
  o += L.temp_bytes;
  L.total = o;
  return L;
}

int build_impl(int esz, int d, const void* Apool, long long a_level_stride,
               long long a_pool_stride, int n_pool, const void* Xpool, long long x_stride, int n_x,
               const void* Ypool, long long y_stride, int n_y, const int* y_idx, const int* x_idx,
               const int* a_idx, int count, int sort_by_y, void* workspace,
               size_t workspace_bytes, const void** pA, const void** pX, const void** pY,
               cudaStream_t s) {
  if (d < 1 || d > MAXD || count < 0 || n_pool < 0 || n_x < 0 || n_y < 0)
    return KMX_ERR_INVALID_ARG;
  if (a_level_stride < 0 || a_pool_stride < 0 || x_stride < 0 || y_stride < 0)
    return KMX_ERR_INVALID_ARG;
  if (count == 0) return KMX_OK;
  if (!Apool || !Xpool || !Ypool || !y_idx || !x_idx || !a_idx || !pA || !pX || !pY)
    return KMX_ERR_NULL_POINTER;
  BuildArgs b;
  b.d = d;
  b.count = count;
  b.A = static_cast<const char*>(Apool);
  b.X = static_cast<const char*>(Xpool);
  b.Y = static_cast<const char*>(Ypool);
  b.a_level = a_level_stride * esz;
  b.a_pool = a_pool_stride * esz;
  b.xs = x_stride * esz;
  b.ys = y_stride * esz;
  b.n_pool = n_pool;
  b.n_x = n_x;
  b.n_y = n_y;
  b.y_idx = y_idx;
  b.x_idx = x_idx;
  b.a_idx = a_idx;
  b.order = nullptr;
  b.pA = pA;
  b.pX = pX;
  b.pY = pY;
  const SortLayout L = sort_layout(count);
  if (sort_by_y && (!workspace || workspace_bytes < L.total)) return KMX_ERR_WORKSPACE;
  int rc = device_status_ptr(&b.status);
  if (rc != KMX_OK) return rc;
  const int threads = 256;
  int blocks = (count + threads - 1) / threads;
  if (blocks > 8192) blocks = 8192;
  if (sort_by_y) {
    unsigned char* w = static_cast<unsigned char*>(workspace);
    int* keys = reinterpret_cast<int*>(w + L.keys);
    int* skeys = reinterpret_cast<int*>(w + L.skeys);
    int* vals = reinterpret_cast<int*>(w + L.vals);
    int* order = reinterpret_cast<int*>(w + L.order);
    iota_kernel<<<blocks, threads, 0, s>>>(y_idx, count, keys, vals);
    if (cudaGetLastError() != cudaSuccess) return KMX_ERR_CUDA;
    int bits = 1;
    while (bits < 31 && (1LL << bits) <= (long long)n_y) ++bits;
    size_t tb = L.temp_bytes;
    if (cub::DeviceRadixSort::SortPairs(w + L.temp, tb, keys, skeys, vals, order, count, 0, bits,
                                        s) != cudaSuccess)
      return KMX_ERR_CUDA;
    b.order = order;
  }
  build_kernel<<<blocks, threads, 0, s>>>(b);
  return cudaGetLastError() == cudaSuccess ? KMX_OK : KMX_ERR_CUDA;
}

}  // namespace
}  // namespace kmx

extern "C" {

size_t kmx_xbatched_build_workspace_bytes(int count) {
  return kmx::sort_layout(count).total;
}

int kmx_xbatched_build_f64(int d, const double* Apool, long long a_level_stride,
                           long long a_pool_stride, int n_pool, const double* Xpool,
                           long long x_stride, int n_x, double* Ypool, long long y_stride, int n_y,
                           const int* y_idx, const int* x_idx, const int* a_idx, int count,
                           int sort_by_y, void* workspace, size_t workspace_bytes,
                           const double** Aarray, const double** pX, double** pY,
                           kmx_stream_t stream) {
  return kmx::build_impl(8, d, Apool, a_level_stride, a_pool_stride, n_pool, Xpool,
                         x_stride, n_x, Ypool, y_stride, n_y, y_idx, x_idx, a_idx, count,
                         sort_by_y, workspace, workspace_bytes,
                         reinterpret_cast<const void**>(Aarray), reinterpret_cast<const void**>(pX),
                         const_cast<const void**>(reinterpret_cast<void**>(pY)),
                         (cudaStream_t)stream);
}

int kmx_xbatched_build_f32(int d, const float* Apool, long long a_level_stride,
                           long long a_pool_stride, int n_pool, const float* Xpool,
                           long long x_stride, int n_x, float* Ypool, long long y_stride, int n_y,
                           const int* y_idx, const int* x_idx, const int* a_idx, int count,
                           int sort_by_y, void* workspace, size_t workspace_bytes,
                           const float** Aarray, const float** pX, float** pY,
                           kmx_stream_t stream) {
  return kmx::build_impl(4, d, Apool, a_level_stride, a_pool_stride, n_pool, Xpool,
                         x_stride, n_x, Ypool, y_stride, n_y, y_idx, x_idx, a_idx, count,
                         sort_by_y, workspace, workspace_bytes,
                         reinterpret_cast<const void**>(Aarray), reinterpret_cast<const void**>(pX),
                         const_cast<const void**>(reinterpret_cast<void**>(pY)),
                         (cudaStream_t)stream);
}

}  // extern "C"
