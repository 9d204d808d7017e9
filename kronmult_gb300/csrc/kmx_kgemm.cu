// kmx_kgemm.cu -- the stand-alone batched tiny-GEMM entry points
// kgemm_nn_batched / kgemm_nt_batched of the reference
// (kgemm_nn_batched.cpp:8-41, kgemm_nt_batched.cpp:8-41).
//
// For every entry e:  C_e = alpha * A_e * op(B_e) + beta * C_e, column-major,
// A_e mm x kk, C_e mm x nn, op(B) = B (kk x nn) or B^T (B nn x kk), each
// matrix with its own leading dimension from a device array.  The epilogue
// keeps the reference's three cases (kgemm_nn.hpp:388-400,
// kgemm_nt.hpp:365-376): beta == 1 adds with an atomic (entries may share C),
// beta == 0 stores, anything else blends beta*C + alpha*c.
//
// Design: the work is (entry, row tile, column tile) items, taken by a
// persistent grid in a grid-stride loop.  A CTA of 256 threads stages a
// BK-deep slice of A (BM x BK) and op(B) (BK x BN) in shared memory, both
// k-major so that one k step reads a row of each, and every thread keeps a
// TM x TN register tile of C.  Tile shapes are picked from the call's shape:
// the kronmult contractions are either short-and-wide (mm = n, nn = n^(d-1))
// or tall-and-narrow (mm = n^(d-1), nn = n), and a square 64 x 64 tile
// would leave most of each tile empty on both.
#include <cuda_runtime.h>

#include "../../include/kronmult_gb300.h"
#include "kmx_engine.cuh"
#include "kmx_launch.cuh"

namespace kmx {
namespace {

template <typename T>
struct KgArgs {
  int mm, nn, kk;
  T alpha, beta;
  const T* const* A;
  const int* ldA;
  const T* const* B;
  const int* ldB;
  T* const* C;
  const int* ldC;
  int tiles_m, tiles_n;
  long long items;
  int* status;
};

// Dot-product accumulator.  FP64: one FP64 fused multiply-add per term.
// FP32: the reference accumulates FP32 data in double (kgemm_nn.hpp:688-701,
// kgemm_nt.hpp:557-571); here the sum is kept as an unevaluated pair of FP32
// values (s + c) with exact products (FMA residual) and an exact two-sum per
// term, about 48 bits, so the stored result carries one rounding to FP32 as
// in the reference, without using the FP64 pipe.
template <typename T>
struct Acc;

template <>
struct Acc<double> {
  double s;
  __device__ __forceinline__ void zero() { s = 0.0; }
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  template <bool TRANS_B>
  __device__ __forceinline__ void store(double* p, double alpha, double beta) const {
    const double v = alpha * s;  // kgemm_nn.hpp:390 / kgemm_nt.hpp:368
    if (beta == 1.0) {
      atomicAdd(p, v);
    } else if (beta == 0.0) {
      *p = v;
    } else {
      *p = fma(beta, *p, v);
    }
  }
};

template <>
struct Acc<float> {
  float s, c;
  __device__ __forceinline__ void zero() { s = c = 0.f; }
  __device__ __forceinline__ void add(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    const float t = __fadd_rn(s, p);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, e));
  }
  template <bool TRANS_B>
  __device__ __forceinline__ void store(float* p, float alpha, float beta) const {
    // renormalise (t, l) = s + c, then alpha*(t + l) with one rounding
    const float t = __fadd_rn(s, c);
    const float l = __fsub_rn(c, __fsub_rn(t, s));
    const float al = __fmul_rn(alpha, l);
    if (beta == 1.f) {
      atomicAdd(p, __fmaf_rn(alpha, t, al));
    } else if (beta == 0.f) {
      *p = __fmaf_rn(alpha, t, al);
    } else if (TRANS_B) {
      // nt blends beta*C + alpha*c before rounding (kgemm_nt.hpp:375)
      const float bc = __fmul_rn(beta, *p);
      const float be = __fmaf_rn(beta, *p, -bc);
      *p = __fadd_rn(__fmaf_rn(alpha, t, bc), __fadd_rn(al, be));
    } else {
      // nn rounds alpha*c first, then blends (kgemm_nn.hpp:390-399)
      *p = __fmaf_rn(beta, *p, __fmaf_rn(alpha, t, al));
    }
  }
};

constexpr int KG_THREADS = 256;
constexpr int KG_BK = 16;

template <typename T, bool TRANS_B, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__(KG_THREADS) kgemm_kernel(KgArgs<T> a) {
  constexpr int RT = BM / TM;  // threads along rows
  constexpr int CT = BN / TN;  // threads along columns
  static_assert(RT * CT == KG_THREADS, "tile does not match the block");
  __shared__ T As[KG_BK][BM + 1];
  __shared__ T Bs[KG_BK][BN + 1];
  const int tid = threadIdx.x;
  const int tr = tid % RT, tc = tid / RT;
  const long long per_entry = (long long)a.tiles_m * a.tiles_n;

  for (long long item = blockIdx.x; item < a.items; item += gridDim.x) {
    const int e = (int)(item / per_entry);
    const int rem = (int)(item - (long long)e * per_entry);
    const int m0 = (rem % a.tiles_m) * BM;
    const int n0 = (rem / a.tiles_m) * BN;
    const T* __restrict__ Ap = a.A[e];
    const T* __restrict__ Bp = a.B[e];
    T* Cp = a.C[e];
    const long long lda = a.ldA[e], ldb = a.ldB[e], ldc = a.ldC[e];
    // uniform over the CTA: every thread reads the same entry
    const bool need_ab = a.kk > 0;
    if (Cp == nullptr || (need_ab && (Ap == nullptr || Bp == nullptr))) {
      if (tid == 0) atomicOr(a.status, DF_NULL_PTR);
      continue;
    }
    if (ldc < a.mm || (need_ab && (lda < a.mm || ldb < (TRANS_B ? a.nn : a.kk)))) {
      if (tid == 0) atomicOr(a.status, DF_BAD_SHAPE);
      continue;
    }
    Acc<T> acc[TM][TN];
#pragma unroll
    for (int r = 0; r < TM; ++r)
#pragma unroll
      for (int c = 0; c < TN; ++c) acc[r][c].zero();

    for (int k0 = 0; k0 < a.kk; k0 += KG_BK) {
      const int kc = min(KG_BK, a.kk - k0);
      __syncthreads();  // the previous slice has been consumed
      for (int idx = tid; idx < BM * kc; idx += KG_THREADS) {
        const int i = idx % BM, k = idx / BM;
        const int gi = m0 + i;
        As[k][i] = gi < a.mm ? Ap[gi + (k0 + k) * lda] : T(0);
      }
      if (TRANS_B) {
        for (int idx = tid; idx < BN * kc; idx += KG_THREADS) {
          const int j = idx % BN, k = idx / BN;
          const int gj = n0 + j;
          Bs[k][j] = gj < a.nn ? Bp[gj + (k0 + k) * ldb] : T(0);
        }
      } else {
        for (int idx = tid; idx < BN * kc; idx += KG_THREADS) {
          const int j = idx / kc, k = idx - j * kc;
          const int gj = n0 + j;
          Bs[k][j] = gj < a.nn ? Bp[(k0 + k) + gj * ldb] : T(0);
        }
      }
      __syncthreads();
      for (int k = 0; k < kc; ++k) {
        T av[TM], bv[TN];
#pragma unroll
        for (int r = 0; r < TM; ++r) av[r] = As[k][tr + r * RT];
#pragma unroll
        for (int c = 0; c < TN; ++c) bv[c] = Bs[k][tc + c * CT];
#pragma unroll
        for (int r = 0; r < TM; ++r)
#pragma unroll
          for (int c = 0; c < TN; ++c) acc[r][c].add(av[r], bv[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < TN; ++c) {
      const int j = n0 + tc + c * CT;
      if (j >= a.nn) continue;
#pragma unroll
      for (int r = 0; r < TM; ++r) {
        const int i = m0 + tr + r * RT;
        if (i >= a.mm) continue;
        acc[r][c].template store<TRANS_B>(Cp + i + j * ldc, a.alpha, a.beta);
      }
    }
  }
}

// Small matrices (mm*nn <= 2048): one warp per entry, each lane computes
// outputs in a strided loop straight from global memory (the entry's A and
// B stay in L1); no shared memory, no block barriers.
template <typename T, bool TRANS_B>
__global__ void __launch_bounds__(KG_THREADS) kgemm_small_kernel(KgArgs<T> a) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (KG_THREADS / 32);
  const int outs = a.mm * a.nn;
  for (long long e = (long long)blockIdx.x * (KG_THREADS / 32) + (threadIdx.x >> 5); e < a.items;
       e += warps) {
    const T* __restrict__ Ap = a.A[e];
    const T* __restrict__ Bp = a.B[e];
    T* Cp = a.C[e];
    const long long lda = a.ldA[e], ldb = a.ldB[e], ldc = a.ldC[e];
    const bool need_ab = a.kk > 0;
    if (Cp == nullptr || (need_ab && (Ap == nullptr || Bp == nullptr))) {
      if (lane == 0) atomicOr(a.status, DF_NULL_PTR);
      continue;
    }
    if (ldc < a.mm || (need_ab && (lda < a.mm || ldb < (TRANS_B ? a.nn : a.kk)))) {
      if (lane == 0) atomicOr(a.status, DF_BAD_SHAPE);
      continue;
    }
    for (int o = lane; o < outs; o += 32) {
      const int j = o / a.mm, i = o - j * a.mm;
      Acc<T> acc;
      acc.zero();
      for (int k = 0; k < a.kk; ++k) {
        const T av = __ldg(Ap + i + k * lda);
        const T bv = TRANS_B ? __ldg(Bp + j + k * ldb) : __ldg(Bp + k + j * ldb);
        acc.add(av, bv);
      }
      acc.template store<TRANS_B>(Cp + i + j * ldc, a.alpha, a.beta);
    }
  }
}

// Streaming kernels (FP32) for the kronmult shapes, whose inner dimensions
// are tiny (kk <= 16) and one output dimension is long:
//   nn (short-wide, mm <= 16): thread = one column j of C; it reads B(:, j)
//     (kk contiguous values), keeps A (mm x kk) in shared memory, writes the
//     mm values of C(:, j) -- a warp sweeps 32 consecutive columns, so B and C
//     stream through in full sectors;
//   nt (tall-narrow, nn <= 16): thread = one row i of C; it reads A(i, :)
//     (kk values, stride ldA), keeps B (nn x kk) in shared memory, writes the
//     nn values of C(i, :) -- consecutive threads take consecutive rows.
// Items are (entry, chunk of 256 columns / rows), grid-stride.
constexpr int KG_SMALL_DIM = 16;
template <typename T, bool TRANS_B>
__global__ void __launch_bounds__(KG_THREADS) kgemm_stream_kernel(KgArgs<T> a) {
  __shared__ T S[KG_SMALL_DIM * KG_SMALL_DIM];  // A (nn form) or B (nt form), column-major
  const int tid = threadIdx.x;
  const int big = TRANS_B ? a.mm : a.nn;         // the long dimension
  const int chunks = (big + KG_THREADS - 1) / KG_THREADS;
  for (long long item = blockIdx.x; item < a.items; item += gridDim.x) {
    const int e = (int)(item / chunks);
    const int c0 = (int)(item - (long long)e * chunks) * KG_THREADS;
    const T* __restrict__ Ap = a.A[e];
    const T* __restrict__ Bp = a.B[e];
    T* Cp = a.C[e];
    const long long lda = a.ldA[e], ldb = a.ldB[e], ldc = a.ldC[e];
    const bool need_ab = a.kk > 0;
    __syncthreads();  // the previous item is done with S
    if (Cp == nullptr || (need_ab && (Ap == nullptr || Bp == nullptr))) {
      if (tid == 0 && c0 == 0) atomicOr(a.status, DF_NULL_PTR);
      continue;
    }
    if (ldc < a.mm || (need_ab && (lda < a.mm || ldb < (TRANS_B ? a.nn : a.kk)))) {
      if (tid == 0 && c0 == 0) atomicOr(a.status, DF_BAD_SHAPE);
      continue;
    }
    // the small operand: A (mm x kk) for nn, B (nn x kk) for nt, as S[r + k*16]
    const int rows = TRANS_B ? a.nn : a.mm;
    for (int idx = tid; idx < rows * a.kk; idx += KG_THREADS) {
      const int r = idx % rows, k = idx / rows;
      S[r + k * KG_SMALL_DIM] = TRANS_B ? Bp[r + k * ldb] : Ap[r + k * lda];
    }
    __syncthreads();
    const int c = c0 + tid;
    if (c >= big) continue;
    T v[KG_SMALL_DIM];
#pragma unroll
    for (int k = 0; k < KG_SMALL_DIM; ++k)
      if (k < a.kk) v[k] = TRANS_B ? __ldg(Ap + c + k * lda) : __ldg(Bp + k + (long long)c * ldb);
#pragma unroll
    for (int r = 0; r < KG_SMALL_DIM; ++r) {
      if (r >= rows) break;
      Acc<T> acc;
      acc.zero();
#pragma unroll
      for (int k = 0; k < KG_SMALL_DIM; ++k)
        if (k < a.kk) acc.add(S[r + k * KG_SMALL_DIM], v[k]);
      // nn: C(r, c); nt: C(c, r)
      T* p = TRANS_B ? Cp + c + r * ldc : Cp + r + (long long)c * ldc;
      acc.template store<TRANS_B>(p, a.alpha, a.beta);
    }
  }
}

struct KgConfig {
  const void* func;
  int bm, bn;
};

template <typename T, bool TB>
KgConfig pick_kgemm(int mm, int nn) {
  if (mm > 64 && nn <= 8) return {(const void*)kgemm_kernel<T, TB, 256, 8, 4, 2>, 256, 8};
  if (mm <= 4) return {(const void*)kgemm_kernel<T, TB, 4, 256, 1, 4>, 4, 256};
  if (mm <= 8) return {(const void*)kgemm_kernel<T, TB, 8, 128, 1, 4>, 8, 128};
  if (mm <= 16) return {(const void*)kgemm_kernel<T, TB, 16, 128, 2, 4>, 16, 128};
  return {(const void*)kgemm_kernel<T, TB, 64, 64, 4, 4>, 64, 64};
}

template <typename T>
int kgemm_impl(bool trans_b, int mm, int nn, int kk, T alpha, const T* const* A, const int* ldA,
               const T* const* B, const int* ldB, T beta, T* const* C, const int* ldC, int batch,
               cudaStream_t s) {
  if (mm < 0 || nn < 0 || kk < 0 || batch < 0) return KMX_ERR_INVALID_ARG;
  if (batch == 0 || mm == 0 || nn == 0) return KMX_OK;
  if (!C || !ldC) return KMX_ERR_NULL_POINTER;
  if (kk > 0 && (!A || !ldA || !B || !ldB)) return KMX_ERR_NULL_POINTER;
  const bool small = (long long)mm * nn <= 2048;
  // streaming: tiny inner and short dimension, long other dimension; FP32
  // only (these shapes are HBM-bound in FP32, FP64-FMA-bound in FP64, where
  // the register tiles' several outputs per thread measure faster)
  const bool stream = sizeof(T) == 4 && !small && kk <= KG_SMALL_DIM &&
                      (trans_b ? (nn <= KG_SMALL_DIM) : (mm <= KG_SMALL_DIM));
  KgConfig cfg = trans_b ? pick_kgemm<T, true>(mm, nn) : pick_kgemm<T, false>(mm, nn);
  if (stream) {
    cfg.func = trans_b ? (const void*)kgemm_stream_kernel<T, true>
                       : (const void*)kgemm_stream_kernel<T, false>;
    // items: (entry, chunk of KG_THREADS along the long dimension)
    cfg.bm = trans_b ? KG_THREADS : mm;
    cfg.bn = trans_b ? nn : KG_THREADS;
  } else if (small) {
    cfg.func = trans_b ? (const void*)kgemm_small_kernel<T, true>
                       : (const void*)kgemm_small_kernel<T, false>;
    cfg.bm = mm;
    cfg.bn = nn;
  }
  KgArgs<T> ka;
  ka.mm = mm;
  ka.nn = nn;
  ka.kk = kk;
  ka.alpha = alpha;
  ka.beta = beta;
  ka.A = A;
  ka.ldA = ldA;
  ka.B = B;
  ka.ldB = ldB;
  ka.C = C;
  ka.ldC = ldC;
  ka.tiles_m = (mm + cfg.bm - 1) / cfg.bm;
  ka.tiles_n = (nn + cfg.bn - 1) / cfg.bn;
  ka.items = (long long)batch * ka.tiles_m * ka.tiles_n;  // small kernel: one item per entry
  int rc = device_status_ptr(&ka.status);
  if (rc != KMX_OK) return rc;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KMX_ERR_CUDA;
  const DeviceInfo di = device_info(dev);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cfg.func, KG_THREADS, 0);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)di.sms * per_sm;
  const long long cta_items = small ? (ka.items + KG_THREADS / 32 - 1) / (KG_THREADS / 32) : ka.items;
  if (grid > cta_items) grid = cta_items;
  void* args[] = {&ka};
  const cudaError_t e = cudaLaunchKernel(cfg.func, dim3((unsigned)grid), dim3(KG_THREADS), args, 0, s);
  return e == cudaSuccess ? KMX_OK : KMX_ERR_CUDA;
}

}  // namespace
}  // namespace kmx

extern "C" {

int kmx_kgemm_nn_batched_f64(int mm, int nn, int kk, double alpha, double* const* Aarray,
                             const int* ldAarray, double* const* Barray, const int* ldBarray,
                             double beta, double* const* Carray, const int* ldCarray,
                             int batchCount, kmx_stream_t stream) {
  return kmx::kgemm_impl<double>(false, mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray,
                                 beta, Carray, ldCarray, batchCount, (cudaStream_t)stream);
}

int kmx_kgemm_nt_batched_f64(int mm, int nn, int kk, double alpha, double* const* Aarray,
                             const int* ldAarray, double* const* Barray, const int* ldBarray,
                             double beta, double* const* Carray, const int* ldCarray,
                             int batchCount, kmx_stream_t stream) {
  return kmx::kgemm_impl<double>(true, mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray,
                                 beta, Carray, ldCarray, batchCount, (cudaStream_t)stream);
}

int kmx_kgemm_nn_batched_f32(int mm, int nn, int kk, float alpha, float* const* Aarray,
                             const int* ldAarray, float* const* Barray, const int* ldBarray,
                             float beta, float* const* Carray, const int* ldCarray,
                             int batchCount, kmx_stream_t stream) {
  return kmx::kgemm_impl<float>(false, mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray,
                                beta, Carray, ldCarray, batchCount, (cudaStream_t)stream);
}

int kmx_kgemm_nt_batched_f32(int mm, int nn, int kk, float alpha, float* const* Aarray,
                             const int* ldAarray, float* const* Barray, const int* ldBarray,
                             float beta, float* const* Carray, const int* ldCarray,
                             int batchCount, kmx_stream_t stream) {
  return kmx::kgemm_impl<float>(true, mm, nn, kk, alpha, Aarray, ldAarray, Barray, ldBarray,
                                beta, Carray, ldCarray, batchCount, (cudaStream_t)stream);
}

}  // extern "C"
