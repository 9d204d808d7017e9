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

// Bulk-copy streaming kernel for FP32 kgemm_nn with mm, kk <= 16 (the
// kronmult short-wide contractions), warp-specialised: items are (entry,
// chunk of 256 columns), grid-stride per CTA, cycling through KB_STAGES
// shared-memory stages.
//   producer warp: for each item, waits until its stage is empty, reads the
//     entry's pointers and leading dimensions, writes A as row pairs
//     (A(2rp, k), A(2rp+1, k)) and an item descriptor into the stage, and
//     fetches the B chunk (kk x 256, contiguous when ldB == kk) and, for beta
//     outside {0, 1}, the C chunk by cp.async.bulk, completing on the stage's
//     "full" mbarrier -- up to KB_STAGES items ahead of the consumers;
//   8 consumer warps: each thread forms one column of C from its B column and
//     A, two rows per instruction on packed FP32 pairs with the same
//     double-length accumulation (exact products, two-sums, one rounding) as
//     Acc<float>; the results leave by one cp.async.bulk store (beta == 0, or
//     the blend) or one cp.reduce.async.bulk .add (beta == 1: element-wise
//     atomic adds, the reference's atomicAdd epilogue); once that copy has
//     read the stage (checked one item later, so the wait is off the item's
//     path) the stage's "empty" mbarrier releases it to the producer.
// Bulk copies cover each chunk from its first 16-byte boundary in whole 16-byte
// units; the few elements before and after are read and written directly.
// Items whose B or C is not contiguous (ldB != kk, ldC != mm) read and write
// global memory directly, with the same arithmetic.  The pointer and A reads
// of the producer run two and one items ahead.  The square shapes n = 2..8
// are compiled with mm = kk = n as constants: with run-time sizes the
// guarded, fully unrolled loops cost 3.7x the instructions (ncu, n = 4).
// Waits are bounded: one that runs out flags DF_WAIT_TIMEOUT, waits once more
// (with the same bound) for every bulk copy the producer may have issued into
// the stages, and leaves.
constexpr int KB_STAGES = 4;
constexpr int KB_CONSUMERS = 256;
constexpr int KB_THREADS = KB_CONSUMERS + 32;

struct KbDesc {
  float* C;
  const float* B;
  long long ldb, ldc;
  int c0, cw, flag;  // flag: 0 direct, 1 bulk, 2 skip (bad pointer or shape)
  // bulk items: the chunk's B (kk*cw floats) and C (mm*cw floats) are read
  // and written by bulk copies from the first 16-byte boundary (head hb, hc
  // floats) for mb, mc floats (multiples of 4); the head and the tail go
  // directly to global memory
  int hb, mb, hc, mc;
  int pad;
};

__device__ __forceinline__ void kb_mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tile::smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void kb_store(float* dst, const float* src, uint32_t bytes, bool add) {
  if (add) {
    asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f32 [%0], [%1], %2;" ::"l"(
                     dst),
                 "r"(tile::smem_u32(src)), "r"(bytes)
                 : "memory");
  } else {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                 "r"(tile::smem_u32(src)), "r"(bytes)
                 : "memory");
  }
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void kb_consumer_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(KB_CONSUMERS) : "memory");
}

// One stage, in floats: B chunk, C chunk (each rounded to 16 bytes), the A
// row pairs [8][16] (u64).  After the stages: full and empty mbarriers, the
// item descriptors and a timeout flag.
// (each chunk area has 4 floats in front for the head's shift)
__host__ __device__ constexpr int kb_c_off(int kk) { return 4 + (kk * KB_CONSUMERS + 3) / 4 * 4; }
__host__ __device__ constexpr int kb_a_off(int mm, int kk) {
  return kb_c_off(kk) + 4 + (mm * KB_CONSUMERS + 3) / 4 * 4;
}
__host__ __device__ constexpr int kb_stage_floats(int mm, int kk) {
  return kb_a_off(mm, kk) + 8 * KG_SMALL_DIM * 2;
}
__host__ __device__ constexpr size_t kb_smem_bytes(int mm, int kk) {
  return (size_t)KB_STAGES * kb_stage_floats(mm, kk) * 4 + 2 * KB_STAGES * 8 +
         KB_STAGES * sizeof(KbDesc) + 16;
}

// MM, KK: the shape as compile-time constants (the square kronmult shapes,
// fully unrolled), or 0 for run-time mm, kk <= 16.
template <int MM, int KK>
__global__ void __launch_bounds__(KB_THREADS) kgemm_bulk_kernel(KgArgs<float> a) {
  using pk2::u64;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x;
  const int mm = MM ? MM : a.mm, kk = KK ? KK : a.kk, nn = a.nn;
  constexpr int QN = KK ? KK : KG_SMALL_DIM;            // k loop bound
  constexpr int RPN = MM ? (MM + 1) / 2 : KG_SMALL_DIM / 2;  // row-pair loop bound
  const int SF = kb_stage_floats(mm, kk), COFF = kb_c_off(kk), AOFF = kb_a_off(mm, kk);
  float* stg = reinterpret_cast<float*>(smem);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)KB_STAGES * SF * 4);
  uint64_t* empty = full + KB_STAGES;
  KbDesc* desc = reinterpret_cast<KbDesc*>(empty + KB_STAGES);
  int* sstop = reinterpret_cast<int*>(desc + KB_STAGES);
  const int chunks = (nn + KB_CONSUMERS - 1) / KB_CONSUMERS;
  const bool beta0 = a.beta == 0.f, beta1 = a.beta == 1.f;
  const int RP = (mm + 1) / 2;
  if (tid == 0) {
    for (int s = 0; s < KB_STAGES; ++s) {
      tile::mbar_init(&full[s], 1);
      tile::mbar_init(&empty[s], 1);
    }
    sstop[0] = 0;
    tile::fence_mbar_init();
  }
  __syncthreads();

  if (tid < 32) {  // ---- producer warp ----
    // Software pipeline: an item's pointers are read two items ahead and its
    // A values one item ahead, so their global latencies overlap the waits
    // for free stages instead of adding up item after item.
    const int lane = tid;
    struct Ptrs {
      const float* A;
      const float* B;
      float* C;
      long long lda, ldb, ldc;
      int e, c0;
      bool ok;  // pointers present and leading dimensions valid
    };
    auto load_ptrs = [&](long long it, Ptrs& p) {
      p.ok = false;
      p.e = 0;
      p.c0 = 0;
      p.A = p.B = nullptr;
      p.C = nullptr;
      p.lda = p.ldb = p.ldc = 0;
      if (it >= a.items) return;
      p.e = (int)(it / chunks);
      p.c0 = (int)(it - (long long)p.e * chunks) * KB_CONSUMERS;
      p.A = a.A[p.e];
      p.B = a.B[p.e];
      p.C = a.C[p.e];
      p.lda = a.ldA[p.e];
      p.ldb = a.ldB[p.e];
      p.ldc = a.ldC[p.e];
    };
    auto check = [&](Ptrs& p) {
      const bool bad_ptr = p.C == nullptr || (kk > 0 && (p.A == nullptr || p.B == nullptr));
      const bool bad_ld = !bad_ptr && (p.ldc < mm || (kk > 0 && (p.lda < mm || p.ldb < kk)));
      p.ok = !bad_ptr && !bad_ld;
      return bad_ptr ? DF_NULL_PTR : (bad_ld ? DF_BAD_SHAPE : 0);
    };
    constexpr int AV = 8 * KG_SMALL_DIM / 32;  // A row-pair slots per lane
    auto load_a = [&](const Ptrs& p, float (&v0)[AV], float (&v1)[AV]) {
#pragma unroll
      for (int j = 0; j < AV; ++j) {
        const int idx = lane + 32 * j;
        v0[j] = v1[j] = 0.f;
        if (p.ok && idx < RP * kk) {
          const int rp = idx / kk, q = idx - rp * kk;
          v0[j] = p.A[2 * rp + q * p.lda];
          if (2 * rp + 1 < mm) v1[j] = p.A[2 * rp + 1 + q * p.lda];
        }
      }
    };
    Ptrs cur, nxt, nn2;
    load_ptrs(blockIdx.x, cur);
    load_ptrs(blockIdx.x + (long long)gridDim.x, nxt);
    int bad_cur = check(cur);
    float a0[AV], a1[AV];
    load_a(cur, a0, a1);
    for (int k = 0;; ++k) {
      const long long it = blockIdx.x + (long long)k * gridDim.x;
      if (it >= a.items) break;
      const int s = k % KB_STAGES;
      load_ptrs(it + 2LL * gridDim.x, nn2);  // two ahead
      if (k >= KB_STAGES) {  // the consumers released the stage's previous item
        bool ok = true;
        if (lane == 0) ok = tile::mbar_wait(&empty[s], (uint32_t)(k / KB_STAGES - 1) & 1u);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) {
          if (lane == 0) atomicOr(a.status, DF_WAIT_TIMEOUT);
          return;  // the consumers' bounded waits end them
        }
      }
      const int cw = min(KB_CONSUMERS, nn - cur.c0);
      float* st = stg + (size_t)s * SF;
      u64* sAp = reinterpret_cast<u64*>(st + AOFF);
#pragma unroll
      for (int j = 0; j < AV; ++j) {
        const int idx = lane + 32 * j;
        if (cur.ok && idx < RP * kk) {
          const int rp = idx / kk, q = idx - rp * kk;
          sAp[rp * KG_SMALL_DIM + q] = pk2::pack(a0[j], a1[j]);
        }
      }
      __syncwarp();
      if (lane == 0) {
        KbDesc dd;
        dd.C = cur.C;
        dd.B = cur.B;
        dd.ldb = cur.ldb;
        dd.ldc = cur.ldc;
        dd.c0 = cur.c0;
        dd.cw = cw;
        dd.flag = 0;
        dd.hb = dd.mb = dd.hc = dd.mc = 0;
        dd.pad = 0;
        if (!cur.ok) {
          dd.flag = 2;
          if (cur.c0 == 0) atomicOr(a.status, bad_cur);
        } else if (kk > 0 && cur.ldb == kk && cur.ldc == mm) {
          dd.flag = 1;
          // aligned middle of each chunk: from the first 16-byte boundary,
          // whole 16-byte units
          const float* gB = cur.B + (long long)cur.c0 * kk;
          const float* gC = cur.C + (long long)cur.c0 * mm;
          const int nb = kk * cw, nc = mm * cw;
          dd.hb = min(nb, (int)(((16 - (reinterpret_cast<uintptr_t>(gB) & 15)) & 15) >> 2));
          dd.mb = (nb - dd.hb) / 4 * 4;
          dd.hc = min(nc, (int)(((16 - (reinterpret_cast<uintptr_t>(gC) & 15)) & 15) >> 2));
          dd.mc = (nc - dd.hc) / 4 * 4;
        }
        desc[s] = dd;
        const bool loadc = !beta0 && !beta1;
        const uint32_t tx = (dd.flag == 1) ? (uint32_t)(dd.mb + (loadc ? dd.mc : 0)) * 4u : 0u;
        if (tx > 0) {
          tile::fence_proxy_async();
          tile::mbar_expect_tx(&full[s], tx);
          if (dd.mb > 0)
            tile::tma_load_1d(st + 4, cur.B + (long long)cur.c0 * kk + dd.hb, (uint32_t)dd.mb * 4u,
                              &full[s]);
          if (loadc && dd.mc > 0)
            tile::tma_load_1d(st + COFF + 4, cur.C + (long long)cur.c0 * mm + dd.hc,
                              (uint32_t)dd.mc * 4u, &full[s]);
        } else {
          kb_mbar_arrive(&full[s]);
        }
      }
      __syncwarp();
      // advance: the next item's A now (its pointers arrived last iteration)
      cur = nxt;
      nxt = nn2;
      bad_cur = check(cur);
      load_a(cur, a0, a1);
    }
    return;
  }

  // ---- consumer warps ----
  const int ct = tid - 32;
  const u64 alpha2 = pk2::bcast(a.alpha), beta2 = pk2::bcast(a.beta);
  int last_stage = -1;
  for (int k = 0;; ++k) {
    const long long it = blockIdx.x + (long long)k * gridDim.x;
    if (it >= a.items) break;
    const int s = k % KB_STAGES;
    const uint32_t par = (uint32_t)(k / KB_STAGES) & 1u;
    if (ct == 0 && !tile::mbar_wait(&full[s], par)) {
      atomicOr(a.status, DF_WAIT_TIMEOUT);
      tile::mbar_wait(&full[s], par);  // the stage's copies, once more
      // The producer may already have issued items k+1 and k+2 (stages are
      // released one item late, so items up to k-2 are free): wait for their
      // copies too, under the same bound, so that no bulk copy is still
      // writing shared memory when the CTA leaves.
      for (int j = 1; j <= KB_STAGES - 2; ++j) {
        if (it + (long long)j * gridDim.x >= a.items) break;
        tile::mbar_wait(&full[(k + j) % KB_STAGES], (uint32_t)((k + j) / KB_STAGES) & 1u);
      }
      sstop[0] = 1;
    }
    kb_consumer_sync();  // stage s has arrived (the leader saw its mbarrier)
    if (sstop[0]) {
      if (ct == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
      return;
    }
    const KbDesc dd = desc[s];
    float* st = stg + (size_t)s * SF;
    const u64* sAp = reinterpret_cast<const u64*>(st + AOFF);
    const bool bulk = dd.flag == 1;
    if (dd.flag != 2 && ct < dd.cw) {
      const int c = dd.c0 + ct;
      // element e of this column's B / C: bulk items index the chunk (B at
      // bb[e0b + q], staged in sB for hb <= e < hb + mb), direct items the
      // column in global memory
      const float* bb = bulk ? dd.B + (long long)dd.c0 * kk : dd.B + (long long)c * dd.ldb;
      float* cb = bulk ? dd.C + (long long)dd.c0 * mm : dd.C + (long long)c * dd.ldc;
      const int e0b = bulk ? ct * kk : 0, e0c = bulk ? ct * mm : 0;
      const int hb = dd.hb, mb = dd.mb, hc = dd.hc, mc = dd.mc;
      const float* sB = st + 4 - hb;
      float* sC = st + COFF + 4 - hc;
      u64 b2[QN], nb2[QN];
      if (KK % 4 == 0 && KK > 0 && bulk && hb == 0 && e0b + QN <= mb) {  // 16-byte loads
#pragma unroll
        for (int q = 0; q < QN; q += 4) {
          const float4 v = *reinterpret_cast<const float4*>(sB + e0b + q);
          const float w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            b2[q + u] = pk2::bcast(w[u]);
            nb2[q + u] = pk2::bcast(-w[u]);
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < QN; ++q) {
          if (KK || q < kk) {
            const int e = e0b + q;
            const float v = (e >= hb && e < hb + mb) ? sB[e] : __ldg(bb + e);
            b2[q] = pk2::bcast(v);
            nb2[q] = pk2::bcast(-v);
          }
        }
      }
#pragma unroll(MM ? RPN : 1)
      for (int rp = 0; rp < (MM ? RPN : RP); ++rp) {
        u64 ns = 0ull, cc = 0ull;
#pragma unroll
        for (int q = 0; q < QN; ++q) {
          if (KK || q < kk) {
            const u64 a2 = sAp[rp * KG_SMALL_DIM + q];
            const u64 qq = pk2::mul(a2, nb2[q]);     // -p, rounded
            const u64 ee = pk2::fma(a2, b2[q], qq);  // a b - p, exact
            u64 t, te;
            pk2::two_sum(ns, qq, t, te);
            ns = t;
            cc = pk2::add(cc, pk2::sub(ee, te));
          }
        }
        // alpha (t + l) with one rounding, t + l = s + c renormalised
        const u64 th = pk2::sub(cc, ns);
        const u64 tl = pk2::sub(cc, pk2::add(th, ns));
        u64 v = pk2::fma(alpha2, th, pk2::mul(alpha2, tl));
        const int r0 = 2 * rp;
        const bool two = r0 + 1 < mm;
        // rows r0, r0 + 1 of column c: elements e, e + 1 (staged or global)
        const int e = e0c + r0;
        const bool in0 = e >= hc && e < hc + mc, in1 = e + 1 >= hc && e + 1 < hc + mc;
        if (!beta0 && !beta1) {  // nn rounds alpha*c, then blends (kgemm_nn.hpp:390-399)
          const float o0 = in0 ? sC[e] : cb[e];
          const float o1 = two ? (in1 ? sC[e + 1] : cb[e + 1]) : 0.f;
          v = pk2::fma(beta2, pk2::pack(o0, o1), v);
        }
        if (MM % 2 == 0 && MM > 0 && hc == 0 && in0 && in1) {  // one 8-byte store
          *reinterpret_cast<u64*>(sC + e) = v;
        } else {
          float v0, v1;
          pk2::unpack(v, v0, v1);
          if (in0) {
            sC[e] = v0;
          } else if (beta1) {
            atomicAdd(cb + e, v0);
          } else {
            cb[e] = v0;
          }
          if (two) {
            if (in1) {
              sC[e + 1] = v1;
            } else if (beta1) {
              atomicAdd(cb + e + 1, v1);
            } else {
              cb[e + 1] = v1;
            }
          }
        }
      }
    }
    if (bulk) tile::fence_proxy_async();  // results visible to the bulk copy
    kb_consumer_sync();                   // every column done; B and C read
    if (ct == 0) {
      // issue this item's result copy, then release the PREVIOUS item's stage
      // once every copy but this one has read its source (waiting for this
      // one's read here would put it on every item's path)
      if (bulk && dd.mc > 0)
        kb_store(dd.C + (long long)dd.c0 * mm + dd.hc, st + COFF + 4, (uint32_t)dd.mc * 4u, beta1);
      else
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");  // an empty group keeps the count
      if (k > 0) {
        asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        kb_mbar_arrive(&empty[(k + KB_STAGES - 1) % KB_STAGES]);
      }
    }
    last_stage = s;
  }
  if (ct == 0) {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    if (last_stage >= 0) kb_mbar_arrive(&empty[last_stage]);
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
  // the nn streaming shapes take the bulk-copy kernel, and so do nn matrices
  // of at most 2048 outputs with 128 or more columns (one item per entry)
  const bool bulk = sizeof(T) == 4 && !trans_b && kk <= KG_SMALL_DIM && mm <= KG_SMALL_DIM &&
                    (stream || nn >= 128);
  KgConfig cfg = trans_b ? pick_kgemm<T, true>(mm, nn) : pick_kgemm<T, false>(mm, nn);
  size_t smem = 0;
  if (bulk) {
    switch (mm == kk ? mm : 0) {
      case 2: cfg.func = (const void*)kgemm_bulk_kernel<2, 2>; break;
      case 3: cfg.func = (const void*)kgemm_bulk_kernel<3, 3>; break;
      case 4: cfg.func = (const void*)kgemm_bulk_kernel<4, 4>; break;
      case 5: cfg.func = (const void*)kgemm_bulk_kernel<5, 5>; break;
      case 6: cfg.func = (const void*)kgemm_bulk_kernel<6, 6>; break;
      case 7: cfg.func = (const void*)kgemm_bulk_kernel<7, 7>; break;
      case 8: cfg.func = (const void*)kgemm_bulk_kernel<8, 8>; break;
      default: cfg.func = (const void*)kgemm_bulk_kernel<0, 0>; break;
    }
    cfg.bm = mm;
    cfg.bn = KB_CONSUMERS;
    smem = kb_smem_bytes(mm, kk);
  } else if (stream) {
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
  if (smem > 0 && ensure_smem(cfg.func, dev, smem) != cudaSuccess) return KMX_ERR_CUDA;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cfg.func, bulk ? KB_THREADS : KG_THREADS,
                                                smem);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)di.sms * per_sm;
  const long long cta_items =
      (small && !bulk) ? (ka.items + KG_THREADS / 32 - 1) / (KG_THREADS / 32) : ka.items;
  if (grid > cta_items) grid = cta_items;
  void* args[] = {&ka};
  const cudaError_t e = cudaLaunchKernel(cfg.func, dim3((unsigned)grid),
                                         dim3(bulk ? KB_THREADS : KG_THREADS), args, smem, s);
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
