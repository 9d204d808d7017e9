// kmx_tc.cuh -- tensor-core form for FP32-stored data (3xTF32).
//
// The Kronecker mat-vec of one entry is d mode contractions; grouping g
// adjacent modes (g = 1 for n = 8, 16; 2 for n = 4) makes each step a GEMM
//   Z'(m, i) = sum_k Z(m, k) * F(i, k),   F = A_l1 (x) ... (x) A_lg,
// with KS = n^g = 8 or 16 columns, and M = n^d / KS rows m = (L, r): L runs
// over the digits before the group, r over those after it (stride R).
// Every GEMM runs on the tensor cores as warp-level mma.sync m16n8k8 TF32:
// a warp owns tiles of 16 rows, the A fragment is the tile of Z, the B
// fragment the factor F (kept in registers for the whole step).
//
// Precision: each operand x is split into big = x rounded to TF32 and
// small = x - big (exact in FP32; its TF32 truncation drops bits below 2^-22
// of x), and the product is big*big + big*small + small*big in FP32
// accumulation (the three-TF32-product scheme; small*small is below FP32
// resolution).  Relative error per product about 2^-21; sums accumulate in
// FP32.
//
// Data path per entry (one CTA, 8 warps):
//   step 0    A fragments straight from X in HBM (each 8-lane group reads
//             32 contiguous bytes); D fragments to shared memory;
//   steps 1.. A and D fragments in shared memory, in place (a warp reads its
//             whole tile before it writes it back);
//   last step D fragments added to Y with RED (FP32, or widened exactly to
//             FP64 for FP64 Y blocks).
// Shared memory holds Z in a swizzled order: word a lives at
//   a ^ (fold2(a >> 5) << 3),  fold2(u) = XOR of the 2-bit groups of u,
// which (by a bank model over every shape built here) makes the fragment
// loads and stores of all steps with r-stride >= 8 conflict-free; the last
// step (stride 1) has 2-way conflicts on its loads only.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "kmx_engine.cuh"
#include "kmx_tile.cuh"

namespace kmx {
namespace tc {

using tile::ipow;

__host__ __device__ constexpr int group_digits(int NN) { return NN == 4 ? 2 : 1; }
__host__ __device__ constexpr int ks_of(int NN) { return ipow(NN, group_digits(NN)); }
// Shapes with a kernel: whole 16-row tiles in every step, Z within 128 KB.
__host__ __device__ constexpr bool supported(int NN, int D) {
  return (NN == 4 || NN == 8 || NN == 16) && D % group_digits(NN) == 0 &&
         ipow(NN, D) / ks_of(NN) >= 16 && ipow(NN, D) <= 32768;
}
constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
__host__ __device__ constexpr int tiles_per_warp_h(int NN, int D) {
  return (ipow(NN, D) / (NN == 4 ? 16 : NN) / 16 + WARPS - 1) / WARPS;
}

__device__ __forceinline__ int swz(int a) {
  int u = a >> 5;
  u ^= u >> 2;
  u ^= u >> 4;
  u ^= u >> 8;
  return a ^ ((u & 3) << 3);
}

__device__ __forceinline__ float to_f32(float x) { return x; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 x) {
  return __uint_as_float(((unsigned)__bfloat16_as_ushort(x)) << 16);
}

// big = x rounded to TF32 (nearest, ties away; integer arithmetic on the
// bits), small = x - big.  Inf/NaN pass through big (small is then NaN/0).
__device__ __forceinline__ void split_tf32(float x, uint32_t& big, uint32_t& small) {
  const uint32_t b = (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u;
  big = b;
  small = __float_as_uint(__fsub_rn(x, __uint_as_float(b)));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Combined factor of step PH at (i, k): product over the group's modes of
// A_l(i_l, k_l), i and k in mixed radix with the first mode most significant.
template <int NN, int PH>
__device__ __forceinline__ float factor(const float* sA, int i, int k) {
  constexpr int NG = group_digits(NN);
  if constexpr (NG == 1) {
    return sA[(PH * NN + i) * NN + k];
  } else {
    const int l0 = PH * 2;
    return __fmul_rn(sA[(l0 * NN + i / NN) * NN + k / NN],
                     sA[((l0 + 1) * NN + i % NN) * NN + k % NN]);
  }
}

template <typename Out>
__device__ __forceinline__ Out widen(float v);
template <>
__device__ __forceinline__ float widen<float>(float v) {
  return v;
}
template <>
__device__ __forceinline__ double widen<double>(float v) {
  return tile::SplitPolicy::to_f64(v, 0);
}

template <typename Out>
__device__ __forceinline__ void add_out(Out* y, float v);
template <>
__device__ __forceinline__ void add_out<float>(float* y, float v) {
  atomicAdd(y, v);
}
template <>
__device__ __forceinline__ void add_out<double>(double* y, float v) {
  atomicAdd(y, tile::SplitPolicy::to_f64(v, 0));
}

// Tiles of one step handled by each warp (compile time, so that a segment's
// running sums can live in registers indexed by it).
template <int NN, int D>
__host__ __device__ constexpr int tiles_per_warp() {
  return (ipow(NN, D) / ks_of(NN) / 16 + WARPS - 1) / WARPS;
}
// Running sums per thread in segment mode: the last step's outputs.
template <int NN, int D>
__host__ __device__ constexpr int seg_values() {
  return tiles_per_warp<NN, D>() * (ks_of(NN) / 8) * 4;
}
// Segment mode keeps the running sums in registers: shapes with few outputs per thread.
__host__ __device__ constexpr bool seg_supported(int NN, int D) {
  return supported(NN, D) &&
         (tiles_per_warp_h(NN, D) * (ks_of(NN) / 8) * 4) <= 16;
}

// One GEMM step of one entry.  SEG: the last step adds into racc instead of Y.
template <int NN, int D, int PH, bool SEG, typename In, typename Out>
__device__ __forceinline__ void step(const In* __restrict__ xp, Out* yp, float* Z, const float* sA,
                                     int warp, int g, int t, Out* racc) {
  constexpr int NG = group_digits(NN);
  constexpr int P = D / NG;
  constexpr int KS = ks_of(NN);
  constexpr int KB = KS / 8;
  constexpr int M = ipow(NN, D) / KS;
  constexpr int TILES = M / 16;
  constexpr int TPW = tiles_per_warp<NN, D>();
  constexpr int R = ipow(NN, D - (PH + 1) * NG);
  // B fragments (k = 8*ks + t + 4*h, i = 8*nt + g), split once per step
  uint32_t bb[KB][KB][2], bs[KB][KB][2];
#pragma unroll
  for (int ks = 0; ks < KB; ++ks)
#pragma unroll
    for (int nt = 0; nt < KB; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h)
        split_tf32(factor<NN, PH>(sA, 8 * nt + g, 8 * ks + t + 4 * h), bb[ks][nt][h],
                   bs[ks][nt][h]);
  auto addr = [](int row, int k) {
    const int L = row / R, r = row - L * R;  // R is a power of two
    return L * KS * R + k * R + r;
  };
  auto do_tile = [&](int jt, int tile) {
    const int m0 = tile * 16;
    float av[KB][4];
#pragma unroll
    for (int ks = 0; ks < KB; ++ks)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int a = addr(m0 + g + 8 * (j & 1), 8 * ks + t + 4 * (j >> 1));
        if constexpr (PH == 0) {
          av[ks][j] = to_f32(xp[a]);
        } else {
          av[ks][j] = Z[swz(a)];
        }
      }
    float acc[KB][4];
#pragma unroll
    for (int nt = 0; nt < KB; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[nt][c] = 0.f;
#pragma unroll
    for (int ks = 0; ks < KB; ++ks) {
      uint32_t ab[4], as[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) split_tf32(av[ks][j], ab[j], as[j]);
#pragma unroll
      for (int nt = 0; nt < KB; ++nt) {
        mma_tf32(acc[nt], as, bb[ks][nt][0], bb[ks][nt][1]);
        mma_tf32(acc[nt], ab, bs[ks][nt][0], bs[ks][nt][1]);
        mma_tf32(acc[nt], ab, bb[ks][nt][0], bb[ks][nt][1]);
      }
    }
#pragma unroll
    for (int nt = 0; nt < KB; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if constexpr (PH == P - 1) {
          if constexpr (SEG) {
            racc[(jt * KB + nt) * 4 + c] += widen<Out>(acc[nt][c]);
          } else {
            add_out<Out>(yp + addr(m0 + g + 8 * (c >> 1), 8 * nt + 2 * t + (c & 1)), acc[nt][c]);
          }
        } else {
          Z[swz(addr(m0 + g + 8 * (c >> 1), 8 * nt + 2 * t + (c & 1)))] = acc[nt][c];
        }
      }
  };
  if constexpr (SEG) {
    // compile-time tile index: the running sums racc are indexed by it
#pragma unroll
    for (int jt = 0; jt < TPW; ++jt)
      if (warp + jt * WARPS < TILES) do_tile(jt, warp + jt * WARPS);
  } else {
#pragma unroll 2
    for (int tile = warp; tile < TILES; tile += WARPS) do_tile(0, tile);
  }
}

template <int NN, int D, int PH, bool SEG, typename In, typename Out>
__device__ __forceinline__ void steps(const In* xp, Out* yp, float* Z, const float* sA, int warp,
                                      int g, int t, Out* racc) {
  constexpr int P = D / group_digits(NN);
  step<NN, D, PH, SEG, In, Out>(xp, yp, Z, sA, warp, g, t, racc);
  if constexpr (PH + 1 < P) {
    __syncthreads();  // step PH's Z complete
    steps<NN, D, PH + 1, SEG, In, Out>(xp, yp, Z, sA, warp, g, t, racc);
  }
}

// Y address of running sum v of this thread (segment mode).
template <int NN, int D>
__device__ __forceinline__ int seg_addr(int v, int warp, int g, int t) {
  constexpr int KS = ks_of(NN);
  constexpr int KB = KS / 8;
  const int c = v & 3, nt = (v >> 2) % KB, jt = (v >> 2) / KB;
  const int row = (warp + jt * WARPS) * 16 + g + 8 * (c >> 1);
  return row * KS + 8 * nt + 2 * t + (c & 1);  // last step: R = 1
}

__host__ __device__ constexpr int smem_bytes(int NN, int D) {
  return (ipow(NN, D) + D * NN * NN) * 4 + 16;  // Z, factors, flag and segment words
}

// Loads the entry's factors into shared memory; returns (in *s_null) whether
// any pointer of the entry is NULL.
template <int NN, int D, typename In>
__device__ __forceinline__ void load_factors(const Problem& p, long long ent, float* sA,
                                             int* s_null) {
  for (int idx = threadIdx.x; idx < D * NN * NN; idx += THREADS) {
    const int l = idx / (NN * NN), rem = idx - l * NN * NN;
    const int i = rem / NN, k = rem - i * NN;
    const In* Ap = tile::a_ptr<In>(p, ent, l);
    float v = 0.f;
    if (Ap) {
      const long long ld = p.ld[l];
      v = to_f32(p.trans ? Ap[k + i * ld] : Ap[i + k * ld]);
    } else {
      *s_null = 1;
    }
    sA[idx] = v;  // sA[l][i][k] = A_l(i, k), or A_l(k, i) when transposed
  }
}

// Persistent kernel.
//   SEG == false: entries in grid-stride order, contributions added to Y
//     with RED.
//   SEG == true (deterministic mode): the CTA pops Y segments -- the entries
//     sharing one Y block, in their original order -- from the device work
//     queue, sums their contributions in registers (every thread owns the
//     same output elements for every entry) and adds the sum to the Y block
//     once, with plain loads and stores (the CTA owns the block).
template <int NN, int D, typename In, typename Out, bool SEG>
__global__ void __launch_bounds__(THREADS, SEG ? 2 : 4) tc_kernel(const Problem p) {
  static_assert(supported(NN, D), "no tensor-core kernel for this shape");
  static_assert(!SEG || seg_supported(NN, D), "segment mode: too many outputs per thread");
  constexpr int N = ipow(NN, D);
  constexpr int NV = SEG ? seg_values<NN, D>() : 1;
  extern __shared__ __align__(16) unsigned char smem[];
  float* Z = reinterpret_cast<float*>(smem);
  float* sA = Z + N;
  int* s_null = reinterpret_cast<int*>(sA + D * NN * NN);
  int* s_seg = s_null + 1;  // [segment id, offset, count]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  if constexpr (!SEG) {
    const long long total = launch_count(p);
    for (long long e = blockIdx.x; e < total; e += gridDim.x) {
      const long long ent = tile::entry_index(p, e);
      if (threadIdx.x == 0) *s_null = 0;
      __syncthreads();  // the previous entry is done with Z and sA
      load_factors<NN, D, In>(p, ent, sA, s_null);
      const In* xp = tile::x_ptr<In>(p, ent);
      Out* yp = tile::y_ptr<Out>(p, ent);
      if (threadIdx.x == 0 && (!xp || !yp)) *s_null = 1;
      __syncthreads();
      if (*s_null) {
        if (threadIdx.x == 0) atomicOr(p.status, DF_NULL_PTR);
        continue;
      }
      steps<NN, D, 0, false, In, Out>(xp, yp, Z, sA, warp, g, t, nullptr);
    }
  } else {
    for (;;) {
      __syncthreads();  // the previous segment is done with s_seg
      if (threadIdx.x == 0) {
        const int q = atomicAdd(p.seg_queue, 1);
        if (q < *p.seg_num) {
          const int sid = p.seg_order[q];
          s_seg[0] = 1;
          s_seg[1] = p.seg_offset[sid];
          s_seg[2] = p.seg_count[sid];
        } else {
          s_seg[0] = 0;
        }
      }
      __syncthreads();
      if (!s_seg[0]) break;
      const int off = s_seg[1], cnt = s_seg[2];
      Out racc[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) racc[v] = Out(0);
      Out* yseg = nullptr;
      for (int j = 0; j < cnt; ++j) {
        const long long ent = p.seg_entries[off + j];
        __syncthreads();  // the previous entry is done with Z, sA and s_null
        if (threadIdx.x == 0) *s_null = 0;
        __syncthreads();
        load_factors<NN, D, In>(p, ent, sA, s_null);
        const In* xp = tile::x_ptr<In>(p, ent);
        Out* yp = tile::y_ptr<Out>(p, ent);
        yseg = yp;  // every entry of a segment has the same Y block
        if (threadIdx.x == 0 && (!xp || !yp)) *s_null = 1;
        __syncthreads();
        if (*s_null) {
          if (threadIdx.x == 0) atomicOr(p.status, DF_NULL_PTR);
          continue;
        }
        steps<NN, D, 0, true, In, Out>(xp, yp, Z, sA, warp, g, t, racc);
      }
      if (yseg) {
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const int jt = (v >> 2) / (ks_of(NN) / 8);
          if (warp + jt * WARPS < N / ks_of(NN) / 16) {
            Out* y = yseg + seg_addr<NN, D>(v, warp, g, t);
            *y += racc[v];
          }
        }
      }
    }
  }
}

}  // namespace tc
}  // namespace kmx
