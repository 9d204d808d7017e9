// kmx_tile.cuh -- register-tiled engine for square factors with compile-time
// n (NN) and d (D), one entry per group of G threads, the entry's
// intermediate in shared memory.
//
// The d mode contractions are grouped into PHASES.  In a phase each thread
// owns whole TILES: all NN (one mode) or NN*NN (two modes, when NN <= 4)
// elements that share the other indices.  A thread loads its tile into
// registers, contracts the phase's mode(s) there, and writes the tile back.
// Phases are ordered so that
//   - the first phase contains mode 0: tile u's elements sit at u + j*NN^(d-1),
//     so consecutive lanes read consecutive X elements straight from HBM;
//   - the last phase excludes mode d-1: consecutive lanes then write runs of
//     consecutive Y elements (whole 32-byte sectors) with FP64 atomics;
//   - the middle phases exchange tiles through shared memory laid out with
//     one pad element per 16 for even NN, which makes every phase's 64-bit
//     accesses free of bank conflicts for NN = 2, 4, 8 (odd NN need no pad).
//
//   NN <= 4:  d=6 {0,1}{4,5}{2,3}   d=5 {0,1}{4}{2,3}   d=4 {0,1}{3}{2}   d=3 {0}{2}{1}
//   NN >= 5:  {0}{d-1}{d-2}...{1}
//
// The result equals the reference's recursion up to the rounding of a
// different (but equally valid) order of the mode products.
#pragma once

#include <cuda_bf16.h>

#include <type_traits>

#include "kmx_engine.cuh"
#include "kmx_pack.cuh"

namespace kmx {
namespace tile {

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

__host__ __device__ constexpr int num_phases(int NN, int D) { return NN <= 4 ? 3 : D; }

// first / second mode of phase p (second = -1 for a one-mode phase)
__host__ __device__ constexpr int phase_a(int NN, int D, int p) {
  return NN <= 4 ? (D == 6 ? (p == 0 ? 0 : p == 1 ? 4 : 2)
                  : D == 5 ? (p == 0 ? 0 : p == 1 ? 4 : 2)
                  : D == 4 ? (p == 0 ? 0 : p == 1 ? 3 : 2)
                           : (p == 0 ? 0 : p == 1 ? 2 : 1))
                 : (p == 0 ? 0 : D - p);
}
__host__ __device__ constexpr int phase_b(int NN, int D, int p) {
  return NN <= 4 ? (D == 6 ? (p == 0 ? 1 : p == 1 ? 5 : 3)
                  : D == 5 ? (p == 0 ? 1 : p == 1 ? -1 : 3)
                  : D == 4 ? (p == 0 ? 1 : -1)
                           : -1)
                 : -1;
}

// elements of one tile in phase p
__host__ __device__ constexpr int tile_size(int NN, int D, int p) {
  return phase_b(NN, D, p) >= 0 ? NN * NN : NN;
}

// threads per entry: one tile per thread in the first phase where possible
// (32..512); a thread may own several factor entries (factors_per_thread)
__host__ __device__ constexpr int round32(int x) { return (x + 31) / 32 * 32; }
__host__ __device__ constexpr int group_threads(int NN, int D) {
  return round32(ipow(NN, D) / tile_size(NN, D, 0)) > 512
             ? 512
             : (round32(ipow(NN, D) / tile_size(NN, D, 0)) < 32
                    ? 32
                    : round32(ipow(NN, D) / tile_size(NN, D, 0)));
}
// whether the packed double-float policy is used for (NN, D): even NN <= 8
// with one first-phase tile per thread (see TilePol in kmx_launch.cuh)
__host__ __device__ constexpr bool packed_pays(int NN, int D) {
  return NN % 2 == 0 && NN <= 8 && ipow(NN, D) / tile_size(NN, D, 0) <= 512;
}
__host__ __device__ constexpr int factors_per_thread(int NN, int D) {
  return (D * NN * NN + group_threads(NN, D) - 1) / group_threads(NN, D);
}

// physical slot of logical element q in the shared intermediate
template <int NN>
__device__ __forceinline__ int slot(int q) {
  if constexpr ((NN & 1) == 0) {
    return q + (q >> 4);
  } else {
    return q;
  }
}

template <int NN, int D>
__host__ __device__ constexpr int buffer_slots() {
  return (NN & 1) == 0 ? ipow(NN, D) + ipow(NN, D) / 16 + 1 : ipow(NN, D);
}

// Base address of tile u in phase p: the modes outside the phase are the
// digits of u in significance order.
template <int NN, int D, int P>
__device__ __forceinline__ int tile_base(int u) {
  constexpr int a = phase_a(NN, D, P);
  constexpr int b = phase_b(NN, D, P);
  constexpr int last = b >= 0 ? b : a;                // phase modes are adjacent
  constexpr int low = ipow(NN, D - 1 - last);          // elements below the phase
  constexpr int span = ipow(NN, D - a);                // the phase's block
  return (u / low) * span + (u % low);
}

// offset of tile element e (row-major over the phase's modes)
template <int NN, int D, int P>
__device__ __forceinline__ constexpr int tile_off(int e) {
  constexpr int a = phase_a(NN, D, P);
  constexpr int b = phase_b(NN, D, P);
  if constexpr (b >= 0) {
    return (e / NN) * ipow(NN, D - 1 - a) + (e % NN) * ipow(NN, D - 1 - b);
  } else {
    return e * ipow(NN, D - 1 - a);
  }
}

// ---------------------------------------------------------------------------
// Arithmetic policies.
// ---------------------------------------------------------------------------

// Factor storage of the policies with one value per factor element: factor
// l is NN*NN values of V, row-major (row = output index).
template <typename V>
struct FlatFactors {
  static constexpr bool PACKED = false;
  template <int NN>
  __host__ __device__ static constexpr int factor_bytes() {
    return NN * NN * (int)sizeof(V);
  }
  template <int NN>
  __device__ __forceinline__ static const void* factor(const unsigned char* base, int l) {
    return base + (size_t)l * factor_bytes<NN>();
  }
  // element idx = l*NN*NN + r*NN + j
  template <int NN>
  __device__ __forceinline__ static void store_factor(unsigned char* base, int idx, V a) {
    reinterpret_cast<V*>(base)[idx] = a;
  }
};

// Double-float with per-entry power-of-two scaling (see kmx_engine.cuh).
struct SplitPolicy : FlatFactors<df> {
  using In = double;
  using V = df;
  using Out = double;
  static constexpr bool SCALED = true;

  // Integer-only split (no conversion instructions: on this GPU they share
  // the narrow FP64 pipe).  hi = leading 24 bits, lo = next 24 bits, both
  // truncated: representation error below 2^-47 relative.
  __device__ __forceinline__ static V make(double x, int eref) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int ef = (int)((b >> 52) & 0x7FF);
    const int fe = ef - eref + 127;
    V r;
    r.hi = 0.f;
    r.lo = 0.f;
    if (ef == 0 || fe <= 0) return r;
    const unsigned mhi = (unsigned)(b >> 29) & 0x7FFFFFu;
    r.hi = __uint_as_float(sign | ((unsigned)fe << 23) | mhi);
    const unsigned rem = (unsigned)b & 0x1FFFFFFFu;  // 29 bits below hi
    if (rem != 0) {
      const int p = 31 - __clz(rem);                  // leading bit of rem
      const unsigned m = (p >= 23) ? (rem >> (p - 23)) : (rem << (23 - p));
      const int el = p + fe - 52;                     // FP32 exponent field of lo
      if (el > 0) r.lo = __uint_as_float(sign | ((unsigned)el << 23) | (m & 0x7FFFFFu));
    }
    return r;
  }

  template <int NN>
  __device__ __forceinline__ static V dot(const V* a, const V* v) {
    return df_dot<NN>(a, v);
  }

  // FP64 value of (hi + lo) * 2^escale: exact exponent arithmetic, one DADD.
  __device__ __forceinline__ static double finish(V o, int escale) {
    return to_f64(o.hi, escale) + to_f64(o.lo, escale);
  }
  __device__ __forceinline__ static double to_f64(float f, int escale) {
    const unsigned u = __float_as_uint(f);
    const int ef = (int)((u >> 23) & 0xFF);
    if (ef == 0) return 0.0;
    int e = ef - 127 + 1023 + escale;
    if (e <= 0) return 0.0;                  // below FP64's normal range
    if (e >= 2047) e = 2047;                 // overflow: +-Inf
    const unsigned long long bits =
        ((unsigned long long)(u & 0x80000000u) << 32) | ((unsigned long long)e << 52) |
        (e == 2047 ? 0ull : ((unsigned long long)(u & 0x7FFFFFu) << 29));
    return __longlong_as_double((long long)bits);
  }
};

// Double-float on packed FP32 pairs (kmx_pack.cuh): two output rows per
// instruction.  Factors are stored as row pairs (high and low parts); the
// arithmetic per value is that of SplitPolicy.
struct PackedSplitPolicy : SplitPolicy {
  static constexpr bool PACKED = true;
  template <int NN>
  __host__ __device__ static constexpr int factor_bytes() {
    return pk2::factor_u64<NN>() * 8;
  }
  template <int NN>
  __device__ __forceinline__ static const void* factor(const unsigned char* base, int l) {
    return base + (size_t)l * factor_bytes<NN>();
  }
  template <int NN>
  __device__ __forceinline__ static void store_factor(unsigned char* base, int idx, df a) {
    constexpr int NN2 = NN * NN;
    const int l = idx / NN2, r = (idx - l * NN2) / NN, j = idx - l * NN2 - r * NN;
    float* f = reinterpret_cast<float*>(base + (size_t)l * factor_bytes<NN>()) +
               ((r >> 1) * NN + j) * 4 + (r & 1);
    f[0] = a.hi;
    f[2] = a.lo;
  }
};

template <typename T>
struct PlainPolicy : FlatFactors<T> {
  using In = T;
  using V = T;
  using Out = T;
  static constexpr bool SCALED = false;
  __device__ __forceinline__ static V make(T x, int) { return x; }
  template <int NN>
  __device__ __forceinline__ static V dot(const V* a, const V* v) {
    V acc = a[0] * v[0];
#pragma unroll
    for (int j = 1; j < NN; ++j) acc = fma(a[j], v[j], acc);
    return acc;
  }
  __device__ __forceinline__ static T finish(V o, int) { return o; }
};

// Low-precision storage with FP32 arithmetic and FP64 results: X and the
// factors are FP32 or BF16 (converted exactly to FP32), the d mode products
// run in FP32, and each contribution is widened exactly to FP64 before it is
// added to the (FP64) Y block, so overlapping contributions accumulate in FP64.
template <typename TIn>
struct WidePolicy : FlatFactors<float> {
  using In = TIn;
  using V = float;
  using Out = double;
  static constexpr bool SCALED = false;
  __device__ __forceinline__ static V make(TIn x, int) { return to_f32(x); }
  __device__ __forceinline__ static float to_f32(float x) { return x; }
  __device__ __forceinline__ static float to_f32(__nv_bfloat16 x) {
    return __uint_as_float(((unsigned)__bfloat16_as_ushort(x)) << 16);
  }
  template <int NN>
  __device__ __forceinline__ static V dot(const V* a, const V* v) {
    V acc = a[0] * v[0];
#pragma unroll
    for (int j = 1; j < NN; ++j) acc = fmaf(a[j], v[j], acc);
    return acc;
  }
  // exact FP32 -> FP64 by exponent arithmetic (no conversion instruction)
  __device__ __forceinline__ static double finish(V o, int) { return SplitPolicy::to_f64(o, 0); }
};

// Packed double-float contraction of a tile (PackedSplitPolicy): the dot
// products of output rows (2rp, 2rp+1) share one instruction stream.
template <int NN, bool PAIR>
__device__ __forceinline__ void contract_tile_packed(df* v, const pk2::RowPair* Fa,
                                                     const pk2::RowPair* Fb) {
  using pk2::u64;
  constexpr int RP = pk2::row_pairs<NN>();
  pk2::PackedRows<NN> A;
  A.load(Fa);
  if constexpr (PAIR) {
    // first mode: columns (fixed second index), rows paired
#pragma unroll
    for (int c = 0; c < NN; ++c) {
      u64 vh[NN], vl[NN], nvh[NN], oh[RP], ol[RP];
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        vh[j] = pk2::bcast(v[j * NN + c].hi);
        vl[j] = pk2::bcast(v[j * NN + c].lo);
        nvh[j] = pk2::bcast(-v[j * NN + c].hi);
      }
#pragma unroll
      for (int rp = 0; rp < RP; ++rp) pk2::dot_pair<NN>(A.pair(rp), vh, vl, nvh, oh[rp], ol[rp]);
#pragma unroll
      for (int rp = 0; rp < RP; ++rp) {
        float h0, h1, l0, l1;
        pk2::unpack(oh[rp], h0, h1);
        pk2::unpack(ol[rp], l0, l1);
        v[2 * rp * NN + c].hi = h0;
        v[2 * rp * NN + c].lo = l0;
        if (2 * rp + 1 < NN) {
          v[(2 * rp + 1) * NN + c].hi = h1;
          v[(2 * rp + 1) * NN + c].lo = l1;
        }
      }
    }
    A.load(Fb);
    // second mode: rows (fixed first index), output columns paired
#pragma unroll
    for (int r0 = 0; r0 < NN; ++r0) {
      u64 vh[NN], vl[NN], nvh[NN], oh[RP], ol[RP];
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        vh[j] = pk2::bcast(v[r0 * NN + j].hi);
        vl[j] = pk2::bcast(v[r0 * NN + j].lo);
        nvh[j] = pk2::bcast(-v[r0 * NN + j].hi);
      }
#pragma unroll
      for (int rp = 0; rp < RP; ++rp) pk2::dot_pair<NN>(A.pair(rp), vh, vl, nvh, oh[rp], ol[rp]);
#pragma unroll
      for (int rp = 0; rp < RP; ++rp) {
        float h0, h1, l0, l1;
        pk2::unpack(oh[rp], h0, h1);
        pk2::unpack(ol[rp], l0, l1);
        v[r0 * NN + 2 * rp].hi = h0;
        v[r0 * NN + 2 * rp].lo = l0;
        if (2 * rp + 1 < NN) {
          v[r0 * NN + 2 * rp + 1].hi = h1;
          v[r0 * NN + 2 * rp + 1].lo = l1;
        }
      }
    }
  } else {
    u64 vh[NN], vl[NN], nvh[NN], oh[RP], ol[RP];
#pragma unroll
    for (int j = 0; j < NN; ++j) {
      vh[j] = pk2::bcast(v[j].hi);
      vl[j] = pk2::bcast(v[j].lo);
      nvh[j] = pk2::bcast(-v[j].hi);
    }
#pragma unroll
    for (int rp = 0; rp < RP; ++rp) pk2::dot_pair<NN>(A.pair(rp), vh, vl, nvh, oh[rp], ol[rp]);
#pragma unroll
    for (int rp = 0; rp < RP; ++rp) {
      float h0, h1, l0, l1;
      pk2::unpack(oh[rp], h0, h1);
      pk2::unpack(ol[rp], l0, l1);
      v[2 * rp].hi = h0;
      v[2 * rp].lo = l0;
      if (2 * rp + 1 < NN) {
        v[2 * rp + 1].hi = h1;
        v[2 * rp + 1].lo = l1;
      }
    }
  }
}

// Contract the tile's mode(s) in registers.  Afirst / Asecond point at the
// phase's factor(s) in shared memory (layout of the policy's factor storage).
template <class Pol, int NN, bool PAIR>
__device__ __forceinline__ void contract_tile(typename Pol::V* v, const void* Afirst_,
                                              const void* Asecond_) {
  using V = typename Pol::V;
  if constexpr (Pol::PACKED) {
    contract_tile_packed<NN, PAIR>(v, static_cast<const pk2::RowPair*>(Afirst_),
                                   static_cast<const pk2::RowPair*>(Asecond_));
    return;
  } else {
  const V* Afirst = static_cast<const V*>(Afirst_);
  const V* Asecond = static_cast<const V*>(Asecond_);
  Rows<V, NN> A;
  A.load(Afirst);
  if constexpr (PAIR) {
    // first mode: columns (fixed second index)
#pragma unroll
    for (int c = 0; c < NN; ++c) {
      V col[NN], out[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) col[j] = v[j * NN + c];
#pragma unroll
      for (int r = 0; r < NN; ++r) out[r] = Pol::template dot<NN>(A.row(r), col);
#pragma unroll
      for (int r = 0; r < NN; ++r) v[r * NN + c] = out[r];
    }
    A.load(Asecond);
#pragma unroll
    for (int r0 = 0; r0 < NN; ++r0) {
      V row[NN], out[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) row[j] = v[r0 * NN + j];
#pragma unroll
      for (int c = 0; c < NN; ++c) out[c] = Pol::template dot<NN>(A.row(c), row);
#pragma unroll
      for (int c = 0; c < NN; ++c) v[r0 * NN + c] = out[c];
    }
  } else {
    V out[NN];
#pragma unroll
    for (int r = 0; r < NN; ++r) out[r] = Pol::template dot<NN>(A.row(r), v);
#pragma unroll
    for (int r = 0; r < NN; ++r) v[r] = out[r];
  }
  }
}

// One middle phase P over all tiles of the group: shared memory -> shared memory.
template <class Pol, int NN, int D, int G, int P>
__device__ __forceinline__ void middle_phase(typename Pol::V* buf, const unsigned char* sA,
                                             int lt) {
  using V = typename Pol::V;
  constexpr int a = phase_a(NN, D, P);
  constexpr int b = phase_b(NN, D, P);
  constexpr int T = tile_size(NN, D, P);
  constexpr int NT = ipow(NN, D) / T;
  for (int u = lt; u < NT; u += G) {
    const int base = tile_base<NN, D, P>(u);
    V v[T];
#pragma unroll
    for (int e = 0; e < T; ++e) v[e] = buf[slot<NN>(base + tile_off<NN, D, P>(e))];
    contract_tile<Pol, NN, (b >= 0)>(v, Pol::template factor<NN>(sA, a),
                                     Pol::template factor<NN>(sA, b >= 0 ? b : a));
#pragma unroll
    for (int e = 0; e < T; ++e) buf[slot<NN>(base + tile_off<NN, D, P>(e))] = v[e];
  }
}

template <class Pol, int NN, int D, int G, int P>
__device__ __forceinline__ void middle_phases(typename Pol::V* buf, const unsigned char* sA,
                                              int lt, int g) {
  if constexpr (P < num_phases(NN, D) - 1) {
    middle_phase<Pol, NN, D, G, P>(buf, sA, lt);
    group_sync(g, G);
    middle_phases<Pol, NN, D, G, P + 1>(buf, sA, lt, g);
  }
}

// ---------------------------------------------------------------------------
// TMA bulk copies and mbarriers.  Every wait is bounded (about 2 s of
// %globaltimer); a wait that runs out sets DF_WAIT_TIMEOUT and the group
// returns.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* ptr) {
  return (uint32_t)__cvta_generic_to_shared(ptr);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// One contiguous global -> shared bulk copy completing on `bar`.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait until the phase of parity `parity` completes; false after ~2 s.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  const unsigned long long t0 = global_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > 2000000000ull) return false;
    __nanosleep(32);
  }
}

// ---------------------------------------------------------------------------
// Entry pointers, one at a time (the pipeline loads them ahead of use).
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long entry_index(const Problem& p, long long e) {
  if (p.order) return (long long)p.order[(p.order_base ? (long long)*p.order_base : 0) + e];
  return e + p.entry_offset;
}
template <typename T>
__device__ __forceinline__ const T* x_ptr(const Problem& p, long long ent) {
  return p.layout == L_BATCHED ? static_cast<const T*>(p.X) + ent * p.Nx
                               : static_cast<T* const*>(p.X)[ent];
}
template <typename T>
__device__ __forceinline__ T* y_ptr(const Problem& p, long long ent) {
  return p.layout == L_BATCHED ? static_cast<T*>(p.Y) + ent * p.Ny
                               : static_cast<T* const*>(p.Y)[ent];
}
template <typename T>
__device__ __forceinline__ const T* a_ptr(const Problem& p, long long ent, int l) {
  if (p.layout == L_BATCHED || p.layout == L_PBATCHED)
    return static_cast<const T*>(p.A) + (ent * p.d + l) * (long long)p.n[0] * p.n[0];
  return static_cast<const T* const*>(p.A)[(p.a_off ? p.a_off[ent] : ent * p.d) + l];
}

// ---------------------------------------------------------------------------
// Shared memory per group:
//   [d*NN*NN factor entries of V]
//   [2 x (MAXD+1) exponent ints][2 flag ints][stage-mode int][pad]   (by entry parity)
//   [2 entry descriptors (long long id, int flags, pad)]
//   [2 x (MAXD+2) cancellation-guard sums (float)]                    (by entry parity)
//   [mbarrier]
//   [X staging block: N x In]
//   [intermediate: buffer_slots x V]
//   [segment accumulator: N x Out]   (deterministic mode only)
// ---------------------------------------------------------------------------
// factor storage first; it also holds MAXD*NN*NN doubles for the FP64
// evaluation of an entry (nonfinite_entry, guard_redo)
template <class Pol, int NN, int D>
__host__ __device__ constexpr int off_ints() {
  return (MAXD * Pol::template factor_bytes<NN>() > MAXD * NN * NN * 8
              ? MAXD * Pol::template factor_bytes<NN>()
              : MAXD * NN * NN * 8 + 15) / 16 * 16;
}
template <class Pol, int NN, int D>
__host__ __device__ constexpr int off_desc() {
  return (off_ints<Pol, NN, D>() + (2 * (MAXD + 1) + 4) * 4 + 15) / 16 * 16;
}
// cancellation-guard sums, by entry parity: ||A_l||^2 (l < MAXD), ||X||^2, ||KX||^2
template <class Pol, int NN, int D>
__host__ __device__ constexpr int off_nrm() {
  return off_desc<Pol, NN, D>() + 2 * 16;
}
constexpr int NRM_STRIDE = MAXD + 2;
template <class Pol, int NN, int D>
__host__ __device__ constexpr int off_bars() {
  return off_nrm<Pol, NN, D>() + 2 * NRM_STRIDE * 4;
}
template <class Pol, int NN, int D>
__host__ __device__ constexpr int off_stage() {
  return off_bars<Pol, NN, D>() + 16;
}
template <class Pol, int NN, int D>
__host__ __device__ constexpr int stage_bytes() {
  return (ipow(NN, D) * (int)sizeof(typename Pol::In) + 15) / 16 * 16;
}
template <class Pol, int NN, int D>
__host__ __device__ constexpr int buf_bytes() {
  return (buffer_slots<NN, D>() * (int)sizeof(typename Pol::V) + 15) / 16 * 16;
}
template <class Pol, int NN, int D>
__host__ __device__ constexpr int acc_bytes() {
  return (ipow(NN, D) * (int)sizeof(typename Pol::Out) + 15) / 16 * 16;
}
// The X staging block is kept when it fits beside the intermediate; without
// it, phase 0 reads X straight from HBM (no TMA prefetch).
template <class Pol, int NN, int D>
__host__ __device__ constexpr bool stages_x() {
  return off_stage<Pol, NN, D>() + stage_bytes<Pol, NN, D>() +
             (buffer_slots<NN, D>() * (int)sizeof(typename Pol::V) + 15) / 16 * 16 +
             (ipow(NN, D) * (int)sizeof(typename Pol::Out) + 15) / 16 * 16 <=
         200 * 1024;
}
template <class Pol, int NN, int D>
__host__ __device__ constexpr int off_buf() {
  return off_stage<Pol, NN, D>() + (stages_x<Pol, NN, D>() ? stage_bytes<Pol, NN, D>() : 0);
}
template <class Pol, int NN, int D>
__host__ __device__ constexpr int off_acc() {
  return off_buf<Pol, NN, D>() + buf_bytes<Pol, NN, D>();
}
template <class Pol, int NN, int D, bool SEG>
__host__ __device__ constexpr int group_smem_bytes() {
  return off_acc<Pol, NN, D>() + (SEG ? acc_bytes<Pol, NN, D>() : 0);
}

// The plain-FP64 evaluation of an entry with Inf/NaN, kept out of line: it
// is rarely taken, and inlined it would sit in the hot loop's instruction
// stream.
template <int NN>
__device__ __noinline__ void nonfinite_entry(const Problem& p, long long ent, double* sA,
                                             double* buf, int lt, int G, int g) {
  EntryPtrs<double> en;
  resolve_entry<double>(p, ent, en);
  sq_plain_entry<double, NN, false>(p, en, sA, buf, lt, G, g);
}

// The cancellation guard fired for this entry (double-float policy only): take
// back what the last phase added -- recomputed from the intermediate, which the
// last phase leaves unchanged, by the same arithmetic, so bitwise the same
// values -- and add the plain FP64 result instead.  Out of line: rarely taken.
template <class Pol, int NN, int D, bool SEG>
__device__ __noinline__ void guard_redo(const Problem& p, long long ent, unsigned char* sA,
                                        typename Pol::V* buf, typename Pol::Out* acc,
                                        typename Pol::Out* yp, int escale, bool last, int lt,
                                        int g) {
  using V = typename Pol::V;
  using Out = typename Pol::Out;
  constexpr int G = group_threads(NN, D);
  constexpr int LP = num_phases(NN, D) - 1;
  constexpr int TL = tile_size(NN, D, LP);
  constexpr int NTL = ipow(NN, D) / TL;
  constexpr bool PAIRL = phase_b(NN, D, LP) >= 0;
  constexpr int aL = phase_a(NN, D, LP);
  constexpr int bL = PAIRL ? phase_b(NN, D, LP) : aL;
  for (int u = lt; u < NTL; u += G) {
    const int base = tile_base<NN, D, LP>(u);
    V v[TL];
#pragma unroll
    for (int t = 0; t < TL; ++t) v[t] = buf[slot<NN>(base + tile_off<NN, D, LP>(t))];
    contract_tile<Pol, NN, PAIRL>(v, Pol::template factor<NN>(sA, aL),
                                  Pol::template factor<NN>(sA, bL));
#pragma unroll
    for (int t = 0; t < TL; ++t) {
      const int q = base + tile_off<NN, D, LP>(t);
      const Out y = Pol::finish(v[t], escale);
      if constexpr (SEG) {
        if (last) {
          yp[q] -= y;
        } else {
          acc[q] -= y;
        }
      } else {
        atomicAdd(yp + q, -y);
      }
    }
  }
  group_sync(g, G);  // factors and intermediate free for the FP64 evaluation
  nonfinite_entry<NN>(p, ent, reinterpret_cast<double*>(sA), reinterpret_cast<double*>(buf), lt,
                      G, g);
  if (lt == 0) count_redo(p.redo_ctr, 0);
}

enum : int { TF_NULL = 1, TF_TIMEOUT = 2 };
enum : int { ED_VALID = 1, ED_FIRST = 2 };  // entry descriptor flags

struct EntryDesc {
  long long ent;
  int flags;
  int pad;
};

// CTA size of the tile kernels, and the CTAs per SM they are compiled for
// (caps registers at 128 per thread for CTAs of <= 256 threads).
__host__ __device__ constexpr int cta_threads(int NN, int D) {
  return group_threads(NN, D) < 256 ? 256 : group_threads(NN, D);
}
__host__ __device__ constexpr int min_ctas(int NN, int D) { return cta_threads(NN, D) > 256 ? 1 : 2; }

// Software-pipelined entry loop of one group.
//
// SEG == false: entries in grid-stride order, contributions added to Y with
//   RED (FP64/FP32 atomic add in L2).
// SEG == true (deterministic mode): the group pops Y segments -- the entries
//   sharing one Y block, in their original order -- from a device work queue;
//   contributions are summed in a shared accumulator in a fixed order and
//   added to the Y block once, by plain loads and stores (the group owns it).
//
// While entry k is contracted, the X block of entry k+1 streams into the
// staging block by TMA (issued once entry k's X is in registers) and entry
// k+1's factor entries are loaded into registers.  Thread 0 runs the entry
// stream and publishes descriptors through shared memory.
template <class Pol, int NN, int D, bool SEG>
__global__ void __launch_bounds__(cta_threads(NN, D), min_ctas(NN, D))
tile_kernel(const Problem p) {
  using V = typename Pol::V;
  using In = typename Pol::In;
  using Out = typename Pol::Out;
  constexpr int G = group_threads(NN, D);
  constexpr int NN2 = NN * NN;
  constexpr int N = ipow(NN, D);
  constexpr int LP = num_phases(NN, D) - 1;
  constexpr int T0 = tile_size(NN, D, 0);
  constexpr int NT0 = N / T0;
  constexpr int TL = tile_size(NN, D, LP);
  constexpr int NTL = N / TL;
  constexpr bool PAIR0 = phase_b(NN, D, 0) >= 0;
  constexpr bool PAIRL = phase_b(NN, D, LP) >= 0;
  constexpr int a0 = phase_a(NN, D, 0);
  constexpr int b0 = PAIR0 ? phase_b(NN, D, 0) : a0;
  constexpr int aL = phase_a(NN, D, LP);
  constexpr int bL = PAIRL ? phase_b(NN, D, LP) : aL;
  constexpr bool ONE = NT0 <= G;
  constexpr uint32_t XBYTES = (uint32_t)N * sizeof(In);

  extern __shared__ __align__(16) unsigned char smem[];
  const int E = p.groups_per_cta;
  const int g = threadIdx.x / G;
  const int lt = threadIdx.x - g * G;
  if (g >= E) return;
  unsigned char* gb = smem + (size_t)g * group_smem_bytes<Pol, NN, D, SEG>();
  unsigned char* sA = gb;  // factor storage (layout of the policy)
  int* sExp = reinterpret_cast<int*>(gb + off_ints<Pol, NN, D>());  // [2][MAXD+1]
  int* sFlag = sExp + 2 * (MAXD + 1);                                 // [2]
  int* sMode = sFlag + 2;                                             // [1]
  EntryDesc* sDesc = reinterpret_cast<EntryDesc*>(gb + off_desc<Pol, NN, D>());  // [2]
  float* sNrm = reinterpret_cast<float*>(gb + off_nrm<Pol, NN, D>());  // [2][NRM_STRIDE]
  uint64_t* bar = reinterpret_cast<uint64_t*>(gb + off_bars<Pol, NN, D>());
  In* stage = reinterpret_cast<In*>(gb + off_stage<Pol, NN, D>());
  V* buf = reinterpret_cast<V*>(gb + off_buf<Pol, NN, D>());
  Out* acc = reinterpret_cast<Out*>(gb + off_acc<Pol, NN, D>());

  // ---- entry stream (thread 0 only) ----
  const long long gstep = (long long)gridDim.x * E;
  long long rr_e = (long long)blockIdx.x * E + g;  // SEG == false: grid-stride position
  int seg_pos = 0, seg_cnt = 0, seg_off = 0;        // SEG == true: current segment
  auto next_desc = [&](EntryDesc& dsc) {
    dsc.flags = 0;
    dsc.ent = 0;
    if constexpr (SEG) {
      if (seg_pos >= seg_cnt) {
        const int s = atomicAdd(p.seg_queue, 1);
        if (s >= *p.seg_num) return;
        const int sid = p.seg_order[s];
        seg_off = p.seg_offset[sid];
        seg_cnt = p.seg_count[sid];
        seg_pos = 0;
        dsc.flags |= ED_FIRST;
      }
      dsc.ent = p.seg_entries[seg_off + seg_pos];
      ++seg_pos;
      dsc.flags |= ED_VALID;
    } else {
      if (rr_e >= launch_count(p)) return;
      dsc.ent = entry_index(p, rr_e);
      rr_e += gstep;
      dsc.flags = ED_VALID | ED_FIRST;
    }
  };

  if (lt < 2 * (MAXD + 1) + 4) sExp[lt] = 0;
  if (lt < 2 * NRM_STRIDE) sNrm[lt] = 0.f;
  if constexpr (Pol::PACKED) {
    // the pad row of an odd NN stays zero (entries write real rows only)
    for (int i = lt; i < off_ints<Pol, NN, D>() / 4; i += G) reinterpret_cast<float*>(sA)[i] = 0.f;
  }
  if (lt == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
    EntryDesc d0;
    next_desc(d0);
    sDesc[0] = d0;
  }
  group_sync(g, G);
  if (!(sDesc[0].flags & ED_VALID)) return;  // nothing for this group (uniform)

  // factor entries owned by this thread: lt, lt + G, ... below d*NN*NN
  constexpr int FPT = factors_per_thread(NN, D);
  bool fthr[FPT];
  int al[FPT], aoff[FPT];
#pragma unroll
  for (int f = 0; f < FPT; ++f) {
    const int idx = lt + f * G;
    fthr[f] = idx < D * NN2;
    al[f] = fthr[f] ? idx / NN2 : 0;
    const int ar = fthr[f] ? (idx - al[f] * NN2) / NN : 0;
    const int aj = fthr[f] ? idx - al[f] * NN2 - ar * NN : 0;
    const int ald = p.ld[al[f]];
    aoff[f] = p.trans ? aj + ar * ald : ar + aj * ald;
  }
  uint32_t uses = 0;  // thread 0: completed phases of the barrier
  auto issue_x = [&](const In* xsrc) {
    int mode = 0;
    if (stages_x<Pol, NN, D>() && xsrc != nullptr &&
        ((reinterpret_cast<uintptr_t>(xsrc) & 15) == 0) && (XBYTES % 16 == 0)) {
      fence_proxy_async();
      mbar_expect_tx(bar, XBYTES);
      tma_load_1d(stage, xsrc, XBYTES, bar);
      mode = 1;
    }
    sMode[0] = mode;
  };

  // ---- prologue: first entry's factor entries and scales, its X block ----
  In af[FPT];
  {
    const long long ent = sDesc[0].ent;
#pragma unroll
    for (int f = 0; f < FPT; ++f) {
      af[f] = In(0);
      if (fthr[f]) {
        const In* Ap = a_ptr<In>(p, ent, al[f]);
        if (Ap) {
          af[f] = Ap[aoff[f]];
          if constexpr (Pol::SCALED) atomicMax(&sExp[al[f]], exp_field(af[f]));
        } else {
          atomicOr(&sFlag[0], TF_NULL);
        }
      }
    }
    if (lt == 0) issue_x(x_ptr<In>(p, ent));
  }
  group_sync(g, G);

  for (int k = 0;; ++k) {
    const int pb = k & 1;
    const EntryDesc dk = sDesc[pb];
    if (!(dk.flags & ED_VALID)) break;
    int* ex_k = sExp + pb * (MAXD + 1);
    int* ex_n = sExp + (pb ^ 1) * (MAXD + 1);
    float* nrm_k = sNrm + pb * NRM_STRIDE;
    float* nrm_n = sNrm + (pb ^ 1) * NRM_STRIDE;
    const long long ent = dk.ent;
    Out* yp = y_ptr<Out>(p, ent);
    const In* xnext = nullptr;
    if (lt == 0) {
      EntryDesc dn;
      next_desc(dn);
      sDesc[pb ^ 1] = dn;
      if (dn.flags & ED_VALID) xnext = x_ptr<In>(p, dn.ent);
    }
#pragma unroll
    for (int f = 0; f < FPT; ++f) {
      float sq = 0.f;
      if (fthr[f]) {
        const V a = Pol::make(af[f], Pol::SCALED ? ex_k[al[f]] : 0);
        Pol::template store_factor<NN>(sA, lt + f * G, a);
        if constexpr (Pol::SCALED) sq = a.hi * a.hi;
      }
      if constexpr (Pol::SCALED) warp_run_add(nrm_k, al[f], sq, fthr[f]);
    }
    if (lt <= MAXD) ex_n[lt] = 0;
    if (lt == 0) {
      sFlag[pb ^ 1] = 0;
      if (sMode[0]) {
        const bool ok = (p.wait_expire && uses == 0) ? false : mbar_wait(bar, uses & 1);
        if (!ok) {
          atomicOr(&sFlag[pb], TF_TIMEOUT);
          // The bulk copy may still be writing the staging block: wait for it
          // once more under the same bound, so that the group never leaves
          // with a copy into shared memory in flight.
          mbar_wait(bar, uses & 1);
        }
        ++uses;
      }
      if (!yp || !x_ptr<In>(p, ent)) atomicOr(&sFlag[pb], TF_NULL);
    }
    group_sync(g, G);  // S1: X staged, factors in shared memory, next descriptor published
    // the other parity's guard sums: entry k-1 has been decided, k+1 starts later
    if (Pol::SCALED && lt < NRM_STRIDE) nrm_n[lt] = 0.f;
    const int flags = sFlag[pb];
    if (flags & TF_TIMEOUT) {
      if (lt == 0) atomicOr(p.status, DF_WAIT_TIMEOUT);
      return;
    }
    const EntryDesc dn = sDesc[pb ^ 1];
    const bool has_next = (dn.flags & ED_VALID) != 0;
    const bool first = (dk.flags & ED_FIRST) != 0;
    const bool last = !has_next || (dn.flags & ED_FIRST);
    const In* anext[FPT];
#pragma unroll
    for (int f = 0; f < FPT; ++f)
      anext[f] = (has_next && fthr[f]) ? a_ptr<In>(p, dn.ent, al[f]) : nullptr;

    auto fetch_next_factor = [&]() {
#pragma unroll
      for (int f = 0; f < FPT; ++f) {
        if (fthr[f] && has_next) {
          if (anext[f]) {
            af[f] = anext[f][aoff[f]];
          } else {
            atomicOr(&sFlag[pb ^ 1], TF_NULL);
          }
        }
      }
    };
    auto reduce_next_scale = [&]() {
      if constexpr (Pol::SCALED) {
#pragma unroll
        for (int f = 0; f < FPT; ++f)
          if (fthr[f] && has_next && anext[f]) atomicMax(&ex_n[al[f]], exp_field(af[f]));
      }
    };
    // Deterministic mode, an entry without a contribution: keep the
    // segment accumulator consistent (start it at zero, flush it at the end).
    auto seg_fixup = [&]() {
      if constexpr (SEG) {
        for (int u = lt; u < NTL; u += G) {
          const int base = tile_base<NN, D, LP>(u);
#pragma unroll
          for (int t = 0; t < TL; ++t) {
            const int q = base + tile_off<NN, D, LP>(t);
            const Out a = first ? Out(0) : acc[q];
            if (last) {
              if (yp) yp[q] += a;
            } else {
              acc[q] = a;
            }
          }
        }
      }
    };
    if (flags & TF_NULL) {
      if (lt == 0) {
        atomicOr(p.status, DF_NULL_PTR);
        if (has_next) issue_x(xnext);
      }
      seg_fixup();
      fetch_next_factor();
      reduce_next_scale();
      group_sync(g, G);
      continue;
    }

    // ---- X tile of phase 0 and the block scale ----
    const In* xs = sMode[0] ? stage : x_ptr<In>(p, ent);
    In xv[ONE ? T0 : 1];
    int ex = 0, escale = 0;
    if constexpr (ONE) {
      if (lt < NT0) {
        const int base = tile_base<NN, D, 0>(lt);
#pragma unroll
        for (int t = 0; t < T0; ++t) xv[t] = xs[base + tile_off<NN, D, 0>(t)];
      }
    }
    if constexpr (Pol::SCALED) {
      int exl = 0;
      if constexpr (ONE) {
        if (lt < NT0) {
#pragma unroll
          for (int t = 0; t < T0; ++t) exl = max(exl, exp_field(xv[t]));
        }
      } else {
        for (int i = lt; i < N; i += G) exl = max(exl, exp_field(xs[i]));
      }
      exl = __reduce_max_sync(0xffffffffu, exl);
      if ((lt & 31) == 0 && exl > 0) atomicMax(&ex_k[MAXD], exl);
    }
    if constexpr (Pol::SCALED || ONE) {
      group_sync(g, G);  // S2: X tiles in registers (stage free), block scale final
    }
    if (ONE && lt == 0 && has_next) issue_x(xnext);
    if constexpr (Pol::SCALED) {
      ex = ex_k[MAXD];
      escale = ex - 1023;
      bool skip = ex == 0, nonfinite = ex == 2047;
#pragma unroll
      for (int l = 0; l < D; ++l) {
        escale += ex_k[l] - 1023;
        skip = skip || ex_k[l] == 0;
        nonfinite = nonfinite || ex_k[l] == 2047;
      }
      if (skip || nonfinite) {
        if (!ONE && lt == 0 && has_next) issue_x(xnext);
        if constexpr (std::is_same<In, double>::value) {
          // Inf/NaN propagate exactly as in FP64: plain FP64 on the same
          // shared memory (an all-zero factor or X contributes exactly zero).
          if (nonfinite) {
            nonfinite_entry<NN>(p, ent, reinterpret_cast<double*>(sA),
                                reinterpret_cast<double*>(buf), lt, G, g);
            group_sync(g, G);
          }
        }
        seg_fixup();
        fetch_next_factor();
        reduce_next_scale();
        group_sync(g, G);
        continue;
      }
    }

    // ---- phase 0: registers -> buf ----
    float gsum = 0.f;  // guard: this thread's part of ||X||^2, then of ||KX||^2
    if constexpr (ONE) {
      if (lt < NT0) {
        V v[T0];
#pragma unroll
        for (int t = 0; t < T0; ++t) {
          v[t] = Pol::make(xv[t], ex);
          if constexpr (Pol::SCALED) gsum = __fmaf_rn(v[t].hi, v[t].hi, gsum);
        }
        contract_tile<Pol, NN, PAIR0>(v, Pol::template factor<NN>(sA, a0),
                                      Pol::template factor<NN>(sA, b0));
        const int base = tile_base<NN, D, 0>(lt);
#pragma unroll
        for (int t = 0; t < T0; ++t) buf[slot<NN>(base + tile_off<NN, D, 0>(t))] = v[t];
      }
    } else {
      for (int u = lt; u < NT0; u += G) {
        const int base = tile_base<NN, D, 0>(u);
        V v[T0];
#pragma unroll
        for (int t = 0; t < T0; ++t) {
          v[t] = Pol::make(xs[base + tile_off<NN, D, 0>(t)], ex);
          if constexpr (Pol::SCALED) gsum = __fmaf_rn(v[t].hi, v[t].hi, gsum);
        }
        contract_tile<Pol, NN, PAIR0>(v, Pol::template factor<NN>(sA, a0),
                                      Pol::template factor<NN>(sA, b0));
#pragma unroll
        for (int t = 0; t < T0; ++t) buf[slot<NN>(base + tile_off<NN, D, 0>(t))] = v[t];
      }
    }
    if constexpr (Pol::SCALED) {
      gsum = warp_sum(gsum);
      if ((lt & 31) == 0) atomicAdd(&nrm_k[MAXD], gsum);
      gsum = 0.f;
    }
    fetch_next_factor();
    group_sync(g, G);  // S3: buf complete; the staging block is free
    if (!ONE && lt == 0 && has_next) issue_x(xnext);
    middle_phases<Pol, NN, D, G, 1>(buf, sA, lt, g);
    // ---- last phase: buf -> Y ----
    for (int u = lt; u < NTL; u += G) {
      const int base = tile_base<NN, D, LP>(u);
      V v[TL];
#pragma unroll
      for (int t = 0; t < TL; ++t) v[t] = buf[slot<NN>(base + tile_off<NN, D, LP>(t))];
      contract_tile<Pol, NN, PAIRL>(v, Pol::template factor<NN>(sA, aL),
                                    Pol::template factor<NN>(sA, bL));
#pragma unroll
      for (int t = 0; t < TL; ++t) {
        const int q = base + tile_off<NN, D, LP>(t);
        if constexpr (Pol::SCALED) gsum = __fmaf_rn(v[t].hi, v[t].hi, gsum);
        const Out y = Pol::finish(v[t], escale);
        if constexpr (SEG) {
          const Out a = first ? y : acc[q] + y;
          if (last) {
            yp[q] += a;
          } else {
            acc[q] = a;
          }
        } else {
          atomicAdd(yp + q, y);
        }
      }
    }
    if constexpr (Pol::SCALED) {
      gsum = warp_sum(gsum);
      if ((lt & 31) == 0) atomicAdd(&nrm_k[MAXD + 1], gsum);
    }
    reduce_next_scale();
    group_sync(g, G);  // trailing: sA, buf reusable; next entry's scales final
    if constexpr (Pol::SCALED) {
      // cancellation guard (uniform over the group): redo in FP64 if rho_F < 1/4
      if (!p.guard_off && guard_fails(nrm_k[MAXD + 1], nrm_k[MAXD], nrm_k, D, N)) {
        guard_redo<Pol, NN, D, SEG>(p, ent, sA, buf, acc, yp, escale, last, lt, g);
        group_sync(g, G);
      }
    }
  }
}

}  // namespace tile
}  // namespace kmx
