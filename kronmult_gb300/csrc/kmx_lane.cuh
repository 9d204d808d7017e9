// kmx_lane.cuh -- one entry per thread, for square entries small enough to
// live in a thread's registers: n^2 <= 16 per factor and n^d <= 16 elements
// (d = 1, 2 with n <= 4; d = 3 with n = 2); and, in namespaces group and
// fiber, d = 2 with n = 5..8 (one group of n lanes per entry) and d >= 3 with
// n^(d-1) <= 32 (one fiber per lane), described there.
//
// The small-entry kernels (kmx_small.cuh) spread an entry over one thread per
// output element, so every per-entry quantity -- the scale exponents of X and
// of each factor, the cancellation guard's norms, the decision to recompute in
// FP64 -- is a reduction across threads with a barrier, and for 4 to 16
// elements those reductions cost more than the arithmetic.  Here a thread
// holds its entry's X, intermediate and the factor being applied in
// registers: the exponents and norms are in-thread maxima and sums, the d mode
// products are fully unrolled register contractions (the reference's mode
// order, A1 first), and an entry whose double-float result would cancel, or
// that holds Inf/NaN, is evaluated in FP64 by the same thread before anything
// is written -- nothing has to be taken back.  Y is updated in place where Y
// blocks are exclusive, with atomics otherwise.
//
// Arithmetic policies: plain FMA in T, FP32 with each dot product rounded once
// (RD, the reference's float semantics), and double-float with per-entry
// power-of-two scales (LaneSplit: the arithmetic of the other double-float
// kernels, the cancellation guard of kmx_engine.cuh, FP64 for Inf/NaN, an
// all-zero X or factor contributing exactly zero).
#pragma once

#include "kmx_engine.cuh"
#include "kmx_tile.cuh"

namespace kmx {
namespace lane {

using tile::ipow;

constexpr int THREADS = 128;

__host__ __device__ constexpr bool supported(int NN, int D) {
  return D >= 1 && D <= 3 && NN >= 2 && NN * NN <= 16 && ipow(NN, D) <= 16;
}

template <typename T, bool RD>
struct LanePlain {
  using S = T;  // storage type
  using V = T;
  static constexpr bool SPLIT = false;
  static constexpr bool ROUNDED = RD;  // each dot product rounded once
  template <int NN>
  __device__ __forceinline__ static V dot(const V* a, const V* v) {
    return dot_n<T, RD, NN>(a, v);
  }
};

struct LaneSplit {
  using S = double;
  using V = df;
  static constexpr bool SPLIT = true;
  template <int NN>
  __device__ __forceinline__ static V dot(const V* a, const V* v) {
    return df_dot<NN>(a, v);
  }
};

// A(i, j) of the applied factor (column-major with leading dimension ld;
// transposed: A(j, i)).
template <typename T>
__device__ __forceinline__ T fac(const T* A, int ld, bool trans, int i, int j) {
  return trans ? A[j + (long long)i * ld] : A[i + (long long)j * ld];
}

// Mode K of a register-resident block: v <- A_K applied along mode K (stride
// NN^(D-1-K)); a[i*NN + j] = A_K(i, j).
template <class Pol, int NN, int D, int K>
__device__ __forceinline__ void apply_mode(typename Pol::V (&v)[ipow(NN, D)],
                                           const typename Pol::V (&a)[NN * NN]) {
  using V = typename Pol::V;
  constexpr int N = ipow(NN, D), S = ipow(NN, D - 1 - K);
  V out[N];
#pragma unroll
  for (int f = 0; f < N / NN; ++f) {
    const int base = (f / S) * NN * S + f % S;
    V fib[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) fib[j] = v[base + j * S];
#pragma unroll
    for (int i = 0; i < NN; ++i) out[base + i * S] = Pol::template dot<NN>(a + i * NN, fib);
  }
#pragma unroll
  for (int q = 0; q < N; ++q) v[q] = out[q];
}

// Plain forms: every mode in T, then Y += the block.
template <class Pol, int NN, int D, int K>
__device__ __forceinline__ void plain_modes(typename Pol::V (&v)[ipow(NN, D)],
                                            const typename Pol::S* const* A, const int* ld,
                                            bool trans) {
  if constexpr (K < D) {
    typename Pol::V a[NN * NN];
#pragma unroll
    for (int i = 0; i < NN; ++i)
#pragma unroll
      for (int j = 0; j < NN; ++j) a[i * NN + j] = fac(A[K], ld[K], trans, i, j);
    apply_mode<Pol, NN, D, K>(v, a);
    plain_modes<Pol, NN, D, K + 1>(v, A, ld, trans);
  }
}

template <class Pol, int NN, int D>
__device__ __forceinline__ void plain_entry(const typename Pol::S* X, typename Pol::S* Y,
                                            const typename Pol::S* const* A, const int* ld,
                                            bool trans, bool excl) {
  constexpr int N = ipow(NN, D);
  typename Pol::V v[N];
#pragma unroll
  for (int q = 0; q < N; ++q) v[q] = X[q];
  plain_modes<Pol, NN, D, 0>(v, A, ld, trans);
#pragma unroll
  for (int q = 0; q < N; ++q) y_accumulate(Y + q, v[q], excl);
}

// The FP64 evaluation of a double-float entry (Inf/NaN, or rejected by the
// guard), out of line so that its registers do not set the kernel's.
template <int NN, int D>
__device__ __noinline__ void fp64_entry(const double* X, double* Y, const double* const* A,
                                        const int* ld, bool trans, bool excl) {
  plain_entry<LanePlain<double, false>, NN, D>(X, Y, A, ld, trans, excl);
}

// Double-float modes: factor K is read, scaled by its largest exponent field
// (ea[K]) and split as it is applied; a2[K] collects its squared norm.
template <int NN, int D, int K>
__device__ __forceinline__ void split_modes(df (&v)[ipow(NN, D)], const double* const* A,
                                            const int* ld, bool trans, int* ea, float* a2) {
  if constexpr (K < D) {
    double raw[NN * NN];
    int e = 0;
#pragma unroll
    for (int i = 0; i < NN; ++i)
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        raw[i * NN + j] = fac(A[K], ld[K], trans, i, j);
        e = max(e, exp_field(raw[i * NN + j]));
      }
    ea[K] = e;
    df a[NN * NN];
    float s2 = 0.f;
#pragma unroll
    for (int t = 0; t < NN * NN; ++t) {
      a[t] = split_scaled(raw[t], e);
      s2 = __fmaf_rn(a[t].hi, a[t].hi, s2);
    }
    a2[K] = s2;
    apply_mode<LaneSplit, NN, D, K>(v, a);
    split_modes<NN, D, K + 1>(v, A, ld, trans, ea, a2);
  }
}

template <int NN, int D>
__device__ __forceinline__ void split_entry(const Problem& p, const double* X, double* Y,
                                            const double* const* A, const int* ld, bool trans,
                                            bool excl) {
  constexpr int N = ipow(NN, D);
  double xr[N];
  int ex = 0;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    xr[q] = X[q];
    ex = max(ex, exp_field(xr[q]));
  }
  df v[N];
  float x2 = 0.f;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    v[q] = split_scaled(xr[q], ex);
    x2 = __fmaf_rn(v[q].hi, v[q].hi, x2);
  }
  int ea[D];
  float a2[D];
  split_modes<NN, D, 0>(v, A, ld, trans, ea, a2);
  bool zero = ex == 0, nonfinite = ex == 2047;
  int escale = ex - 1023;
#pragma unroll
  for (int l = 0; l < D; ++l) {
    zero = zero || ea[l] == 0;
    nonfinite = nonfinite || ea[l] == 2047;
    escale += ea[l] - 1023;
  }
  if (nonfinite) {  // Inf/NaN propagate exactly as in FP64 (0 * Inf included)
    fp64_entry<NN, D>(X, Y, A, ld, trans, excl);
    return;
  }
  if (zero) return;  // an all-zero factor or X: kron(...) X is exactly zero
  float out2 = 0.f;
#pragma unroll
  for (int q = 0; q < N; ++q) out2 = __fmaf_rn(v[q].hi, v[q].hi, out2);
  if (!p.guard_off && guard_fails(out2, x2, a2, D, N)) {  // cancellation: FP64 instead
    fp64_entry<NN, D>(X, Y, A, ld, trans, excl);
    count_redo(p.redo_ctr, 0);
    return;
  }
#pragma unroll
  for (int q = 0; q < N; ++q)
    y_accumulate(Y + q, f32_to_f64_scaled(v[q].hi, escale) + f32_to_f64_scaled(v[q].lo, escale),
                 excl);
}

// Thread t of CTA b takes entries b*THREADS + t, then every (grid*THREADS)-th.
template <class Pol, int NN, int D>
__global__ void __launch_bounds__(THREADS) lane_kernel(const Problem p) {
  using S = typename Pol::S;
  const long long count = launch_count(p);
  const bool excl = p.y_exclusive != 0;
  const bool trans = p.trans != 0;
  int ld[D];
#pragma unroll
  for (int l = 0; l < D; ++l) ld[l] = p.ld[l];
  for (long long e = (long long)blockIdx.x * THREADS + threadIdx.x; e < count;
       e += (long long)gridDim.x * THREADS) {
    const long long ent = tile::entry_index(p, e);
    const S* X = tile::x_ptr<S>(p, ent);
    S* Y = tile::y_ptr<S>(p, ent);
    const S* A[D];
    bool null = X == nullptr || Y == nullptr;
#pragma unroll
    for (int l = 0; l < D; ++l) {
      A[l] = tile::a_ptr<S>(p, ent, l);
      null = null || A[l] == nullptr;
    }
    if (null) {
      atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    if constexpr (Pol::SPLIT) {
      split_entry<NN, D>(p, X, Y, A, ld, trans, excl);
    } else {
      plain_entry<Pol, NN, D>(X, Y, A, ld, trans, excl);
    }
  }
}

// ---------------------------------------------------------------------------
// d = 2 with n = 5..8: one group of n lanes per entry (32/n groups per warp).
//
// With the X block as the n x n matrix M(j1, j2) = X[j1*n + j2], lane r of
// the group first holds column r of M (loads of consecutive elements across
// the group) and forms column r of T = A1 M (mode 1, the reference's order);
// T goes through the group's shared memory, and lane r then holds row r of T
// and forms row r of Y = T A2^T (mode 2), which it adds to Y.  Every factor
// row is read by all lanes of the group from shared memory, where each lane
// stores the column it loaded.  Per-entry quantities (exponents, guard norms)
// are reduced by n shuffles within the group; there is no block barrier, and
// groups run independently (shuffles and syncs carry the group's mask).
// Double-float dots run on packed FP32 pairs (two rows of the factor per
// instruction, kmx_pack.cuh); entries the guard rejects or holding Inf/NaN
// are evaluated in FP64 by the same group, mode by mode, before anything is
// written.
// ---------------------------------------------------------------------------
namespace group {

constexpr int THREADS = 128;
constexpr int WARPS = THREADS / 32;

__host__ __device__ constexpr bool supported(int NN, int D) {
  return D == 2 && NN >= 5 && NN <= 8;
}

// Shared memory of one group, in 8-byte words: the two factors (row pairs
// of (hi, lo) for the double-float form, else row-major T) and the n x (n+1)
// transpose tile; rounded to 2 mod 16 words so that the groups of a warp start
// on different banks.
template <class Pol, int NN>
struct Layout {
  static constexpr int RP = (NN + 1) / 2;
  static constexpr int FAC_WORDS =
      Pol::SPLIT ? 2 * RP * NN : (int)((NN * NN * sizeof(typename Pol::S) + 7) / 8);
  static constexpr int TILE_WORDS = (int)((NN * (NN + 1) * sizeof(typename Pol::S) + 7) / 8);
  static constexpr int RAW = 2 * FAC_WORDS + TILE_WORDS;
  static constexpr int WORDS = (RAW + 13) / 16 * 16 + 2;
  static constexpr int GPW = 32 / NN;
  static constexpr int CTA_WORDS = WARPS * GPW * WORDS;
};

// The group's maximum: n shuffles for n <= 6; one __reduce_max_sync for
// n = 7, 8, where it needs fewer registers (the shuffles measured faster at
// n = 5, 6, where the reduction raised the register count).
template <int NN>
__device__ __forceinline__ int gmax(int v, unsigned gm, int base) {
  if constexpr (NN >= 7) {
    return (int)__reduce_max_sync(gm, (unsigned)v);
  } else {
    int m = v;
#pragma unroll
    for (int k = 0; k < NN; ++k) m = max(m, __shfl_sync(gm, v, base + k));
    return m;
  }
}
// the group's sum, added in lane order (the same value in every lane)
template <int NN>
__device__ __forceinline__ float gsum(float v, unsigned gm, int base) {
  float s = __shfl_sync(gm, v, base);
#pragma unroll
  for (int k = 1; k < NN; ++k) s = __fadd_rn(s, __shfl_sync(gm, v, base + k));
  return s;
}

// Plain forms (and the FP64 evaluation of double-float entries): factors
// read as rows from fr (row-major, shared memory) or, with fr == nullptr,
// from global memory; the tile holds T.
template <typename T, bool RD, int NN>
__device__ __forceinline__ void plain_modes(const T* X, T* Y, const T* A0, const T* A1, int ld0,
                                            int ld1, bool trans, bool excl, const T* f0,
                                            const T* f1, T* tile, int r, unsigned gm) {
  T v[NN], yo[NN];
#pragma unroll
  for (int j = 0; j < NN; ++j) v[j] = X[j * NN + r];  // column r of M
  if (excl) {  // row r of Y, loaded with X (no load latency at the end)
#pragma unroll
    for (int i = 0; i < NN; ++i) yo[i] = Y[r * NN + i];
  }
#pragma unroll
  for (int i = 0; i < NN; ++i) {
    T a[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) a[j] = f0 ? f0[i * NN + j] : fac(A0, ld0, trans, i, j);
    tile[i * (NN + 1) + r] = dot_n<T, RD, NN>(a, v);
  }
  __syncwarp(gm);
#pragma unroll
  for (int j = 0; j < NN; ++j) v[j] = tile[r * (NN + 1) + j];  // row r of T
#pragma unroll
  for (int i = 0; i < NN; ++i) {
    T a[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) a[j] = f1 ? f1[i * NN + j] : fac(A1, ld1, trans, i, j);
    const T y = dot_n<T, RD, NN>(a, v);
    if (excl) {
      Y[r * NN + i] = yo[i] + y;
    } else {
      atomicAdd(Y + r * NN + i, y);
    }
  }
}

template <int NN>
__device__ __noinline__ void fp64_group_entry(const double* X, double* Y, const double* A0,
                                              const double* A1, int ld0, int ld1, bool trans,
                                              bool excl, double* tile, int r, unsigned gm) {
  __syncwarp(gm);  // every lane is done with the tile
  plain_modes<double, false, NN>(X, Y, A0, A1, ld0, ld1, trans, excl, nullptr, nullptr, tile, r,
                                 gm);
}

// Packed double-float dots of one mode: out[i] (i < NN) = sum_j A(i, j) v[j]
// for the factor's row pairs fp (RowPair (rp, j) at fp[rp*NN + j]).
template <int NN>
__device__ __forceinline__ void split_mode(const pk2::RowPair* fp, const df (&v)[NN],
                                           df (&out)[NN]) {
  using pk2::u64;
  u64 vh[NN], vl[NN], nvh[NN];
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    vh[j] = pk2::bcast(v[j].hi);
    vl[j] = pk2::bcast(v[j].lo);
    nvh[j] = pk2::bcast(-v[j].hi);
  }
#pragma unroll
  for (int rp = 0; rp < (NN + 1) / 2; ++rp) {
    u64 oh, ol;
    pk2::dot_pair<NN>(fp + rp * NN, vh, vl, nvh, oh, ol);
    float h0, h1, l0, l1;
    pk2::unpack(oh, h0, h1);
    pk2::unpack(ol, l0, l1);
    out[2 * rp] = df{h0, l0};
    if (2 * rp + 1 < NN) out[2 * rp + 1] = df{h1, l1};
  }
}

// Column r of factor a (a[i] = A(i, r), split with exponent e) into row
// pairs: RowPair (rp, r) = ((A(2rp, r), A(2rp+1, r)) high parts, low parts).
template <int NN>
__device__ __forceinline__ float store_column(pk2::RowPair* fp, const double (&a)[NN], int e,
                                              int r) {
  float s2 = 0.f;
#pragma unroll
  for (int rp = 0; rp < (NN + 1) / 2; ++rp) {
    const df x0 = split_scaled(a[2 * rp], e);
    const df x1 = 2 * rp + 1 < NN ? split_scaled(a[2 * rp + 1], e) : df{0.f, 0.f};
    s2 = __fmaf_rn(x0.hi, x0.hi, s2);
    s2 = __fmaf_rn(x1.hi, x1.hi, s2);
    pk2::RowPair q;
    q.hi = pk2::pack(x0.hi, x1.hi);
    q.lo = pk2::pack(x0.lo, x1.lo);
    fp[rp * NN + r] = q;
  }
  return s2;
}

template <int NN>
__device__ __forceinline__ void split_group_entry(const Problem& p, const double* X, double* Y,
                                                  const double* A0, const double* A1, int ld0,
                                                  int ld1, bool trans, bool excl, uint64_t* region,
                                                  int r, unsigned gm, int base) {
  using L = Layout<LaneSplit, NN>;
  pk2::RowPair* f0 = reinterpret_cast<pk2::RowPair*>(region);
  pk2::RowPair* f1 = f0 + L::RP * NN;
  df* tile = reinterpret_cast<df*>(region + 2 * L::FAC_WORDS);
  double xr[NN], c0[NN], c1[NN];
  int ex = 0, e0 = 0, e1 = 0;
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    xr[j] = X[j * NN + r];
    c0[j] = fac(A0, ld0, trans, j, r);
    c1[j] = fac(A1, ld1, trans, j, r);
    ex = max(ex, exp_field(xr[j]));
    e0 = max(e0, exp_field(c0[j]));
    e1 = max(e1, exp_field(c1[j]));
  }
  ex = gmax<NN>(ex, gm, base);
  e0 = gmax<NN>(e0, gm, base);
  e1 = gmax<NN>(e1, gm, base);
  df v[NN];
  float x2 = 0.f;
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    v[j] = split_scaled(xr[j], ex);
    x2 = __fmaf_rn(v[j].hi, v[j].hi, x2);
  }
  float a2[2];
  a2[0] = store_column<NN>(f0, c0, e0, r);
  a2[1] = store_column<NN>(f1, c1, e1, r);
  __syncwarp(gm);
  df t[NN];
  split_mode<NN>(f0, v, t);  // column r of T
#pragma unroll
  for (int i = 0; i < NN; ++i) tile[i * (NN + 1) + r] = t[i];
  __syncwarp(gm);
#pragma unroll
  for (int j = 0; j < NN; ++j) v[j] = tile[r * (NN + 1) + j];  // row r of T
  split_mode<NN>(f1, v, t);  // row r of Y
  float out2 = 0.f;
#pragma unroll
  for (int i = 0; i < NN; ++i) out2 = __fmaf_rn(t[i].hi, t[i].hi, out2);
  x2 = gsum<NN>(x2, gm, base);
  a2[0] = gsum<NN>(a2[0], gm, base);
  a2[1] = gsum<NN>(a2[1], gm, base);
  out2 = gsum<NN>(out2, gm, base);
  const bool nonfinite = ex == 2047 || e0 == 2047 || e1 == 2047;
  const bool zero = ex == 0 || e0 == 0 || e1 == 0;
  if (nonfinite) {  // Inf/NaN propagate exactly as in FP64 (0 * Inf included)
    fp64_group_entry<NN>(X, Y, A0, A1, ld0, ld1, trans, excl, reinterpret_cast<double*>(tile), r,
                         gm);
    return;
  }
  if (zero) return;  // an all-zero factor or X: kron(...) X is exactly zero
  if (!p.guard_off && guard_fails(out2, x2, a2, 2, NN * NN)) {  // cancellation: FP64 instead
    fp64_group_entry<NN>(X, Y, A0, A1, ld0, ld1, trans, excl, reinterpret_cast<double*>(tile), r,
                         gm);
    if (r == 0) count_redo(p.redo_ctr, 0);
    return;
  }
  const int escale = (ex - 1023) + (e0 - 1023) + (e1 - 1023);
  // Y by atomic adds even where blocks are exclusive: the add runs in L2, off
  // this kernel's busiest pipe (FP64: the widening adds and the split's
  // int -> float conversions), and with one writer per block it rounds once,
  // exactly as a read-modify-write would
#pragma unroll
  for (int i = 0; i < NN; ++i)
    atomicAdd(Y + r * NN + i,
              f32_to_f64_scaled(t[i].hi, escale) + f32_to_f64_scaled(t[i].lo, escale));
}

// Group g of warp w takes entries (blockIdx.x*WARPS + w)*GPW + g, then every
// (gridDim.x*WARPS*GPW)-th; lanes beyond the last whole group stay idle.
// Double-float, n = 6 is held to 6 CTAs per SM (80 registers) and n = 7, 8
// to 5 (96): measured 3-8 % faster than the compiler's choice (96 / 112 / 122
// registers), with at most 28 bytes of spill.
template <class Pol, int NN>
__global__ void __launch_bounds__(THREADS, Pol::SPLIT ? (NN >= 7 ? 5 : (NN == 6 ? 6 : 0)) : 0)
    group_kernel(const Problem p) {
  using S = typename Pol::S;
  using L = Layout<Pol, NN>;
  __shared__ __align__(16) uint64_t sm[L::CTA_WORDS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane / NN, r = lane - g * NN;
  if (g >= L::GPW) return;
  const int base = g * NN;
  const unsigned gm = ((1u << NN) - 1u) << base;
  uint64_t* region = sm + (warp * L::GPW + g) * L::WORDS;
  const long long count = launch_count(p);
  const bool excl = p.y_exclusive != 0;
  const bool trans = p.trans != 0;
  const int ld0 = p.ld[0], ld1 = p.ld[1];
  const long long stride = (long long)gridDim.x * WARPS * L::GPW;
  for (long long e = ((long long)blockIdx.x * WARPS + warp) * L::GPW + g; e < count; e += stride) {
    const long long ent = tile::entry_index(p, e);
    const S* X = tile::x_ptr<S>(p, ent);
    S* Y = tile::y_ptr<S>(p, ent);
    const S* A0 = tile::a_ptr<S>(p, ent, 0);
    const S* A1 = tile::a_ptr<S>(p, ent, 1);
    if (X == nullptr || Y == nullptr || A0 == nullptr || A1 == nullptr) {
      if (r == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    if constexpr (Pol::SPLIT) {
      split_group_entry<NN>(p, X, Y, A0, A1, ld0, ld1, trans, excl, region, r, gm, base);
    } else {
      S* f0 = reinterpret_cast<S*>(region);
      S* f1 = f0 + NN * NN;
      S* tl = reinterpret_cast<S*>(region + 2 * L::FAC_WORDS);
#pragma unroll
      for (int i = 0; i < NN; ++i) {  // column r of each factor, stored row-major
        f0[i * NN + r] = fac(A0, ld0, trans, i, r);
        f1[i * NN + r] = fac(A1, ld1, trans, i, r);
      }
      __syncwarp(gm);
      plain_modes<S, Pol::ROUNDED, NN>(X, Y, A0, A1, ld0, ld1, trans, excl, f0, f1, tl, r, gm);
    }
    __syncwarp(gm);  // the group's shared memory is free for the next entry
  }
}

}  // namespace group

// ---------------------------------------------------------------------------
// d >= 3 with n^(d-1) <= 32 (d = 3 with n = 3..5, d = 4 with n = 2, 3, d = 5, 6
// with n = 2): one group of L = n^(d-1) lanes per entry, one fiber per lane
// and mode.
//
// Mode k contracts index k (stride S_k = n^(d-1-k)); lane l's fiber in mode k
// starts at b_k(l) = (l / S_k) n S_k + l % S_k, so mode 0 reads X with
// consecutive lanes on consecutive elements (b_0(l) = l) and mode d-1 leaves
// lane l the contiguous row Y[l n .. l n + n).  The intermediates live in the
// group's shared memory with one pad word per n (row reads conflict-free);
// each lane overwrites its own fiber in place (fibers of one mode partition
// the block), with a group sync between modes.  Lane l < n^2 loads entry
// (l % n, l / n) of every factor (a column-major sweep) and stores it,
// split, into the factor's row layout.  Reductions: butterflies when L is a
// power of two, else L shuffles (sums) and __reduce_max_sync (maxima); the
// double-float dots, the guard and the FP64 path are those of the group kernel.
// ---------------------------------------------------------------------------
namespace fiber {

constexpr int THREADS = 128;
constexpr int WARPS = THREADS / 32;

__host__ __device__ constexpr bool supported(int NN, int D) {
  return D >= 3 && D <= 6 && NN >= 2 && ipow(NN, D - 1) <= 32 && !lane::supported(NN, D);
}

template <class Pol, int NN, int D>
struct Layout {
  static constexpr int L = ipow(NN, D - 1);
  static constexpr int N = NN * L;
  static constexpr int RP = (NN + 1) / 2;
  static constexpr int FAC_WORDS =
      Pol::SPLIT ? 2 * RP * NN : (int)((NN * NN * sizeof(typename Pol::S) + 7) / 8);
  static constexpr int TILE_ELEMS = N + L;  // one pad per n
  static constexpr int TILE_WORDS = (int)((TILE_ELEMS * sizeof(typename Pol::S) + 7) / 8);
  static constexpr int RAW = D * FAC_WORDS + TILE_WORDS;
  static constexpr int WORDS = (RAW + 13) / 16 * 16 + 2;
  static constexpr int GPW = 32 / L;
  static constexpr int CTA_WORDS = WARPS * GPW * WORDS;
};

template <int NN>
__device__ __forceinline__ int pq(int q) {
  return q + q / NN;
}
template <int NN, int D>
__device__ __forceinline__ int fiber_base(int l, int k) {
  const int S = ipow(NN, D - 1 - k);
  return (l / S) * NN * S + l % S;
}

// Group-wide max and sum (every lane gets the same value).
template <int L>
__device__ __forceinline__ int fmax_g(int v, unsigned gm, int base) {
  if constexpr ((L & (L - 1)) == 0) {
#pragma unroll
    for (int o = 1; o < L; o <<= 1) v = max(v, __shfl_xor_sync(gm, v, o));
    return v;
  } else {
    return (int)__reduce_max_sync(gm, (unsigned)v);
  }
}
template <int L>
__device__ __forceinline__ float fsum_g(float v, unsigned gm, int base) {
  if constexpr ((L & (L - 1)) == 0) {
    // a butterfly: each level adds the same two partial sums in every lane
#pragma unroll
    for (int o = 1; o < L; o <<= 1) v = __fadd_rn(v, __shfl_xor_sync(gm, v, o));
    return v;
  } else {
    return group::gsum<L>(v, gm, base);
  }
}

// Plain forms and the FP64 path: factors as rows from f (shared memory) or,
// with f == nullptr, from global memory; T the intermediate tile.
template <typename T, bool RD, int NN, int D>
__device__ __forceinline__ void plain_fibers(const T* X, T* Y, const T* const* A, const int* ld,
                                             bool trans, bool excl, const T* f, T* tile, int l,
                                             unsigned gm) {
  constexpr int L = ipow(NN, D - 1), NN2 = NN * NN;
  T v[NN], yo[NN];
#pragma unroll
  for (int j = 0; j < NN; ++j) v[j] = X[l + j * L];
  if (excl) {
#pragma unroll
    for (int i = 0; i < NN; ++i) yo[i] = Y[l * NN + i];
  }
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int S = ipow(NN, D - 1 - k);
    const int b = fiber_base<NN, D>(l, k);
    if (k > 0) {
      __syncwarp(gm);  // mode k-1 is complete
#pragma unroll
      for (int j = 0; j < NN; ++j) v[j] = tile[pq<NN>(b + j * S)];
    }
    T out[NN];
#pragma unroll
    for (int i = 0; i < NN; ++i) {
      T a[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j)
        a[j] = f ? f[k * NN2 + i * NN + j] : fac(A[k], ld[k], trans, i, j);
      out[i] = dot_n<T, RD, NN>(a, v);
    }
    if (k < D - 1) {
#pragma unroll
      for (int i = 0; i < NN; ++i) tile[pq<NN>(b + i * S)] = out[i];
    } else {
#pragma unroll
      for (int i = 0; i < NN; ++i) {
        if (excl) {
          Y[l * NN + i] = yo[i] + out[i];
        } else {
          atomicAdd(Y + l * NN + i, out[i]);
        }
      }
    }
  }
}

template <int NN, int D>
__device__ __noinline__ void fp64_fiber_entry(const double* X, double* Y, const double* const* A,
                                              const int* ld, bool trans, bool excl, double* tile,
                                              int l, unsigned gm) {
  __syncwarp(gm);  // every lane is done with the tile
  plain_fibers<double, false, NN, D>(X, Y, A, ld, trans, excl, nullptr, tile, l, gm);
}

template <int NN, int D>
__device__ __forceinline__ void split_fiber_entry(const Problem& p, const double* X, double* Y,
                                                  const double* const* A, const int* ld,
                                                  bool trans, bool excl, uint64_t* region, int l,
                                                  unsigned gm, int base) {
  using Lay = Layout<LaneSplit, NN, D>;
  constexpr int L = Lay::L, NN2 = NN * NN;
  float* ff = reinterpret_cast<float*>(region);  // factor k: RowPairs at word k*FAC_WORDS
  const pk2::RowPair* fp = reinterpret_cast<const pk2::RowPair*>(region);
  df* tile = reinterpret_cast<df*>(region + D * Lay::FAC_WORDS);
  double xr[NN], c[D];
  int ex = 0, ea[D];
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    xr[j] = X[l + j * L];
    ex = max(ex, exp_field(xr[j]));
  }
  const int fi = l % NN, fj = l / NN;  // the factor entry this lane loads (l < n^2)
#pragma unroll
  for (int k = 0; k < D; ++k) {
    c[k] = l < NN2 ? fac(A[k], ld[k], trans, fi, fj) : 0.0;
    ea[k] = exp_field(c[k]);
  }
  ex = fmax_g<L>(ex, gm, base);
#pragma unroll
  for (int k = 0; k < D; ++k) ea[k] = fmax_g<L>(ea[k], gm, base);
  df v[NN], t[NN];
  float x2 = 0.f, a2[D];
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    v[j] = split_scaled(xr[j], ex);
    x2 = __fmaf_rn(v[j].hi, v[j].hi, x2);
  }
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const df a = split_scaled(c[k], ea[k]);
    a2[k] = __fmul_rn(a.hi, a.hi);
    if (l < NN2) {
      // RowPair (fi/2, fj) of factor k: floats [hi(2rp), hi(2rp+1), lo(2rp), lo(2rp+1)]
      float* q = ff + 2 * k * Lay::FAC_WORDS + 4 * ((fi >> 1) * NN + fj);
      q[fi & 1] = a.hi;
      q[2 + (fi & 1)] = a.lo;
      if ((NN & 1) && fi == NN - 1) {  // the zero pad row of an odd n
        q[1] = 0.f;
        q[3] = 0.f;
      }
    }
  }
  __syncwarp(gm);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int S = ipow(NN, D - 1 - k);
    const int b = fiber_base<NN, D>(l, k);
    if (k > 0) {
      __syncwarp(gm);  // mode k-1 is complete
#pragma unroll
      for (int j = 0; j < NN; ++j) v[j] = tile[pq<NN>(b + j * S)];
    }
    group::split_mode<NN>(fp + k * (Lay::FAC_WORDS / 2), v, t);
    if (k < D - 1) {
#pragma unroll
      for (int i = 0; i < NN; ++i) tile[pq<NN>(b + i * S)] = t[i];
    }
  }
  float out2 = 0.f;
#pragma unroll
  for (int i = 0; i < NN; ++i) out2 = __fmaf_rn(t[i].hi, t[i].hi, out2);
  x2 = fsum_g<L>(x2, gm, base);
#pragma unroll
  for (int k = 0; k < D; ++k) a2[k] = fsum_g<L>(a2[k], gm, base);
  out2 = fsum_g<L>(out2, gm, base);
  bool nonfinite = ex == 2047, zero = ex == 0;
  int escale = ex - 1023;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    nonfinite = nonfinite || ea[k] == 2047;
    zero = zero || ea[k] == 0;
    escale += ea[k] - 1023;
  }
  if (nonfinite) {  // Inf/NaN propagate exactly as in FP64 (0 * Inf included)
    fp64_fiber_entry<NN, D>(X, Y, A, ld, trans, excl, reinterpret_cast<double*>(tile), l, gm);
    return;
  }
  if (zero) return;  // an all-zero factor or X: kron(...) X is exactly zero
  if (!p.guard_off && guard_fails(out2, x2, a2, D, Lay::N)) {  // cancellation: FP64 instead
    fp64_fiber_entry<NN, D>(X, Y, A, ld, trans, excl, reinterpret_cast<double*>(tile), l, gm);
    if (l == 0) count_redo(p.redo_ctr, 0);
    return;
  }
  // Y by atomic adds even where blocks are exclusive (as in the group kernel)
#pragma unroll
  for (int i = 0; i < NN; ++i)
    atomicAdd(Y + l * NN + i,
              f32_to_f64_scaled(t[i].hi, escale) + f32_to_f64_scaled(t[i].lo, escale));
}

// Group g of warp w takes entries (blockIdx.x*WARPS + w)*GPW + g, then every
// (gridDim.x*WARPS*GPW)-th; lanes beyond the last whole group stay idle.
template <class Pol, int NN, int D>
__global__ void __launch_bounds__(THREADS) fiber_kernel(const Problem p) {
  using S = typename Pol::S;
  using Lay = Layout<Pol, NN, D>;
  constexpr int L = Lay::L;
  __shared__ __align__(16) uint64_t sm[Lay::CTA_WORDS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane / L, l = lane - g * L;
  if (g >= Lay::GPW) return;
  const int base = g * L;
  const unsigned gm = (L == 32 ? 0xffffffffu : ((1u << L) - 1u)) << base;
  uint64_t* region = sm + (warp * Lay::GPW + g) * Lay::WORDS;
  const long long count = launch_count(p);
  const bool excl = p.y_exclusive != 0;
  const bool trans = p.trans != 0;
  int ld[D];
#pragma unroll
  for (int k = 0; k < D; ++k) ld[k] = p.ld[k];
  const long long stride = (long long)gridDim.x * WARPS * Lay::GPW;
  for (long long e = ((long long)blockIdx.x * WARPS + warp) * Lay::GPW + g; e < count;
       e += stride) {
    const long long ent = tile::entry_index(p, e);
    const S* X = tile::x_ptr<S>(p, ent);
    S* Y = tile::y_ptr<S>(p, ent);
    const S* A[D];
    bool null = X == nullptr || Y == nullptr;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      A[k] = tile::a_ptr<S>(p, ent, k);
      null = null || A[k] == nullptr;
    }
    if (null) {
      if (l == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    if constexpr (Pol::SPLIT) {
      split_fiber_entry<NN, D>(p, X, Y, A, ld, trans, excl, region, l, gm, base);
    } else {
      S* f = reinterpret_cast<S*>(region);  // factor k row-major at f + k*n^2
      S* tl = reinterpret_cast<S*>(region + D * Lay::FAC_WORDS);
      constexpr int NN2 = NN * NN;
      if (l < NN2) {
#pragma unroll
        for (int k = 0; k < D; ++k)
          f[k * NN2 + (l % NN) * NN + l / NN] = fac(A[k], ld[k], trans, l % NN, l / NN);
      }
      __syncwarp(gm);
      plain_fibers<S, Pol::ROUNDED, NN, D>(X, Y, A, ld, trans, excl, f, tl, l, gm);
    }
    __syncwarp(gm);  // the group's shared memory is free for the next entry
  }
}

}  // namespace fiber

}  // namespace lane
}  // namespace kmx
