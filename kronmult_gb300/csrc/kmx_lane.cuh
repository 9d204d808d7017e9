// kmx_lane.cuh -- one entry per thread, for square entries small enough to
// live in a thread's registers: n^2 <= 16 per factor and n^d <= 16 elements
// (d = 1, 2 with n <= 4; d = 3 with n = 2).
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

}  // namespace lane
}  // namespace kmx
