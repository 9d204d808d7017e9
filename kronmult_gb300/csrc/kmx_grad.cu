// kmx_grad.cu -- fused forward + backward of the batched Kronecker mat-vec.
//
// For one entry, with Y = (A_1 x ... x A_d) X and an upstream gradient G
// (loss = sum G .* Y):
//   F_k = X with modes l < k contracted by A_l        (forward intermediates)
//   B_k = G with modes l > k contracted by A_l^T      (backward intermediates)
//   dA_k(a, b) = sum over the other indices of B_k[.., a, ..] * F_k[.., b, ..]
//   dX = A_1^T applied to B_1  ( = (A_1^T x ... x A_d^T) G )
//   Y  = A_d applied to F_d
// (0-based in the code: modes 0..d-1.)  The forward intermediates are
// recomputed from X on chip -- a forward call stores nothing -- and kept in
// shared memory when they fit, else in a per-group slot of the caller's
// workspace.  The B sweep runs in place in shared memory; each Gram is
// accumulated per thread in registers and reduced with shared-memory atomics.
// Every output is accumulated into (Y +=, dX +=, dA +=) like Y in the forward
// entry points.  Flops: 3d mode products versus d for the forward.
#include <cuda_runtime.h>

#include "../../include/kronmult_gb300.h"
#include "kmx_engine.cuh"
#include "kmx_grad.h"
#include "kmx_launch.cuh"

namespace kmx {

namespace {

template <typename T, int NN>
__device__ __forceinline__ void mode_apply(const T* src, T* dst, const T* A, bool transA, int s,
                                           int F, int lt, int G) {
  // dst[o, a, r] = sum_j A(a, j) src[o, j, r] along the mode of stride s; dst may equal src
  const FastDiv fd((unsigned)s);
  for (int f = lt; f < F; f += G) {
    const unsigned o = fd((unsigned)f);
    const int r0 = f - (int)o * s;
    const long long base = (long long)o * NN * s + r0;
    T v[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) v[j] = src[base + (long long)j * s];
#pragma unroll
    for (int a = 0; a < NN; ++a) {
      // A(a, j) = A[a*NN + j]; its transpose reads A[j*NN + a]
      T acc = (transA ? A[0 * NN + a] : A[a * NN + 0]) * v[0];
#pragma unroll
      for (int j = 1; j < NN; ++j) acc = fma(transA ? A[j * NN + a] : A[a * NN + j], v[j], acc);
      dst[base + (long long)a * s] = acc;
    }
  }
}

// sdA[q] += the sum over the G threads of acc[q] (q < NN^2), with one FP64 add
// per partial: neighbouring lanes pre-add their partials (one shuffle and one
// add each), halving the shared-memory partials, then 32-wide chunks are
// summed and the chunk sums added.  Every thread of the block calls it.
template <typename T, int NN>
__device__ __forceinline__ void gram_reduce(const T (&acc)[NN * NN], T* sdA, T* sRed, int lt,
                                            int G) {
  constexpr int NN2 = NN * NN;
  const int GH = G / 2;
#pragma unroll
  for (int q = 0; q < NN2; ++q) {
    const T other = __shfl_down_sync(0xffffffffu, acc[q], 1);
    if ((lt & 1) == 0) sRed[q * GH + (lt >> 1)] = acc[q] + other;
  }
  __syncthreads();
  const int nch = GH / 32;
  T* sRed2 = sRed + NN2 * GH;
  for (int t = lt; t < NN2 * nch; t += G) {
    const int q = t / nch, c = t - q * nch;
    const T* src = sRed + q * GH + c * 32;
    T v = src[0];
#pragma unroll 8
    for (int i = 1; i < 32; ++i) v += src[i];
    sRed2[t] = v;
  }
  __syncthreads();
  for (int q = lt; q < NN2; q += G) {
    T v = sRed2[q * nch];
    for (int c = 1; c < nch; ++c) v += sRed2[q * nch + c];
    sdA[q] += v;
  }
}

// Gram along the mode of stride s: dA(a, b) += sum over fibers B[a] * Fk[b].
//
// NN <= 5: a thread owns whole fibers, loads each fiber's NN values of B and
// of Fk once (Fk may live in global memory) and accumulates all NN^2 products
// in registers.  The G x NN^2 partial sums are then reduced through shared
// memory (sRed: NN^2 x G, sRed2: NN^2 x G/32) with one FP64 add per partial --
// a shuffle tree would spend five adds per partial on the narrow FP64 pipe.
// NN > 5 (NN^2 accumulators would not fit in registers): thread t owns the
// pair (a, b) = t mod NN^2 and every (G / NN^2)-th fiber; one atomic each.
template <typename T, int NN>
__device__ __forceinline__ void mode_gram(const T* B, const T* Fk, T* sdA, T* sRed, int s, int F,
                                          int lt, int G) {
  constexpr int NN2 = NN * NN;
  const FastDiv fd((unsigned)s);
  if constexpr (NN <= 5) {
    T acc[NN2];
#pragma unroll
    for (int q = 0; q < NN2; ++q) acc[q] = T(0);
    for (int f = lt; f < F; f += G) {
      const unsigned o = fd((unsigned)f);
      const int r = f - (int)o * s;
      const long long base = (long long)o * NN * s + r;
      T bv[NN], x[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        bv[j] = B[base + (long long)j * s];
        x[j] = Fk[base + (long long)j * s];
      }
#pragma unroll
      for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int b = 0; b < NN; ++b) acc[a * NN + b] = fma(bv[a], x[b], acc[a * NN + b]);
    }
    gram_reduce<T, NN>(acc, sdA, sRed, lt, G);
  } else {
    const int chunks = G / NN2;
    if (lt >= chunks * NN2) return;
    const int pr = lt % NN2, c0 = lt / NN2;
    const int a = pr / NN, b = pr - a * NN;
    T acc = T(0);
    for (int f = c0; f < F; f += chunks) {
      const unsigned o = fd((unsigned)f);
      const int r = f - (int)o * s;
      const long long base = (long long)o * NN * s + r;
      acc = fma(B[base + (long long)a * s], Fk[base + (long long)b * s], acc);
    }
    atomicAdd(&sdA[pr], acc);
  }
}

// One entry, FP64 (or FP32) arithmetic.  sA holds A_l row-major:
// sA[l*NN*NN + a*NN + j] = A_l(a, j).  Every thread of the block calls it.
template <typename T, int NN>
__device__ __forceinline__ void grad_entry(const GradProblem& gp, long long e, T* sA, T* sdA,
                                           T* sB, T* sRed, T* Fst, int lt, int G) {
  constexpr int NN2 = NN * NN;
  const int d = gp.d, N = gp.N, F = N / NN;
  const T* Ae = static_cast<const T*>(gp.A) + e * d * NN2;
  for (int i = lt; i < d * NN2; i += G) {
    const int l = i / NN2, r = i - l * NN2, a = r / NN, j = r - a * NN;
    sA[i] = Ae[l * NN2 + a + j * NN];
    sdA[i] = T(0);
  }
  __syncthreads();
  const T* Xe = static_cast<const T*>(gp.X) + e * N;
  const T* Ge = static_cast<const T*>(gp.G) + e * N;
  // forward sweep: F_{k+1} = mode k of F_k, F_0 = X
  int s = N / NN;
  for (int k = 0; k < d - 1; ++k, s /= NN) {
    const T* src = k == 0 ? Xe : Fst + (long long)(k - 1) * N;
    mode_apply<T, NN>(src, Fst + (long long)k * N, sA + k * NN2, false, s, F, lt, G);
    __syncthreads();
  }
  // forward output (s is now 1: the last mode)
  if (gp.Y) {
    T* Ye = static_cast<T*>(gp.Y) + e * N;
    const T* src = d == 1 ? Xe : Fst + (long long)(d - 2) * N;
    const T* Ad = sA + (d - 1) * NN2;
    for (int i = lt; i < N; i += G) {
      const int f = i / NN, a = i - f * NN;
      T acc = Ad[a * NN] * src[(long long)f * NN];
#pragma unroll
      for (int j = 1; j < NN; ++j) acc = fma(Ad[a * NN + j], src[(long long)f * NN + j], acc);
      Ye[i] += acc;
    }
  }
  // backward sweep from B = G
  for (int i = lt; i < N; i += G) sB[i] = Ge[i];
  __syncthreads();
  s = 1;
  for (int k = d - 1; k >= 0; --k, s *= NN) {
    const T* Fk = k == 0 ? Xe : Fst + (long long)(k - 1) * N;
    if (gp.dA) mode_gram<T, NN>(sB, Fk, sdA + k * NN2, sRed, s, F, lt, G);
    if (k > 0) {
      __syncthreads();  // the Gram read sB before it is overwritten
      mode_apply<T, NN>(sB, sB, sA + k * NN2, true, s, F, lt, G);
      __syncthreads();
    } else if (gp.dX) {
      T* dXe = static_cast<T*>(gp.dX) + e * N;
      // dX += A_0^T along mode 0 (stride N / NN), one output per thread
      const FastDiv fd((unsigned)s);
      for (int f = lt; f < F; f += G) {
        const unsigned o = fd((unsigned)f);
        const int r0 = f - (int)o * s;
        const long long base = (long long)o * NN * s + r0;
        T v[NN];
#pragma unroll
        for (int j = 0; j < NN; ++j) v[j] = sB[base + (long long)j * s];
#pragma unroll
        for (int a = 0; a < NN; ++a) {
          T acc = sA[0 * NN + a] * v[0];
#pragma unroll
          for (int j = 1; j < NN; ++j) acc = fma(sA[j * NN + a], v[j], acc);
          dXe[base + (long long)a * s] += acc;
        }
      }
    }
  }
  __syncthreads();
  if (gp.dA) {
    T* dAe = static_cast<T*>(gp.dA) + e * d * NN2;
    for (int i = lt; i < d * NN2; i += G) {
      const int l = i / NN2, r = i - l * NN2, a = r / NN, b = r - a * NN;
      dAe[l * NN2 + a + b * NN] += sdA[i];
    }
  }
  __syncthreads();
}

// Shared memory of the fused kernels, in T-sized elements: factors, dA
// accumulators, the backward intermediate, the Gram partials (n <= 5), and the
// forward intermediates when they fit.
template <typename T, int NN>
struct GradSmem {
  T *sA, *sdA, *sB, *sRed, *sF;
  __device__ GradSmem(unsigned char* smem, int N, int G) {
    constexpr int NN2 = NN * NN;
    sA = reinterpret_cast<T*>(smem);
    sdA = sA + MAXD * NN2;
    sB = sdA + MAXD * NN2;
    sRed = sB + N;
    sF = sRed + (NN <= 5 ? NN2 * (G / 2 + G / 64) : 0);
  }
};

template <typename T, int NN>
__global__ void __launch_bounds__(NN <= 5 ? 512 : 256) grad_kernel(const GradProblem gp) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lt = threadIdx.x, G = blockDim.x;
  const GradSmem<T, NN> m(smem, gp.N, G);
  const long long slot = blockIdx.x;
  T* Fst = gp.f_in_smem ? m.sF : (gp.W ? static_cast<T*>(gp.W) + slot * gp.wslot : nullptr);
  if (Fst == nullptr) {
    if (lt == 0) atomicOr(gp.status, DF_NULL_PTR);
    return;
  }
  for (long long e = blockIdx.x; e < gp.batch; e += gridDim.x)
    grad_entry<T, NN>(gp, e, m.sA, m.sdA, m.sB, m.sRed, Fst, lt, G);
}

// ---------------------------------------------------------------------------
// Split (double-float) form of the fused kernel, FP64 only: the mode products
// and the Gram sums run on the FP32 pipe with every FP64 value carried as an
// unevaluated FP32 pair, as in the forward split kernels.  Per entry, X, G
// and each factor are scaled by the powers of two of their largest exponent
// fields (sx, sg, sa_l); the stored pairs then carry
//   F_k: sx + sum_{l<k} sa_l,   B_k: sg + sum_{l>k} sa_l,
//   dA_k: sg + sx + sum_{l!=k} sa_l,   Y and dX: sx (sg) + sum_l sa_l,
// and are widened to FP64 by exponent arithmetic where they leave.  The Gram
// partials of a block are reduced as pairs and widened once per output.
// Entries with Inf/NaN or an all-zero X, G or factor run grad_entry in FP64
// (so IEEE propagation and exact zeros are those of FP64).
// ---------------------------------------------------------------------------


__device__ __forceinline__ double widen_pair(df v, int escale) {
  return f32_to_f64_scaled(v.hi, escale) + f32_to_f64_scaled(v.lo, escale);
}

// a + b for normalised pairs (same scale): exact two-sum of the high parts,
// low parts and error added, renormalised.
__device__ __forceinline__ df df_add(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  df r;
  r.hi = __fadd_rn(s, e);
  r.lo = __fsub_rn(e, __fsub_rn(r.hi, s));
  return r;
}

// The pair form of gram_reduce: the G threads' partials (all at one scale)
// are summed as pairs on the FP32 pipe and widened once per output,
// sdA[q] += 2^escale * sum.  sRed holds pairs in the FP64 slots.  Every
// thread of the block calls it.
template <int NN>
__device__ __forceinline__ void gram_reduce_df(const df (&acc)[NN * NN], double* sdA,
                                               double* sRed, int escale, int lt, int G) {
  constexpr int NN2 = NN * NN;
  df* sR = reinterpret_cast<df*>(sRed);
  const int GH = G / 2;
#pragma unroll
  for (int q = 0; q < NN2; ++q) {
    df other;
    other.hi = __shfl_down_sync(0xffffffffu, acc[q].hi, 1);
    other.lo = __shfl_down_sync(0xffffffffu, acc[q].lo, 1);
    if ((lt & 1) == 0) sR[q * GH + (lt >> 1)] = df_add(acc[q], other);
  }
  __syncthreads();
  const int nch = GH / 32;
  df* sR2 = sR + NN2 * GH;
  for (int t = lt; t < NN2 * nch; t += G) {
    const int q = t / nch, c = t - q * nch;
    const df* src = sR + q * GH + c * 32;
    df v = src[0];
#pragma unroll 8
    for (int i = 1; i < 32; ++i) v = df_add(v, src[i]);
    sR2[t] = v;
  }
  __syncthreads();
  for (int q = lt; q < NN2; q += G) {
    df v = sR2[q * nch];
    for (int c = 1; c < nch; ++c) v = df_add(v, sR2[q * nch + c]);
    sdA[q] += widen_pair(v, escale);
  }
}

// One fiber's NN values: FP64 X split on the fly (FROM_X), else stored pairs.
template <int NN, bool FROM_X>
__device__ __forceinline__ void load_fiber(df (&v)[NN], const double* X, int ex, const df* src,
                                           long long base, int s) {
#pragma unroll
  for (int j = 0; j < NN; ++j)
    v[j] = FROM_X ? split_scaled(__ldg(X + base + (long long)j * s), ex) : src[base + (long long)j * s];
}

// dst[o, a, r] = sum_j A(a, j) src[o, j, r] along the mode of stride s (pairs;
// dst may equal src).  With OUT the results are widened by 2^escale and added
// to the FP64 array out instead.
template <int NN, bool FROM_X, bool OUT>
__device__ __forceinline__ void mode_apply_df(const double* X, int ex, const df* src, df* dst,
                                              double* out, int escale, const df* A, bool transA,
                                              int s, int F, int lt, int G) {
  const FastDiv fd((unsigned)s);
  for (int f = lt; f < F; f += G) {
    const unsigned o = fd((unsigned)f);
    const int r0 = f - (int)o * s;
    const long long base = (long long)o * NN * s + r0;
    df v[NN];
    load_fiber<NN, FROM_X>(v, X, ex, src, base, s);
    // rows one at a time above n = 5: all NN^2 factor pairs in registers at
    // once would cost the occupancy these small-block launches need
#pragma unroll(NN <= 5 ? NN : 1)
    for (int a = 0; a < NN; ++a) {
      df ar[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) ar[j] = transA ? A[j * NN + a] : A[a * NN + j];
      const df r = df_dot<NN>(ar, v);
      if (OUT) {
        out[base + (long long)a * s] += widen_pair(r, escale);
      } else {
        dst[base + (long long)a * s] = r;
      }
    }
  }
}

// Gram of pairs: sdA(a, b) += 2^escale * sum over fibers B[a] * Fk[b].
template <int NN, bool FROM_X>
__device__ __forceinline__ void mode_gram_df(const df* B, const double* X, int ex, const df* Fk,
                                             double* sdA, double* sRed, int escale, int s, int F,
                                             int lt, int G) {
  constexpr int NN2 = NN * NN;
  const FastDiv fd((unsigned)s);
  if constexpr (NN <= 5) {
    DfSum acc[NN2];
#pragma unroll
    for (int q = 0; q < NN2; ++q) acc[q].zero();
    for (int f = lt; f < F; f += G) {
      const unsigned o = fd((unsigned)f);
      const int r = f - (int)o * s;
      const long long base = (long long)o * NN * s + r;
      df bv[NN], x[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) bv[j] = B[base + (long long)j * s];
      load_fiber<NN, FROM_X>(x, X, ex, Fk, base, s);
#pragma unroll
      for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int b = 0; b < NN; ++b) acc[a * NN + b].add(bv[a], x[b]);
    }
    df w[NN2];
#pragma unroll
    for (int q = 0; q < NN2; ++q) w[q] = acc[q].pair();
    gram_reduce_df<NN>(w, sdA, sRed, escale, lt, G);
  } else {
    const int chunks = G / NN2;
    if (lt >= chunks * NN2) return;
    const int pr = lt % NN2, c0 = lt / NN2;
    const int a = pr / NN, b = pr - a * NN;
    DfSum acc;
    acc.zero();
    for (int f = c0; f < F; f += chunks) {
      const unsigned o = fd((unsigned)f);
      const int r = f - (int)o * s;
      const long long base = (long long)o * NN * s + r;
      const df xb = FROM_X ? split_scaled(__ldg(X + base + (long long)b * s), ex)
                           : Fk[base + (long long)b * s];
      acc.add(B[base + (long long)a * s], xb);
    }
    atomicAdd(&sdA[pr], acc.widen(escale));
  }
}

// The FP64 path for the split kernel's special entries, out of line so that
// its registers do not set the kernel's.
template <int NN>
__device__ __noinline__ void grad_entry_fp64(const GradProblem& gp, long long e, double* sA,
                                             double* sdA, double* sB, double* sRed, double* Fst,
                                             int lt, int G) {
  grad_entry<double, NN>(gp, e, sA, sdA, sB, sRed, Fst, lt, G);
}

// n > 5 is held to 64 registers (four 256-thread CTAs per SM): small entries
// such as d=3 n=8 launch 64-thread CTAs and are latency-bound (0.210 ms at 108
// registers, 0.193 at 64, measured on GB300).
template <int NN>
__global__ void __launch_bounds__(NN <= 5 ? 512 : 256, NN <= 5 ? 0 : 4) grad_split_kernel(const GradProblem gp) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NN2 = NN * NN;
  const int d = gp.d, N = gp.N, F = N / NN;
  const int lt = threadIdx.x, G = blockDim.x;
  const GradSmem<double, NN> m(smem, N, G);  // pairs occupy the FP64 slots
  int* sExp = reinterpret_cast<int*>(smem + gp.exp_off);  // [MAXD] factors, X, G
  const long long slot = blockIdx.x;
  double* Fst = gp.f_in_smem ? m.sF
                             : (gp.W ? static_cast<double*>(gp.W) + slot * gp.wslot : nullptr);
  if (Fst == nullptr) {
    if (lt == 0) atomicOr(gp.status, DF_NULL_PTR);
    return;
  }
  df* sA = reinterpret_cast<df*>(m.sA);
  df* sB = reinterpret_cast<df*>(m.sB);
  df* Fs = reinterpret_cast<df*>(Fst);
  for (long long e = blockIdx.x; e < gp.batch; e += gridDim.x) {
    const double* Ae = static_cast<const double*>(gp.A) + e * d * NN2;
    const double* Xe = static_cast<const double*>(gp.X) + e * N;
    const double* Ge = static_cast<const double*>(gp.G) + e * N;
    // --- scales: largest exponent field of each factor, of X and of G ---
    if (lt < MAXD + 2) sExp[lt] = 0;
    __syncthreads();
    for (int l = 0; l < d; ++l) {
      int em = 0;
      for (int i = lt; i < NN2; i += G) em = max(em, exp_field(Ae[l * NN2 + i]));
      em = __reduce_max_sync(0xffffffffu, em);  // one shared atomic per warp
      if ((lt & 31) == 0 && em > 0) atomicMax(&sExp[l], em);
    }
    {
      int ex = 0, eg = 0;
      for (int i = lt; i < N; i += G) {
        ex = max(ex, exp_field(__ldg(Xe + i)));
        eg = max(eg, exp_field(__ldg(Ge + i)));
      }
      ex = __reduce_max_sync(0xffffffffu, ex);
      eg = __reduce_max_sync(0xffffffffu, eg);
      if ((lt & 31) == 0) {
        if (ex > 0) atomicMax(&sExp[MAXD], ex);
        if (eg > 0) atomicMax(&sExp[MAXD + 1], eg);
      }
    }
    __syncthreads();
    const int ex = sExp[MAXD], eg = sExp[MAXD + 1];
    bool special = ex == 0 || ex == 2047 || eg == 0 || eg == 2047;
    int sa[MAXD], sum_a = 0;
#pragma unroll
    for (int l = 0; l < MAXD; ++l) {
      sa[l] = l < d ? sExp[l] - 1023 : 0;
      if (l < d) special = special || sExp[l] == 0 || sExp[l] == 2047;
      sum_a += sa[l];
    }
    // (sExp is reset only by the next entry, after this entry's last barrier)
    if (special) {
      grad_entry_fp64<NN>(gp, e, m.sA, m.sdA, m.sB, m.sRed, Fst, lt, G);
      continue;
    }
    const int sx = ex - 1023, sg = eg - 1023;
    // --- factors as pairs, row-major: sA[l*NN2 + a*NN + j] = A_l(a, j) ---
    for (int i = lt; i < d * NN2; i += G) {
      const int l = i / NN2, r = i - l * NN2, a = r / NN, j = r - a * NN;
      sA[i] = split_scaled(Ae[l * NN2 + a + j * NN], sExp[l]);
      m.sdA[i] = 0.0;
    }
    __syncthreads();
    // forward sweep: F_{k+1} = mode k of F_k, F_0 = X
    int s = N / NN;
    for (int k = 0; k < d - 1; ++k, s /= NN) {
      if (k == 0) {
        mode_apply_df<NN, true, false>(Xe, ex, nullptr, Fs, nullptr, 0, sA, false, s, F, lt, G);
      } else {
        mode_apply_df<NN, false, false>(nullptr, 0, Fs + (long long)(k - 1) * N,
                                        Fs + (long long)k * N, nullptr, 0, sA + k * NN2, false, s,
                                        F, lt, G);
      }
      __syncthreads();
    }
    if (gp.Y) {  // the last mode (stride 1) into Y
      double* Ye = static_cast<double*>(gp.Y) + e * N;
      if (d == 1) {
        mode_apply_df<NN, true, true>(Xe, ex, nullptr, nullptr, Ye, sx + sum_a, sA, false, 1, F,
                                      lt, G);
      } else {
        mode_apply_df<NN, false, true>(nullptr, 0, Fs + (long long)(d - 2) * N, nullptr, Ye,
                                       sx + sum_a, sA + (d - 1) * NN2, false, 1, F, lt, G);
      }
    }
    // backward sweep from B = G
    for (int i = lt; i < N; i += G) sB[i] = split_scaled(__ldg(Ge + i), eg);
    __syncthreads();
    s = 1;
    for (int k = d - 1; k >= 0; --k, s *= NN) {
      if (gp.dA) {
        const int esc = sg + sx + sum_a - sa[k];
        if (k == 0) {
          mode_gram_df<NN, true>(sB, Xe, ex, nullptr, m.sdA, m.sRed, esc, s, F, lt, G);
        } else {
          mode_gram_df<NN, false>(sB, nullptr, 0, Fs + (long long)(k - 1) * N, m.sdA + k * NN2,
                                  m.sRed, esc, s, F, lt, G);
        }
      }
      if (k > 0) {
        __syncthreads();  // the Gram read sB before it is overwritten
        mode_apply_df<NN, false, false>(nullptr, 0, sB, sB, nullptr, 0, sA + k * NN2, true, s, F,
                                        lt, G);
        __syncthreads();
      } else if (gp.dX) {
        double* dXe = static_cast<double*>(gp.dX) + e * N;
        mode_apply_df<NN, false, true>(nullptr, 0, sB, nullptr, dXe, sg + sum_a, sA, true, s, F,
                                       lt, G);
      }
    }
    __syncthreads();
    if (gp.dA) {
      double* dAe = static_cast<double*>(gp.dA) + e * d * NN2;
      for (int i = lt; i < d * NN2; i += G) {
        const int l = i / NN2, r = i - l * NN2, a = r / NN, b = r - a * NN;
        dAe[l * NN2 + a + b * NN] += m.sdA[i];
      }
    }
    __syncthreads();
  }
}

template <int NN>
const void* grad_split_func() {
  return reinterpret_cast<const void*>(&grad_split_kernel<NN>);
}

const void* pick_grad_split(int n) {
  switch (n) {
    case 2: return grad_split_func<2>();
    case 3: return grad_split_func<3>();
    case 4: return grad_split_func<4>();
    case 5: return grad_split_func<5>();
    case 6: return grad_split_func<6>();
    case 7: return grad_split_func<7>();
    case 8: return grad_split_func<8>();
    default: return nullptr;
  }
}

template <typename T, int NN>
const void* grad_func() {
  return reinterpret_cast<const void*>(&grad_kernel<T, NN>);
}

template <typename T>
const void* pick_grad(int n) {
  switch (n) {
    case 2: return grad_func<T, 2>();
    case 3: return grad_func<T, 3>();
    case 4: return grad_func<T, 4>();
    case 5: return grad_func<T, 5>();
    case 6: return grad_func<T, 6>();
    case 7: return grad_func<T, 7>();
    case 8: return grad_func<T, 8>();
    default: return nullptr;
  }
}

// Launch shape and memory plan of the fused kernel for (d, n).
struct GradPlan {
  int threads;
  size_t smem;
  int f_in_smem;
  size_t slot_bytes;  // workspace per concurrent entry when !f_in_smem
  bool ok;
};

// Threads: one fiber per thread up to 512 for n <= 5 and 256 above (the
// fused kernel is FP64-pipe bound and needs many warps to hide the FP64 and
// shared-memory latency; large entries hold one CTA per SM in shared memory;
// n > 5 keeps 256 so that its kernels are not capped at 128 registers),
// multiples of 64 (the Gram reduction pairs lanes).  Falls back to fewer
// threads when the Gram scratch does not fit.
template <typename T>
GradPlan grad_plan(int d, int n, long long N, int max_smem) {
  GradPlan g;
  int threads = (int)((N / n + 63) / 64 * 64);
  if (threads < 64) threads = 64;
  if (threads > (n <= 5 ? 512 : 256)) threads = n <= 5 ? 512 : 256;  // the kernels' launch bounds
  for (;; threads /= 2) {
    g.threads = threads;
    const size_t red = n <= 5 ? (size_t)n * n * (threads / 2 + threads / 64) * sizeof(T) : 0;
    const size_t head = 2 * (size_t)MAXD * n * n * sizeof(T) + red;
    const size_t with_f = head + (size_t)N * sizeof(T) * (d > 1 ? d : 1);
    const size_t without_f = head + (size_t)N * sizeof(T);
    g.slot_bytes = (size_t)(d > 1 ? d - 1 : 1) * N * sizeof(T);
    if (with_f <= 200 * 1024) {
      g.f_in_smem = 1;
      g.smem = with_f;
      g.ok = true;
    } else {
      g.f_in_smem = 0;
      g.smem = without_f;
      g.ok = without_f <= (size_t)max_smem;
    }
    if (g.ok || threads <= 64) return g;
  }
}

// form: KMX_FORM_PLAIN runs FP64 (FP32) arithmetic; any other form runs the
// double-float kernel for FP64 data.
// engine: KMX_ENGINE_PER_MODE runs the CTA-per-entry kernels above; any other
// value runs FP64 data one warp per entry (kmx_grad_warp.cu) where the entry's
// factors and intermediates fit in the warp's share of shared memory.
template <typename T>
int grad_impl(int d, int n, const T* A, const T* X, const T* G, T* Y, T* dX, T* dA, T* W,
              size_t Wbytes, int batch, int form, int engine, cudaStream_t s) {
  if (d < 1 || d > MAXD || n < 1 || batch < 0) return KMX_ERR_INVALID_ARG;
  if (form != KMX_FORM_AUTO && form != KMX_FORM_PLAIN && form != KMX_FORM_SPLIT &&
      form != KMX_FORM_DIGITS)
    return KMX_ERR_INVALID_ARG;
  if (batch == 0) return KMX_OK;
  if (!A || !X || !G) return KMX_ERR_NULL_POINTER;
  const bool split = sizeof(T) == 8 && form != KMX_FORM_PLAIN;
  const void* func = split ? pick_grad_split(n) : pick_grad<T>(n);
  if (!func) return KMX_ERR_UNSUPPORTED;
  long long N = 1;
  for (int i = 0; i < d; ++i) N *= n;
  if (N > (1LL << 28)) return KMX_ERR_UNSUPPORTED;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KMX_ERR_CUDA;
  const DeviceInfo di = device_info(dev);
  GradProblem gp;
  gp.d = d;
  gp.N = (int)N;
  gp.batch = batch;
  gp.A = A;
  gp.X = X;
  gp.G = G;
  gp.Y = Y;
  gp.dX = dX;
  gp.dA = dA;
  gp.W = W;
  gp.wslot = (long long)(d > 1 ? d - 1 : 1) * N;
  if (sizeof(T) == 8 && engine != KMX_ENGINE_PER_MODE && grad_warp_bytes(d, n) > 0) {
    int rc = device_status_ptr(&gp.status);
    if (rc != KMX_OK) return rc;
    gp.W = nullptr;
    gp.wslot = 0;
    gp.nslots = 0;
    gp.f_in_smem = 1;
    gp.exp_off = 0;
    return launch_grad_warp(gp, n, split, s);
  }
  const GradPlan plan = grad_plan<T>(d, n, N, di.max_smem_optin);
  if (!plan.ok) return KMX_ERR_UNSUPPORTED;
  const int threads = plan.threads;
  // the split kernel keeps its per-entry exponents after the plan's layout
  gp.exp_off = (int)((plan.smem + 15) / 16 * 16);
  const size_t smem = split ? (size_t)gp.exp_off + 64 : plan.smem;
  if (smem > (size_t)di.max_smem_optin) return KMX_ERR_UNSUPPORTED;
  gp.f_in_smem = plan.f_in_smem;
  if (plan.f_in_smem) {
    gp.nslots = batch;
  } else {
    gp.nslots = W ? (int)(Wbytes / plan.slot_bytes < (size_t)batch ? Wbytes / plan.slot_bytes : batch) : 0;
    if (gp.nslots < 1) return KMX_ERR_WORKSPACE;
  }
  int rc = device_status_ptr(&gp.status);
  if (rc != KMX_OK) return rc;
  cudaError_t e = ensure_smem(func, dev, smem);
  if (e != cudaSuccess) return KMX_ERR_CUDA;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, threads, smem);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)di.sms * per_sm;
  if (grid > batch) grid = batch;
  if (!gp.f_in_smem && grid > gp.nslots) grid = gp.nslots;
  void* args[] = {&gp};
  e = cudaLaunchKernel(func, dim3((unsigned)grid), dim3(threads), args, smem, s);
  return e == cudaSuccess ? KMX_OK : KMX_ERR_CUDA;
}

}  // namespace
}  // namespace kmx

extern "C" size_t kmx_grad_workspace_bytes(int d, int n, int batchCount, int fp64) {
  if (d < 1 || d > kmx::MAXD || n < 1 || batchCount <= 0) return 0;
  long long N = 1;
  for (int i = 0; i < d; ++i) N *= n;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  const kmx::DeviceInfo di = kmx::device_info(dev);
  const kmx::GradPlan g = fp64 ? kmx::grad_plan<double>(d, n, N, di.max_smem_optin)
                               : kmx::grad_plan<float>(d, n, N, di.max_smem_optin);
  if (!g.ok || g.f_in_smem) return 0;
  long long slots = (long long)di.sms * 2;
  if (slots > batchCount) slots = batchCount;
  return (size_t)slots * g.slot_bytes;
}

static int default_form() {
  kmx_options o;
  kmx_get_default_options(&o);
  return o.form;
}

extern "C" int kmx_kronmult_batched_grad_f64(int d, int n, const double* A, const double* X,
                                             const double* G, double* Y, double* dX, double* dA,
                                             double* W, size_t Wcapacity_bytes, int batchCount,
                                             kmx_stream_t stream) {
  return kmx::grad_impl<double>(d, n, A, X, G, Y, dX, dA, W, Wcapacity_bytes, batchCount,
                                default_form(), KMX_ENGINE_TUNED,
                                reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int kmx_kronmult_batched_grad_f64_ex(int d, int n, const double* A, const double* X,
                                                const double* G, double* Y, double* dX,
                                                double* dA, double* W, size_t Wcapacity_bytes,
                                                int batchCount, const kmx_options* opt,
                                                kmx_stream_t stream) {
  return kmx::grad_impl<double>(d, n, A, X, G, Y, dX, dA, W, Wcapacity_bytes, batchCount,
                                opt ? opt->form : default_form(),
                                opt ? opt->engine : KMX_ENGINE_TUNED,
                                reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int kmx_kronmult_batched_grad_f32(int d, int n, const float* A, const float* X,
                                             const float* G, float* Y, float* dX, float* dA,
                                             float* W, size_t Wcapacity_bytes, int batchCount,
                                             kmx_stream_t stream) {
  return kmx::grad_impl<float>(d, n, A, X, G, Y, dX, dA, W, Wcapacity_bytes, batchCount,
                               KMX_FORM_PLAIN, KMX_ENGINE_TUNED,
                               reinterpret_cast<cudaStream_t>(stream));
}
