// kmx_grad_warp.cu -- fused forward + backward of small entries: one warp per
// entry, every intermediate in the warp's own region of shared memory.
//
// The fused kernels of kmx_grad.cu give each entry a CTA.  An entry of a few
// hundred elements (d = 3, n = 8: 512) then keeps most of that CTA waiting at
// block barriers between steps that each hold a few fibers per thread.  Here
// a warp takes one entry at a time with its factors and d + 1 slots of its own
// region of shared memory, so every step is ordered by warp barriers alone:
//   forward   X -> slot 0, F_{k+1} = A_k x_k F_k into slot k+1 (a lane owns
//             whole mode-k fibers, two at a time), then Y += A_{d-1} x_{d-1}
//             F_{d-1} (staged in slot d, added with coalesced loads/stores);
//   backward  B = G into slot d; for k = d-1 .. 0: the Gram dA_k(a, b) += sum
//             over the mode-k fibers of B[a] F_k[b] (lane (a, s) sums row a
//             over every S-th fiber; each output adds its S partials in lane
//             order), then B = A_k^T x_k B in place; at k = 0, dX += A_0^T
//             x_0 B, staged in slot 0 (X is dead once the last Gram has run).
// Global memory is touched only by coalesced staging loads and the Y, dX and
// dA updates.  The shapes are compile-time (n, d), so every stride folds.
// FP64 data, in double-float (the split kernels' arithmetic and per-entry
// power-of-two scales, as grad_split_kernel) or native FP64 (the plain form,
// and in the split kernel the entries with Inf/NaN or an all-zero X, G or
// factor).  Flops: 3d mode products, as the CTA kernels.
#include <cuda_runtime.h>

#include <type_traits>

#include "../../include/kronmult_gb300.h"
#include "kmx_engine.cuh"
#include "kmx_grad.h"
#include "kmx_launch.cuh"
#include "kmx_pack.cuh"

namespace kmx {
namespace gw {

// Largest per-warp region taken (at least seven warps per SM).
constexpr size_t KMX_GRAD_WARP_MAX_BYTES = 32 * 1024;

// physical position of element q in a slot: one pad word per 16 for even n,
// so that mode strides that are multiples of 16 words spread over the banks
template <int NN>
__device__ __forceinline__ int ps(int q) {
  if constexpr ((NN & 1) == 0) {
    return q + (q >> 4);
  } else {
    return q;
  }
}
__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }
__host__ __device__ constexpr int slot_words(int n, int N) {
  return (n & 1) == 0 ? N + N / 16 + 1 : N;
}
// Per-warp region in 8-byte words: the factors (FP64 row-major, or for the
// packed double-float form two row-pair copies, A_l and A_l^T), d+1 slots and
// the Gram partials [32][n].
__host__ __device__ constexpr bool packed_form(int n) { return (n & 1) == 0 && n <= 4; }
__host__ __device__ constexpr int factor_words(int n, int d) {
  return (packed_form(n) ? 2 : 1) * d * n * n;
}
__host__ __device__ constexpr int warp_words(int d, int n) {
  return (factor_words(n, d) + (d + 1) * slot_words(n, ipow(n, d)) + 32 * n + 1) / 2 * 2;
}
__host__ __device__ constexpr bool warp_fits(int d, int n) {
  return d >= 3 && d <= MAXD && n >= 2 && n <= 8 &&
         (long long)warp_words(d, n) * 8 <= (long long)KMX_GRAD_WARP_MAX_BYTES;
}

// ---- arithmetic policies ---------------------------------------------------

// Double-float pairs at per-entry power-of-two scales (kmx_engine.cuh).
struct WDf {
  using V = df;
  static constexpr bool PACKED = false;
  __device__ static __forceinline__ V make(double x, int e) { return split_scaled(x, e); }
  template <int NN>
  __device__ static __forceinline__ V dot(const V* a, const V* v) {
    return df_dot<NN>(a, v);
  }
  __device__ static __forceinline__ double widen(V v, int esc) {
    return f32_to_f64_scaled(v.hi, esc) + f32_to_f64_scaled(v.lo, esc);
  }
  // a + b of normalised pairs at one scale
  __device__ static __forceinline__ V add(V a, V b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    V r;
    r.hi = __fadd_rn(s, e);
    r.lo = __fsub_rn(e, __fsub_rn(r.hi, s));
    return r;
  }
  struct Acc {
    DfSum s;
    __device__ __forceinline__ void zero() { s.zero(); }
    __device__ __forceinline__ void add(V a, V b) { s.add(a, b); }
    __device__ __forceinline__ V get() const { return s.pair(); }
  };
};

// Native FP64 (the scales are ignored).
struct WF64 {
  using V = double;
  static constexpr bool PACKED = false;
  __device__ static __forceinline__ V make(double x, int) { return x; }
  template <int NN>
  __device__ static __forceinline__ V dot(const V* a, const V* v) {
    double acc = __dmul_rn(a[0], v[0]);
#pragma unroll
    for (int j = 1; j < NN; ++j) acc = __fma_rn(a[j], v[j], acc);
    return acc;
  }
  __device__ static __forceinline__ double widen(V v, int) { return v; }
  __device__ static __forceinline__ V add(V a, V b) { return __dadd_rn(a, b); }
  struct Acc {
    double s;
    __device__ __forceinline__ void zero() { s = 0.0; }
    __device__ __forceinline__ void add(V a, V b) { s = __fma_rn(a, b, s); }
    __device__ __forceinline__ V get() const { return s; }
  };
};

// Double-float on packed FP32 pairs (kmx_pack.cuh), n = 2, 4: the mode
// products form the dot products of two output rows per instruction from
// factor row pairs (A_l and A_l^T each stored as row pairs), and the Gram sums
// accumulate two columns b, b+1 per instruction.  Values in the slots, the
// widening and the partial sums are those of WDf.  (Measured on GB300: d=4
// n=4 0.105 -> 0.091 ms, d=6 n=2 0.163 -> 0.155; n = 6, 8 gained nothing, d=3
// n=6 lost 5 %, so they keep the scalar pairs and half the factor storage.)
struct WPk : WDf {
  static constexpr bool PACKED = true;
};

// Running double-float sums of two columns: the negated sum of the high
// products (ns) and the FP32 sum of everything else (c), as in pk2::dot_pair.
struct PkSum {
  pk2::u64 ns, c;
  __device__ __forceinline__ void zero() { ns = c = 0ull; }
  // += (fh, fl) * b for the pair of values (fh, fl) and b = (bh, bl) broadcast
  __device__ __forceinline__ void add(pk2::u64 fh, pk2::u64 fl, pk2::u64 bh, pk2::u64 bl,
                                      pk2::u64 nbh) {
    const pk2::u64 q = pk2::mul(fh, nbh);  // -p, rounded
    pk2::u64 e = pk2::fma(fh, bh, q);      // f b - p, exact
    e = pk2::fma(fh, bl, e);
    e = pk2::fma(fl, bh, e);
    pk2::u64 t, te;
    pk2::two_sum(ns, q, t, te);  // -(s + p) exactly as t + te
    ns = t;
    c = pk2::add(c, pk2::sub(e, te));
  }
  // the two sums as normalised pairs
  __device__ __forceinline__ void get(df& v0, df& v1) const {
    const pk2::u64 hi = pk2::sub(c, ns);
    const pk2::u64 lo = pk2::sub(c, pk2::add(hi, ns));
    pk2::unpack(hi, v0.hi, v1.hi);
    pk2::unpack(lo, v0.lo, v1.lo);
  }
};

// ---- steps of one entry (every lane of the warp calls them) -----------------
// N = NN^D; mode K has stride S = NN^(D-1-K) and NF = N/NN fibers.

// Mode K in shared memory, fibers f = lane, lane + 32, ..., two per pass
// (their dot products share each factor row):
//   dst[o, a, r] = sum_j A(a, j) src[o, j, r],   A(a, j) = Ak[a*NN + j], or
//   Ak[j*NN + a] with TR.  dst may equal src: a lane reads its fibers whole
//   before writing them.
template <class P, int NN, int D, int K, bool TR>
__device__ __forceinline__ void mode_step(const typename P::V* src, typename P::V* dst,
                                          const typename P::V* Ak, int lane) {
  using V = typename P::V;
  constexpr int S = ipow(NN, D - 1 - K), NF = ipow(NN, D - 1);
  for (int f0 = lane; f0 < NF; f0 += 64) {
    const int f1 = f0 + 32;
    const bool two = f1 < NF;
    const int b0 = (f0 / S) * NN * S + f0 % S;
    const int b1 = two ? (f1 / S) * NN * S + f1 % S : b0;
    V v0[NN], v1[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) {
      v0[j] = src[ps<NN>(b0 + j * S)];
      v1[j] = src[ps<NN>(b1 + j * S)];
    }
    // rows one at a time above n = 5 (all NN^2 factor values at once would
    // not fit beside the fibers in the registers two CTAs per SM allow)
#pragma unroll(NN <= 5 ? NN : 1)
    for (int a = 0; a < NN; ++a) {
      V ar[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) ar[j] = TR ? Ak[j * NN + a] : Ak[a * NN + j];
      const V r0 = P::template dot<NN>(ar, v0);
      const V r1 = P::template dot<NN>(ar, v1);
      dst[ps<NN>(b0 + a * S)] = r0;
      if (two) dst[ps<NN>(b1 + a * S)] = r1;
    }
  }
}

// Packed form of mode_step: one fiber at a time, each input value broadcast
// to both halves (and negated: kmx_pack.cuh), the dot products of output rows
// (2rp, 2rp+1) from the row pairs F[rp*NN + j] of A_K (or of A_K^T).
template <int NN, int D, int K>
__device__ __forceinline__ void mode_step_pk(const df* src, df* dst, const pk2::RowPair* F,
                                             int lane) {
  using pk2::u64;
  constexpr int S = ipow(NN, D - 1 - K), NF = ipow(NN, D - 1), RP = NN / 2;
  for (int f = lane; f < NF; f += 32) {
    const int base = (f / S) * NN * S + f % S;
    u64 vh[NN], vl[NN], nvh[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) {
      const df v = src[ps<NN>(base + j * S)];
      vh[j] = pk2::bcast(v.hi);
      vl[j] = pk2::bcast(v.lo);
      nvh[j] = pk2::bcast(-v.hi);
    }
#pragma unroll(NN <= 4 ? RP : 2)
    for (int rp = 0; rp < RP; ++rp) {
      u64 oh, ol;
      pk2::dot_pair<NN>(F + rp * NN, vh, vl, nvh, oh, ol);
      df o0, o1;
      pk2::unpack(oh, o0.hi, o1.hi);
      pk2::unpack(ol, o0.lo, o1.lo);
      dst[ps<NN>(base + 2 * rp * S)] = o0;
      dst[ps<NN>(base + (2 * rp + 1) * S)] = o1;
    }
  }
}

// out[q] += 2^esc src[q], q < N: coalesced, four loads in flight per lane.
template <class P, int NN, int N>
__device__ __forceinline__ void add_out(double* out, const typename P::V* src, int esc, int lane) {
  for (int q0 = lane; q0 < N; q0 += 128) {
    double o[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) o[u] = q0 + 32 * u < N ? out[q0 + 32 * u] : 0.0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int q = q0 + 32 * u;
      if (q < N) out[q] = o[u] + P::widen(src[ps<NN>(q)], esc);
    }
  }
}

// Gram along mode K: dAk(a, b) += 2^esc sum over the fibers of B[a] F[b]
// (dAk column-major).  Lane (a, sub) = a*SG + sub, a < NN, sub < SG = 32/NN,
// sums row a over the fibers sub, sub + SG, ...; the partials go through
// `part` ([32][NN]) and each output adds its SG partials in lane order, so the
// result does not depend on timing.
template <class P, int NN, int D, int K>
__device__ __forceinline__ void gram_step(const typename P::V* B, const typename P::V* Fk,
                                          typename P::V* part, double* dAk, int esc, int lane) {
  using V = typename P::V;
  constexpr int S = ipow(NN, D - 1 - K), NF = ipow(NN, D - 1);
  constexpr int SG = 32 / NN;
  const int a = lane / SG, sub = lane - a * SG;
  if (a < NN) {
    if constexpr (P::PACKED) {
      PkSum acc[NN / 2];
#pragma unroll
      for (int b = 0; b < NN / 2; ++b) acc[b].zero();
#pragma unroll 2
      for (int f = sub; f < NF; f += SG) {
        const int base = (f / S) * NN * S + f % S;
        const df bv = B[ps<NN>(base + a * S)];
        const pk2::u64 bh = pk2::bcast(bv.hi), bl = pk2::bcast(bv.lo), nbh = pk2::bcast(-bv.hi);
#pragma unroll
        for (int b = 0; b < NN / 2; ++b) {
          const df f0 = Fk[ps<NN>(base + 2 * b * S)], f1 = Fk[ps<NN>(base + (2 * b + 1) * S)];
          acc[b].add(pk2::pack(f0.hi, f1.hi), pk2::pack(f0.lo, f1.lo), bh, bl, nbh);
        }
      }
#pragma unroll
      for (int b = 0; b < NN / 2; ++b) acc[b].get(part[lane * NN + 2 * b], part[lane * NN + 2 * b + 1]);
    } else {
      typename P::Acc acc[NN];
#pragma unroll
      for (int b = 0; b < NN; ++b) acc[b].zero();
#pragma unroll 2
      for (int f = sub; f < NF; f += SG) {
        const int base = (f / S) * NN * S + f % S;
        const V bv = B[ps<NN>(base + a * S)];
#pragma unroll
        for (int b = 0; b < NN; ++b) acc[b].add(bv, Fk[ps<NN>(base + b * S)]);
      }
#pragma unroll
      for (int b = 0; b < NN; ++b) part[lane * NN + b] = acc[b].get();
    }
  }
  __syncwarp();
  for (int t = lane; t < NN * NN; t += 32) {
    const int aa = t / NN, bb = t - aa * NN;
    V v = part[(aa * SG) * NN + bb];
#pragma unroll
    for (int u = 1; u < SG; ++u) v = P::add(v, part[(aa * SG + u) * NN + bb]);
    dAk[aa + bb * NN] += P::widen(v, esc);
  }
  __syncwarp();  // partials and the Gram's inputs read before they change
}

// Region of one warp: factors, slots 0..D (slot k: F_k, slot 0: X; slot D:
// Y staging, then B), Gram partials.
template <class P, int NN, int D>
struct Region {
  using V = typename P::V;
  static constexpr int SL = slot_words(NN, ipow(NN, D));
  V* sA;
  V* slots;
  V* Bs;
  V* part;
  __device__ __forceinline__ explicit Region(double* wbase) {
    sA = reinterpret_cast<V*>(wbase);
    slots = sA + factor_words(NN, D);
    Bs = slots + D * SL;
    part = Bs + SL;
  }
};

// Mode K with A_K (TR: A_K^T) from src into dst, in the policy's arithmetic.
// Factor storage: FP64 / WDf row-major sA[K*NN2 + a*NN + j]; WPk row pairs,
// A_K at (2K)*NN2/2 and A_K^T at (2K+1)*NN2/2 RowPairs.
template <class P, int NN, int D, int K, bool TR>
__device__ __forceinline__ void apply_mode(const Region<P, NN, D>& r, const typename P::V* src,
                                           typename P::V* dst, int lane) {
  if constexpr (P::PACKED) {
    const pk2::RowPair* F = reinterpret_cast<const pk2::RowPair*>(r.sA) + (2 * K + (TR ? 1 : 0)) * (NN * NN / 2);
    mode_step_pk<NN, D, K>(src, dst, F, lane);
  } else {
    mode_step<P, NN, D, K, TR>(src, dst, r.sA + K * NN * NN, lane);
  }
}

template <class P, int NN, int D, int K>
__device__ __forceinline__ void fwd_sweep(const Region<P, NN, D>& r, int lane) {
  if constexpr (K + 1 < D) {
    apply_mode<P, NN, D, K, false>(r, r.slots + K * r.SL, r.slots + (K + 1) * r.SL, lane);
    __syncwarp();
    fwd_sweep<P, NN, D, K + 1>(r, lane);
  }
}

template <class P, int NN, int D, int K>
__device__ __forceinline__ void bwd_sweep(const Region<P, NN, D>& r, double* dAe, double* dXe,
                                          const int* sa, int esc_dA, int esc_dX, int lane) {
  if (dAe)
    gram_step<P, NN, D, K>(r.Bs, r.slots + K * r.SL, r.part, dAe + K * NN * NN, esc_dA - sa[K],
                           lane);
  if constexpr (K > 0) {
    apply_mode<P, NN, D, K, true>(r, r.Bs, r.Bs, lane);
    __syncwarp();
    bwd_sweep<P, NN, D, K - 1>(r, dAe, dXe, sa, esc_dA, esc_dX, lane);
  } else if (dXe) {  // slot 0 is free once the last Gram has read X
    apply_mode<P, NN, D, 0, true>(r, r.Bs, r.slots, lane);
    __syncwarp();
    add_out<P, NN, ipow(NN, D)>(dXe, r.slots, esc_dX, lane);
  }
}

// One entry, with X (slot 0) and the factors (sA, row-major: sA[l*NN2 + a*NN
// + j] = A_l(a, j)) already staged as FP64 values.  ea[l], ex, eg: the
// exponent fields that scale factor l, X and G (1023 = no scaling for WF64).
template <class P, int NN, int D>
__device__ __forceinline__ void warp_entry(const GradProblem& gp, long long e, double* wbase,
                                           const int* ea, int ex, int eg, int lane) {
  using V = typename P::V;
  constexpr int NN2 = NN * NN, N = ipow(NN, D);
  const Region<P, NN, D> r(wbase);
  int sa[MAXD], sa_sum = 0;
#pragma unroll
  for (int l = 0; l < MAXD; ++l) {
    sa[l] = l < D ? ea[l] - 1023 : 0;
    sa_sum += sa[l];
  }
  const int sx = ex - 1023, sg = eg - 1023;
  if constexpr (P::PACKED) {
    // FP64 row-major -> row pairs of A_l and of A_l^T (twice the space, so
    // every lane reads its values before any lane writes)
    constexpr int RP = NN / 2, NRP = D * NN2, PER = (NRP + 31) / 32;
    const double* raw = reinterpret_cast<const double*>(r.sA);
    double x0[PER], x1[PER];
#pragma unroll
    for (int t = 0; t < PER; ++t) {
      const int idx = lane + 32 * t;
      x0[t] = x1[t] = 0.0;
      if (idx < NRP) {
        const int j = idx % NN, rp = (idx / NN) % RP, lo = idx / (NN * RP);  // lo = 2l + TR
        const double* Al = raw + (lo >> 1) * NN2;
        if (lo & 1) {  // A^T(2rp, j) = A(j, 2rp)
          x0[t] = Al[j * NN + 2 * rp];
          x1[t] = Al[j * NN + 2 * rp + 1];
        } else {
          x0[t] = Al[(2 * rp) * NN + j];
          x1[t] = Al[(2 * rp + 1) * NN + j];
        }
      }
    }
    __syncwarp();
    pk2::RowPair* pk = reinterpret_cast<pk2::RowPair*>(r.sA);
#pragma unroll
    for (int t = 0; t < PER; ++t) {
      const int idx = lane + 32 * t;
      if (idx < NRP) {
        const int e = ea[idx / (NN * RP * 2)];
        const df s0 = split_scaled(x0[t], e), s1 = split_scaled(x1[t], e);
        pk[idx].hi = pk2::pack(s0.hi, s1.hi);
        pk[idx].lo = pk2::pack(s0.lo, s1.lo);
      }
    }
  } else if constexpr (!std::is_same<V, double>::value) {
    for (int i = lane; i < D * NN2; i += 32)
      r.sA[i] = P::make(reinterpret_cast<const double*>(r.sA)[i], ea[i / NN2]);
  }
  if constexpr (!std::is_same<V, double>::value) {
    // X: FP64 -> scaled pairs in place (each lane converts what it staged)
    for (int q = lane; q < N; q += 32)
      r.slots[ps<NN>(q)] = P::make(reinterpret_cast<const double*>(r.slots)[ps<NN>(q)], ex);
    __syncwarp();
  }
  fwd_sweep<P, NN, D, 0>(r, lane);
  if (gp.Y) {  // the last mode into slot D, then Y += it
    apply_mode<P, NN, D, D - 1, false>(r, r.slots + (D - 1) * r.SL, r.Bs, lane);
    __syncwarp();
    add_out<P, NN, N>(static_cast<double*>(gp.Y) + e * N, r.Bs, sx + sa_sum, lane);
    __syncwarp();
  }
  {  // B = G into slot D
    const double* Ge = static_cast<const double*>(gp.G) + e * N;
    for (int q0 = lane; q0 < N; q0 += 128) {
      double g[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) g[u] = q0 + 32 * u < N ? __ldg(Ge + q0 + 32 * u) : 0.0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = q0 + 32 * u;
        if (q < N) r.Bs[ps<NN>(q)] = P::make(g[u], eg);
      }
    }
    __syncwarp();
  }
  bwd_sweep<P, NN, D, D - 1>(r, gp.dA ? static_cast<double*>(gp.dA) + e * D * NN2 : nullptr,
                             gp.dX ? static_cast<double*>(gp.dX) + e * N : nullptr, sa,
                             sg + sx + sa_sum, sg + sa_sum, lane);
  __syncwarp();  // the region is free for the next entry
}

// The FP64 evaluation inside the double-float kernel, out of line so that its
// registers do not set the kernel's.
template <int NN, int D>
__device__ __noinline__ void warp_entry_f64(const GradProblem& gp, long long e, double* wbase,
                                            int lane) {
  int ea[MAXD];
#pragma unroll
  for (int l = 0; l < MAXD; ++l) ea[l] = 1023;
  warp_entry<WF64, NN, D>(gp, e, wbase, ea, 1023, 1023, lane);
}

// Warp w of CTA b takes entries b*W + w, then every (grid*W)-th.  The entry's
// factors and X are staged as FP64 first (the split kernel takes the
// exponents from the staged values and G's from a scan of G).  SPLIT: the
// double-float kernel, which runs entries with Inf/NaN, or an all-zero X, G or
// factor, in FP64, so that IEEE propagation and exact zeros are those of FP64.
template <int NN, int D, bool SPLIT>
__global__ void __launch_bounds__(256, 2) grad_warp_kernel(const GradProblem gp) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NN2 = NN * NN, N = ipow(NN, D);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, W = blockDim.x >> 5;
  double* wbase = reinterpret_cast<double*>(smem) + (size_t)w * warp_words(D, NN);
  double* sA = wbase;
  double* slot0 = wbase + factor_words(NN, D);
  for (long long e = (long long)blockIdx.x * W + w; e < gp.batch; e += (long long)gridDim.x * W) {
    const double* Ae = static_cast<const double*>(gp.A) + e * D * NN2;
    const double* Xe = static_cast<const double*>(gp.X) + e * N;
    int ea[MAXD];
#pragma unroll
    for (int l = 0; l < MAXD; ++l) ea[l] = 0;
    for (int i = lane; i < D * NN2; i += 32) {
      const int l = i / NN2, rr = i - l * NN2, a = rr / NN, j = rr - a * NN;
      const double v = Ae[l * NN2 + a + j * NN];
      sA[i] = v;
      if constexpr (SPLIT) {
        const int ef = exp_field(v);
#pragma unroll
        for (int q = 0; q < MAXD; ++q)
          if (q == l) ea[q] = max(ea[q], ef);
      }
    }
    int mx = 0, mg = 0;
    for (int q0 = lane; q0 < N; q0 += 128) {
      double x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = q0 + 32 * u < N ? __ldg(Xe + q0 + 32 * u) : 0.0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = q0 + 32 * u;
        if (q < N) slot0[ps<NN>(q)] = x[u];
        if (SPLIT) mx = max(mx, exp_field(x[u]));
      }
    }
    if constexpr (!SPLIT) {
      __syncwarp();
#pragma unroll
      for (int l = 0; l < MAXD; ++l) ea[l] = 1023;
      warp_entry<WF64, NN, D>(gp, e, wbase, ea, 1023, 1023, lane);
    } else {
      const double* Ge = static_cast<const double*>(gp.G) + e * N;
      for (int q0 = lane; q0 < N; q0 += 128) {
        double g[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) g[u] = q0 + 32 * u < N ? __ldg(Ge + q0 + 32 * u) : 0.0;
#pragma unroll
        for (int u = 0; u < 4; ++u) mg = max(mg, exp_field(g[u]));
      }
      __syncwarp();
      const int ex = __reduce_max_sync(0xffffffffu, mx);
      const int eg = __reduce_max_sync(0xffffffffu, mg);
      bool special = ex == 0 || ex == 2047 || eg == 0 || eg == 2047;
#pragma unroll
      for (int l = 0; l < MAXD; ++l) {
        ea[l] = __reduce_max_sync(0xffffffffu, ea[l]);
        if (l < D) special = special || ea[l] == 0 || ea[l] == 2047;
      }
      if (special) {
        warp_entry_f64<NN, D>(gp, e, wbase, lane);
      } else {
        using Pol = typename std::conditional<packed_form(NN), WPk, WDf>::type;
        warp_entry<Pol, NN, D>(gp, e, wbase, ea, ex, eg, lane);
      }
    }
  }
}

template <int NN, int D, bool SPLIT>
const void* warp_func() {
  static_assert(warp_fits(D, NN), "shape beyond the warp kernel's region");
  return reinterpret_cast<const void*>(&grad_warp_kernel<NN, D, SPLIT>);
}

// the shapes with warp_fits(d, n) (checked by the static_assert)
template <bool SPLIT>
const void* pick_warp(int n, int d) {
  switch (d * 10 + n) {
    case 32: return warp_func<2, 3, SPLIT>();
    case 33: return warp_func<3, 3, SPLIT>();
    case 34: return warp_func<4, 3, SPLIT>();
    case 35: return warp_func<5, 3, SPLIT>();
    case 36: return warp_func<6, 3, SPLIT>();
    case 37: return warp_func<7, 3, SPLIT>();
    case 38: return warp_func<8, 3, SPLIT>();
    case 42: return warp_func<2, 4, SPLIT>();
    case 43: return warp_func<3, 4, SPLIT>();
    case 44: return warp_func<4, 4, SPLIT>();
    case 45: return warp_func<5, 4, SPLIT>();
    case 52: return warp_func<2, 5, SPLIT>();
    case 53: return warp_func<3, 5, SPLIT>();
    case 62: return warp_func<2, 6, SPLIT>();
    default: return nullptr;
  }
}

}  // namespace gw

// d >= 3: d <= 2 entries hold too little work per warp step (measured slower
// than the CTA kernels in plain FP64 on GB300)
size_t grad_warp_bytes(int d, int n) {
  if (!gw::warp_fits(d, n) || gw::pick_warp<true>(n, d) == nullptr) return 0;
  return (size_t)gw::warp_words(d, n) * 8;
}

int launch_grad_warp(const GradProblem& gp, int n, bool split, cudaStream_t s) {
  const size_t bytes = grad_warp_bytes(gp.d, n);
  const void* func = split ? gw::pick_warp<true>(n, gp.d) : gw::pick_warp<false>(n, gp.d);
  if (bytes == 0 || func == nullptr) return KMX_ERR_UNSUPPORTED;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KMX_ERR_CUDA;
  const DeviceInfo di = device_info(dev);
  // one to eight warps (entries) per CTA: the count that keeps the most warps
  // resident per SM (shared memory is reserved per CTA as well), the larger
  // CTA on a tie
  int wmax = (int)((size_t)di.max_smem_optin / bytes);
  if (wmax > 8) wmax = 8;
  if (wmax < 1) return KMX_ERR_UNSUPPORTED;
  if (ensure_smem(func, dev, bytes * wmax) != cudaSuccess) return KMX_ERR_CUDA;
  int wpc = 1, per_sm = 0, best = -1;
  for (int w = 1; w <= wmax; ++w) {
    int c = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, func, 32 * w, bytes * w) != cudaSuccess)
      return KMX_ERR_CUDA;
    if (c * w >= best) {
      best = c * w;
      wpc = w;
      per_sm = c;
    }
  }
  if (per_sm < 1) per_sm = 1;
  const size_t smem = bytes * wpc;
  long long grid = (long long)di.sms * per_sm;
  const long long need = (gp.batch + wpc - 1) / wpc;
  if (grid > need) grid = need;
  GradProblem g = gp;
  void* args[] = {&g};
  const cudaError_t e = cudaLaunchKernel(func, dim3((unsigned)grid), dim3(32 * wpc), args, smem, s);
  return e == cudaSuccess ? KMX_OK : KMX_ERR_CUDA;
}

}  // namespace kmx
