// kmx_cluster.cuh -- double-float entries too large for one SM's shared memory
// (square n <= 8 with n^d beyond it: d=5 n=8, d=6 n=6, 7, 8), on chip, by a
// thread-block cluster of n CTAs with distributed shared memory.
//
// Cluster c takes one (entry, i1) item at a time: the output block
// Y(i1, :, ..., :) of n^(d-1) elements.  CTA r of the cluster:
//   0. loads and splits the factors (per-entry scales), finds the largest
//      exponent of its slice X(:, r, :) and publishes it to the cluster;
//   A. applies mode 1 for row i1 to its slice:
//        W1_r(t) = sum_j1 A1(i1, j1) X(j1, r, t),   t < S2 = n^(d-2),
//      into its shared memory;
//   B. reads every CTA's W1 slice through distributed shared memory and
//      applies mode 2 for row i2 = r:
//        W2(t) = sum_j2 A2(r, j2) W1_j2(t),
//      the (i1, r) block of the intermediate after two modes;
//   C. applies modes 3..d to W2 with the register-tiled phases of the
//      (n, d-2) problem and adds the result to Y(i1, r, :) (S2 elements).
// Every multiply of the recursion happens once (modes 1 and 2 split by output
// rows, the rest local); X is read from L2 by n clusters per entry.  Cluster
// barriers: after the exponent exchange, after step A (slices complete),
// after step B (slices no longer read).
//
// The cancellation guard of kmx_engine.cuh applies per (i1, r) block with the
// block's operator a1(i1,:) (x) a2(r,:) (x) A3 (x) ... (x) Ad; a rejected
// block, and a block of an entry with Inf/NaN, is recomputed in FP64 by its
// CTA alone (fp64_block).
#pragma once

#include <stdint.h>

#include <type_traits>

#include "kmx_tile.cuh"

namespace kmx {
namespace clus {

using tile::ipow;

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_index() {
  unsigned r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_count() {
  unsigned r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// every thread of every CTA of the cluster; shared-memory writes before it
// are visible to the cluster after it
__device__ __forceinline__ void cluster_sync() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::
          : "memory");
}
// shared::cluster address of a local shared-memory location in CTA `rank`
__device__ __forceinline__ uint32_t peer_addr(const void* local, unsigned rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(tile::smem_u32(local)), "r"(rank));
  return r;
}
__device__ __forceinline__ df ld_peer_df(uint32_t a) {
  df v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.hi), "=f"(v.lo) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ int ld_peer_i32(uint32_t a) {
  int v;
  asm volatile("ld.shared::cluster.b32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ float ld_peer_f32(uint32_t a) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}

__host__ __device__ constexpr bool supported(int NN, int D) {
  return NN >= 2 && NN <= 8 && (D == 5 || D == 6);
}

// Threads per CTA: those of the (n, d-2) tile problem.
__host__ __device__ constexpr int cta_threads(int NN, int D) { return tile::group_threads(NN, D - 2); }

// Tile policy of the trailing problem.
template <int NN, int D>
using SubPol = typename std::conditional<tile::packed_pays(NN, D - 2), tile::PackedSplitPolicy,
                                         tile::SplitPolicy>::type;

// Shared memory of one CTA.
template <int NN, int D>
struct Layout {
  using Pol = SubPol<NN, D>;
  static constexpr int S2 = ipow(NN, D - 2);
  static constexpr int FAC = (D * Pol::template factor_bytes<NN>() > D * NN * NN * 8
                                  ? D * Pol::template factor_bytes<NN>()
                                  : D * NN * NN * 8 + 15) / 16 * 16;
  static constexpr int ROW1 = FAC;                    // A1 row i1, NN df
  static constexpr int ROW2 = ROW1 + NN * 8;          // A2 row r, NN df
  // scalars, 96 bytes: int exps[8] (factor l, then X at [D]); int published
  // slice exponent; float norms[8] (factor l, X at [D], output at [D+1]);
  // float published slice norm
  static constexpr int INTS = (ROW2 + NN * 8 + 15) / 16 * 16;
  static constexpr int EXPS = INTS, PUB_EXP = INTS + 32, NORMS = INTS + 48, PUB_NRM = INTS + 80;
  static constexpr int BUF1 = INTS + 96;                       // W1 slice: S2 df
  static constexpr int BUF2 = (BUF1 + S2 * 8 + 15) / 16 * 16;  // W2: buffer_slots df
  static constexpr int BYTES = (BUF2 + tile::buffer_slots<NN, D - 2>() * 8 + 15) / 16 * 16;
};

// Y(i1, r, :) += the (i1, r) block in FP64, computed by this CTA alone from
// X and the factors in global memory, modes in the recursion's order (so that
// Inf/NaN propagate as they do there); buf holds S2 doubles.
template <int NN, int D>
__device__ __noinline__ void fp64_block(const Problem& p, const EntryPtrs<double>& en, int i1,
                                        int r, double* buf, bool excl) {
  constexpr int S2 = ipow(NN, D - 2);
  constexpr int N1 = ipow(NN, D - 1);
  const int G = blockDim.x;
  auto A = [&](int l, int row, int col) -> double {
    const long long ld = en.ld[l];
    return p.trans ? en.A[l][col + row * ld] : en.A[l][row + col * ld];
  };
  for (int t = threadIdx.x; t < S2; t += G) {
    double acc = 0.0;
    for (int j2 = 0; j2 < NN; ++j2) {
      double w1 = 0.0;
      for (int j1 = 0; j1 < NN; ++j1)
        w1 = fma(A(0, i1, j1), en.X[(long long)j1 * N1 + (long long)j2 * S2 + t], w1);
      acc = fma(A(1, r, j2), w1, acc);
    }
    buf[t] = acc;
  }
  __syncthreads();
  // modes 3..d of the (i1, r) block, in place, the last one into Y
  double* yb = en.Y + ((long long)i1 * NN + r) * S2;
#pragma unroll
  for (int m = 0; m < D - 2; ++m) {
    const int s = ipow(NN, D - 3 - m);  // stride of the mode's index
    const int l = m + 2;
    if (m < D - 3) {
      for (int f = threadIdx.x; f < S2 / NN; f += G) {
        const int o = f / s, r0 = f - o * s;
        double* base = buf + (long long)o * NN * s + r0;
        double v[NN];
#pragma unroll
        for (int j = 0; j < NN; ++j) v[j] = base[j * s];
#pragma unroll
        for (int a = 0; a < NN; ++a) {
          double acc = 0.0;
#pragma unroll
          for (int j = 0; j < NN; ++j) acc = fma(A(l, a, j), v[j], acc);
          base[a * s] = acc;
        }
      }
    } else {
      for (int q = threadIdx.x; q < S2; q += G) {
        const int f = q / NN, a = q - f * NN;
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < NN; ++j) acc = fma(A(l, a, j), buf[f * NN + j], acc);
        y_accumulate(yb + q, acc, excl);
      }
    }
    __syncthreads();
  }
}

template <int NN, int D>
__global__ void __launch_bounds__(cta_threads(NN, D)) cluster_kernel(const Problem p) {
  static_assert(supported(NN, D), "no cluster kernel for this shape");
  using Pol = SubPol<NN, D>;
  using V = df;
  using L = Layout<NN, D>;
  constexpr int G = cta_threads(NN, D);
  constexpr int NN2 = NN * NN;
  constexpr int S2 = L::S2;
  constexpr long long N1 = ipow(NN, D - 1);
  constexpr long long NFULL = (long long)ipow(NN, D);
  constexpr int DS = D - 2;  // the trailing tile problem
  constexpr int LP = tile::num_phases(NN, DS) - 1;
  constexpr int TL = tile::tile_size(NN, DS, LP);
  constexpr int NTL = S2 / TL;
  constexpr bool PAIRL = tile::phase_b(NN, DS, LP) >= 0;
  constexpr int aL = tile::phase_a(NN, DS, LP);
  constexpr int bL = PAIRL ? tile::phase_b(NN, DS, LP) : aL;
  constexpr int FPT = (D * NN2 + G - 1) / G;

  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* sA = smem;  // the D factors (Pol layout)
  df* sRow1 = reinterpret_cast<df*>(smem + L::ROW1);
  df* sRow2 = reinterpret_cast<df*>(smem + L::ROW2);
  int* sExp = reinterpret_cast<int*>(smem + L::EXPS);       // [D+1]: factors, X
  int* sXexp = reinterpret_cast<int*>(smem + L::PUB_EXP);   // this slice's exponent
  float* sNrm = reinterpret_cast<float*>(smem + L::NORMS);  // [D+2]: factors, X, Y
  float* sXn = reinterpret_cast<float*>(smem + L::PUB_NRM); // this slice's ||X||^2
  df* buf1 = reinterpret_cast<df*>(smem + L::BUF1);
  V* buf2 = reinterpret_cast<V*>(smem + L::BUF2);
  const int lt = threadIdx.x;
  const unsigned r = cluster_rank();
  const bool excl = p.y_exclusive != 0;
  const long long items = launch_count(p) * NN;

  if constexpr (Pol::PACKED) {
    // the pad row of an odd NN stays zero (entries write real rows only)
    for (int i = lt; i < L::FAC / 4; i += G) reinterpret_cast<float*>(sA)[i] = 0.f;
  }
  for (long long it = cluster_index(); it < items; it += cluster_count()) {
    const long long epos = it / NN;
    const int i1 = (int)(it - epos * NN);
    const long long ent = tile::entry_index(p, epos);
    EntryPtrs<double> en;
    const bool valid = resolve_entry<double>(p, ent, en);
    // ---- 0. factors and their scales; the slice's exponent ----
    // (the published slots were last read before the previous item's barrier #3)
    if (lt < 24) reinterpret_cast<int*>(smem + L::INTS)[lt] = 0;
    __syncthreads();
    double af[FPT];
    int al[FPT], ar[FPT], ac[FPT];
#pragma unroll
    for (int f = 0; f < FPT; ++f) {
      const int idx = lt + f * G;
      al[f] = idx / NN2;
      ar[f] = (idx - al[f] * NN2) / NN;
      ac[f] = idx - al[f] * NN2 - ar[f] * NN;
      af[f] = 0.0;
      if (valid && idx < D * NN2) {
        const long long ld = en.ld[al[f]];
        af[f] = p.trans ? en.A[al[f]][ac[f] + ar[f] * ld] : en.A[al[f]][ar[f] + ac[f] * ld];
        const int ef = exp_field(af[f]);
        if (ef) atomicMax(&sExp[al[f]], ef);
      }
    }
    int xe = 0;
    if (valid) {
      for (int q = lt; q < NN * S2; q += G) {
        const int j1 = q / S2, t = q - j1 * S2;
        xe = max(xe, exp_field(en.X[(long long)j1 * N1 + (long long)r * S2 + t]));
      }
    }
    xe = __reduce_max_sync(0xffffffffu, xe);
    if ((lt & 31) == 0 && xe) atomicMax(sXexp, xe);
    __syncthreads();
#pragma unroll
    for (int f = 0; f < FPT; ++f) {
      const int idx = lt + f * G;
      const bool own = idx < D * NN2;
      float sq = 0.f;  // sNrm[0], [1]: rows i1 of A1 and r of A2 only
      if (own) {
        const df s = tile::SplitPolicy::make(af[f], sExp[al[f]]);
        Pol::template store_factor<NN>(sA, idx, s);
        if (al[f] == 0 && ar[f] == i1) {
          sRow1[ac[f]] = s;
          sq = s.hi * s.hi;
        } else if (al[f] == 1 && ar[f] == (int)r) {
          sRow2[ac[f]] = s;
          sq = s.hi * s.hi;
        } else if (al[f] >= 2) {
          sq = s.hi * s.hi;
        }
      }
      warp_run_add(sNrm, own ? al[f] : 0, sq, own);
    }
    cluster_sync();  // #1: every CTA's slice exponent published
    if (lt == 0) {
      int ex = 0;
      for (unsigned k = 0; k < (unsigned)NN; ++k) ex = max(ex, ld_peer_i32(peer_addr(sXexp, k)));
      sExp[D] = ex;
    }
    __syncthreads();
    const int ex = sExp[D];
    bool zero = ex == 0, nonfinite = ex == 2047;
    int escale = ex - 1023;
#pragma unroll
    for (int l = 0; l < D; ++l) {
      zero = zero || sExp[l] == 0;
      nonfinite = nonfinite || sExp[l] == 2047;
      escale += sExp[l] - 1023;
    }
    const bool run = valid && !zero && !nonfinite;  // uniform over the cluster
    // ---- A. mode 1 on this CTA's slice X(:, r, :) for row i1 ----
    float xs = 0.f;
    if (run) {
      for (int t = lt; t < S2; t += G) {
        df v[NN];
#pragma unroll
        for (int j = 0; j < NN; ++j) {
          v[j] = tile::SplitPolicy::make(en.X[(long long)j * N1 + (long long)r * S2 + t], ex);
          xs = __fmaf_rn(v[j].hi, v[j].hi, xs);
        }
        buf1[t] = df_dot<NN>(sRow1, v);
      }
    }
    xs = warp_sum(xs);
    if ((lt & 31) == 0) atomicAdd(sXn, xs);  // this slice's ||X||^2, read by the cluster
    cluster_sync();  // #2: every W1 slice complete
    // ---- B. mode 2 for row r from every CTA's slice ----
    if (run) {
      uint32_t base[NN];
#pragma unroll
      for (int k = 0; k < NN; ++k) base[k] = peer_addr(buf1, (unsigned)k);
      for (int t = lt; t < S2; t += G) {
        df w[NN];
#pragma unroll
        for (int k = 0; k < NN; ++k) w[k] = ld_peer_df(base[k] + (uint32_t)t * 8u);
        buf2[tile::slot<NN>(t)] = df_dot<NN>(sRow2, w);
      }
    }
    if (lt == 0) {
      float x2 = 0.f;
      for (unsigned k = 0; k < (unsigned)NN; ++k) x2 += ld_peer_f32(peer_addr(sXn, k));
      sNrm[D] = x2;  // ||X||^2 of the whole entry
    }
    cluster_sync();  // #3: slices and published values no longer read
    if (!valid) {
      if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    if (zero) continue;
    double* yblk = en.Y + ((long long)i1 * NN + r) * S2;
    if (nonfinite) {  // Inf/NaN propagate as in FP64
      fp64_block<NN, D>(p, en, i1, (int)r, reinterpret_cast<double*>(buf2), excl);
      continue;
    }
    // ---- C. modes 3..d with the register-tiled phases of the (n, d-2) problem ----
    const unsigned char* sSub = sA + 2 * Pol::template factor_bytes<NN>();
    tile::middle_phases<Pol, NN, DS, G, 0>(buf2, sSub, lt, 0);
    float os = 0.f;
    auto last_phase = [&](bool neg) {
      for (int u = lt; u < NTL; u += G) {
        const int basei = tile::tile_base<NN, DS, LP>(u);
        V v[TL];
#pragma unroll
        for (int e = 0; e < TL; ++e) v[e] = buf2[tile::slot<NN>(basei + tile::tile_off<NN, DS, LP>(e))];
        tile::contract_tile<Pol, NN, PAIRL>(v, Pol::template factor<NN>(sSub, aL),
                                            Pol::template factor<NN>(sSub, bL));
#pragma unroll
        for (int e = 0; e < TL; ++e) {
          const int q = basei + tile::tile_off<NN, DS, LP>(e);
          if (!neg) os = __fmaf_rn(v[e].hi, v[e].hi, os);
          const double y = Pol::finish(v[e], escale);
          y_accumulate(yblk + q, neg ? -y : y, excl);
        }
      }
    };
    last_phase(false);
    os = warp_sum(os);
    if ((lt & 31) == 0) atomicAdd(&sNrm[D + 1], os);
    __syncthreads();
    // cancellation guard of the (i1, r) block (norms of row i1 of A1 and row r
    // of A2 in place of those factors' Frobenius norms)
    if (!p.guard_off && guard_fails(sNrm[D + 1], sNrm[D], sNrm, D, NFULL)) {
      last_phase(true);  // take the double-float contribution back
      __syncthreads();
      fp64_block<NN, D>(p, en, i1, (int)r, reinterpret_cast<double*>(buf2), excl);
      if (lt == 0) count_redo(p.redo_ctr, 0);
    }
    __syncthreads();
  }
}

}  // namespace clus
}  // namespace kmx
