// kmx_small.cuh -- many small entries per CTA: square factors, d <= 3 and
// n^d <= 256 elements per X/Y block (the shapes of kronmult1..3 with small
// n, for which one group of threads per entry leaves most lanes idle).
//
// A CTA takes a CHUNK of K consecutive entries at a time (K sized for about
// 32 KB of shared memory):
//   1. the chunk's X blocks and factors are staged in shared memory -- for
//      the contiguous batched layout with 128-bit loads over the whole chunk
//      (every byte of a sector used), otherwise entry by entry through the
//      pointer arrays; the factors are stored column-major as applied, so
//      the threads of a mode, which read different rows at the same column,
//      read consecutive words (a row-major copy put every row on the same
//      banks: 136 shared-memory bank conflicts per d=2 n=8 entry), and the
//      batched layout's column-major factors copy straight across;
//   2. the d modes are applied in the reference's order (A1 first), one
//      thread per output element and mode, ping-ponging between two
//      shared-memory buffers: the last mode adds its outputs to Y
//      (read-modify-write where Y blocks are exclusive, atomics otherwise),
//      consecutive threads on consecutive Y elements.  In the batched
//      layout the chunk's Y blocks are staged with X (128-bit loads), so the
//      last mode stores Y without waiting on a load.
// Several CTAs per SM overlap one chunk's loads with another's arithmetic.
//
// Arithmetic policies: plain FMA in T; FP32 with each dot product rounded once
// (RD, the reference's float semantics); and double-float (SmallSplit) with
// per-entry power-of-two scales, the cancellation guard of kmx_engine.cuh, and
// plain FP64 for entries holding Inf/NaN.
#pragma once

#include <stdint.h>

#include "kmx_engine.cuh"
#include "kmx_tile.cuh"

namespace kmx {
namespace small {

using tile::ipow;

constexpr int THREADS = 256;
constexpr int MAX_ELEMS = 256;  // n^d
constexpr int CHUNK_BYTES = 32 * 1024;

__host__ __device__ constexpr bool supported(int NN, int D) {
  return D >= 1 && D <= 3 && NN >= 2 && ipow(NN, D) <= MAX_ELEMS;
}

// Plain forms: V == In == Out == T.
// dot(a, v, vs): sum_j a[j * NN] v[j * vs] (a: one row of a column-major
// factor).
template <typename T, bool RD>
struct SmallPlain {
  using In = T;
  using V = T;
  static constexpr bool SPLIT = false;
  template <int NN>
  __device__ __forceinline__ static V dot(const V* a, const V* v, int vs) {
    V av[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) av[j] = a[j * NN];
    return dot_n<T, RD, NN>(av, v, vs);
  }
};

// Double-float with per-entry scales.
struct SmallSplit {
  using In = double;
  using V = df;
  static constexpr bool SPLIT = true;
  template <int NN>
  __device__ __forceinline__ static V dot(const V* a, const V* v, int vs) {
    df av[NN], vv[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) {
      av[j] = a[j * NN];
      vv[j] = v[j * vs];
    }
    return df_dot<NN>(av, vv);
  }
};

// Entry flags of the split policy.
enum : int { SF_NULL = 1, SF_SKIP = 2, SF_FP64 = 4, SF_GUARD = 8 };

template <class Pol, int NN, int D>
struct Layout {
  using V = typename Pol::V;
  static constexpr int N = ipow(NN, D);
  static constexpr int NA = D * NN * NN;
  static constexpr int NBUF = D >= 2 ? 2 : 1;
  // the double-float form keeps the squares of the last mode's outputs for
  // the guard's per-entry norm (one float per output)
  static constexpr int SQ = Pol::SPLIT ? N * 4 : 0;
  static constexpr int PER_ENTRY = (NA + NBUF * N) * (int)sizeof(V) + N * (int)sizeof(V) + SQ +
                                   (D + 2) * 8 + 4 * (D + 1) + 4 * (D + 2) + 4;
  static constexpr int K0 = CHUNK_BYTES / PER_ENTRY;
  static constexpr int K = K0 < 1 ? 1 : (K0 > 512 ? 512 : K0);
  // byte offsets, every region 16-byte aligned (the staging stores are 128-bit)
  __host__ __device__ static constexpr int al16(int x) { return (x + 15) / 16 * 16; }
  static constexpr int A_OFF = 0;
  static constexpr int W0_OFF = al16(A_OFF + K * NA * (int)sizeof(V));
  static constexpr int W1_OFF = al16(W0_OFF + K * N * (int)sizeof(V));
  static constexpr int YS_OFF = al16(W1_OFF + (NBUF == 2 ? K * N * (int)sizeof(V) : 0));  // staged Y
  static constexpr int SQ_OFF = al16(YS_OFF + K * N * (int)sizeof(V));
  static constexpr int PX_OFF = al16(SQ_OFF + K * SQ);
  static constexpr int PY_OFF = PX_OFF + K * 8;
  static constexpr int PA_OFF = PY_OFF + K * 8;
  static constexpr int EXP_OFF = al16(PA_OFF + K * D * 8);        // [K][D+1] ints (split)
  static constexpr int NRM_OFF = al16(EXP_OFF + K * (D + 1) * 4);  // [K][D+2] floats (split)
  static constexpr int FLAG_OFF = al16(NRM_OFF + K * (D + 2) * 4); // [K] ints
  static constexpr int BYTES = al16(FLAG_OFF + K * 4 + 16);        // + redo count
};

// Row i_k of factor k of chunk entry e (column-major: its entries NN apart).
template <int NN, int D, typename V>
__device__ __forceinline__ const V* factor_row(const V* sA, int e, int k, int i) {
  return sA + (e * D + k) * NN * NN + i;
}

// The FP64 recursion of one chunk entry, by the whole CTA, on its slices of
// the shared buffers (reinterpreted as double): factors and X from global
// memory, Y += result.  For split entries with Inf/NaN and for entries the
// cancellation guard rejected.
template <int NN, int D>
__device__ __noinline__ void fp64_entry(const Problem& p, const double* xp, double* yp,
                                        const double* const* ap, double* a, double* w0, double* w1,
                                        bool excl) {
  constexpr int N = ipow(NN, D);
  for (int idx = threadIdx.x; idx < D * NN * NN; idx += THREADS) {
    const int l = idx / (NN * NN), r = (idx / NN) % NN, c = idx % NN;
    const long long ld = p.ld[l];
    a[idx] = p.trans ? ap[l][c + r * ld] : ap[l][r + c * ld];
  }
  for (int i = threadIdx.x; i < N; i += THREADS) w0[i] = xp[i];
  __syncthreads();
  double* src = w0;
  double* dst = w1;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const int s = ipow(NN, D - 1 - k);
    for (int q = threadIdx.x; q < N; q += THREADS) {
      const int t = q / s, r = q - t * s, i = t % NN, o = t / NN;
      const double v = dot_n<double, false, NN>(a + (k * NN + i) * NN, src + o * NN * s + r, s);
      if (k == D - 1) {
        y_accumulate(yp + q, v, excl);
      } else {
        dst[q] = v;
      }
    }
    __syncthreads();
    double* t = src;
    src = dst;
    dst = t;
  }
}

template <class Pol, int NN, int D>
__global__ void __launch_bounds__(THREADS) small_kernel(const Problem p) {
  static_assert(supported(NN, D), "no small kernel for this shape");
  using In = typename Pol::In;
  using V = typename Pol::V;
  using L = Layout<Pol, NN, D>;
  constexpr int N = L::N, NA = L::NA, K = L::K;
  extern __shared__ __align__(16) unsigned char smem[];
  V* sA = reinterpret_cast<V*>(smem + L::A_OFF);
  V* sW0 = reinterpret_cast<V*>(smem + L::W0_OFF);
  V* sW1 = reinterpret_cast<V*>(smem + L::W1_OFF);
  const In** sPX = reinterpret_cast<const In**>(smem + L::PX_OFF);
  In** sPY = reinterpret_cast<In**>(smem + L::PY_OFF);
  const In** sPA = reinterpret_cast<const In**>(smem + L::PA_OFF);
  int* sExp = reinterpret_cast<int*>(smem + L::EXP_OFF);
  float* sNrm = reinterpret_cast<float*>(smem + L::NRM_OFF);
  int* sFlag = reinterpret_cast<int*>(smem + L::FLAG_OFF);
  float* sSq = reinterpret_cast<float*>(smem + L::SQ_OFF);  // [K][N] (split)
  In* sYs = reinterpret_cast<In*>(smem + L::YS_OFF);        // [K][N] staged Y (batched)
  const bool excl = p.y_exclusive != 0;
  const long long total = launch_count(p);
  const long long nchunks = (total + K - 1) / K;
  const bool contig = p.layout == L_BATCHED && !p.order;
  const bool ystaged = contig && excl;
  // per-entry reductions of the double-float form: ES threads per entry (a
  // warp when the entry has 64 or more values, else one thread)
  constexpr int ES = (N + NA >= 64) ? 32 : 1;
  const int ei = threadIdx.x % ES;                 // lane within the entry's threads
  const int e0 = threadIdx.x / ES;                 // first entry of this thread
  constexpr int estep = THREADS / ES;
  for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const long long pos0 = ch * K;
    const int kc = (int)((total - pos0) < K ? (total - pos0) : K);
    // ---- pointers of the chunk's entries ----
    for (int e = threadIdx.x; e < kc; e += THREADS) {
      const long long ent = tile::entry_index(p, pos0 + e);
      const In* xp = tile::x_ptr<In>(p, ent);
      In* yp = tile::y_ptr<In>(p, ent);
      int fl = (xp && yp) ? 0 : SF_NULL;
#pragma unroll
      for (int l = 0; l < D; ++l) {
        const In* ap = tile::a_ptr<In>(p, ent, l);
        sPA[e * D + l] = ap;
        if (!ap) fl |= SF_NULL;
      }
      sPX[e] = xp;
      sPY[e] = yp;
      sFlag[e] = fl;
    }
    __syncthreads();
    // ---- stage X and the factors (raw values in the V-sized slots) ----
    // In and V have the same size in every policy (SmallSplit: double and df,
    // 8 bytes), so the raw values are staged in the slots they are split into
    In* rawX = reinterpret_cast<In*>(sW0);
    In* rawA = reinterpret_cast<In*>(sA);
    static_assert(sizeof(In) == sizeof(V), "raw staging needs In-sized slots");
    if (contig) {
      const long long ent0 = pos0 + p.entry_offset;
      const In* xg = static_cast<const In*>(p.X) + ent0 * N;
      const int nx = kc * N;
      // X, and Y where the blocks are exclusive, into shared memory
      auto stage = [&](const In* g, In* sm) {
        if ((reinterpret_cast<uintptr_t>(g) & 15) == 0) {
          constexpr int PV = 16 / (int)sizeof(In);  // values per 128-bit load
          const int nv = nx / PV;
          for (int i = threadIdx.x; i < nv; i += THREADS) {
            const uint4 u = __ldg(reinterpret_cast<const uint4*>(g) + i);
            *reinterpret_cast<uint4*>(sm + i * PV) = u;
          }
          for (int i = nv * PV + threadIdx.x; i < nx; i += THREADS) sm[i] = __ldg(g + i);
        } else {
          for (int i = threadIdx.x; i < nx; i += THREADS) sm[i] = __ldg(g + i);
        }
      };
      stage(xg, rawX);
      if (ystaged) stage(static_cast<const In*>(p.Y) + ent0 * N, sYs);
      // factors: (n, n, d, batch) column-major, ld = n: the same layout
      // (transposed factors swap row and column)
      const In* ag = static_cast<const In*>(p.A) + ent0 * NA;
      for (int i = threadIdx.x; i < kc * NA; i += THREADS) {
        int dst = i;
        if (p.trans) {
          const int e = i / NA, m = i - e * NA, l = m / (NN * NN), rc = m - l * NN * NN;
          const int row = rc % NN, col = rc / NN;  // stored A(row, col)
          dst = (e * D + l) * NN * NN + row * NN + col;
        }
        rawA[dst] = __ldg(ag + i);
      }
    } else {
      for (int i = threadIdx.x; i < kc * N; i += THREADS) {
        const int e = i / N, q = i - e * N;
        const In* xp = sPX[e];
        rawX[i] = xp ? xp[q] : In(0);
      }
      for (int i = threadIdx.x; i < kc * NA; i += THREADS) {
        const int e = i / NA, m = i - e * NA, l = m / (NN * NN), rc = m - l * NN * NN;
        const int row = rc % NN, col = rc / NN;  // applied M(row, col), column-major
        const In* ap = sPA[e * D + l];
        const long long ld = p.ld[l];
        rawA[i] = ap ? (p.trans ? ap[col + row * ld] : ap[row + col * ld]) : In(0);
      }
    }
    if constexpr (Pol::SPLIT) {
      __syncthreads();
      // per-entry exponents of the X block and of every factor (a warp per
      // entry, or a thread per entry when entries are small)
      for (int e = e0; e < kc; e += estep) {
        int ex[D + 1];
#pragma unroll
        for (int l = 0; l <= D; ++l) ex[l] = 0;
        for (int i = ei; i < N; i += ES) ex[D] = max(ex[D], exp_field(rawX[e * N + i]));
#pragma unroll
        for (int l = 0; l < D; ++l)
          for (int i = ei; i < NN * NN; i += ES)
            ex[l] = max(ex[l], exp_field(rawA[e * NA + l * NN * NN + i]));
        if constexpr (ES == 32) {
#pragma unroll
          for (int l = 0; l <= D; ++l) ex[l] = __reduce_max_sync(0xffffffffu, ex[l]);
        }
        if (ei == 0) {
          int fl = sFlag[e];
#pragma unroll
          for (int l = 0; l <= D; ++l) {
            sExp[e * (D + 1) + l] = ex[l];
            if (ex[l] == 0) fl |= SF_SKIP;     // an all-zero factor or X: contributes zero
            if (ex[l] == 2047) fl |= SF_FP64;  // Inf/NaN: exact IEEE propagation in FP64
          }
          sFlag[e] = fl;
        }
      }
      __syncthreads();
      // split in place, scaled per entry
      for (int i = threadIdx.x; i < kc * N; i += THREADS) {
        const int e = i / N;
        sW0[i] = tile::SplitPolicy::make(rawX[i], sExp[e * (D + 1) + D]);
      }
      for (int i = threadIdx.x; i < kc * NA; i += THREADS) {
        const int e = i / NA, l = (i - e * NA) / (NN * NN);
        sA[i] = tile::SplitPolicy::make(rawA[i], sExp[e * (D + 1) + l]);
      }
      __syncthreads();
      // the guard's norms of X and of the factors
      for (int e = e0; e < kc; e += estep) {
        float x2 = 0.f;
        for (int i = ei; i < N; i += ES) x2 = __fmaf_rn(sW0[e * N + i].hi, sW0[e * N + i].hi, x2);
        if constexpr (ES == 32) x2 = warp_sum(x2);
        if (ei == 0) sNrm[e * (D + 2) + D] = x2;
#pragma unroll
        for (int l = 0; l < D; ++l) {
          float a2 = 0.f;
          for (int i = ei; i < NN * NN; i += ES) {
            const float h = sA[e * NA + l * NN * NN + i].hi;
            a2 = __fmaf_rn(h, h, a2);
          }
          if constexpr (ES == 32) a2 = warp_sum(a2);
          if (ei == 0) sNrm[e * (D + 2) + l] = a2;
        }
      }
    }
    __syncthreads();
    // ---- the d modes, A1 first; the last adds to Y ----
    // first pass (only < 0, neg false) with staged Y: plain stores of the
    // staged value plus the contribution; other passes read-modify-write
    auto last_mode = [&](const V* src, bool neg, bool norm, int only) {
      constexpr int k = D - 1;
      const bool st = ystaged && only < 0 && !neg;
      for (int i = threadIdx.x; i < kc * N; i += THREADS) {
        const int e = i / N, q = i - e * N;
        if (only >= 0 && e != only) continue;
        const int t = q, i_k = t % NN, o = t / NN;  // s = 1 for the last mode
        const V v = Pol::template dot<NN>(factor_row<NN, D>(sA, e, k, i_k), src + e * N + o * NN, 1);
        const int fl = sFlag[e];
        if constexpr (Pol::SPLIT) {
          if (norm) sSq[i] = v.hi * v.hi;
          if (fl & (SF_NULL | SF_SKIP | SF_FP64)) continue;
          int escale = 0;
#pragma unroll
          for (int l = 0; l <= D; ++l) escale += sExp[e * (D + 1) + l] - 1023;
          const double y = tile::SplitPolicy::finish(v, escale);
          if (st) {
            sPY[e][q] = sYs[i] + y;
          } else {
            y_accumulate(sPY[e] + q, neg ? -y : y, excl);
          }
        } else {
          if (fl & SF_NULL) continue;
          if (st) {
            sPY[e][q] = sYs[i] + v;
          } else {
            y_accumulate(sPY[e] + q, v, excl);
          }
        }
      }
    };
    const V* src = sW0;
    V* dst = sW1;
#pragma unroll
    for (int k = 0; k < D - 1; ++k) {
      const int s = ipow(NN, D - 1 - k);
      for (int i = threadIdx.x; i < kc * N; i += THREADS) {
        const int e = i / N, q = i - e * N;
        const int t = q / s, r = q - t * s, i_k = t % NN, o = t / NN;
        dst[i] = Pol::template dot<NN>(factor_row<NN, D>(sA, e, k, i_k), src + e * N + o * NN * s + r, s);
      }
      __syncthreads();
      const V* tsrc = dst;
      dst = const_cast<V*>(src);
      src = tsrc;
    }
    last_mode(src, false, true, -1);
    if (!contig || Pol::SPLIT) {
      int* redo_n = reinterpret_cast<int*>(smem + L::FLAG_OFF + K * 4);
      __syncthreads();
      if constexpr (Pol::SPLIT) {
        // cancellation guard, entries with Inf/NaN: the FP64 recursion
        if (threadIdx.x == 0) *redo_n = 0;
        __syncthreads();
        for (int e = e0; e < kc; e += estep) {
          float o2 = 0.f;
          for (int i = ei; i < N; i += ES) o2 += sSq[e * N + i];
          if constexpr (ES == 32) o2 = warp_sum(o2);
          if (ei != 0) continue;
          sNrm[e * (D + 2) + D + 1] = o2;
          int fl = sFlag[e];
          if (!(fl & (SF_NULL | SF_SKIP | SF_FP64)) && !p.guard_off &&
              guard_fails(sNrm[e * (D + 2) + D + 1], sNrm[e * (D + 2) + D], sNrm + e * (D + 2), D, N)) {
            fl |= SF_GUARD;
            sFlag[e] = fl;
          }
          if (fl & (SF_GUARD | SF_FP64)) atomicAdd(redo_n, 1);
        }
        __syncthreads();
        if (*redo_n) {
          for (int e = 0; e < kc; ++e) {
            const int fl = sFlag[e];
            if (fl & SF_NULL) continue;
            if (fl & SF_GUARD) {
              last_mode(src, true, false, e);  // take the double-float contribution back
              __syncthreads();
            }
            if (fl & (SF_GUARD | SF_FP64)) {
              fp64_entry<NN, D>(p, reinterpret_cast<const double*>(sPX[e]),
                                reinterpret_cast<double*>(sPY[e]),
                                reinterpret_cast<const double* const*>(sPA + e * D),
                                reinterpret_cast<double*>(sA + e * NA),
                                reinterpret_cast<double*>(sW0 + e * N),
                                reinterpret_cast<double*>(sW1 + e * N), excl);
              if (threadIdx.x == 0 && (fl & SF_GUARD)) count_redo(p.redo_ctr, 0);
            }
          }
        }
      }
      for (int e = threadIdx.x; e < kc; e += THREADS)
        if (sFlag[e] & SF_NULL) atomicOr(p.status, DF_NULL_PTR);
    }
    __syncthreads();  // the chunk's shared memory is free
  }
}

}  // namespace small
}  // namespace kmx
