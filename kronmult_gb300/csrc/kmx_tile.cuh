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

#include "kmx_engine.cuh"

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
__host__ __device__ constexpr int group_threads(int NN, int D) {
  return (ipow(NN, D) / tile_size(NN, D, 0) + 31) / 32 * 32 > 512
             ? 512
             : ((ipow(NN, D) / tile_size(NN, D, 0) + 31) / 32 * 32 < 32
                    ? 32
                    : (ipow(NN, D) / tile_size(NN, D, 0) + 31) / 32 * 32);
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

// Double-float with per-entry power-of-two scaling (see kmx_engine.cuh).
struct SplitPolicy {
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

template <typename T>
struct PlainPolicy {
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

// Contract the tile's mode(s) in registers.  sA points at the phase's
// factor(s) in shared memory, rows of NN values of V.
template <class Pol, int NN, bool PAIR>
__device__ __forceinline__ void contract_tile(typename Pol::V* v, const typename Pol::V* Afirst,
                                              const typename Pol::V* Asecond) {
  using V = typename Pol::V;
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

// One middle phase P over all tiles of the group: shared memory -> shared memory.
template <class Pol, int NN, int D, int G, int P>
__device__ __forceinline__ void middle_phase(typename Pol::V* buf, const typename Pol::V* sA,
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
    contract_tile<Pol, NN, (b >= 0)>(v, sA + a * NN * NN, sA + (b >= 0 ? b : a) * NN * NN);
#pragma unroll
    for (int e = 0; e < T; ++e) buf[slot<NN>(base + tile_off<NN, D, P>(e))] = v[e];
  }
}

template <class Pol, int NN, int D, int G, int P>
__device__ __forceinline__ void middle_phases(typename Pol::V* buf, const typename Pol::V* sA,
                                              int lt, int g) {
  if constexpr (P < num_phases(NN, D) - 1) {
    middle_phase<Pol, NN, D, G, P>(buf, sA, lt);
    group_sync(g, G);
    middle_phases<Pol, NN, D, G, P + 1>(buf, sA, lt, g);
  }
}

// Shared memory per group: [d*NN*NN factor entries of V][MAXD+2 ints][buffer].
template <class Pol, int NN, int D>
__host__ __device__ constexpr int group_smem_bytes() {
  return ((MAXD * NN * NN * (int)sizeof(typename Pol::V) + (MAXD + 2) * 4 + 15) / 16) * 16 +
         ((buffer_slots<NN, D>() * (int)sizeof(typename Pol::V) + 15) / 16) * 16;
}

template <class Pol, int NN, int D>
__global__ void __launch_bounds__(group_threads(NN, D) < 256 ? 256 : group_threads(NN, D))
tile_kernel(const Problem p) {
  using V = typename Pol::V;
  using In = typename Pol::In;
  constexpr int G = group_threads(NN, D);
  constexpr int NN2 = NN * NN;
  constexpr int N = ipow(NN, D);
  constexpr int LP = num_phases(NN, D) - 1;  // the last phase
  constexpr int T0 = tile_size(NN, D, 0);
  constexpr int NT0 = N / T0;
  constexpr int TL = tile_size(NN, D, LP);
  constexpr int NTL = N / TL;
  constexpr bool PAIR0 = phase_b(NN, D, 0) >= 0;
  constexpr bool PAIRL = phase_b(NN, D, LP) >= 0;
  constexpr int aL = phase_a(NN, D, LP);
  constexpr int bL = PAIRL ? phase_b(NN, D, LP) : aL;

  extern __shared__ __align__(16) unsigned char smem[];
  const int E = p.groups_per_cta;
  const int g = threadIdx.x / G;
  const int lt = threadIdx.x - g * G;
  if (g >= E) return;
  unsigned char* gbase = smem + (size_t)g * group_smem_bytes<Pol, NN, D>();
  V* sA = reinterpret_cast<V*>(gbase);
  int* sExp = reinterpret_cast<int*>(gbase + MAXD * NN2 * sizeof(V));
  V* buf = reinterpret_cast<V*>(
      gbase + ((MAXD * NN2 * (int)sizeof(V) + (MAXD + 2) * 4 + 15) / 16) * 16);
  const bool excl = p.y_exclusive != 0;
  if (lt < MAXD + 2) sExp[lt] = 0;
  group_sync(g, G);

  const long long step = (long long)gridDim.x * E;
  for (long long e = (long long)blockIdx.x * E + g; e < p.count; e += step) {
    const long long entry = p.order ? (long long)p.order[e] : e + p.entry_offset;
    EntryPtrs<In> en;
    if (!resolve_entry<In>(p, entry, en)) {
      if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    // ---- factor entries and their scales ----
    In af = In(0);
    const bool has_a = lt < D * NN2;
    int al = 0, aidx = 0;
    if (has_a) {
      al = lt / NN2;
      const int r = lt - al * NN2, ar = r / NN, aj = r - ar * NN;
      aidx = lt;
      af = p.trans ? en.A[al][aj + (long long)ar * en.ld[al]] : en.A[al][ar + (long long)aj * en.ld[al]];
    }
    for (int i = lt + G; i < D * NN2; i += G) {
      // more factor entries than threads (large NN): stage raw values
      const int l = i / NN2, r = i - l * NN2, ar = r / NN, aj = r - ar * NN;
      const In v = p.trans ? en.A[l][aj + (long long)ar * en.ld[l]] : en.A[l][ar + (long long)aj * en.ld[l]];
      if constexpr (Pol::SCALED) atomicMax(&sExp[l], exp_field(v));
      reinterpret_cast<In*>(buf)[i] = v;
    }
    // ---- first tile(s) of X; with one tile per thread they stay in registers ----
    constexpr bool ONE = NT0 <= G;
    In xv[ONE ? T0 : 1];
    if constexpr (Pol::SCALED) {
      int ex = 0;
      if constexpr (ONE) {
        if (lt < NT0) {
#pragma unroll
          for (int t = 0; t < T0; ++t) {
            xv[t] = __ldg(en.X + tile_base<NN, D, 0>(lt) + tile_off<NN, D, 0>(t));
            ex = max(ex, exp_field(xv[t]));
          }
        }
      } else {
        for (int i = lt; i < N; i += G) ex = max(ex, exp_field(__ldg(en.X + i)));
      }
      ex = __reduce_max_sync(0xffffffffu, ex);
      if ((lt & 31) == 0 && ex > 0) atomicMax(&sExp[MAXD], ex);
      if (has_a) atomicMax(&sExp[al], exp_field(af));
    } else if constexpr (ONE) {
      if (lt < NT0) {
#pragma unroll
        for (int t = 0; t < T0; ++t) xv[t] = __ldg(en.X + tile_base<NN, D, 0>(lt) + tile_off<NN, D, 0>(t));
      }
    }
    group_sync(g, G);
    int escale = 0, ex = 0;
    if constexpr (Pol::SCALED) {
      bool skip = false, nonfinite = sExp[MAXD] == 2047;
      ex = sExp[MAXD];
      escale = ex - 1023;
#pragma unroll
      for (int l = 0; l < D; ++l) {
        escale += sExp[l] - 1023;
        nonfinite = nonfinite || sExp[l] == 2047;
        skip = skip || sExp[l] == 0;
      }
      skip = skip || ex == 0;
      if (skip || nonfinite) {
        group_sync(g, G);  // every thread has read sExp
        if (lt < MAXD + 2) sExp[lt] = 0;
        if constexpr (sizeof(In) == 8) {
          // Inf/NaN must propagate exactly as in FP64: evaluate this entry in
          // plain FP64 on the same shared memory (an all-zero factor or X
          // without Inf/NaN contributes exactly zero and is skipped).
          if (nonfinite) {
            sq_plain_entry<double, NN, false>(p, *reinterpret_cast<EntryPtrs<double>*>(&en),
                                              reinterpret_cast<double*>(sA),
                                              reinterpret_cast<double*>(buf), lt, G, g);
          }
        }
        group_sync(g, G);
        continue;
      }
    }
    if (has_a) sA[aidx] = Pol::make(af, Pol::SCALED ? sExp[al] : 0);
    for (int i = lt + G; i < D * NN2; i += G) {
      const int l = i / NN2;
      sA[i] = Pol::make(reinterpret_cast<In*>(buf)[i], Pol::SCALED ? sExp[l] : 0);
    }
    group_sync(g, G);  // sA ready; buf staging free; sExp read by all
    if (lt < MAXD + 2) sExp[lt] = 0;  // for the next entry (read above, before the barrier)

    // ---- phase 0: X (HBM) -> registers -> contract -> buf ----
    if constexpr (ONE) {
      if (lt < NT0) {
        V v[T0];
#pragma unroll
        for (int t = 0; t < T0; ++t) v[t] = Pol::make(xv[t], ex);
        contract_tile<Pol, NN, PAIR0>(v, sA + phase_a(NN, D, 0) * NN2,
                                      sA + (PAIR0 ? phase_b(NN, D, 0) : 0) * NN2);
        const int base = tile_base<NN, D, 0>(lt);
#pragma unroll
        for (int t = 0; t < T0; ++t) buf[slot<NN>(base + tile_off<NN, D, 0>(t))] = v[t];
      }
    } else {
      for (int u = lt; u < NT0; u += G) {
        const int base = tile_base<NN, D, 0>(u);
        V v[T0];
#pragma unroll
        for (int t = 0; t < T0; ++t) v[t] = Pol::make(__ldg(en.X + base + tile_off<NN, D, 0>(t)), ex);
        contract_tile<Pol, NN, PAIR0>(v, sA + phase_a(NN, D, 0) * NN2,
                                      sA + (PAIR0 ? phase_b(NN, D, 0) : 0) * NN2);
#pragma unroll
        for (int t = 0; t < T0; ++t) buf[slot<NN>(base + tile_off<NN, D, 0>(t))] = v[t];
      }
    }
    group_sync(g, G);
    // ---- middle phases: buf -> buf ----
    middle_phases<Pol, NN, D, G, 1>(buf, sA, lt, g);
    // ---- last phase: buf -> contract -> Y (HBM) ----
    for (int u = lt; u < NTL; u += G) {
      const int base = tile_base<NN, D, LP>(u);
      V v[TL];
#pragma unroll
      for (int t = 0; t < TL; ++t) v[t] = buf[slot<NN>(base + tile_off<NN, D, LP>(t))];
      contract_tile<Pol, NN, PAIRL>(v, sA + aL * NN2, sA + bL * NN2);
#pragma unroll
      for (int t = 0; t < TL; ++t) {
        const auto y = Pol::finish(v[t], escale);
        y_accumulate(en.Y + base + tile_off<NN, D, LP>(t), y, excl);
      }
    }
    group_sync(g, G);
  }
}

}  // namespace tile
}  // namespace kmx
