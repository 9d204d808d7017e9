// kmx_oz.cuh -- FP64 Kronecker mat-vec on the FP16 tensor cores by exact
// integer-digit products (the "digits" form).
//
// Each entry is contracted in steps of K = 16 (n = 4: two modes, factor
// F = A_a (x) A_b; n = 16: one mode), as a GEMM  Z'(i, c) = sum_k F(i, k) Z(k, c)
// with F as the 16 x 16 A operand and the intermediate Z as the B operand
// (c runs over the other digits).  Both operands are held as 7 base-2^9
// digit planes with one exponent per entry (block floating point):
//   Z = 2^E  * sum_s z_s 2^(-9(s+1)),   F = 2^EF * sum_t f_t 2^(-9(t+1)),
// digits exact in FP16.  mma.sync m16n8k16 (FP16 in, FP32 accumulate)
// forms every digit product with s + t <= 6 and adds it to the accumulator
// of its level L = s + t.  X digits are unsigned (|z| <= 511), all others
// balanced (|f|, |z| <= 256, F scaled below 1/2), so each level's sum stays
// below 7 * 16 * 511 * 256 < 2^24: every accumulator is an exact integer.
//
// Between steps the level sums are carried into balanced digits again with
// FP32 arithmetic (exact: rint by the 1.5 * 2^23 shift), the entry's
// leading digit position is found by a block vote, and the next step reads
// the 7 planes from there.  The last step combines the levels as an
// unevaluated FP32 pair (exact two-sums), widens it exactly to FP64 and adds
// it to Y with RED.F64.
//
// Accuracy: digits are kept to 63 bits below the entry's scale and products
// to level 6; everything dropped is below 2^-57 of the scale.  An entry whose
// result (at any step) comes out more than 2^-10 below its scale -- heavy
// cancellation, or factors/X with extreme ranges -- would keep fewer bits,
// so it is not written: its index goes to a redo list, which the
// double-float kernel then processes.  So are entries with Inf/NaN.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "kmx_engine.cuh"
#include "kmx_tile.cuh"

namespace kmx {
namespace oz {

using tile::ipow;

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr int NP = 7;      // digit planes of an operand
constexpr int LMAX = 6;    // highest product level kept
constexpr int NPLANE = 8;  // stored output planes (positions 0..7)

__host__ __device__ constexpr int group_digits(int NN) { return NN == 4 ? 2 : 1; }
__host__ __device__ constexpr bool supported(int NN, int D) {
  return (NN == 4 && (D == 4 || D == 6)) || (NN == 16 && (D == 2 || D == 3));
}

// rint(v) for |v| < 2^22, exact, FP32 pipe only
__device__ __forceinline__ float rint_s(float v) {
  return __fsub_rn(__fadd_rn(v, 12582912.0f), 12582912.0f);
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
  const __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ void mma_f16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                        uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared memory of one CTA (one entry at a time).
template <int NN, int D>
struct Smem {
  static constexpr int N = ipow(NN, D);
  static constexpr int G = group_digits(NN);
  static constexpr int P = D / G;
  __half z[NPLANE][N];         // digit planes of the intermediate, natural index order
  __half f[P][NP][16][16];     // digit planes of each step's factor, [i][k]
  double a[D][NN][NN];         // the entry's factors, [l][i][k] (transposed if asked)
  int ef[P];                   // per-step factor exponent (|F| < 2^(ef-1))
  int emax;                    // X block: largest biased exponent
  int flags;                   // OZ_* bits of the entry
  int top[P];                  // per step: bit 0 a digit at position 0, bit 1 at position 1
  float gn[P + 2];             // cancellation guard: ||F_ph||^2 (2^(ef-1021) units), ||X||^2
                               // (2^(emax-1023) units), ||KX||^2 (2^es units)
};

// |x| as a 63-bit fraction of 2^E (E = emax - 1022): digit s (0..6) is bits
// [62 - 9s - 8, 62 - 9s], unsigned; the sign is returned separately.
__device__ __forceinline__ void x_digits(double x, int emax, float (&dg)[NP]) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  int ee = e;
  if (e == 0) {
    ee = 1;  // subnormal: no implicit bit
  } else {
    m |= 1ull << 52;
  }
  const int sh = ee - emax + 10;  // m << sh is the 63-bit fraction
  unsigned long long f;
  if (sh >= 0) {
    f = m << sh;
  } else if (sh > -64) {
    f = m >> (-sh);
  } else {
    f = 0;
  }
  const bool neg = (b >> 63) != 0;
#pragma unroll
  for (int s = 0; s < NP; ++s) {
    const float v = (float)(unsigned)((f >> (54 - 9 * s)) & 511u);
    dg[s] = neg ? -v : v;
  }
}

// Level sums acc[L] (position L+2) -> balanced digits at positions 0..7.
__device__ __forceinline__ void carry(const float (&acc)[LMAX + 1], float (&dg)[NPLANE]) {
  float a[LMAX + 1];
#pragma unroll
  for (int L = 0; L <= LMAX; ++L) a[L] = acc[L];
  // position 8 (level 6) is not stored; its carry goes up
#pragma unroll
  for (int L = LMAX; L >= 1; --L) {
    const float c = rint_s(__fmul_rn(a[L], 1.0f / 512.0f));
    if (L + 2 < NPLANE) dg[L + 2] = __fmaf_rn(-512.0f, c, a[L]);
    a[L - 1] = __fadd_rn(a[L - 1], c);
  }
  const float c1 = rint_s(__fmul_rn(a[0], 1.0f / 512.0f));
  dg[2] = __fmaf_rn(-512.0f, c1, a[0]);
  const float c0 = rint_s(__fmul_rn(c1, 1.0f / 512.0f));
  dg[1] = __fmaf_rn(-512.0f, c0, c1);
  dg[0] = c0;
}

// Natural index of GEMM element (k or i within the group, column c).
template <int NN, int D, int PH>
__device__ __forceinline__ int nat(int k, int c) {
  constexpr int G = group_digits(NN);
  constexpr int R = ipow(NN, D - (PH + 1) * G);  // stride of the group's last digit
  const int L = c / R, r = c - L * R;
  return (L * 16 + k) * R + r;
}

// Physical half index of natural element a in a digit plane: 32-bit words
// XOR-swizzled (w ^ (w >> 5) & 31), which keeps the fragment loads and the
// digit stores of every step within 2-way bank conflicts.
__device__ __forceinline__ int zsw(int a) {
  const int w = a >> 1;
  return ((w ^ ((w >> 5) & 31)) << 1) | (a & 1);
}

template <int NN, int D>
struct Shape {
  static constexpr int N = ipow(NN, D);
  static constexpr int G = group_digits(NN);
  static constexpr int P = D / G;
  static constexpr int NC = N / 16;                        // GEMM columns per step
  static constexpr int NT = NC / 8;                        // n-tiles per step
  static constexpr int TPW = (NT + WARPS - 1) / WARPS;     // n-tiles per warp
};

// Digits of F for step PH, as A fragments (7 planes x 4 registers).
template <int NN, int D, int PH>
__device__ __forceinline__ void load_f(const Smem<NN, D>& S, int g, int t, uint32_t (&af)[NP][4]) {
#pragma unroll
  for (int s = 0; s < NP; ++s) {
    const __half* f = &S.f[PH][s][0][0];
    af[s][0] = *reinterpret_cast<const uint32_t*>(f + g * 16 + 2 * t);
    af[s][1] = *reinterpret_cast<const uint32_t*>(f + (g + 8) * 16 + 2 * t);
    af[s][2] = *reinterpret_cast<const uint32_t*>(f + g * 16 + 2 * t + 8);
    af[s][3] = *reinterpret_cast<const uint32_t*>(f + (g + 8) * 16 + 2 * t + 8);
  }
}

__device__ __forceinline__ uint32_t pack_raw(__half lo, __half hi) {
  return (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
}

// One step over the warp's n-tiles.  Returns (through flags in shared
// memory) which leading positions were nonzero; the last step leaves the
// outputs in ov (hi, lo per element) for the caller to add to Y.
template <int NN, int D, int PH>
__device__ __forceinline__ void run_step(Smem<NN, D>& S, const double (&xv)[Shape<NN, D>::TPW][4],
                                         int top, int warp, int g, int t,
                                         float (&ov)[Shape<NN, D>::TPW][4][2], bool& big) {
  using SH = Shape<NN, D>;
  uint32_t af[NP][4];
  load_f<NN, D, PH>(S, g, t, af);
  bool nz0 = false, nz1 = false;
#pragma unroll
  for (int j = 0; j < SH::TPW; ++j) {
    const int nt = warp + j * WARPS;
    if (nt >= SH::NT) break;
    const int c = nt * 8 + g;
    uint32_t b0[NP], b1[NP];
    if constexpr (PH == 0) {
      float d0[NP], d1[NP], d8[NP], d9[NP];
      x_digits(xv[j][0], S.emax, d0);
      x_digits(xv[j][1], S.emax, d1);
      x_digits(xv[j][2], S.emax, d8);
      x_digits(xv[j][3], S.emax, d9);
#pragma unroll
      for (int s = 0; s < NP; ++s) {
        b0[s] = pack_h2(d0[s], d1[s]);
        b1[s] = pack_h2(d8[s], d9[s]);
      }
    } else {
      const int a0 = nat<NN, D, PH>(2 * t, c), a1 = nat<NN, D, PH>(2 * t + 1, c);
      const int a8 = nat<NN, D, PH>(2 * t + 8, c), a9 = nat<NN, D, PH>(2 * t + 9, c);
      const int p0 = zsw(a0), p1 = zsw(a1), p8 = zsw(a8), p9 = zsw(a9);
#pragma unroll
      for (int s = 0; s < NP; ++s) {
        const __half* z = S.z[top + s];
        b0[s] = pack_raw(z[p0], z[p1]);
        b1[s] = pack_raw(z[p8], z[p9]);
      }
    }
    float acc[LMAX + 1][4];
#pragma unroll
    for (int L = 0; L <= LMAX; ++L)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[L][q] = 0.f;
#pragma unroll
    for (int s = 0; s < NP; ++s)
#pragma unroll
      for (int tt = 0; tt < NP; ++tt)
        if (s + tt <= LMAX) mma_f16(acc[s + tt], af[tt], b0[s], b1[s]);
    // element q: row i = g + 8*(q >> 1), column 8*nt + 2*t + (q & 1)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float lv[LMAX + 1];
#pragma unroll
      for (int L = 0; L <= LMAX; ++L) lv[L] = acc[L][q];
      const int i = g + 8 * (q >> 1), col = nt * 8 + 2 * t + (q & 1);
      if constexpr (PH + 1 < SH::P) {
        float dg[NPLANE];
        carry(lv, dg);
        nz0 = nz0 || dg[0] != 0.f;
        nz1 = nz1 || dg[1] != 0.f;
        const int pa = zsw(nat<NN, D, PH>(i, col));
#pragma unroll
        for (int pl = 0; pl < NPLANE; ++pl) S.z[pl][pa] = __float2half_rn(dg[pl]);
      } else {
        // value / 2^scale = sum_L lv[L] 2^(-9(L+2)), as an unevaluated FP32 pair
        float hi = __fmul_rn(lv[0], 0x1p-18f), lo = 0.f;
#pragma unroll
        for (int L = 1; L <= LMAX; ++L) {
          const float v = __fmul_rn(lv[L], __int_as_float((127 - 9 * (L + 2)) << 23));
          const float s2 = __fadd_rn(hi, v);
          const float bp = __fsub_rn(s2, hi);
          lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s2, bp)), __fsub_rn(v, bp)));
          hi = s2;
        }
        const float h2 = __fadd_rn(hi, lo);
        ov[j][q][0] = h2;
        ov[j][q][1] = __fsub_rn(lo, __fsub_rn(h2, hi));
        big = big || fabsf(h2) >= 0x1p-10f;
      }
    }
  }
  if constexpr (PH + 1 < SH::P) {
    nz0 = __any_sync(0xffffffffu, nz0);
    nz1 = __any_sync(0xffffffffu, nz1);
    if ((threadIdx.x & 31) == 0 && (nz0 || nz1)) atomicOr(&S.top[PH], (nz0 ? 1 : 0) | (nz1 ? 2 : 0));
  }
}

enum : int { OZ_REDO = 1, OZ_NULL = 2, OZ_BIG = 4 };

template <int NN, int D, int PH>
__device__ __forceinline__ void steps(Smem<NN, D>& S, const double (&xv)[Shape<NN, D>::TPW][4],
                                      int top, int E, int warp, int g, int t, double* yp) {
  using SH = Shape<NN, D>;
  float ov[SH::TPW][4][2];
  bool big = false;
  run_step<NN, D, PH>(S, xv, top, warp, g, t, ov, big);
  const int efs = S.ef[PH] - 1021;  // F = 2^efs * sum_t f_t 2^(-9(t+1))
  if constexpr (PH + 1 < SH::P) {
    __syncthreads();  // digits of step PH stored, leading positions voted
    const int tf = S.top[PH];
    const int ntop = (tf & 1) ? 0 : (tf & 2) ? 1 : -1;
    if (ntop < 0) {
      // the result fell more than 2^-10 below the block scale: redo in double-float
      if (threadIdx.x == 0) atomicOr(&S.flags, OZ_REDO);
      return;
    }
    steps<NN, D, PH + 1>(S, xv, ntop, E + efs + 9 * (1 - ntop), warp, g, t, yp);
  } else {
    if (__any_sync(0xffffffffu, big) && (threadIdx.x & 31) == 0) atomicOr(&S.flags, OZ_BIG);
    float o2 = 0.f;
#pragma unroll
    for (int j = 0; j < SH::TPW; ++j) {
      if (warp + j * WARPS >= SH::NT) break;
#pragma unroll
      for (int q = 0; q < 4; ++q) o2 = __fmaf_rn(ov[j][q][0], ov[j][q][0], o2);
    }
    o2 = warp_sum(o2);
    if ((threadIdx.x & 31) == 0) atomicAdd(&S.gn[SH::P + 1], o2);
    __syncthreads();
    const int es = E + efs;
    // cancellation guard of the double-float forms (kmx_engine.cuh), with the
    // three norms brought to one scale: the output carries 2^es, X 2^(emax-1023),
    // factor F_ph 2^(ef_ph-1021)
    int delta = es - (S.emax - 1023);
#pragma unroll
    for (int ph = 0; ph < SH::P; ++ph) delta -= S.ef[ph] - 1021;
    float rhs = S.gn[SH::P];
#pragma unroll
    for (int ph = 0; ph < SH::P; ++ph) rhs *= S.gn[ph];
    const bool cancel =
        delta < 0 || delta > 60 ||
        S.gn[SH::P + 1] * __int_as_float((127 + 2 * delta) << 23) * (float)SH::N * GUARD_INV_TAU2 <
            rhs;
    if (!(S.flags & OZ_BIG) || cancel) {
      if (threadIdx.x == 0) atomicOr(&S.flags, OZ_REDO);
      return;
    }
#pragma unroll
    for (int j = 0; j < SH::TPW; ++j) {
      const int nt = warp + j * WARPS;
      if (nt >= SH::NT) break;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = g + 8 * (q >> 1), col = nt * 8 + 2 * t + (q & 1);
        const double y = tile::SplitPolicy::to_f64(ov[j][q][0], es) +
                         tile::SplitPolicy::to_f64(ov[j][q][1], es);
        atomicAdd(yp + nat<NN, D, PH>(i, col), y);
      }
    }
  }
}

// Persistent: one entry per CTA at a time, grid-stride over the launch.
// Entries that need the double-float path are appended to redo[].
template <int NN, int D>
__global__ void __launch_bounds__(THREADS, 1) oz_kernel(const Problem p, int* redo, int* redo_count) {
  static_assert(supported(NN, D), "no digits kernel for this shape");
  using SH = Shape<NN, D>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem<NN, D>& S = *reinterpret_cast<Smem<NN, D>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const long long total = launch_count(p);
  for (long long e = blockIdx.x; e < total; e += gridDim.x) {
    const long long ent = tile::entry_index(p, e);
    __syncthreads();  // the previous entry is done with shared memory
    if (threadIdx.x < SH::P) {
      S.ef[threadIdx.x] = 0;
      S.top[threadIdx.x] = 0;
    }
    if (threadIdx.x < SH::P + 2) S.gn[threadIdx.x] = 0.f;
    if (threadIdx.x == 0) {
      S.flags = 0;
      S.emax = 0;
    }
    __syncthreads();
    // factors (FP64) and their exponents
    for (int idx = threadIdx.x; idx < D * NN * NN; idx += THREADS) {
      const int l = idx / (NN * NN), rem = idx - l * NN * NN;
      const int i = rem / NN, k = rem - i * NN;
      const double* Ap = tile::a_ptr<double>(p, ent, l);
      double v = 0.0;
      if (Ap) {
        const long long ld = p.ld[l];
        v = p.trans ? Ap[k + i * ld] : Ap[i + k * ld];
        if (exp_field(v) == 2047) atomicOr(&S.flags, OZ_REDO);
      } else {
        atomicOr(&S.flags, OZ_NULL);
      }
      S.a[l][i][k] = v;
    }
    const double* xp = tile::x_ptr<double>(p, ent);
    double* yp = tile::y_ptr<double>(p, ent);
    if (threadIdx.x == 0 && (!xp || !yp)) atomicOr(&S.flags, OZ_NULL);
    __syncthreads();
    if (S.flags & OZ_NULL) {
      if (threadIdx.x == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    // X values of this thread's step-0 fragments, and the block exponent
    double xv[SH::TPW][4];
    int xe = 0;
#pragma unroll
    for (int j = 0; j < SH::TPW; ++j) {
      const int nt = warp + j * WARPS;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = 2 * t + (q & 1) + 8 * (q >> 1);
        xv[j][q] = nt < SH::NT ? xp[nat<NN, D, 0>(k, nt * 8 + g)] : 0.0;
        xe = max(xe, exp_field(xv[j][q]));
      }
    }
    xe = __reduce_max_sync(0xffffffffu, xe);
    if (lane == 0) atomicMax(&S.emax, xe);
    __syncthreads();  // block exponent of X final (for the guard's norm of X)
    {
      float x2 = 0.f;
#pragma unroll
      for (int j = 0; j < SH::TPW; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float h = split_scaled(xv[j][q], S.emax).hi;
          x2 = __fmaf_rn(h, h, x2);
        }
      x2 = warp_sum(x2);
      if (lane == 0) atomicAdd(&S.gn[SH::P], x2);
    }
    // combined factors of every step; their block exponents
    for (int idx = threadIdx.x; idx < SH::P * 256; idx += THREADS) {
      const int ph = idx >> 8, i = (idx >> 4) & 15, k = idx & 15;
      double f;
      if constexpr (NN == 4) {
        f = S.a[2 * ph][i >> 2][k >> 2] * S.a[2 * ph + 1][i & 3][k & 3];
      } else {
        f = S.a[ph][i][k];
      }
      atomicMax(&S.ef[ph], exp_field(f));
    }
    __syncthreads();
    bool skip = S.emax == 0;  // X is zero: nothing to add
    for (int ph = 0; ph < SH::P; ++ph) skip = skip || S.ef[ph] == 0;
    if (S.emax == 2047) {
      if (threadIdx.x == 0) atomicOr(&S.flags, OZ_REDO);
    }
    for (int ph = 0; ph < SH::P; ++ph)
      if (S.ef[ph] == 2047 && threadIdx.x == 0) atomicOr(&S.flags, OZ_REDO);
    __syncthreads();
    if (S.flags & OZ_REDO) {
      if (threadIdx.x == 0) {
        redo[atomicAdd(redo_count, 1)] = (int)ent;
        count_redo(p.redo_ctr, 1);
      }
      continue;
    }
    if (skip) continue;
    // factor digits: F * 2^-(ef-1021) in (-1/2, 1/2), 7 balanced base-2^9 digits
    for (int idx = threadIdx.x; idx < SH::P * 256; idx += THREADS) {
      const int ph = idx >> 8, i = (idx >> 4) & 15, k = idx & 15;
      double f;
      if constexpr (NN == 4) {
        f = S.a[2 * ph][i >> 2][k >> 2] * S.a[2 * ph + 1][i & 3][k & 3];
      } else {
        f = S.a[ph][i][k];
      }
      df u = split_scaled(f, S.ef[ph] + 2);
      const float fn = warp_sum(u.hi * u.hi);  // a warp's 32 elements share ph
      if ((threadIdx.x & 31) == 0) atomicAdd(&S.gn[ph], fn);
      float hi = u.hi, lo = u.lo;
#pragma unroll
      for (int sd = 0; sd < NP; ++sd) {
        const float tt = __fmul_rn(hi, 512.0f);
        const float dgt = rint_s(tt);
        const float rh = __fsub_rn(tt, dgt), rl = __fmul_rn(lo, 512.0f);
        hi = __fadd_rn(rh, rl);
        lo = __fsub_rn(rl, __fsub_rn(hi, rh));
        S.f[ph][sd][i][k] = __float2half_rn(dgt);
      }
    }
    __syncthreads();
    steps<NN, D, 0>(S, xv, 0, S.emax - 1022, warp, g, t, yp);
    __syncthreads();
    if ((S.flags & OZ_REDO) && threadIdx.x == 0) {
      redo[atomicAdd(redo_count, 1)] = (int)ent;
      count_redo(p.redo_ctr, 1);
    }
  }
}

template <int NN, int D>
constexpr int smem_bytes() {
  return (int)sizeof(Smem<NN, D>);
}

}  // namespace oz
}  // namespace kmx
