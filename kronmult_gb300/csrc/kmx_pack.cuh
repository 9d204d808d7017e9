// kmx_pack.cuh -- double-float dot products on packed FP32 pairs.
//
// sm_100+ executes FP32 add / mul / fma on a pair of FP32 values per lane in
// one instruction (PTX add/sub/mul/fma.rn.f32x2).  The double-float mode
// contraction of the register-tiled kernels evaluates the dot products of two
// output rows (r, r+1) at once: the factor is stored as row pairs
// (A(r,j), A(r+1,j)) and each input value v_j is broadcast to both halves.
// Every operation of the scalar double-float dot (exact product by FMA,
// error-free two-sums, FP32 sums of the cross terms and errors) maps one to
// one onto the packed form, so the results carry the same ~2^-48 relative
// accuracy while the FP32 instruction count halves.
//
// The exact error of a product p = fl(a v) is fma(a, v, -p).  PTX has no
// packed negation, so each input's high part is also broadcast negated: the
// products are formed as q = fl(a (-v)) = -p (round-to-nearest is symmetric)
// and the error as fma(a, v, q); the two-sums then run on the negated
// products, and the result is (c - s) for their negated sum s and the FP32
// sum c of everything else.  (Keeping the factor's negated high parts instead
// costs a third more factor registers and measured 1.6 % slower.)
#pragma once

#include <stdint.h>

namespace kmx {
namespace pk2 {

typedef unsigned long long u64;

__device__ __forceinline__ u64 pack(float a, float b) {
  u64 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ u64 bcast(float a) { return pack(a, a); }
__device__ __forceinline__ void unpack(u64 v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ u64 add(u64 a, u64 b) {
  u64 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 sub(u64 a, u64 b) {
  u64 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 mul(u64 a, u64 b) {
  u64 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 fma(u64 a, u64 b, u64 c) {
  u64 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// Exact sum of two pairs: s + e == a + b per half (Knuth's two-sum).
__device__ __forceinline__ void two_sum(u64 a, u64 b, u64& s, u64& e) {
  s = add(a, b);
  const u64 bp = sub(s, a);
  e = add(sub(a, sub(s, bp)), sub(b, bp));
}

// One factor row pair: column j holds (A(r,j), A(r+1,j)) split as high and
// low parts.
struct RowPair {
  u64 hi, lo;
};

// Factor l in shared memory as RP = ceil(NN/2) row pairs x NN columns of
// RowPair (16 bytes each); an odd NN pads a zero row.
template <int NN>
__host__ __device__ constexpr int row_pairs() {
  return (NN + 1) / 2;
}
template <int NN>
__host__ __device__ constexpr int factor_u64() {
  return 2 * row_pairs<NN>() * NN;
}

// Dot products of row pair rp with the NN values (vh[j], vl[j]) (each already
// broadcast to both halves; nvh[j] = -vh[j]): out = sum_j A(r,j) v_j for
// r = 2rp, 2rp+1.
template <int NN>
__device__ __forceinline__ void dot_pair(const RowPair* ap, const u64* vh, const u64* vl,
                                         const u64* nvh, u64& ohi, u64& olo) {
  u64 q[NN], c = 0;
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    const RowPair a = ap[j];
    q[j] = mul(a.hi, nvh[j]);            // -p, rounded
    u64 e = fma(a.hi, vh[j], q[j]);      // a v - p, exact
    e = fma(a.hi, vl[j], e);
    e = fma(a.lo, vh[j], e);
    c = j == 0 ? e : add(c, e);
  }
  // pairwise two-sums of the negated products; their errors come out negated
#pragma unroll
  for (int w = 1; w < NN; w *= 2) {
#pragma unroll
    for (int j = 0; j + w < NN; j += 2 * w) {
      u64 s, e;
      two_sum(q[j], q[j + w], s, e);
      q[j] = s;
      c = sub(c, e);
    }
  }
  // value = s + c with s = -q[0] (|s| >= |c|): fast two-sum into (hi, lo)
  ohi = sub(c, q[0]);
  olo = sub(c, add(ohi, q[0]));
}

// Factor rows of one mode: in registers for NN <= 4 (at most 8 row pairs,
// 32 registers), read from shared memory at each use otherwise.
template <int NN>
struct PackedRows {
  static constexpr int RP = row_pairs<NN>();
  static constexpr bool REG = NN <= 4;
  RowPair r[REG ? RP * NN : 1];
  const RowPair* s;
  __device__ __forceinline__ void load(const RowPair* src) {
    s = src;
    if constexpr (REG) {
#pragma unroll
      for (int i = 0; i < RP * NN; ++i) r[i] = src[i];
    }
  }
  __device__ __forceinline__ const RowPair* pair(int rp) const {
    if constexpr (REG) {
      return r + rp * NN;
    } else {
      return s + rp * NN;
    }
  }
};

}  // namespace pk2
}  // namespace kmx
