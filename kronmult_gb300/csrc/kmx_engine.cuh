// kmx_engine.cuh -- device engine of the batched Kronecker mat-vec on sm_103a.
//
//   Y(:,k) += kron(A1(:,:,k), ..., Ad(:,:,k)) * X(:,k)
//
// One "entry" k is processed by a GROUP of G threads (G a multiple of 32);
// a CTA holds E = blockDim/G groups, each with its own shared-memory region
// and its own stream of entries (grid-stride over entries).  For one entry
// the d mode contractions run on chip:
//
//   mode 0      reads the X block straight from HBM (the mode-0 fibers are
//               the n slices of X, so lane f reads X[j*s + f]: coalesced) and
//               writes the first intermediate to shared memory;
//   modes 1..d-2 update the intermediate IN PLACE: a lane owns whole fibers
//               (n elements at stride s), reads them, forms the n outputs and
//               writes them back to the same slots;
//   mode d-1    reads shared memory and adds its outputs to the Y block in
//               HBM, one output per lane so consecutive lanes touch
//               consecutive Y elements (coalesced FP64 atomics / RMW).
//
// The reference evaluates the same contractions in the same mode order (A1
// first) as a recursion of tiny GEMMs with every intermediate in global
// memory (kronmultv.hpp:19-148, kgemm_nt.hpp:215-385, kgemm_nn.hpp:227-406).
//
// Arithmetic forms:
//   FormPlain<T>  T = double or float, fused multiply-add in T.
//   FormSplit     FP64 in/out, carried as FP32 (hi, lo) pairs ("double-float"):
//                 every product hi*hi is split exactly with an FMA, the sums of
//                 hi parts are error-free (two-sum), the cross terms and the
//                 errors are summed in FP32.  GB300 runs FP32 ~70x faster than
//                 FP64, so this form trades ~2^-47 relative per operation for
//                 ~6x throughput.  Each entry is first scaled by powers of two
//                 (per factor and for X) so every carried value is <= 2 in
//                 magnitude; the scale is folded back into the exponent of the
//                 FP64 result.  Entries holding Inf/NaN take the plain path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kmx {

constexpr int MAXD = 6;
constexpr int MAX_THREADS = 512;

enum Layout : int { L_BATCHED = 0, L_PBATCHED = 1, L_XBATCHED = 2, L_VBATCHED = 3, L_MIXED = 4 };

// Bits of the device status word.
enum DevFlag : int { DF_NULL_PTR = 1, DF_WAIT_TIMEOUT = 2, DF_BAD_SHAPE = 4, DF_NONFINITE_SPLIT = 8, DF_OVERLAP = 16 };

// Everything a launch needs.  Shapes are those of the APPLIED operator:
// mode l maps n[l] -> m[l]; with trans != 0 factor l is read transposed
// (the host then passes m/n of A_l^T).
struct Problem {
  int layout;
  int d;
  int m[MAXD], n[MAXD], ld[MAXD];
  long long Nx, Ny;      // input / output block lengths
  long long sxw;         // largest intermediate (elements)
  int count;             // entries in this launch
  int entry_offset;      // index of the first entry (sub-batches)
  const void* A;         // batched/pbatched: T base (n,n,d,batch); x/v: const T* const*
  const void* X;         // batched: T base; otherwise T* const*
  void* Y;               // batched: T base; otherwise T* const*
  const int* order;      // optional processing order of entries (may be null)
  int trans;             // read every factor transposed
  int y_exclusive;       // Y blocks of distinct entries never overlap
  int* status;           // device status word
  // execution shape
  int group_threads;     // G
  int groups_per_cta;    // E
  int group_smem;        // bytes of shared memory per group
  // global-memory workspace for entries that do not fit on chip
  int wmode;             // 0 none, 1 per-entry pointer array, 2 slot pointer pairs, 3 base+stride slots
  void* const* pW;       // wmode 1: pW[entry]; wmode 2: pW[2*slot]
  void* Wbase;           // wmode 3
  long long w_stride;    // wmode 3: elements between slots
  int nslots;            // concurrent workspace slots (grid*E must not exceed it)
  // deterministic mode: entries grouped into Y segments (device arrays)
  const int* seg_entries;  // entry ids sorted by Y block, original order within a block
  const int* seg_offset;   // first position of segment s in seg_entries
  const int* seg_count;    // entries of segment s
  const int* seg_order;    // processing order of segments (longest first)
  const int* seg_num;      // number of segments (device scalar)
  int* seg_queue;          // work-queue counter, zero at launch
  const int* seg_key;      // mixed shapes: class of each entry; only seg_class's are taken
  int seg_class;
  // mixed-shape batches: this launch covers order[*order_base .. *order_base + *count_dev)
  const long long* a_off;  // L_MIXED: first factor pointer of instance i in A
  const int* count_dev;    // when set, the entry count is read from device memory
  const int* order_base;   // when set, offset of this launch's entries in order[]
  // diagnostic counters (may be null): [0] double-float entries recomputed in
  // FP64 by the cancellation guard, [1] digits-form entries handed to the
  // double-float pass
  unsigned long long* redo_ctr;
  int guard_off;         // nonzero: double-float without the cancellation guard
  // test hook (set from the host environment, see run_problem): nonzero makes
  // each group's first wait on a staged copy report that it ran out, so that
  // the timeout path -- drain the copy, flag DF_WAIT_TIMEOUT, leave -- runs
  // without a real stall
  int wait_expire;
};

// ---------------------------------------------------------------------------
// Cancellation guard of the double-float forms.
//
// Double-float carries about 48 bits, so its error on one entry is about
// 2^-48 |K||X| (elementwise), where plain FP64's is about 2^-53 d n |K||X|:
// when KX is much smaller than |K||X| (cancellation), the double-float result
// loses accuracy first.  |K||X| is not available cheaply, but its norm is
// bounded by prod_l ||A_l||_F ||X||_2, and for random (isotropic) data
//     rho_F = ||KX||_2 sqrt(N) / (prod_l ||A_l||_F ||X||_2)
// stays near 1 (above 0.2 for every shape at the 1e-4 quantile, measured on
// Gaussian and uniform inputs), falling in proportion to the cancellation.
// An entry with rho_F < 1/4 is recomputed in plain FP64: the double-float
// error times rho_F stays below about 8e-14, so the entries it keeps are
// within about 3e-13 even in the worst case measured and within 1e-13 on
// every cancelling family tested.  The three norms are summed in FP32 from
// the scaled high parts (the scale factors cancel in rho_F).
// ---------------------------------------------------------------------------
constexpr float GUARD_INV_TAU2 = 16.f;  // 1 / tau^2 with tau = 1/4

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sums[key] += v for every lane of the warp whose `valid` is set, where key
// does not decrease with the lane index (invalid lanes last): each run of
// equal keys is summed by shuffles and its first lane adds the run's sum with
// one shared-memory atomic, so no two lanes of a warp add to one address (a
// factor's n*n squared entries otherwise queue on one word).  Every lane of
// the warp calls it.
__device__ __forceinline__ void warp_run_add(float* sums, int key, float v, bool valid) {
  const int lane = threadIdx.x & 31;
  if (!valid) {
    key = 0x7fffffff;
    v = 0.f;
  }
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const float t = __shfl_down_sync(0xffffffffu, v, off);
    const int tk = __shfl_down_sync(0xffffffffu, key, off);
    if (lane + off < 32 && tk == key) v += t;
  }
  const int pk = __shfl_up_sync(0xffffffffu, key, 1);
  if (valid && (lane == 0 || pk != key)) atomicAdd(&sums[key], v);
}

// true when the entry must be recomputed in FP64: out2 = ||KX||^2, x2 = ||X||^2,
// a2[l] = ||A_l||_F^2 (all of scaled values), N = length of X (for m_l x n_l
// factors E||A v||^2 = ||A||_F^2 ||v||^2 / n_l, so prod n_l is the normaliser)
__device__ __forceinline__ bool guard_fails(float out2, float x2, const float* a2, int d, long long N) {
  float rhs = x2;
  for (int l = 0; l < d; ++l) rhs *= a2[l];
  return out2 * (float)N * GUARD_INV_TAU2 < rhs;
}

__device__ __forceinline__ void count_redo(const unsigned long long* ctr_base, int which) {
  if (ctr_base) atomicAdd(const_cast<unsigned long long*>(ctr_base) + which, 1ull);
}

// Entries of a launch (device-side count when the host does not know it).
__device__ __forceinline__ long long launch_count(const Problem& p) {
  return p.count_dev ? (long long)*p.count_dev : (long long)p.count;
}

// The entries one group processes, in order: grid-stride over the launch's
// entries (through p.order when given), or, with segments (deterministic
// mode), every entry of each segment the group takes -- segments grid-stride
// in the longest-first order -- in their stored order.  A segment's entries
// share one Y block, so the group that owns it adds their contributions in a
// fixed order (plain read-modify-write, y_exclusive).  With seg_key (mixed
// shapes) the segments span every class and each class's launch takes only
// its own entries; launches run class after class on the stream, so a Y
// block's contributions still arrive in one fixed order.  Uniform over a group.
struct EntryStream {
  long long pos, step, end, obase;
  int j, cnt, off;
  __device__ EntryStream(const Problem& p, long long slot0, long long step_)
      : pos(slot0), step(step_), j(0), cnt(0), off(0) {
    end = p.seg_entries ? (long long)*p.seg_num : launch_count(p);
    obase = p.order_base ? (long long)*p.order_base : 0;
  }
  __device__ bool next(const Problem& p, long long& entry) {
    if (p.seg_entries) {
      for (;;) {
        while (j >= cnt) {
          if (pos >= end) return false;
          const int sid = p.seg_order[pos];
          off = p.seg_offset[sid];
          cnt = p.seg_count[sid];
          j = 0;
          pos += step;
        }
        entry = p.seg_entries[off + j++];
        if (!p.seg_key || p.seg_key[entry] == p.seg_class) return true;
      }
    }
    if (pos >= end) return false;
    entry = p.order ? (long long)p.order[obase + pos] : pos + p.entry_offset;
    pos += step;
    return true;
  }
};

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------

// Division by a run-time constant (round-up method), exact for n < 2^31.
struct FastDiv {
  unsigned mul;
  int shift;
  unsigned div;
  __host__ __device__ FastDiv() : mul(1), shift(0), div(1) {}
  __host__ __device__ explicit FastDiv(unsigned s) : div(s) {
    shift = 0;
    while ((1u << shift) < s) ++shift;
    mul = (unsigned)(((1ull << 32) * ((1ull << shift) - s)) / s + 1);
  }
  __device__ __forceinline__ unsigned operator()(unsigned x) const {
    return (__umulhi(mul, x) + x) >> shift;
  }
};

__device__ __forceinline__ void group_sync(int g, int G) {
  if (G == (int)blockDim.x) {
    __syncthreads();
  } else if (G == 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(G) : "memory");
  }
}

template <typename T>
struct EntryPtrs {
  const T* X;
  T* Y;
  const T* A[MAXD];
  int ld[MAXD];
};

// Resolve the pointers of entry e.  Returns false if any is NULL.
template <typename T>
__device__ __forceinline__ bool resolve_entry(const Problem& p, long long e, EntryPtrs<T>& en) {
  const int d = p.d;
  if (p.layout == L_BATCHED || p.layout == L_PBATCHED) {
    if (p.layout == L_BATCHED) {
      en.X = static_cast<const T*>(p.X) + e * p.Nx;
      en.Y = static_cast<T*>(p.Y) + e * p.Ny;
    } else {
      en.X = static_cast<T* const*>(p.X)[e];
      en.Y = static_cast<T* const*>(p.Y)[e];
    }
    const long long nn = (long long)p.n[0] * p.n[0];
#pragma unroll
    for (int l = 0; l < MAXD; ++l) {
      if (l < d) {
        en.A[l] = static_cast<const T*>(p.A) + (e * d + l) * nn;
        en.ld[l] = p.ld[l];
      }
    }
  } else {
    en.X = static_cast<T* const*>(p.X)[e];
    en.Y = static_cast<T* const*>(p.Y)[e];
    const T* const* Ap = static_cast<const T* const*>(p.A) + (p.a_off ? p.a_off[e] : e * d);
#pragma unroll
    for (int l = 0; l < MAXD; ++l) {
      if (l < d) {
        en.A[l] = Ap[l];
        en.ld[l] = p.ld[l];
      }
    }
  }
  bool ok = (en.X != nullptr) && (en.Y != nullptr);
#pragma unroll
  for (int l = 0; l < MAXD; ++l)
    if (l < d) ok = ok && (en.A[l] != nullptr);
  return ok;
}

// Global workspace of one group: two buffers of sxw elements (the second
// only for rectangular shapes).  Returns false if none is available.
template <typename T>
__device__ __forceinline__ bool workspace(const Problem& p, long long entry, long long slot, T*& w0,
                                          T*& w1) {
  w0 = w1 = nullptr;
  if (p.wmode == 1) {
    w0 = static_cast<T*>(p.pW[entry]);
  } else if (p.wmode == 2) {
    w0 = static_cast<T*>(p.pW[2 * slot]);
    w1 = static_cast<T*>(p.pW[2 * slot + 1]);
  } else if (p.wmode == 3) {
    w0 = static_cast<T*>(p.Wbase) + slot * p.w_stride;
    w1 = w0 + p.sxw;
  }
  return w0 != nullptr;
}

template <typename T>
__device__ __forceinline__ void y_accumulate(T* y, T v, bool exclusive) {
  if (exclusive) {
    *y += v;
  } else {
    atomicAdd(y, v);
  }
}

// ---------------------------------------------------------------------------
// Double-float ("split") arithmetic.  Explicit _rn intrinsics keep the
// compiler from fusing the error-free transformations.
// ---------------------------------------------------------------------------
struct df {
  float hi, lo;
};

// Biased FP64 exponent field of x (0 for zero/subnormal, 2047 for Inf/NaN).
__device__ __forceinline__ int exp_field(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// Split x * 2^-(eref-1023) into (hi, lo) with integer operations only (no
// FP64 pipe).  hi keeps the leading 24 significant bits (truncated), lo the
// next 29 rounded to 24.  Values far below the scale (FP32 underflow) become
// zero, which is below 2^-126 relative to the block's largest magnitude.
__device__ __forceinline__ df split_scaled(double x, int eref) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int ef = (int)((b >> 52) & 0x7FF);
  const int fe = ef - eref + 127;  // FP32 biased exponent of the scaled value
  df r;
  if (ef == 0 || fe <= 0) {
    r.hi = 0.f;
    r.lo = 0.f;
    return r;
  }
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  r.hi = __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)(mant >> 29));
  const unsigned rem = (unsigned)(mant & 0x1FFFFFFFu);
  if (rem == 0) {
    r.lo = 0.f;
  } else {
    // rem * 2^(fe-127-52): scale the FP32 value of rem by adding to its exponent.
    const unsigned fb = __float_as_uint(__uint2float_rn(rem));
    const int e2 = (int)((fb >> 23) & 0xFF) + fe - 179;
    r.lo = (e2 > 0) ? __uint_as_float(sign | ((unsigned)e2 << 23) | (fb & 0x7FFFFFu)) : 0.f;
  }
  return r;
}

// Exact FP64 value of an FP32 number times 2^escale, by exponent arithmetic.
// Normal-range results only; otherwise falls back to an FP64 multiply.
__device__ __forceinline__ double f32_to_f64_scaled(float f, int escale) {
  const unsigned u = __float_as_uint(f);
  const int ef = (int)((u >> 23) & 0xFF);
  if (ef == 0) return 0.0;  // zero, or an FP32 subnormal (negligible at this scale)
  const int e = ef - 127 + 1023 + escale;
  if (e <= 0 || e >= 2047) return (double)f * exp2((double)escale);
  const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)e << 52) |
                               ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)b);
}

// Exact sum of two FP32 values: s + e == a + b (Knuth's two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// sum_j a[j]*v[j] in double-float.  Every product's high part is exact as
// (pr, pe) by FMA; the high parts are added by a pairwise tree of exact
// two-sums (depth log2(NN) instead of NN-1, the same operations), and the
// low parts, the two-sum errors and the cross terms a.hi*v.lo + a.lo*v.hi
// are summed in FP32 beside them.
template <int NN>
__device__ __forceinline__ df df_dot(const df* a, const df* v) {
  float pr[NN], c = 0.f;
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    pr[j] = __fmul_rn(a[j].hi, v[j].hi);
    float e = __fmaf_rn(a[j].hi, v[j].hi, -pr[j]);
    e = __fmaf_rn(a[j].hi, v[j].lo, e);
    e = __fmaf_rn(a[j].lo, v[j].hi, e);
    c = j == 0 ? e : __fadd_rn(c, e);
  }
#pragma unroll
  for (int w = 1; w < NN; w *= 2) {
#pragma unroll
    for (int j = 0; j + w < NN; j += 2 * w) {
      float s, e;
      two_sum(pr[j], pr[j + w], s, e);
      pr[j] = s;
      c = __fadd_rn(c, e);
    }
  }
  df r;
  r.hi = __fadd_rn(pr[0], c);
  r.lo = __fsub_rn(c, __fsub_rn(r.hi, pr[0]));
  return r;
}

// Running double-float sum of products of pairs.
struct DfSum {
  float s, c;
  __device__ __forceinline__ void zero() { s = c = 0.f; }
  __device__ __forceinline__ void add(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    float t, te;
    two_sum(s, p, t, te);
    s = t;
    c = __fadd_rn(c, __fadd_rn(te, e));
  }
  // the sum as a normalised pair
  __device__ __forceinline__ df pair() const {
    df r;
    r.hi = __fadd_rn(s, c);
    r.lo = __fsub_rn(c, __fsub_rn(r.hi, s));
    return r;
  }
  // the sum times 2^escale, in FP64
  __device__ __forceinline__ double widen(int escale) const {
    const df r = pair();
    return f32_to_f64_scaled(r.hi, escale) + f32_to_f64_scaled(r.lo, escale);
  }
};

// Same with a run-time length (generic path).
__device__ __forceinline__ df df_dot_rt(const df* a, int astride, const df* v, long long vstride,
                                        int nn) {
  float s = __fmul_rn(a[0].hi, v[0].hi);
  float c = __fmaf_rn(a[0].hi, v[0].hi, -s);
  c = __fmaf_rn(a[0].hi, v[0].lo, c);
  c = __fmaf_rn(a[0].lo, v[0].hi, c);
  for (int j = 1; j < nn; ++j) {
    const df aj = a[j * astride];
    const df vj = v[j * vstride];
    const float pr = __fmul_rn(aj.hi, vj.hi);
    const float pe = __fmaf_rn(aj.hi, vj.hi, -pr);
    const float t = __fadd_rn(s, pr);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(pr, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, pe));
    c = __fmaf_rn(aj.hi, vj.lo, c);
    c = __fmaf_rn(aj.lo, vj.hi, c);
  }
  df r;
  r.hi = __fadd_rn(s, c);
  r.lo = __fsub_rn(c, __fsub_rn(r.hi, s));
  return r;
}


// Factor rows of one mode: kept in registers when small enough (NN*NN
// values of S), otherwise read from shared memory at each use.
template <typename S, int NN>
struct Rows {
  static constexpr bool REG = (NN * NN * sizeof(S) <= 128);
  S r[REG ? NN * NN : 1];
  const S* s;
  __device__ __forceinline__ void load(const S* src) {
    s = src;
    if constexpr (REG) {
#pragma unroll
      for (int i = 0; i < NN * NN; ++i) r[i] = src[i];
    }
  }
  __device__ __forceinline__ const S* row(int a) const {
    if constexpr (REG) {
      return r + a * NN;
    } else {
      return s + a * NN;
    }
  }
};

// ---------------------------------------------------------------------------
// Dot products of the plain kernels.  RD == false: fused multiply-add in T.
// RD == true (FP32 data): every product exact as an FP32 pair, the pairs
// summed with error-free two-sums and the sum rounded once to FP32 -- what
// the reference's float kernels get by accumulating each dot product in
// double and rounding it when stored (kgemm_nt.hpp:557-571,
// kgemm_nn.hpp:688-701), to within about 2^-48 before that rounding.
// ---------------------------------------------------------------------------
template <typename T, bool RD>
struct DotAcc {
  T s;
  __device__ __forceinline__ void first(T a, T v) { s = a * v; }
  __device__ __forceinline__ void add(T a, T v) { s = fma(a, v, s); }
  __device__ __forceinline__ T get() const { return s; }
};
template <>
struct DotAcc<float, true> {
  float s, c;
  __device__ __forceinline__ void first(float a, float v) {
    s = __fmul_rn(a, v);
    c = __fmaf_rn(a, v, -s);
  }
  __device__ __forceinline__ void add(float a, float v) {
    const float p = __fmul_rn(a, v);
    const float e = __fmaf_rn(a, v, -p);
    float t, te;
    two_sum(s, p, t, te);
    s = t;
    c = __fadd_rn(c, __fadd_rn(te, e));
  }
  __device__ __forceinline__ float get() const { return __fadd_rn(s, c); }
};

// sum_j a[j] * v[j*vs], j < NN
template <typename T, bool RD, int NN>
__device__ __forceinline__ T dot_n(const T* a, const T* v, long long vs = 1) {
  DotAcc<T, RD> acc;
  acc.first(a[0], v[0]);
#pragma unroll
  for (int j = 1; j < NN; ++j) acc.add(a[j], v[(long long)j * vs]);
  return acc.get();
}
// run-time length nk
template <typename T, bool RD>
__device__ __forceinline__ T dot_rt(const T* a, const T* v, long long vs, int nk) {
  DotAcc<T, RD> acc;
  acc.first(a[0], v[0]);
  for (int j = 1; j < nk; ++j) acc.add(a[j], v[(long long)j * vs]);
  return acc.get();
}

// ---------------------------------------------------------------------------
// Plain form, square factors, compile-time n = NN.
// Shared memory per group: [d*NN*NN factor entries][N intermediates].
// With GBUF the intermediate lives in a global workspace instead.
// ---------------------------------------------------------------------------
template <typename T, int NN, bool GBUF, bool RD = false>
__device__ __forceinline__ void sq_plain_entry(const Problem& p, const EntryPtrs<T>& en, T* sA,
                                               T* buf, int lt, int G, int g) {
  constexpr int NN2 = NN * NN;
  const int d = p.d;
  const int N = (int)p.Nx;
  const int F = N / NN;  // fibers per mode
  for (int i = lt; i < d * NN2; i += G) {
    const int l = i / NN2, r = i - l * NN2, a = r / NN, j = r - a * NN;
    const T* Al = en.A[l];
    sA[i] = p.trans ? Al[j + (long long)a * en.ld[l]] : Al[a + (long long)j * en.ld[l]];
  }
  group_sync(g, G);
  const bool excl = p.y_exclusive != 0;
  if (d == 1) {
    for (int i = lt; i < NN; i += G) {
      T xv[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) xv[j] = __ldg(en.X + j);
      y_accumulate(en.Y + i, dot_n<T, RD, NN>(sA + i * NN, xv), excl);
    }
    return;
  }
  // mode 0: X (HBM) -> buf.  Fibers f = 0..F-1 at stride F.
  {
    Rows<T, NN> a;
    a.load(sA);
    for (int f = lt; f < F; f += G) {
      T v[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) v[j] = __ldg(en.X + (long long)j * F + f);
#pragma unroll
      for (int r = 0; r < NN; ++r) buf[(long long)r * F + f] = dot_n<T, RD, NN>(a.row(r), v);
    }
  }
  group_sync(g, G);
  // modes 1..d-2 in place
  int s = F / NN;
  for (int k = 1; k < d - 1; ++k, s /= NN) {
    Rows<T, NN> a;
    a.load(sA + k * NN2);
    const FastDiv fd((unsigned)s);
    for (int f = lt; f < F; f += G) {
      const unsigned o = fd((unsigned)f);
      const int r0 = f - (int)o * s;
      T* base = buf + (long long)o * NN * s + r0;
      T v[NN];
#pragma unroll
      for (int j = 0; j < NN; ++j) v[j] = base[(long long)j * s];
#pragma unroll
      for (int r = 0; r < NN; ++r) base[(long long)r * s] = dot_n<T, RD, NN>(a.row(r), v);
    }
    group_sync(g, G);
  }
  // last mode: buf -> Y, one output per lane (consecutive lanes, consecutive Y)
  {
    const T* Ad = sA + (d - 1) * NN2;
    for (int i = lt; i < N; i += G) {
      const int f = i / NN, r = i - f * NN;
      const T* v = buf + (long long)f * NN;
      y_accumulate(en.Y + i, dot_n<T, RD, NN>(Ad + r * NN, v), excl);
    }
  }
}

template <typename T, int NN, bool GBUF, bool RD = false>
__global__ void __launch_bounds__(MAX_THREADS) sq_plain_kernel(const Problem p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = p.group_threads;
  const int E = p.groups_per_cta;
  const int g = threadIdx.x / G;
  const int lt = threadIdx.x - g * G;
  if (g >= E) return;
  constexpr int NN2 = NN * NN;
  T* sA = reinterpret_cast<T*>(smem + (size_t)g * p.group_smem);
  T* sbuf = sA + ((MAXD * NN2 * sizeof(T) + 15) / 16 * 16) / sizeof(T);
  const long long slot0 = (long long)blockIdx.x * E + g;
  const long long step = (long long)gridDim.x * E;
  const long long count = launch_count(p);
  const long long obase = p.order_base ? (long long)*p.order_base : 0;
  for (long long e = slot0; e < count; e += step) {
    const long long entry = p.order ? (long long)p.order[obase + e] : e + p.entry_offset;
    EntryPtrs<T> en;
    if (!resolve_entry<T>(p, entry, en)) {
      if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    T* buf = sbuf;
    if (GBUF) {
      T* w1;
      if (!workspace<T>(p, entry, slot0, buf, w1)) {
        if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
        continue;
      }
    }
    sq_plain_entry<T, NN, GBUF, RD>(p, en, sA, buf, lt, G, g);
    group_sync(g, G);
  }
}

// ---------------------------------------------------------------------------
// Split (double-float) form, square factors, compile-time NN.  Same data flow
// as the plain form; the shared intermediate holds (hi, lo) pairs.  An entry
// whose inputs hold Inf/NaN is evaluated by the plain FP64 code instead.
// With the intermediate in the global workspace (GBUF: entries of 16K+
// elements, groups of 512 threads) the kernel waits on L2 and needs two CTAs
// per SM, so for n <= 8 it is held to 64 registers (measured on GB300, d=6
// n=8: 2321 GFLOP/s at 64 registers against 1963 at the 116 the compiler
// otherwise takes); a minimum of 0 CTAs leaves the on-chip variants' register
// choice to the compiler.
// ---------------------------------------------------------------------------
// Shared-memory head of the split per-mode kernels: d*NN*NN factor pairs,
// MAXD+2 exponent ints, 2 x (MAXD+2) cancellation-guard sums.
__host__ __device__ constexpr size_t sq_split_head(int nn) {
  return ((size_t)MAXD * nn * nn * 8 + (MAXD + 2) * 4 + 2 * (MAXD + 2) * 4 + 15) / 16 * 16;
}

template <int NN, bool GBUF>
__global__ void __launch_bounds__(MAX_THREADS, (GBUF && NN <= 8) ? 2 : 0) sq_split_kernel(const Problem p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = p.group_threads;
  const int E = p.groups_per_cta;
  const int g = threadIdx.x / G;
  const int lt = threadIdx.x - g * G;
  if (g >= E) return;
  constexpr int NN2 = NN * NN;
  const int d = p.d;
  const int N = (int)p.Nx;
  const int F = N / NN;
  unsigned char* gbase = smem + (size_t)g * p.group_smem;
  df* sA = reinterpret_cast<df*>(gbase);                        // d*NN2 pairs
  int* sExp = reinterpret_cast<int*>(gbase + MAXD * NN2 * sizeof(df));  // MAXD+2 ints
  float* sNrm0 = reinterpret_cast<float*>(sExp + MAXD + 2);     // [2][MAXD+2] guard sums
  unsigned char* sbuf_raw = gbase + sq_split_head(NN);
  const long long slot0 = (long long)blockIdx.x * E + g;
  const long long step = (long long)gridDim.x * E;
  const bool excl = p.y_exclusive != 0;
  const long long count = launch_count(p);
  const long long obase = p.order_base ? (long long)*p.order_base : 0;
  int par = 0;  // guard sums alternate between two slots (entry parity)
  for (long long e = slot0; e < count; e += step) {
    const long long entry = p.order ? (long long)p.order[obase + e] : e + p.entry_offset;
    EntryPtrs<double> en;
    if (!resolve_entry<double>(p, entry, en)) {
      if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    unsigned char* bufp = sbuf_raw;
    if (GBUF) {
      double *w0, *w1;
      if (!workspace<double>(p, entry, slot0, w0, w1)) {
        if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
        continue;
      }
      bufp = reinterpret_cast<unsigned char*>(w0);
    }
    df* buf = reinterpret_cast<df*>(bufp);
    // --- scales: max exponent field per factor and of X ---
    float* sNrm = sNrm0 + par * (MAXD + 2);
    par ^= 1;
    if (lt < MAXD + 2) {
      sExp[lt] = 0;
      sNrm[lt] = 0.f;
    }
    group_sync(g, G);
    {
      int emax[MAXD];
#pragma unroll
      for (int l = 0; l < MAXD; ++l) emax[l] = 0;
      for (int i = lt; i < d * NN2; i += G) {
        const int l = i / NN2, r = i - l * NN2, a = r / NN, j = r - a * NN;
        const double* Al = en.A[l];
        const double v = p.trans ? Al[j + (long long)a * en.ld[l]] : Al[a + (long long)j * en.ld[l]];
        const int ef = exp_field(v);
#pragma unroll
        for (int q = 0; q < MAXD; ++q)
          if (q == l) emax[q] = max(emax[q], ef);
      }
      int ex = 0;
      for (int i = lt; i < N; i += G) ex = max(ex, exp_field(__ldg(en.X + i)));
      // one shared atomic per warp (groups are whole warps)
#pragma unroll
      for (int l = 0; l < MAXD; ++l) {
        if (l < d) {
          const int m = __reduce_max_sync(0xffffffffu, emax[l]);
          if ((lt & 31) == 0 && m > 0) atomicMax(&sExp[l], m);
        }
      }
      ex = __reduce_max_sync(0xffffffffu, ex);
      if ((lt & 31) == 0 && ex > 0) atomicMax(&sExp[MAXD], ex);
    }
    group_sync(g, G);
    int nonfinite = (sExp[MAXD] == 2047);
    int escale = sExp[MAXD] - 1023;
    for (int l = 0; l < d; ++l) {
      nonfinite |= (sExp[l] == 2047);
      escale += sExp[l] - 1023;
    }
    const bool zero_block = (sExp[MAXD] == 0);
    bool anyzero = zero_block;
    for (int l = 0; l < d; ++l) anyzero = anyzero || (sExp[l] == 0);
    if (nonfinite) {
      // Inf/NaN must propagate exactly as in FP64 (0 * Inf included): evaluate
      // with the plain form on the same (double-sized) buffer.
      double* sAd = reinterpret_cast<double*>(gbase);
      sq_plain_entry<double, NN, GBUF>(p, en, sAd, reinterpret_cast<double*>(bufp), lt, G, g);
      group_sync(g, G);
      continue;
    }
    if (anyzero) {
      // kron(...) X is exactly zero: nothing to add.
      group_sync(g, G);
      continue;
    }
    // --- factors, scaled and split (warp-uniform trip count: the norm
    // sums run over whole warps) ---
    for (int i0 = 0; i0 < d * NN2; i0 += G) {
      const int i = i0 + lt;
      const bool own = i < d * NN2;
      const int l = own ? i / NN2 : 0;
      float sq = 0.f;
      if (own) {
        const int r = i - l * NN2, a = r / NN, j = r - a * NN;
        const double* Al = en.A[l];
        const double v = p.trans ? Al[j + (long long)a * en.ld[l]] : Al[a + (long long)j * en.ld[l]];
        const df s = split_scaled(v, sExp[l]);
        sA[i] = s;
        sq = s.hi * s.hi;
      }
      warp_run_add(sNrm, l, sq, own);
    }
    const int ex = sExp[MAXD];
    group_sync(g, G);
    float gsum = 0.f;  // guard: this thread's part of ||X||^2, then of ||KX||^2
    // The last mode (d == 1: the only one), adding sign * its contribution to Y.
    auto last_mode = [&](bool neg, bool norm) {
      if (d == 1) {
        for (int i = lt; i < NN; i += G) {
          df v[NN];
#pragma unroll
          for (int j = 0; j < NN; ++j) v[j] = split_scaled(__ldg(en.X + j), ex);
          const df o = df_dot<NN>(sA + i * NN, v);
          if (norm) gsum = __fmaf_rn(o.hi, o.hi, gsum);
          const double y = f32_to_f64_scaled(o.hi, escale) + f32_to_f64_scaled(o.lo, escale);
          y_accumulate(en.Y + i, neg ? -y : y, excl);
        }
        return;
      }
      const df* Ad = sA + (d - 1) * NN2;
      for (int i = lt; i < N; i += G) {
        const int f = i / NN, r = i - f * NN;
        df v[NN], a[NN];
#pragma unroll
        for (int j = 0; j < NN; ++j) {
          v[j] = buf[(long long)f * NN + j];
          a[j] = Ad[r * NN + j];
        }
        const df o = df_dot<NN>(a, v);
        if (norm) gsum = __fmaf_rn(o.hi, o.hi, gsum);
        const double y = f32_to_f64_scaled(o.hi, escale) + f32_to_f64_scaled(o.lo, escale);
        y_accumulate(en.Y + i, neg ? -y : y, excl);
      }
    };
    if (d == 1) {
      if (lt < NN) {
        const df x = split_scaled(__ldg(en.X + lt), ex);
        gsum = x.hi * x.hi;
      }
    } else {
      // mode 0: X (HBM) -> buf
      {
        Rows<df, NN> a;
        a.load(sA);
        for (int f = lt; f < F; f += G) {
          df v[NN];
#pragma unroll
          for (int j = 0; j < NN; ++j) {
            v[j] = split_scaled(__ldg(en.X + (long long)j * F + f), ex);
            gsum = __fmaf_rn(v[j].hi, v[j].hi, gsum);
          }
#pragma unroll
          for (int r = 0; r < NN; ++r) buf[(long long)r * F + f] = df_dot<NN>(a.row(r), v);
        }
      }
    }
    gsum = warp_sum(gsum);
    if ((lt & 31) == 0) atomicAdd(&sNrm[MAXD], gsum);
    gsum = 0.f;
    if (d == 1) {
      last_mode(false, true);
    } else {
    group_sync(g, G);
    int s = F / NN;
    for (int k = 1; k < d - 1; ++k, s /= NN) {
      Rows<df, NN> a;
      a.load(sA + k * NN2);
      const FastDiv fd((unsigned)s);
      for (int f = lt; f < F; f += G) {
        const unsigned o = fd((unsigned)f);
        const int r0 = f - (int)o * s;
        df* base = buf + (long long)o * NN * s + r0;
        df v[NN];
#pragma unroll
        for (int j = 0; j < NN; ++j) v[j] = base[(long long)j * s];
#pragma unroll
        for (int r = 0; r < NN; ++r) base[(long long)r * s] = df_dot<NN>(a.row(r), v);
      }
      group_sync(g, G);
    }
    last_mode(false, true);
    }
    gsum = warp_sum(gsum);
    if ((lt & 31) == 0) atomicAdd(&sNrm[MAXD + 1], gsum);
    group_sync(g, G);
    // cancellation guard (uniform over the group): take the contribution back
    // (the intermediate is unchanged, the same arithmetic gives the same
    // values) and add the plain FP64 result instead
    if (!p.guard_off && guard_fails(sNrm[MAXD + 1], sNrm[MAXD], sNrm, d, N)) {
      last_mode(true, false);
      group_sync(g, G);
      sq_plain_entry<double, NN, GBUF>(p, en, reinterpret_cast<double*>(gbase),
                                       reinterpret_cast<double*>(bufp), lt, G, g);
      if (lt == 0) count_redo(p.redo_ctr, 0);
      group_sync(g, G);
    }
  }
}

// ---------------------------------------------------------------------------
// Generic path: run-time shapes (rectangular, or n without a compile-time
// specialisation), plain form.  Square modes update the intermediate in
// place (a lane owns whole fibers; n <= GEN_MAXN); a rectangular mode writes
// the other of two buffers (sxw elements each).  Buffers are in shared
// memory, or in the global workspace with GBUF.
// Shared memory per group: [sum_l m_l*n_l factor entries][sxw][sxw if rectangular].
// ---------------------------------------------------------------------------
constexpr int GEN_MAXN = 64;

// One entry of the generic plain kernel (also the Inf/NaN fallback of the
// generic split kernel): factors into sA, modes through b0/b1, Y += result.
template <typename T, bool RD = false>
__device__ __forceinline__ void gen_plain_entry(const Problem& p, const EntryPtrs<T>& en, T* sA,
                                                T* b0, T* b1, int lt, int G, int g) {
  const int d = p.d;
  int aoff[MAXD + 1];
  aoff[0] = 0;
#pragma unroll
  for (int l = 0; l < MAXD; ++l) aoff[l + 1] = aoff[l] + (l < d ? p.m[l] * p.n[l] : 0);
  const bool excl = p.y_exclusive != 0;
  for (int l = 0; l < d; ++l) {
    const int ml = p.m[l], nl = p.n[l];
    for (int i = lt; i < ml * nl; i += G) {
      const int a = i / nl, j = i - a * nl;
      sA[aoff[l] + i] = p.trans ? en.A[l][j + (long long)a * en.ld[l]]
                                : en.A[l][a + (long long)j * en.ld[l]];
    }
  }
  group_sync(g, G);
  const T* src = en.X;
  T* cur = b0;
  unsigned outer = 1;
  for (int k = 0; k < d; ++k) {
    unsigned s = 1;
    for (int l = k + 1; l < d; ++l) s *= (unsigned)p.n[l];
    const int mk = p.m[k], nk = p.n[k];
    const T* Ak = sA + aoff[k];
    const bool last = (k == d - 1);
    if (!last && k > 0 && mk == nk) {
      // square middle mode: in place on cur, one fiber per lane
      const FastDiv fs(s);
      const unsigned F = outer * s;
      for (unsigned f = lt; f < F; f += G) {
        const unsigned o = fs(f);
        const unsigned r0 = f - o * s;
        T* base = cur + (long long)o * nk * s + r0;
        T v[GEN_MAXN];
        for (int j = 0; j < nk; ++j) v[j] = base[(long long)j * s];
        for (int a = 0; a < mk; ++a) base[(long long)a * s] = dot_rt<T, RD>(Ak + a * nk, v, 1, nk);
      }
    } else {
      // out of place: one output element per lane
      T* dst = last ? en.Y : ((k == 0) ? cur : (cur == b0 ? b1 : b0));
      const FastDiv fs(s), fm((unsigned)mk);
      const unsigned total = outer * (unsigned)mk * s;
      for (unsigned q = lt; q < total; q += G) {
        const unsigned t = fs(q);
        const unsigned rr = q - t * s;
        const unsigned o = fm(t);
        const int a = (int)(t - o * (unsigned)mk);
        const T* v = src + (long long)o * nk * s + rr;
        const T acc = dot_rt<T, RD>(Ak + a * nk, v, s, nk);
        if (last) {
          y_accumulate(dst + q, acc, excl);
        } else {
          dst[q] = acc;
        }
      }
      if (!last) cur = dst;
    }
    group_sync(g, G);
    src = cur;
    outer *= (unsigned)mk;
  }
}

template <typename T, bool GBUF, bool RD = false>
__global__ void __launch_bounds__(MAX_THREADS) gen_plain_kernel(const Problem p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = p.group_threads;
  const int E = p.groups_per_cta;
  const int g = threadIdx.x / G;
  const int lt = threadIdx.x - g * G;
  if (g >= E) return;
  const int d = p.d;
  int nfac = 0;
  for (int l = 0; l < d; ++l) nfac += p.m[l] * p.n[l];
  T* sA = reinterpret_cast<T*>(smem + (size_t)g * p.group_smem);
  T* sb0 = sA + ((nfac * sizeof(T) + 15) / 16 * 16) / sizeof(T);
  T* sb1 = sb0 + ((p.sxw * sizeof(T) + 15) / 16 * 16) / sizeof(T);
  const long long slot0 = (long long)blockIdx.x * E + g;
  const long long step = (long long)gridDim.x * E;
  EntryStream es(p, slot0, step);
  for (long long entry; es.next(p, entry);) {
    EntryPtrs<T> en;
    if (!resolve_entry<T>(p, entry, en)) {
      if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    T* b0 = sb0;
    T* b1 = sb1;
    if (GBUF) {
      if (!workspace<T>(p, entry, slot0, b0, b1)) {
        if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
        continue;
      }
    }
    gen_plain_entry<T, RD>(p, en, sA, b0, b1, lt, G, g);
  }
}

// ---------------------------------------------------------------------------
// Generic path, split form: run-time (and rectangular) shapes in double-float,
// the same mode structure as gen_plain_kernel.  X is split into the first
// buffer (scaled by its block exponent), every factor by its own exponent and
// stored transposed (column j of A_l contiguous), so the R rows one lane
// accumulates are adjacent.  With two buffers every mode runs out of place: a
// lane owns R outputs of one fiber (R independent two-sum chains sharing each
// input load; the launcher picks R = 4 for large entries and R = 2 for small
// ones, where the extra registers cost more occupancy than they win).  With
// one buffer (an entry too large for two on chip, or a large one whose modes
// but the last are all square with n <= GEN_SPLIT_MAXN) those modes run in
// place, the lane holding its fiber.  The last mode widens to FP64 and adds
// to Y.  Entries with Inf/NaN run the plain entry.
// Shared memory per group: [factors as pairs][MAXD+2 exponents, 2 x (MAXD+2)
// guard sums: GEN_SPLIT_HDR bytes][sxw pairs][sxw pairs when two buffers]
// (buffers in the workspace with GBUF).
// ---------------------------------------------------------------------------
constexpr int GEN_SPLIT_MAXN = 16;
constexpr int GEN_SPLIT_HDR = 128;

// A mode the generic split kernel can apply in place.
__host__ __device__ inline bool gen_split_in_place(int m, int n) {
  return m == n && n <= GEN_SPLIT_MAXN;
}

// R running double-float dot products sharing one input value per term.
template <int R>
struct DfRows {
  float s[R], c[R];
  __device__ __forceinline__ void first(const df* a, df v) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      s[r] = __fmul_rn(a[r].hi, v.hi);
      float e = __fmaf_rn(a[r].hi, v.hi, -s[r]);
      e = __fmaf_rn(a[r].hi, v.lo, e);
      c[r] = __fmaf_rn(a[r].lo, v.hi, e);
    }
  }
  __device__ __forceinline__ void add(const df* a, df v) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float pr = __fmul_rn(a[r].hi, v.hi);
      float e = __fmaf_rn(a[r].hi, v.hi, -pr);
      e = __fmaf_rn(a[r].hi, v.lo, e);
      e = __fmaf_rn(a[r].lo, v.hi, e);
      float t, te;
      two_sum(s[r], pr, t, te);
      s[r] = t;
      c[r] = __fadd_rn(c[r], __fadd_rn(te, e));
    }
  }
  __device__ __forceinline__ df get(int r) const {
    df o;
    o.hi = __fadd_rn(s[r], c[r]);
    o.lo = __fsub_rn(c[r], __fsub_rn(o.hi, s[r]));
    return o;
  }
};

// One entry of the generic double-float kernel (shape from p, which may be
// a per-entry copy): scales, split, the d modes, the cancellation guard.
// gbase: the group's shared memory (factors, exponents); w0/w1: its buffers
// (shared memory, or the global workspace); two: both buffers usable.
template <int R>
__device__ __forceinline__ void gen_split_entry(const Problem& p, const EntryPtrs<double>& en,
                                                unsigned char* gbase, double* w0, double* w1,
                                                int* sExp, float* sNrm, bool two, int lt, int G,
                                                int g) {
  const int d = p.d;
  int aoff[MAXD + 1];
  aoff[0] = 0;
#pragma unroll
  for (int l = 0; l < MAXD; ++l) aoff[l + 1] = aoff[l] + (l < d ? p.m[l] * p.n[l] : 0);
  df* sA = reinterpret_cast<df*>(gbase);
  const bool excl = p.y_exclusive != 0;
  const long long Nx = p.Nx;
  // --- scales: max exponent field per factor and of X ---
  if (lt < MAXD + 2) {
    sExp[lt] = 0;
    sNrm[lt] = 0.f;
  }
  group_sync(g, G);
  for (int l = 0; l < d; ++l) {
    const int ml = p.m[l], nl = p.n[l];
    int em = 0;
    for (int i = lt; i < ml * nl; i += G) {
      const int a = i / nl, j = i - a * nl;
      em = max(em, exp_field(p.trans ? en.A[l][j + (long long)a * en.ld[l]]
                                     : en.A[l][a + (long long)j * en.ld[l]]));
    }
    em = __reduce_max_sync(0xffffffffu, em);  // one shared atomic per warp
    if ((lt & 31) == 0 && em > 0) atomicMax(&sExp[l], em);
  }
  {
    int ex = 0;
    for (long long i = lt; i < Nx; i += G) ex = max(ex, exp_field(__ldg(en.X + i)));
    ex = __reduce_max_sync(0xffffffffu, ex);
    if ((lt & 31) == 0 && ex > 0) atomicMax(&sExp[MAXD], ex);
  }
  group_sync(g, G);
  int nonfinite = (sExp[MAXD] == 2047);
  int escale = sExp[MAXD] - 1023;
  bool anyzero = sExp[MAXD] == 0;
  for (int l = 0; l < d; ++l) {
    nonfinite |= (sExp[l] == 2047);
    escale += sExp[l] - 1023;
    anyzero = anyzero || sExp[l] == 0;
  }
  if (nonfinite) {
    // Inf/NaN propagate exactly as in FP64 (0 * Inf included): the plain
    // entry on the same memory
    gen_plain_entry<double>(p, en, reinterpret_cast<double*>(gbase), w0, w1, lt, G, g);
    group_sync(g, G);
    return;
  }
  if (anyzero) {  // kron(...) X is exactly zero
    group_sync(g, G);
    return;
  }
  // --- factors (transposed: sA[aoff[l] + j*m_l + a] = A_l(a, j)) and X, split ---
  for (int l = 0; l < d; ++l) {
    const int ml = p.m[l], nl = p.n[l];
    float an = 0.f;
    for (int i = lt; i < ml * nl; i += G) {
      const int j = i / ml, a = i - j * ml;
      const df s = split_scaled(p.trans ? en.A[l][j + (long long)a * en.ld[l]]
                                        : en.A[l][a + (long long)j * en.ld[l]],
                                sExp[l]);
      sA[aoff[l] + i] = s;
      an = __fmaf_rn(s.hi, s.hi, an);
    }
    an = warp_sum(an);
    if ((lt & 31) == 0) atomicAdd(&sNrm[l], an);
  }
  df* b0 = reinterpret_cast<df*>(w0);
  df* b1 = reinterpret_cast<df*>(w1);
  const int ex = sExp[MAXD];
  float gsum = 0.f;  // guard: this thread's part of ||X||^2, then of ||KX||^2
  for (long long i = lt; i < Nx; i += G) {
    const df s = split_scaled(__ldg(en.X + i), ex);
    b0[i] = s;
    gsum = __fmaf_rn(s.hi, s.hi, gsum);
  }
  gsum = warp_sum(gsum);
  if ((lt & 31) == 0) atomicAdd(&sNrm[MAXD], gsum);
  gsum = 0.f;
  group_sync(g, G);
  // Out of place: a lane owns rows a0..a0+R-1 of one fiber of mode k.  The
  // last mode (dst == nullptr) adds its outputs to Y, or subtracts them (neg).
  auto out_of_place = [&](int k, unsigned outer, const df* src, df* dst, bool neg) {
    unsigned s = 1;
    for (int l = k + 1; l < d; ++l) s *= (unsigned)p.n[l];
    const int mk = p.m[k], nk = p.n[k];
    const df* At = sA + aoff[k];
    const int nb = (mk + R - 1) / R;
    const FastDiv fs(s), fb((unsigned)nb);
    const unsigned total = outer * (unsigned)nb * s;
    for (unsigned q = lt; q < total; q += G) {
      const unsigned t = fs(q);
      const unsigned rr = q - t * s;
      const unsigned o = fb(t);
      const int a0 = (int)(t - o * (unsigned)nb) * R;
      const df* v = src + (long long)o * nk * s + rr;
      df av[R];
      DfRows<R> acc;
#pragma unroll
      for (int r = 0; r < R; ++r) av[r] = At[min(a0 + r, mk - 1)];
      acc.first(av, v[0]);
      for (int j = 1; j < nk; ++j) {
#pragma unroll
        for (int r = 0; r < R; ++r) av[r] = At[j * mk + min(a0 + r, mk - 1)];
        acc.add(av, v[(long long)j * s]);
      }
      const long long obase_q = ((long long)o * mk + a0) * s + rr;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (a0 + r < mk) {
          const df o2 = acc.get(r);
          if (dst == nullptr) {
            if (!neg) gsum = __fmaf_rn(o2.hi, o2.hi, gsum);
            const double y =
                f32_to_f64_scaled(o2.hi, escale) + f32_to_f64_scaled(o2.lo, escale);
            y_accumulate(en.Y + obase_q + (long long)r * s, neg ? -y : y, excl);
          } else {
            dst[obase_q + (long long)r * s] = o2;
          }
        }
      }
    }
  };
  df* cur = b0;
  unsigned outer = 1, outer_last = 1;
  for (int k = 0; k < d; ++k) {
    unsigned s = 1;
    for (int l = k + 1; l < d; ++l) s *= (unsigned)p.n[l];
    const int mk = p.m[k], nk = p.n[k];
    const df* At = sA + aoff[k];
    const bool last = (k == d - 1);
    const int nb = (mk + R - 1) / R;
    if (!last && !two && gen_split_in_place(mk, nk)) {
      // one buffer: in place on cur, one fiber per lane
      const FastDiv fs(s);
      const unsigned F = outer * s;
      for (unsigned f = lt; f < F; f += G) {
        const unsigned o = fs(f);
        const unsigned r0 = f - o * s;
        df* base = cur + (long long)o * nk * s + r0;
        df v[GEN_SPLIT_MAXN];
        for (int j = 0; j < nk; ++j) v[j] = base[(long long)j * s];
        for (int ab = 0; ab < nb; ++ab) {
          const int a0 = ab * R;
          df av[R];
          DfRows<R> acc;
#pragma unroll
          for (int r = 0; r < R; ++r) av[r] = At[min(a0 + r, mk - 1)];
          acc.first(av, v[0]);
          for (int j = 1; j < nk; ++j) {
#pragma unroll
            for (int r = 0; r < R; ++r) av[r] = At[j * mk + min(a0 + r, mk - 1)];
            acc.add(av, v[j]);
          }
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (a0 + r < mk) base[(long long)(a0 + r) * s] = acc.get(r);
        }
      }
    } else {
      df* dst = last ? nullptr : (cur == b0 ? b1 : b0);
      if (last) outer_last = outer;
      out_of_place(k, outer, cur, dst, false);
      if (!last) cur = dst;
    }
    group_sync(g, G);
    outer *= (unsigned)mk;
  }
  gsum = warp_sum(gsum);
  if ((lt & 31) == 0) atomicAdd(&sNrm[MAXD + 1], gsum);
  group_sync(g, G);
  // cancellation guard (uniform over the group): take the contribution back
  // (the last mode leaves its input unchanged, the same arithmetic gives the
  // same values) and add the plain FP64 result instead
  if (!p.guard_off && guard_fails(sNrm[MAXD + 1], sNrm[MAXD], sNrm, d, Nx)) {
    out_of_place(d - 1, outer_last, cur, nullptr, true);
    group_sync(g, G);
    gen_plain_entry<double>(p, en, reinterpret_cast<double*>(gbase), w0, w1, lt, G, g);
    if (lt == 0) count_redo(p.redo_ctr, 0);
  }
}

template <bool GBUF, int R>
__global__ void __launch_bounds__(MAX_THREADS) gen_split_kernel(const Problem p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = p.group_threads;
  const int E = p.groups_per_cta;
  const int g = threadIdx.x / G;
  const int lt = threadIdx.x - g * G;
  if (g >= E) return;
  const int d = p.d;
  int aoff[MAXD + 1];
  aoff[0] = 0;
#pragma unroll
  for (int l = 0; l < MAXD; ++l) aoff[l + 1] = aoff[l] + (l < d ? p.m[l] * p.n[l] : 0);
  unsigned char* gbase = smem + (size_t)g * p.group_smem;
  const size_t fac_bytes = ((size_t)aoff[d] * 8 + 15) / 16 * 16;
  int* sExp = reinterpret_cast<int*>(gbase + fac_bytes);  // MAXD + 2 ints
  float* sNrm0 = reinterpret_cast<float*>(sExp + MAXD + 2);  // [2][MAXD + 2] guard sums
  unsigned char* braw = gbase + fac_bytes + GEN_SPLIT_HDR;
  const size_t bbytes = ((size_t)p.sxw * 8 + 15) / 16 * 16;
  const bool two = GBUF || (size_t)p.group_smem >= fac_bytes + GEN_SPLIT_HDR + 2 * bbytes;
  const long long slot0 = (long long)blockIdx.x * E + g;
  const long long step = (long long)gridDim.x * E;
  int par = 0;  // guard sums alternate between two slots (entry parity)
  EntryStream es(p, slot0, step);
  for (long long entry; es.next(p, entry);) {
    EntryPtrs<double> en;
    if (!resolve_entry<double>(p, entry, en)) {
      if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
      continue;
    }
    float* sNrm = sNrm0 + par * (MAXD + 2);
    par ^= 1;
    double *w0 = reinterpret_cast<double*>(braw), *w1 = reinterpret_cast<double*>(braw + bbytes);
    if (GBUF) {
      if (!workspace<double>(p, entry, slot0, w0, w1)) {
        if (lt == 0) atomicOr(p.status, DF_NULL_PTR);
        continue;
      }
    }
    gen_split_entry<R>(p, en, gbase, w0, w1, sExp, sNrm, two, lt, G, g);
  }
}

}  // namespace kmx
