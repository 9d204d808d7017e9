/*
 * kron_oracle.c -- CPU oracle for the batched Kronecker mat-vec.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark load it.  The CUDA
 * product path never links, loads or calls it.
 *
 * It restates, in plain C with OpenMP, the algorithm of hipdac-lab/kronmult:
 *
 *   Y(:,k) += kron(A1(:,:,k), ..., Ad(:,:,k)) * X(:,k)
 *
 * evaluated by the "tail-recursive reshape" of kronmultv.hpp:19-148:
 *   W_i(n2..nd x m1) = X_i(n2..nd x n1) * transpose(A1)   (kgemm_nt, beta=0)
 *   recurse on d-1 factors with nvec*m1 vectors, X and W swapped
 *   base case: Y(m1 x nvec) += A1 * X(n1 x nvec)          (kgemm_nn, beta=1)
 *
 * Every dot product is a plain sum over k = 0..kk-1 starting from zero, in
 * the same order as kgemm_nt_v1 / kgemm_nn_v1 (kgemm_nt.hpp:330-357,
 * kgemm_nn.hpp:340-384).  Build with -ffp-contract=off so that no multiply
 * and add are fused; the results are then bit-identical to the reference's
 * CPU build on x86-64, where g++ emits no FMA by default.
 *
 * FP32 storage follows the reference's float specialisation: each dot
 * product accumulates in double and is rounded to float when stored
 * (kgemm_nt.hpp:557-571, kgemm_nn.hpp:688-701, kronmultv.hpp:200-238).
 *
 * Overlapping Y blocks are accumulated with an OpenMP atomic update, as the
 * reference's CPU atomicAdd does (kroncommon.hpp:38-64).
 */
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KMO_MAXD 6

/* ------------------------------------------------------------------ */
/* Tiny GEMMs of the reference, restated.                             */
/* ------------------------------------------------------------------ */

/* C(mm x nn) = A(mm x kk) * transpose(B(nn x kk)), beta = 0.
 * kgemm_nt.hpp:541-555 with beta == 0 (store path kgemm_nt.hpp:371-379). */
static void gemm_nt_f64(int mm, int nn, int kk, const double* A, int ldA,
                        const double* B, int ldB, double* C, int ldC) {
  for (int j = 0; j < nn; ++j)
    for (int i = 0; i < mm; ++i) {
      double c = 0;
      for (int k = 0; k < kk; ++k) c += A[i + (size_t)k * ldA] * B[j + (size_t)k * ldB];
      C[i + (size_t)j * ldC] = c;
    }
}

/* C(mm x nn) += A(mm x kk) * B(kk x nn), beta = 1 -> atomic accumulate.
 * kgemm_nn.hpp:669-682, atomic epilogue kgemm_nn.hpp:392-400. */
static void gemm_nn_acc_f64(int mm, int nn, int kk, const double* A, int ldA,
                            const double* B, int ldB, double* C, int ldC) {
  for (int j = 0; j < nn; ++j)
    for (int i = 0; i < mm; ++i) {
      double c = 0;
      for (int k = 0; k < kk; ++k) c += A[i + (size_t)k * ldA] * B[k + (size_t)j * ldB];
      double* p = &C[i + (size_t)j * ldC];
#pragma omp atomic update
      *p += c;
    }
}

static void gemm_nt_f32(int mm, int nn, int kk, const float* A, int ldA,
                        const float* B, int ldB, float* C, int ldC) {
  for (int j = 0; j < nn; ++j)
    for (int i = 0; i < mm; ++i) {
      double c = 0;
      for (int k = 0; k < kk; ++k) c += (double)A[i + (size_t)k * ldA] * (double)B[j + (size_t)k * ldB];
      C[i + (size_t)j * ldC] = (float)c;
    }
}

static void gemm_nn_acc_f32(int mm, int nn, int kk, const float* A, int ldA,
                            const float* B, int ldB, float* C, int ldC) {
  for (int j = 0; j < nn; ++j)
    for (int i = 0; i < mm; ++i) {
      double c = 0;
      for (int k = 0; k < kk; ++k) c += (double)A[i + (size_t)k * ldA] * (double)B[k + (size_t)j * ldB];
      float* p = &C[i + (size_t)j * ldC];
      float v = (float)c;
#pragma omp atomic update
      *p += v;
    }
}

/* ------------------------------------------------------------------ */
/* The recursion of kronmultv.hpp:19-148 (rectangular factors).        */
/* m[l] x n[l] is factor l, ld[l] its leading dimension.               */
/* X holds nvec vectors of length n[0]*...*n[d-1]; it is clobbered as  */
/* workspace when d >= 3, exactly as in the reference.                 */
/* ------------------------------------------------------------------ */
#define DEFINE_KRONMULTV(SUF, T)                                                        \
  static void kronmultv_##SUF(int d, const int* m, const int* n, const T* const* A,     \
                              const int* ld, int nvec, T* X, T* Y, T* W) {              \
    if (d == 1) {                                                                       \
      /* kronmultv.hpp:152-195: Y(m1 x nvec) += A1 * X(n1 x nvec) */                    \
      gemm_nn_acc_##SUF(m[0], nvec, n[0], A[0], ld[0], X, n[0], Y, m[0]);               \
      return;                                                                           \
    }                                                                                   \
    size_t n26 = 1;                                                                     \
    for (int l = 1; l < d; ++l) n26 *= (size_t)n[l];                                    \
    size_t ldX = n26 * (size_t)n[0], ldW = n26 * (size_t)m[0];                          \
    /* kronmultv.hpp:82-128: W_i = X_i * transpose(A1), one gemm per vector */          \
    for (int i = 0; i < nvec; ++i)                                                      \
      gemm_nt_##SUF((int)n26, m[0], n[0], X + i * ldX, (int)n26, A[0], ld[0],          \
                    W + i * ldW, (int)n26);                                             \
    /* kronmultv.hpp:130-146: recurse with X and W swapped */                           \
    kronmultv_##SUF(d - 1, m + 1, n + 1, A + 1, ld + 1, nvec * m[0], W, Y, X);          \
  }

DEFINE_KRONMULTV(f64, double)
DEFINE_KRONMULTV(f32, float)

/* Size in elements of the larger of X and every intermediate W of one
 * entry, kronmult_vbatched.hpp:136-153 (sizeXW). */
static size_t size_xw(int d, const int* m, const int* n) {
  size_t sx = 1;
  for (int l = 0; l < d; ++l) sx *= (size_t)n[l];
  size_t best = sx;
  for (int k = 1; k <= d; ++k) {
    size_t s = 1;
    for (int l = 0; l < k; ++l) s *= (size_t)m[l];
    for (int l = k; l < d; ++l) s *= (size_t)n[l];
    if (s > best) best = s;
  }
  return best;
}

size_t kmo_size_xw(int d, const int* m, const int* n) { return size_xw(d, m, n); }

static size_t ipow(int n, int d) {
  size_t r = 1;
  for (int i = 0; i < d; ++i) r *= (size_t)n;
  return r;
}

void kmo_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

int kmo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* kronmult{d}_batched: kronmult6_batched.hpp:14-94.                   */
/* A is (n,n,d,batch), X, Y, W are (n^d, batch).  X and W clobbered.   */
/* ------------------------------------------------------------------ */
#define DEFINE_BATCHED(SUF, T)                                                            \
  void kmo_batched_##SUF(int d, int n, const T* A, T* X, T* Y, T* W, int batch) {         \
    size_t N = ipow(n, d);                                                                \
    int mm[KMO_MAXD], nn[KMO_MAXD], ld[KMO_MAXD];                                         \
    for (int l = 0; l < d; ++l) { mm[l] = n; nn[l] = n; ld[l] = n; }                      \
    _Pragma("omp parallel for schedule(static)")                                          \
    for (int b = 0; b < batch; ++b) {                                                     \
      const T* Ak[KMO_MAXD];                                                              \
      for (int l = 0; l < d; ++l) Ak[l] = A + ((size_t)l + (size_t)b * d) * n * n;        \
      kronmultv_##SUF(d, mm, nn, Ak, ld, 1, X + b * N, Y + b * N, W + b * N);             \
    }                                                                                     \
  }

DEFINE_BATCHED(f64, double)
DEFINE_BATCHED(f32, float)

/* kronmult{d}_pbatched: kronmult6_pbatched.hpp:14-81.  Same, with X, Y, W
 * given as pointer arrays; Y blocks may alias. */
#define DEFINE_PBATCHED(SUF, T)                                                           \
  void kmo_pbatched_##SUF(int d, int n, const T* A, T* const* pX, T* const* pY,           \
                          T* const* pW, int batch) {                                      \
    int mm[KMO_MAXD], nn[KMO_MAXD], ld[KMO_MAXD];                                         \
    for (int l = 0; l < d; ++l) { mm[l] = n; nn[l] = n; ld[l] = n; }                      \
    _Pragma("omp parallel for schedule(static)")                                          \
    for (int b = 0; b < batch; ++b) {                                                     \
      const T* Ak[KMO_MAXD];                                                              \
      for (int l = 0; l < d; ++l) Ak[l] = A + ((size_t)l + (size_t)b * d) * n * n;        \
      kronmultv_##SUF(d, mm, nn, Ak, ld, 1, pX[b], pY[b], pW[b]);                         \
    }                                                                                     \
  }

DEFINE_PBATCHED(f64, double)
DEFINE_PBATCHED(f32, float)

/* kronmult{d}_xbatched: kronmult_xbatched.hpp:19-157.
 * Aarray is (d, batch) pointers, common lda.  Sub-batches of subbatch
 * entries; with batch > 1 entry iz of a sub-batch copies X into pW[2*iz]
 * and uses pW[2*iz+1] as W (X preserved); with batch == 1 X itself is
 * the workspace and pW[0] is W (kronmult_xbatched.hpp:121-133). */
#define DEFINE_XBATCHED(SUF, T)                                                           \
  void kmo_xbatched_##SUF(int d, int n, const T* const* Aarray, int lda, T* const* pX,    \
                          T* const* pY, T* const* pW, int batch, int subbatch) {          \
    if (subbatch <= 0) subbatch = (batch / 2 > 1) ? batch / 2 : 1;                        \
    size_t N = ipow(n, d);                                                                \
    int mm[KMO_MAXD], nn[KMO_MAXD], ld[KMO_MAXD];                                         \
    for (int l = 0; l < d; ++l) { mm[l] = n; nn[l] = n; ld[l] = (lda == 0) ? n : lda; }   \
    for (int start = 0; start < batch; start += subbatch) {                               \
      int cnt = (batch - start < subbatch) ? batch - start : subbatch;                    \
      _Pragma("omp parallel for schedule(static)")                                        \
      for (int iz = 0; iz < cnt; ++iz) {                                                  \
        int b = start + iz;                                                               \
        T* Xp = (batch > 1) ? pW[2 * iz] : pX[b];                                         \
        T* Wp = (batch > 1) ? pW[2 * iz + 1] : pW[b];                                     \
        if (Xp != pX[b]) memcpy(Xp, pX[b], N * sizeof(T));                                \
        kronmultv_##SUF(d, mm, nn, Aarray + (size_t)b * d, ld, 1, Xp, pY[b], Wp);         \
      }                                                                                   \
    }                                                                                     \
  }

DEFINE_XBATCHED(f64, double)
DEFINE_XBATCHED(f32, float)

/* kronmult{d}_vbatched: kronmult_vbatched.hpp:19-248.
 * Rectangular factors m[l] x n[l], uniform over the batch, ld = m[l].
 * One workspace W of Wcap bytes holds (X copy, W) slot pairs of sizeXW
 * elements each; subbatch = min(batch, Wcap / (2*sizeXW*sizeof(T))).
 * Returns -1 if the workspace holds no slot pair, else 0. */
#define DEFINE_VBATCHED(SUF, T)                                                           \
  int kmo_vbatched_##SUF(int d, const int* m, const int* n, const T* const* Aarray,       \
                         T* const* pX, T* const* pY, T* W, size_t Wcap, int batch) {      \
    size_t sxw = size_xw(d, m, n);                                                        \
    size_t sx = 1;                                                                        \
    for (int l = 0; l < d; ++l) sx *= (size_t)n[l];                                       \
    size_t fit = Wcap / (2 * sxw * sizeof(T));                                            \
    if (fit < 1) return -1;                                                               \
    int subbatch = (fit < (size_t)batch) ? (int)fit : batch;                              \
    int ld[KMO_MAXD];                                                                     \
    for (int l = 0; l < d; ++l) ld[l] = m[l];                                             \
    for (int start = 0; start < batch; start += subbatch) {                               \
      int cnt = (batch - start < subbatch) ? batch - start : subbatch;                    \
      _Pragma("omp parallel for schedule(static)")                                        \
      for (int iz = 0; iz < cnt; ++iz) {                                                  \
        int b = start + iz;                                                               \
        T* Xp = W + (size_t)iz * 2 * sxw;                                                 \
        T* Wp = Xp + sxw;                                                                 \
        memcpy(Xp, pX[b], sx * sizeof(T));                                                \
        kronmultv_##SUF(d, m, n, Aarray + (size_t)b * d, ld, 1, Xp, pY[b], Wp);           \
      }                                                                                   \
    }                                                                                     \
    return 0;                                                                             \
  }

DEFINE_VBATCHED(f64, double)
DEFINE_VBATCHED(f32, float)

/* ------------------------------------------------------------------ */
/* Index-triple form of xbatched: entry e is (y_idx[e], x_idx[e],      */
/* a_idx[e*d + l]) into pools X (N x nx), Y (N x ny) and per-dimension */
/* factor pools A[l] (lda x n x pool), column-major.  Same recursion;  */
/* each entry uses a private copy of its X block, so X is preserved.   */
/* This is the layout the benchmark builds its pointer arrays from.   */
/* ------------------------------------------------------------------ */
void kmo_xbatched_idx_f64(int d, int n, const double* Apool, int lda, int pool,
                          const double* Xpool, double* Ypool, const int* y_idx,
                          const int* x_idx, const int* a_idx, int nentries) {
  size_t N = ipow(n, d);
  int mm[KMO_MAXD], nn[KMO_MAXD], ld[KMO_MAXD];
  for (int l = 0; l < d; ++l) { mm[l] = n; nn[l] = n; ld[l] = lda; }
#pragma omp parallel
  {
    double* Xp = (double*)malloc(2 * N * sizeof(double));
    double* Wp = Xp + N;
#pragma omp for schedule(static)
    for (int e = 0; e < nentries; ++e) {
      const double* Ak[KMO_MAXD];
      for (int l = 0; l < d; ++l)
        Ak[l] = Apool + ((size_t)l * pool + (size_t)a_idx[(size_t)e * d + l]) * (size_t)lda * n;
      memcpy(Xp, Xpool + (size_t)x_idx[e] * N, N * sizeof(double));
      kronmultv_f64(d, mm, nn, Ak, ld, 1, Xp, Ypool + (size_t)y_idx[e] * N, Wp);
    }
    free(Xp);
  }
}

/* ------------------------------------------------------------------ */
/* Explicit-Kronecker oracle (test_kronmult6_batched.cpp:394-458):     */
/* Yout(ic) = sum_jc prod_l A_l(i_l, j_l) X(jc), last index fastest.  */
/* Accumulates in long double.  Overwrites Yout.  Small sizes only.   */
/* ------------------------------------------------------------------ */
void kmo_explicit_f64(int d, const int* m, const int* n, const double* const* A,
                      const int* ld, const double* X, double* Yout) {
  size_t M = 1, Nn = 1;
  for (int l = 0; l < d; ++l) { M *= (size_t)m[l]; Nn *= (size_t)n[l]; }
#pragma omp parallel for schedule(static)
  for (size_t ic = 0; ic < M; ++ic) {
    int ii[KMO_MAXD];
    size_t r = ic;
    for (int l = d - 1; l >= 0; --l) { ii[l] = (int)(r % (size_t)m[l]); r /= (size_t)m[l]; }
    long double acc = 0;
    for (size_t jc = 0; jc < Nn; ++jc) {
      size_t s = jc;
      long double c = 1;
      for (int l = d - 1; l >= 0; --l) {
        int jl = (int)(s % (size_t)n[l]);
        s /= (size_t)n[l];
        c *= (long double)A[l][ii[l] + (size_t)jl * ld[l]];
      }
      acc += c * (long double)X[jc];
    }
    Yout[ic] = (double)acc;
  }
}

/* Single-entry recursion, exported for the tests (one entry, nvec = 1,
 * caller's X is not modified: a private copy is used). */
void kmo_kronmultv_f64(int d, const int* m, const int* n, const double* const* A,
                       const int* ld, const double* X, double* Y) {
  size_t sxw = size_xw(d, m, n), sx = 1;
  for (int l = 0; l < d; ++l) sx *= (size_t)n[l];
  double* buf = (double*)malloc(2 * sxw * sizeof(double));
  memcpy(buf, X, sx * sizeof(double));
  kronmultv_f64(d, m, n, A, ld, 1, buf, Y, buf + sxw);
  free(buf);
}

void kmo_kronmultv_f32(int d, const int* m, const int* n, const float* const* A,
                       const int* ld, const float* X, float* Y) {
  size_t sxw = size_xw(d, m, n), sx = 1;
  for (int l = 0; l < d; ++l) sx *= (size_t)n[l];
  float* buf = (float*)malloc(2 * sxw * sizeof(float));
  memcpy(buf, X, sx * sizeof(float));
  kronmultv_f32(d, m, n, A, ld, 1, buf, Y, buf + sxw);
  free(buf);
}

/* kron_flops of kroncommon.hpp:204-234: flops of one entry. */
double kmo_kron_flops(int d, const int* m, const int* n) {
  if (d == 1) return 2.0 * m[0] * n[0];
  double rest = 1;
  for (int l = 1; l < d; ++l) rest *= n[l];
  double f1 = 2.0 * rest * n[0] * m[0];
  return f1 + kmo_kron_flops(d - 1, m + 1, n + 1) * m[0];
}

/* ------------------------------------------------------------------ */
/* Stand-alone batched tiny GEMMs: kgemm_nn_batched / kgemm_nt_batched */
/* ------------------------------------------------------------------ */

/* Entry ib: C = alpha * A * op(B) + beta * C, A mm x kk, C mm x nn,
 * op(B) = B (kk x nn) for "nn", transpose(B) with B nn x kk for "nt".
 * Follows kgemm_nn_batched.hpp:8-81 / kgemm_nt_batched.hpp:8-79 (one entry
 * after another) and the per-element epilogue of kgemm_nn_v1
 * (kgemm_nn.hpp:388-400) / kgemm_nt_v1 (kgemm_nt.hpp:365-376):
 *   beta == 1: C += alpha*c with an atomic update (entries may share C);
 *   beta == 0: C  = alpha*c;
 *   otherwise: C  = beta*C + alpha*c.
 * The nn epilogue rounds alpha*c to T before it is used (kgemm_nn.hpp:390);
 * the nt epilogue blends beta*C + alpha*c in the accumulation type and
 * rounds once (kgemm_nt.hpp:375).  For FP64 the two are the same.
 * The dot product c starts from zero and runs over k in increasing order.
 * FP32 follows the reference's float specialisation (kgemm_nn.hpp:688-701,
 * kgemm_nt.hpp:557-571): accumulate, scale and blend in double, round when
 * stored. */
#define DEFINE_KGEMM(NAME, T, TRANSB)                                                     \
  void NAME(int mm, int nn, int kk, T alpha, const T* const* Aarray, const int* ldAarray, \
            const T* const* Barray, const int* ldBarray, T beta, T* const* Carray,        \
            const int* ldCarray, int batch) {                                             \
    const double al = (double)alpha, be = (double)beta;                                   \
    _Pragma("omp parallel for schedule(dynamic, 1)")                                      \
    for (int ib = 0; ib < batch; ++ib) {                                                  \
      const T* A = Aarray[ib];                                                            \
      const T* B = Barray[ib];                                                            \
      T* C = Carray[ib];                                                                  \
      const size_t ldA = (size_t)ldAarray[ib], ldB = (size_t)ldBarray[ib];                \
      const size_t ldC = (size_t)ldCarray[ib];                                            \
      for (int j = 0; j < nn; ++j)                                                        \
        for (int i = 0; i < mm; ++i) {                                                    \
          double c = 0;                                                                   \
          for (int k = 0; k < kk; ++k) {                                                  \
            const double b = TRANSB ? (double)B[j + k * ldB] : (double)B[k + j * ldB];    \
            c += (double)A[i + k * ldA] * b;                                              \
          }                                                                               \
          T* p = &C[i + j * ldC];                                                         \
          const T ac = (T)(al * c);                                                       \
          if (be == 1.0) {                                                                \
            _Pragma("omp atomic update") *p += ac;                                        \
          } else if (be == 0.0) {                                                         \
            *p = ac;                                                                      \
          } else {                                                                        \
            *p = TRANSB ? (T)(be * (double)*p + al * c) : (T)(be * (double)*p + (double)ac); \
          }                                                                               \
        }                                                                                 \
    }                                                                                     \
  }

DEFINE_KGEMM(kmo_kgemm_nn_batched_f64, double, 0)
DEFINE_KGEMM(kmo_kgemm_nt_batched_f64, double, 1)
DEFINE_KGEMM(kmo_kgemm_nn_batched_f32, float, 0)
DEFINE_KGEMM(kmo_kgemm_nt_batched_f32, float, 1)
