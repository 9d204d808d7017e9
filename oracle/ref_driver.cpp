// Parity-reference driver: instantiates hipdac-lab/kronmult's own CPU
// (OpenMP) templates from the reference source tree and exposes them with a
// C ABI, so the tests can run the unmodified reference algorithm on the same
// inputs as the CUDA path.  Test infrastructure only; built by
// oracle/Makefile into oracle/_ref/ and never shipped.
//
// Entry points wrapped (reference file:line):
//   kronmult{d}_batched<T>   kronmult6_batched.hpp:14-94
//   kronmult{d}_pbatched<T>  kronmult6_pbatched.hpp:14-81
//   kronmult{d}_xbatched<T>  kronmult6_xbatched.hpp:14-46 -> kronmult_xbatched.hpp:19-157
//   kronmult{d}_vbatched<T>  kronmult6_vbatched.hpp:14-58 -> kronmult_vbatched.hpp:19-248
//   kgemm_nn_batched<T>      kgemm_nn_batched.hpp:8-81
//   kgemm_nt_batched<T>      kgemm_nt_batched.hpp:8-79
#include <cstddef>
#include "kronmult1_batched.hpp"
#include "kronmult2_batched.hpp"
#include "kronmult3_batched.hpp"
#include "kronmult4_batched.hpp"
#include "kronmult5_batched.hpp"
#include "kronmult6_batched.hpp"
#include "kronmult1_pbatched.hpp"
#include "kronmult2_pbatched.hpp"
#include "kronmult3_pbatched.hpp"
#include "kronmult4_pbatched.hpp"
#include "kronmult5_pbatched.hpp"
#include "kronmult6_pbatched.hpp"
#include "kronmult1_xbatched.hpp"
#include "kronmult2_xbatched.hpp"
#include "kronmult3_xbatched.hpp"
#include "kronmult4_xbatched.hpp"
#include "kronmult5_xbatched.hpp"
#include "kronmult6_xbatched.hpp"
#include "kronmult1_vbatched.hpp"
#include "kronmult2_vbatched.hpp"
#include "kronmult3_vbatched.hpp"
#include "kronmult4_vbatched.hpp"
#include "kronmult5_vbatched.hpp"
#include "kronmult6_vbatched.hpp"
#include "kgemm_nn_batched.hpp"
#include "kgemm_nt_batched.hpp"

template <typename T>
static int batched(int d, int n, const T* A, T* X, T* Y, T* W, int b) {
  switch (d) {
    case 1: kronmult1_batched<T>(n, A, X, Y, W, b); return 0;
    case 2: kronmult2_batched<T>(n, A, X, Y, W, b); return 0;
    case 3: kronmult3_batched<T>(n, A, X, Y, W, b); return 0;
    case 4: kronmult4_batched<T>(n, A, X, Y, W, b); return 0;
    case 5: kronmult5_batched<T>(n, A, X, Y, W, b); return 0;
    case 6: kronmult6_batched<T>(n, A, X, Y, W, b); return 0;
  }
  return -1;
}

template <typename T>
static int pbatched(int d, int n, const T* A, T** X, T** Y, T** W, int b) {
  switch (d) {
    case 1: kronmult1_pbatched<T>(n, A, X, Y, W, b); return 0;
    case 2: kronmult2_pbatched<T>(n, A, X, Y, W, b); return 0;
    case 3: kronmult3_pbatched<T>(n, A, X, Y, W, b); return 0;
    case 4: kronmult4_pbatched<T>(n, A, X, Y, W, b); return 0;
    case 5: kronmult5_pbatched<T>(n, A, X, Y, W, b); return 0;
    case 6: kronmult6_pbatched<T>(n, A, X, Y, W, b); return 0;
  }
  return -1;
}

template <typename T>
static int xbatched(int d, int n, const T* const* A, int lda, T** X, T** Y, T** W, int b, int sub) {
  switch (d) {
    case 1: kronmult1_xbatched<T>(n, A, lda, X, Y, W, b, sub); return 0;
    case 2: kronmult2_xbatched<T>(n, A, lda, X, Y, W, b, sub); return 0;
    case 3: kronmult3_xbatched<T>(n, A, lda, X, Y, W, b, sub); return 0;
    case 4: kronmult4_xbatched<T>(n, A, lda, X, Y, W, b, sub); return 0;
    case 5: kronmult5_xbatched<T>(n, A, lda, X, Y, W, b, sub); return 0;
    case 6: kronmult6_xbatched<T>(n, A, lda, X, Y, W, b, sub); return 0;
  }
  return -1;
}

template <typename T>
static int vbatched(int d, const int* m, const int* n, const T* const* A, T** X, T** Y, T* W,
                    size_t cap, int b) {
  switch (d) {
    case 1: kronmult1_vbatched<T>(m[0], n[0], A, X, Y, W, cap, b); return 0;
    case 2: kronmult2_vbatched<T>(m[0], n[0], m[1], n[1], A, X, Y, W, cap, b); return 0;
    case 3: kronmult3_vbatched<T>(m[0], n[0], m[1], n[1], m[2], n[2], A, X, Y, W, cap, b); return 0;
    case 4: kronmult4_vbatched<T>(m[0], n[0], m[1], n[1], m[2], n[2], m[3], n[3], A, X, Y, W, cap, b); return 0;
    case 5: kronmult5_vbatched<T>(m[0], n[0], m[1], n[1], m[2], n[2], m[3], n[3], m[4], n[4], A, X, Y, W, cap, b); return 0;
    case 6: kronmult6_vbatched<T>(m[0], n[0], m[1], n[1], m[2], n[2], m[3], n[3], m[4], n[4], m[5], n[5], A, X, Y, W, cap, b); return 0;
  }
  return -1;
}

extern "C" {
int ref_batched_f64(int d, int n, const double* A, double* X, double* Y, double* W, int b) { return batched<double>(d, n, A, X, Y, W, b); }
int ref_batched_f32(int d, int n, const float* A, float* X, float* Y, float* W, int b) { return batched<float>(d, n, A, X, Y, W, b); }
int ref_pbatched_f64(int d, int n, const double* A, double** X, double** Y, double** W, int b) { return pbatched<double>(d, n, A, X, Y, W, b); }
int ref_pbatched_f32(int d, int n, const float* A, float** X, float** Y, float** W, int b) { return pbatched<float>(d, n, A, X, Y, W, b); }
int ref_xbatched_f64(int d, int n, const double* const* A, int lda, double** X, double** Y, double** W, int b, int sub) { return xbatched<double>(d, n, A, lda, X, Y, W, b, sub); }
int ref_xbatched_f32(int d, int n, const float* const* A, int lda, float** X, float** Y, float** W, int b, int sub) { return xbatched<float>(d, n, A, lda, X, Y, W, b, sub); }
int ref_vbatched_f64(int d, const int* m, const int* n, const double* const* A, double** X, double** Y, double* W, size_t cap, int b) { return vbatched<double>(d, m, n, A, X, Y, W, cap, b); }
int ref_vbatched_f32(int d, const int* m, const int* n, const float* const* A, float** X, float** Y, float* W, size_t cap, int b) { return vbatched<float>(d, m, n, A, X, Y, W, cap, b); }

int ref_kgemm_nn_batched_f64(int mm, int nn, int kk, double alpha, double* const* A, const int* ldA, double* const* B, const int* ldB, double beta, double* const* C, const int* ldC, int b) { kgemm_nn_batched<double>(mm, nn, kk, alpha, A, ldA, B, ldB, beta, C, ldC, b); return 0; }
int ref_kgemm_nt_batched_f64(int mm, int nn, int kk, double alpha, double* const* A, const int* ldA, double* const* B, const int* ldB, double beta, double* const* C, const int* ldC, int b) { kgemm_nt_batched<double>(mm, nn, kk, alpha, A, ldA, B, ldB, beta, C, ldC, b); return 0; }
int ref_kgemm_nn_batched_f32(int mm, int nn, int kk, float alpha, float* const* A, const int* ldA, float* const* B, const int* ldB, float beta, float* const* C, const int* ldC, int b) { kgemm_nn_batched<float>(mm, nn, kk, alpha, A, ldA, B, ldB, beta, C, ldC, b); return 0; }
int ref_kgemm_nt_batched_f32(int mm, int nn, int kk, float alpha, float* const* A, const int* ldA, float* const* B, const int* ldB, float beta, float* const* C, const int* ldC, int b) { kgemm_nt_batched<float>(mm, nn, kk, alpha, A, ldA, B, ldB, beta, C, ldC, b); return 0; }
}
