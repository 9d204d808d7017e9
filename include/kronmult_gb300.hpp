// kronmult_gb300.hpp -- C++ drop-in for hipdac-lab/kronmult's host entry points.
//
// Same names, argument order and meaning as the reference's host wrappers
// (kronmult6_batched.cpp:5-25, kronmult6_pbatched.cpp:5-25,
// kronmult6_xbatched.cpp:5-39) and, for vbatched (which the reference only
// has as a __global__ template, kronmult6_vbatched.hpp:16-29), the template's
// argument list as a host function.  All arrays are device pointers; the
// launch is asynchronous on the default stream.  Like the reference, these
// return void and stop on an error through assert(); call the C ABI
// (kronmult_gb300.h) directly to get status codes instead.
#ifndef KRONMULT_GB300_HPP
#define KRONMULT_GB300_HPP

#include <cassert>
#include <cstddef>

#include "kronmult_gb300.h"

namespace kmx_detail {
inline void check(int status) {
  (void)status;
  assert(status == KMX_OK && "kronmult_gb300 call failed");
}
}  // namespace kmx_detail

#define KMX_DROPIN_SQUARE(D)                                                                    \
  inline void kronmult##D##_batched(int const n, double const Aarray_[], double Xarray_[],      \
                                    double Yarray_[], double Warray_[], int const batchCount) { \
    kmx_detail::check(                                                                          \
        kmx_kronmult_batched_f64(D, n, Aarray_, Xarray_, Yarray_, Warray_, batchCount, 0));     \
  }                                                                                             \
  inline void kronmult##D##_batched(int const n, float const Aarray_[], float Xarray_[],        \
                                    float Yarray_[], float Warray_[], int const batchCount) {   \
    kmx_detail::check(                                                                          \
        kmx_kronmult_batched_f32(D, n, Aarray_, Xarray_, Yarray_, Warray_, batchCount, 0));     \
  }                                                                                             \
  inline void kronmult##D##_pbatched(int const n, double const Aarray_[], double* Xarray_[],    \
                                     double* Yarray_[], double* Warray_[],                      \
                                     int const batchCount) {                                    \
    kmx_detail::check(                                                                          \
        kmx_kronmult_pbatched_f64(D, n, Aarray_, Xarray_, Yarray_, Warray_, batchCount, 0));    \
  }                                                                                             \
  inline void kronmult##D##_pbatched(int const n, float const Aarray_[], float* Xarray_[],      \
                                     float* Yarray_[], float* Warray_[], int const batchCount) { \
    kmx_detail::check(                                                                          \
        kmx_kronmult_pbatched_f32(D, n, Aarray_, Xarray_, Yarray_, Warray_, batchCount, 0));    \
  }                                                                                             \
  inline void kronmult##D##_xbatched(int const n, double const* const Aarray_[], int const lda, \
                                     double* Xarray_[], double* Yarray_[], double* Warray_[],   \
                                     int const batchCount, int const subbatchCount = 0) {       \
    kmx_detail::check(kmx_kronmult_xbatched_f64(D, n, Aarray_, lda, Xarray_, Yarray_, Warray_,  \
                                                batchCount, subbatchCount, 0));                 \
  }                                                                                             \
  inline void kronmult##D##_xbatched(int const n, float const* const Aarray_[], int const lda,  \
                                     float* Xarray_[], float* Yarray_[], float* Warray_[],      \
                                     int const batchCount, int const subbatchCount = 0) {       \
    kmx_detail::check(kmx_kronmult_xbatched_f32(D, n, Aarray_, lda, Xarray_, Yarray_, Warray_,  \
                                                batchCount, subbatchCount, 0));                 \
  }

KMX_DROPIN_SQUARE(1)
KMX_DROPIN_SQUARE(2)
KMX_DROPIN_SQUARE(3)
KMX_DROPIN_SQUARE(4)
KMX_DROPIN_SQUARE(5)
KMX_DROPIN_SQUARE(6)
#undef KMX_DROPIN_SQUARE

// kgemm_{nn,nt}_batched (kgemm_nn_batched.cpp:8-41, kgemm_nt_batched.cpp:8-41)
inline void kgemm_nn_batched(int const mm, int const nn, int const kk, double const alpha,
                             double* const Aarray_[], int const ldAarray_[],
                             double* const Barray_[], int const ldBarray_[], double const beta,
                             double* const Carray_[], int const ldCarray_[],
                             int const batchCount) {
  kmx_detail::check(kmx_kgemm_nn_batched_f64(mm, nn, kk, alpha, Aarray_, ldAarray_, Barray_,
                                             ldBarray_, beta, Carray_, ldCarray_, batchCount, 0));
}
inline void kgemm_nt_batched(int const mm, int const nn, int const kk, double const alpha,
                             double* const Aarray_[], int const ldAarray_[],
                             double* const Barray_[], int const ldBarray_[], double const beta,
                             double* const Carray_[], int const ldCarray_[],
                             int const batchCount) {
  kmx_detail::check(kmx_kgemm_nt_batched_f64(mm, nn, kk, alpha, Aarray_, ldAarray_, Barray_,
                                             ldBarray_, beta, Carray_, ldCarray_, batchCount, 0));
}
inline void kgemm_nn_batched(int const mm, int const nn, int const kk, float const alpha,
                             float* const Aarray_[], int const ldAarray_[],
                             float* const Barray_[], int const ldBarray_[], float const beta,
                             float* const Carray_[], int const ldCarray_[],
                             int const batchCount) {
  kmx_detail::check(kmx_kgemm_nn_batched_f32(mm, nn, kk, alpha, Aarray_, ldAarray_, Barray_,
                                             ldBarray_, beta, Carray_, ldCarray_, batchCount, 0));
}
inline void kgemm_nt_batched(int const mm, int const nn, int const kk, float const alpha,
                             float* const Aarray_[], int const ldAarray_[],
                             float* const Barray_[], int const ldBarray_[], float const beta,
                             float* const Carray_[], int const ldCarray_[],
                             int const batchCount) {
  kmx_detail::check(kmx_kgemm_nt_batched_f32(mm, nn, kk, alpha, Aarray_, ldAarray_, Barray_,
                                             ldBarray_, beta, Carray_, ldCarray_, batchCount, 0));
}

// vbatched: (m1,n1, ..., md,nd, Aarray, pX, pY, W, Wcapacity_bytes, batchCount)
template <typename T>
inline int kmx_vbatched_dispatch(int d, const int* m, const int* n, T const* const Aarray_[],
                                 T* pX_[], T* pY_[], T* W_, size_t cap, int batchCount);
template <>
inline int kmx_vbatched_dispatch<double>(int d, const int* m, const int* n,
                                         double const* const Aarray_[], double* pX_[],
                                         double* pY_[], double* W_, size_t cap, int batchCount) {
  return kmx_kronmult_vbatched_f64(d, m, n, Aarray_, pX_, pY_, W_, cap, batchCount, 0);
}
template <>
inline int kmx_vbatched_dispatch<float>(int d, const int* m, const int* n,
                                        float const* const Aarray_[], float* pX_[], float* pY_[],
                                        float* W_, size_t cap, int batchCount) {
  return kmx_kronmult_vbatched_f32(d, m, n, Aarray_, pX_, pY_, W_, cap, batchCount, 0);
}

template <typename T>
inline void kronmult1_vbatched(int m1, int n1, T const* const Aarray_[], T* pX_[], T* pY_[], T* W_,
                               size_t const Wcapacity_bytes, int const batchCount) {
  const int m[] = {m1}, n[] = {n1};
  kmx_detail::check(kmx_vbatched_dispatch<T>(1, m, n, Aarray_, pX_, pY_, W_, Wcapacity_bytes, batchCount));
}
template <typename T>
inline void kronmult2_vbatched(int m1, int n1, int m2, int n2, T const* const Aarray_[], T* pX_[],
                               T* pY_[], T* W_, size_t const Wcapacity_bytes, int const batchCount) {
  const int m[] = {m1, m2}, n[] = {n1, n2};
  kmx_detail::check(kmx_vbatched_dispatch<T>(2, m, n, Aarray_, pX_, pY_, W_, Wcapacity_bytes, batchCount));
}
template <typename T>
inline void kronmult3_vbatched(int m1, int n1, int m2, int n2, int m3, int n3,
                               T const* const Aarray_[], T* pX_[], T* pY_[], T* W_,
                               size_t const Wcapacity_bytes, int const batchCount) {
  const int m[] = {m1, m2, m3}, n[] = {n1, n2, n3};
  kmx_detail::check(kmx_vbatched_dispatch<T>(3, m, n, Aarray_, pX_, pY_, W_, Wcapacity_bytes, batchCount));
}
template <typename T>
inline void kronmult4_vbatched(int m1, int n1, int m2, int n2, int m3, int n3, int m4, int n4,
                               T const* const Aarray_[], T* pX_[], T* pY_[], T* W_,
                               size_t const Wcapacity_bytes, int const batchCount) {
  const int m[] = {m1, m2, m3, m4}, n[] = {n1, n2, n3, n4};
  kmx_detail::check(kmx_vbatched_dispatch<T>(4, m, n, Aarray_, pX_, pY_, W_, Wcapacity_bytes, batchCount));
}
template <typename T>
inline void kronmult5_vbatched(int m1, int n1, int m2, int n2, int m3, int n3, int m4, int n4,
                               int m5, int n5, T const* const Aarray_[], T* pX_[], T* pY_[], T* W_,
                               size_t const Wcapacity_bytes, int const batchCount) {
  const int m[] = {m1, m2, m3, m4, m5}, n[] = {n1, n2, n3, n4, n5};
  kmx_detail::check(kmx_vbatched_dispatch<T>(5, m, n, Aarray_, pX_, pY_, W_, Wcapacity_bytes, batchCount));
}
template <typename T>
inline void kronmult6_vbatched(int m1, int n1, int m2, int n2, int m3, int n3, int m4, int n4,
                               int m5, int n5, int m6, int n6, T const* const Aarray_[], T* pX_[],
                               T* pY_[], T* W_, size_t const Wcapacity_bytes, int const batchCount) {
  const int m[] = {m1, m2, m3, m4, m5, m6}, n[] = {n1, n2, n3, n4, n5, n6};
  kmx_detail::check(kmx_vbatched_dispatch<T>(6, m, n, Aarray_, pX_, pY_, W_, Wcapacity_bytes, batchCount));
}

#endif  // KRONMULT_GB300_HPP
