/* Force-included when the reference's CPU (OpenMP) path is compiled as the
 * parity reference.  Its GPU-only tiny-GEMM variants (kgemm_nt_v2,
 * kgemm_nn_v2) name CUDA built-ins outside #ifdef USE_GPU; they are never
 * called on the CPU path, but the names must exist for the templates to
 * parse.  Nothing here executes. */
#ifndef KMX_REF_CPU_SHIM_H
#define KMX_REF_CPU_SHIM_H
#include <cstdio> /* the vbatched debug print uses printf without including it */
struct kmx_ref_dim3 { unsigned x, y, z; };
static const kmx_ref_dim3 threadIdx = {0, 0, 0};
static const kmx_ref_dim3 blockIdx = {0, 0, 0};
static const kmx_ref_dim3 blockDim = {1, 1, 1};
static const kmx_ref_dim3 gridDim = {1, 1, 1};
static inline void __syncthreads() {}
#endif
