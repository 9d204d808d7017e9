/*
 * kronmult_gb300.h -- C ABI of the GB300 (sm_103a) batched Kronecker mat-vec.
 *
 *   Y(:,k) += kron(A1(:,:,k), ..., Ad(:,:,k)) * X(:,k),   d = 1..6
 *
 * Conventions, identical to hipdac-lab/kronmult:
 *   - factors are column-major with a leading dimension; A_l(i,j) = A_l[i + j*ld];
 *   - an X/Y block is a vector whose LAST Kronecker index runs fastest, so
 *     kron(A1,...,Ad) has A1's index slowest (test_kronmult6_batched.cpp:418-436);
 *   - Y is accumulated into, never overwritten (kronmultv.hpp:178);
 *   - every array and every pointer array is DEVICE memory; the pointer arrays
 *     themselves live on the device (test_kronmult6_xbatched.cpp:318-321);
 *   - calls are asynchronous on the given stream (0 = legacy default stream);
 *     the caller synchronises, as with the reference (test_kronmult6_batched.cpp:248).
 *
 * The library looks up the device addresses of its own device variables (the
 * status word, the diagnostic counters, the no-allocation scratch) once per
 * device and keeps them for the life of the process: do not use it across a
 * cudaDeviceReset of a device it has run on.
 *
 * Differences from the reference, all supersets of its contract:
 *   - each call returns a kmx_status instead of asserting;
 *   - X is never modified (the reference may clobber X in batched/pbatched);
 *   - W is used only when one entry does not fit on chip; it may then be
 *     clobbered exactly as in the reference.
 */
#ifndef KRONMULT_GB300_H
#define KRONMULT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without pulling in cuda_runtime.h. */
typedef struct CUstream_st* kmx_stream_t;

typedef enum kmx_status {
  KMX_OK = 0,
  KMX_ERR_INVALID_ARG = 1,   /* d outside 1..6, n < 1, batch < 0, lda < n, ... */
  KMX_ERR_NULL_POINTER = 2,  /* a required array pointer is NULL */
  KMX_ERR_WORKSPACE = 3,     /* workspace missing or too small for an entry */
  KMX_ERR_UNSUPPORTED = 4,   /* shape or option the library does not handle */
  KMX_ERR_CUDA = 5,          /* a CUDA runtime call failed (see kmx_last_cuda_error) */
  KMX_ERR_DEVICE = 6,        /* a kernel reported an error through the device status word */
  KMX_ERR_OVERLAP = 7        /* deterministic mode: Y blocks partially overlap (reported
                                through the device status word, bit 16) */
} kmx_status;

/* Arithmetic form.  FP64 entry points: AUTO, PLAIN, SPLIT, SPLIT_RAW, DIGITS
 * (the fused backward: PLAIN runs FP64, the others double-float).  FP32 entry
 * points (the _f32 functions): AUTO and SPLIT round each dot product once, as
 * the reference's float kernels do; PLAIN is FP32 fused multiply-add; TF32X3
 * the tensor cores.  kmx_kronmult_xbatched_wide: FP32 fused multiply-add
 * unless TF32X3 is asked for. */
typedef enum kmx_form {
  KMX_FORM_AUTO = 0,   /* square shapes: per-(d,n) choice from the tuning table;
                          other shapes: SPLIT once an X or Y block has 512 or more
                          elements, PLAIN below */
  KMX_FORM_PLAIN = 1,  /* native FP64 fused multiply-add */
  KMX_FORM_SPLIT = 2,  /* double-float: FP64 values carried as FP32 (hi, lo) pairs,
                          ~2^-48 relative to |K||X| per entry, FP64 in and out.  An entry
                          whose result cancels (rho_F = ||KX|| sqrt(prod n_l) /
                          (prod ||A_l||_F ||X||) below 1/4) is recomputed in FP64, so the
                          form is as accurate as PLAIN wherever PLAIN holds 1e-13
                          (kmx_read_redo_counters counts those entries), except on the
                          smallest blocks: n = 2 (and d = 1, n = 3) measured up to 4e-13
                          per block; AUTO runs FP64 for every n = 2 shape and every
                          block under 8 elements */
  KMX_FORM_DIGITS = 4, /* FP64 data on the FP16 tensor cores: X and factors as 7 base-2^9
                          digits with one exponent per entry, exact digit products
                          (mma.sync), exact FP32 level sums, FP64 out.  Square n = 4
                          (d = 4, 6) and n = 16 (d = 2, 3), atomic mode; entries whose
                          result falls far below the entry's scale, or with Inf/NaN, are
                          recomputed in double-float.  Other shapes: SPLIT. */
  KMX_FORM_SPLIT_RAW = 5, /* SPLIT without the cancellation guard (accuracy studies):
                             error about 2^-48 ||(|K||X|)|| */
  KMX_FORM_TF32X3 = 3  /* FP32-stored data only: tensor cores (mma.sync TF32), each
                          operand split into two TF32 parts, three products, FP32
                          accumulation (~2^-21 relative per product).  Square n = 4
                          (d = 4, 6), n = 8 (d = 3..5), n = 16 (d = 2, 3), atomic mode;
                          other shapes and the deterministic mode use FP32 FMA. */
} kmx_form;

/* How contributions of entries that share a Y block are combined. */
typedef enum kmx_accumulate {
  KMX_ACC_ATOMIC = 0,        /* FP64/FP32 atomic add per element (reference semantics) */
  KMX_ACC_DETERMINISTIC = 1  /* entries grouped by Y block on the device, each block summed
                                in a fixed order by one group: bitwise reproducible.  Every
                                shape of the FP64 and FP32 entry points (square n = 2..8
                                and d >= 3 in register-tiled segment kernels, the others
                                in the generic kernels); kmx_kronmult_xbatched_wide:
                                register-tiled shapes only; mixed-shape calls: the generic
                                kernels, class after class over one set of segments */
} kmx_accumulate;

/* Kernel family for square factors. */
typedef enum kmx_engine {
  KMX_ENGINE_TUNED = 0,    /* the committed tuning table's choice for (form, d, n) */
  KMX_ENGINE_PER_MODE = 1, /* one mode contraction per pass over shared memory */
  KMX_ENGINE_TILED = 2,    /* register tiles of one or two modes, TMA-prefetched X */
  KMX_ENGINE_SMALL = 3,    /* d <= 3 with n^d <= 256: many entries per CTA, staged with
                              128-bit loads, one thread per output element and mode */
  KMX_ENGINE_PERSISTENT = 4 /* kmx_kronmult_mixed_f64 with form AUTO or SPLIT and atomic
                              accumulation: ONE persistent launch over every class, instances
                              taken from a device work queue in class order, each run by the
                              generic double-float kernel with its own (d, n) (the default runs
                              one tuned launch per class, measured faster); other calls treat
                              it as TUNED */,
  KMX_ENGINE_CLUSTER = 5   /* double-float entries beyond one SM's shared memory (square
                              d=5 n=8, d=6 n=6..8, atomic accumulation): a thread-block
                              cluster of n CTAs per (entry, i1) sharing mode 2 through
                              distributed shared memory, no workspace.  Every engine takes
                              it for these shapes when the call passes no workspace; with
                              a workspace the per-mode kernels run (measured faster) unless
                              this engine is asked for; other shapes treat it as TUNED */,
  KMX_ENGINE_LANE = 6      /* one entry per thread with the entry in registers: square
                              n^2 <= 16 and n^d <= 16 (d = 1, 2 with n <= 4; d = 3 with
                              n = 2); d = 2 with n = 5..8, one group of n lanes per
                              entry; d >= 3 with n^(d-1) <= 32, one fiber per lane;
                              atomic or exclusive accumulation; other shapes treat it
                              as TUNED */
} kmx_engine;

typedef struct kmx_options {
  int form;        /* kmx_form */
  int accumulate;  /* kmx_accumulate */
  int transpose;   /* nonzero: use A_l^T for every factor (the backward dX product) */
  int engine;      /* kmx_engine */
  /* Deterministic mode only: device workspace of at least
   * kmx_deterministic_workspace_bytes(batchCount) bytes.  NULL: the library
   * keeps one stream-ordered workspace per device (cudaMallocAsync on first
   * use and on growth), which calls on different streams must not share. */
  void* workspace;
  size_t workspace_bytes;
  /* Launch shape; 0 takes the tuning table's choice for the call's (form,
   * layout, d, n) with engine TUNED, else the built-in default.
   * group_threads: threads per entry of the per-mode kernels (a multiple of
   * 32, at most 512; the register-tiled and small-entry kernels fix their
   * own); groups_per_cta: entries processed side by side in one CTA;
   * ctas_per_sm: cap on the CTAs per SM the grid is sized for. */
  int group_threads;
  int groups_per_cta;
  int ctas_per_sm;
} kmx_options;

/* ---------------------------------------------------------------------- */
/* Drop-in entry points (FP64), argument order of the reference.           */
/* ---------------------------------------------------------------------- */

/* kronmult{d}_batched (reference kronmult6_batched.cpp:5-25).
 * A is (n,n,d,batch); X, Y, W are (n^d, batch), contiguous. */
int kmx_kronmult_batched_f64(int d, int n, const double* A, double* X, double* Y, double* W,
                             int batchCount, kmx_stream_t stream);

/* kronmult{d}_pbatched (reference kronmult6_pbatched.cpp:5-25).
 * A is (n,n,d,batch); pX/pY/pW are arrays of batch device pointers to
 * n^d-element blocks; Y blocks may alias. */
int kmx_kronmult_pbatched_f64(int d, int n, const double* A, double* const* pX,
                              double* const* pY, double* const* pW, int batchCount,
                              kmx_stream_t stream);

/* kronmult{d}_xbatched (reference kronmult6_xbatched.cpp:5-39).
 * Aarray is (d, batch) pointers to n x n factors with leading dimension lda
 * (0 means n); Y blocks may alias.  pW holds 2*subbatchCount workspace
 * pointers when batchCount > 1 (subbatchCount 0 means max(1, batch/2)) and
 * one when batchCount == 1, exactly as the reference; it is read only when an
 * entry does not fit on chip. */
int kmx_kronmult_xbatched_f64(int d, int n, const double* const* Aarray, int lda,
                              double* const* pX, double* const* pY, double* const* pW,
                              int batchCount, int subbatchCount, kmx_stream_t stream);

/* kronmult{d}_vbatched (reference kronmult6_vbatched.hpp:16-29, which has no
 * host wrapper).  Factor l is m[l] x n[l] with leading dimension m[l],
 * uniform over the batch; Aarray is (d, batch).  W is one workspace of
 * Wcapacity_bytes, used only when an entry does not fit on chip. */
int kmx_kronmult_vbatched_f64(int d, const int* m, const int* n, const double* const* Aarray,
                              double* const* pX, double* const* pY, double* W,
                              size_t Wcapacity_bytes, int batchCount, kmx_stream_t stream);

/* FP32 storage forms of the same four entry points (the reference's float
 * templates).  By default (form AUTO or SPLIT) each dot product is formed from
 * exact products summed as an FP32 pair and rounded once to FP32, stage by
 * stage in the reference's mode order (A1 first), which is what the
 * reference's float kernels compute by accumulating in double
 * (kgemm_nt.hpp:557-571, kgemm_nn.hpp:688-701): results agree with its float
 * build to within one FP32 ulp per element where the summation order of
 * overlapping Y blocks is the same (deterministic mode).  _ex with form PLAIN
 * runs FP32 fused multiply-add instead (faster, ~2^-24 per product), TF32X3
 * the tensor cores. */
int kmx_kronmult_batched_f32(int d, int n, const float* A, float* X, float* Y, float* W,
                             int batchCount, kmx_stream_t stream);
int kmx_kronmult_pbatched_f32(int d, int n, const float* A, float* const* pX, float* const* pY,
                              float* const* pW, int batchCount, kmx_stream_t stream);
int kmx_kronmult_xbatched_f32(int d, int n, const float* const* Aarray, int lda,
                              float* const* pX, float* const* pY, float* const* pW,
                              int batchCount, int subbatchCount, kmx_stream_t stream);
int kmx_kronmult_vbatched_f32(int d, const int* m, const int* n, const float* const* Aarray,
                              float* const* pX, float* const* pY, float* W,
                              size_t Wcapacity_bytes, int batchCount, kmx_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Extended entry points: same arguments plus options (NULL = defaults).   */
/* ---------------------------------------------------------------------- */
int kmx_kronmult_batched_f64_ex(int d, int n, const double* A, double* X, double* Y, double* W,
                                int batchCount, const kmx_options* opt, kmx_stream_t stream);
int kmx_kronmult_pbatched_f64_ex(int d, int n, const double* A, double* const* pX,
                                 double* const* pY, double* const* pW, int batchCount,
                                 const kmx_options* opt, kmx_stream_t stream);
int kmx_kronmult_xbatched_f64_ex(int d, int n, const double* const* Aarray, int lda,
                                 double* const* pX, double* const* pY, double* const* pW,
                                 int batchCount, int subbatchCount, const kmx_options* opt,
                                 kmx_stream_t stream);
int kmx_kronmult_vbatched_f64_ex(int d, const int* m, const int* n,
                                 const double* const* Aarray, double* const* pX,
                                 double* const* pY, double* W, size_t Wcapacity_bytes,
                                 int batchCount, const kmx_options* opt, kmx_stream_t stream);

int kmx_kronmult_batched_f32_ex(int d, int n, const float* A, float* X, float* Y, float* W,
                                int batchCount, const kmx_options* opt, kmx_stream_t stream);
int kmx_kronmult_pbatched_f32_ex(int d, int n, const float* A, float* const* pX, float* const* pY,
                                 float* const* pW, int batchCount, const kmx_options* opt,
                                 kmx_stream_t stream);
int kmx_kronmult_xbatched_f32_ex(int d, int n, const float* const* Aarray, int lda,
                                 float* const* pX, float* const* pY, float* const* pW,
                                 int batchCount, int subbatchCount, const kmx_options* opt,
                                 kmx_stream_t stream);
int kmx_kronmult_vbatched_f32_ex(int d, const int* m, const int* n, const float* const* Aarray,
                                 float* const* pX, float* const* pY, float* W,
                                 size_t Wcapacity_bytes, int batchCount, const kmx_options* opt,
                                 kmx_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Low-precision storage with FP64 accumulation (no counterpart in the     */
/* reference, whose float path stores and accumulates Y in FP32).          */
/* ---------------------------------------------------------------------- */
typedef enum kmx_in_type {
  KMX_IN_F32 = 1,   /* X and factors stored as FP32 */
  KMX_IN_BF16 = 2   /* X and factors stored as bfloat16 */
} kmx_in_type;

/* xbatched with X and factors of in_type, FP32 arithmetic, and each entry's
 * contribution widened exactly to FP64 and accumulated into FP64 Y blocks
 * (so many overlapping contributions sum in FP64).  Square n = 2..8 with
 * d = 3..6, and n = 16 with d = 3. */
int kmx_kronmult_xbatched_wide(int in_type, int d, int n, const void* const* Aarray, int lda,
                               const void* const* pX, double* const* pY, int batchCount,
                               const kmx_options* opt, kmx_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Construction of the xbatched arrays from index triples (no counterpart  */
/* in the reference, whose tests build them on the host,                   */
/* test_kronmult6_xbatched.cpp:253-321).                                   */
/* ---------------------------------------------------------------------- */

/* Writes, for each entry e < count, the kmx_kronmult_xbatched_* arrays
 *   pY[e]           = Ypool + y_idx[e] * y_stride
 *   pX[e]           = Xpool + x_idx[e] * x_stride
 *   Aarray[e*d + l] = Apool + l * a_level_stride + a_idx[e*d + l] * a_pool_stride
 * (strides in elements; y_idx, x_idx, a_idx are int32 device arrays; the
 * outputs are device arrays of count, count and d*count pointers).  An index
 * outside [0, n_y), [0, n_x) or [0, n_pool) yields a NULL pointer and sets
 * the device status word.  With sort_by_y nonzero the entries are first
 * ordered by y_idx (stable, on the device), which keeps the atomic updates of
 * one Y block close together in time; this needs a device workspace of
 * kmx_xbatched_build_workspace_bytes(count) bytes.  Asynchronous, no host
 * synchronisation. */
size_t kmx_xbatched_build_workspace_bytes(int count);
int kmx_xbatched_build_f64(int d, const double* Apool, long long a_level_stride,
                           long long a_pool_stride, int n_pool, const double* Xpool,
                           long long x_stride, int n_x, double* Ypool, long long y_stride, int n_y,
                           const int* y_idx, const int* x_idx, const int* a_idx, int count,
                           int sort_by_y, void* workspace, size_t workspace_bytes,
                           const double** Aarray, const double** pX, double** pY,
                           kmx_stream_t stream);
int kmx_xbatched_build_f32(int d, const float* Apool, long long a_level_stride,
                           long long a_pool_stride, int n_pool, const float* Xpool,
                           long long x_stride, int n_x, float* Ypool, long long y_stride, int n_y,
                           const int* y_idx, const int* x_idx, const int* a_idx, int count,
                           int sort_by_y, void* workspace, size_t workspace_bytes,
                           const float** Aarray, const float** pX, float** pY,
                           kmx_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Stand-alone batched tiny GEMMs (reference kgemm_nn_batched.cpp:8-41,    */
/* kgemm_nt_batched.cpp:8-41; templates kgemm_nn_batched.hpp:8-81,         */
/* kgemm_nt_batched.hpp:8-79).                                             */
/* ---------------------------------------------------------------------- */

/* For each entry e < batchCount, column-major:
 *   nn: C_e = alpha * A_e * B_e   + beta * C_e,  B_e kk x nn (ldBarray[e] >= kk)
 *   nt: C_e = alpha * A_e * B_e^T + beta * C_e,  B_e nn x kk (ldBarray[e] >= nn)
 * with A_e mm x kk (ldAarray[e] >= mm) and C_e mm x nn (ldCarray[e] >= mm).
 * The pointer arrays and the leading-dimension arrays are device arrays.
 * beta == 1 adds alpha*A*op(B) into C with atomics, so entries may share one
 * C; beta == 0 overwrites C; any other beta blends beta*C + alpha*A*op(B)
 * (entries must not share C), as the reference's epilogue does
 * (kgemm_nn.hpp:388-400, kgemm_nt.hpp:365-376).  An entry with a NULL
 * pointer or a leading dimension below its row count is skipped and flagged
 * in the device status word.  FP32 keeps each dot product as a pair of FP32
 * values (exact products, exact two-sums: about 48 bits) and rounds once when
 * stored, like the reference's accumulation of FP32 data in double. */
int kmx_kgemm_nn_batched_f64(int mm, int nn, int kk, double alpha, double* const* Aarray,
                             const int* ldAarray, double* const* Barray, const int* ldBarray,
                             double beta, double* const* Carray, const int* ldCarray,
                             int batchCount, kmx_stream_t stream);
int kmx_kgemm_nt_batched_f64(int mm, int nn, int kk, double alpha, double* const* Aarray,
                             const int* ldAarray, double* const* Barray, const int* ldBarray,
                             double beta, double* const* Carray, const int* ldCarray,
                             int batchCount, kmx_stream_t stream);
int kmx_kgemm_nn_batched_f32(int mm, int nn, int kk, float alpha, float* const* Aarray,
                             const int* ldAarray, float* const* Barray, const int* ldBarray,
                             float beta, float* const* Carray, const int* ldCarray,
                             int batchCount, kmx_stream_t stream);
int kmx_kgemm_nt_batched_f32(int mm, int nn, int kk, float alpha, float* const* Aarray,
                             const int* ldAarray, float* const* Barray, const int* ldBarray,
                             float beta, float* const* Carray, const int* ldCarray,
                             int batchCount, kmx_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Differentiation (no counterpart in the reference, which has no backward).  */
/* ---------------------------------------------------------------------- */

/* Fused forward + backward of the batched layout for loss = sum(G .* Y):
 *   Y  += (A1 x ... x Ad) X          (when Y != NULL)
 *   dX += (A1^T x ... x Ad^T) G      (when dX != NULL)
 *   dA_k += sum over the other indices of B_k[.., a, ..] F_k[.., b, ..]  (when dA != NULL)
 * with F_k = X contracted by A_l for l < k and B_k = G contracted by A_l^T for
 * l > k, recomputed on chip.  A, dA are (n,n,d,batch) column-major; X, G, Y, dX
 * are (n^d, batch).  Square n = 2..8.  W (Wcapacity_bytes) holds (d-1)*n^d
 * elements per concurrent entry when the intermediates exceed shared memory
 * (about 200 KB per entry); otherwise it may be NULL. */
/* Workspace bytes the fused kernel wants for (d, n, batchCount) on the current
 * device: 0 when the intermediates fit in shared memory (W may be NULL);
 * otherwise slots for the concurrently processed entries. */
size_t kmx_grad_workspace_bytes(int d, int n, int batchCount, int fp64);

/* FP64 arithmetic form: the library default (kmx_set_default_options), whose
 * AUTO runs the mode products and Gram sums in double-float on the FP32 pipe
 * (entries holding Inf/NaN or an all-zero X, G or factor in FP64); _ex takes
 * it from opt->form (KMX_FORM_PLAIN: native FP64).  FP32 data: FP32 FMA.
 * Kernels for FP64 data: one warp per entry, every intermediate in shared
 * memory, for d >= 3 entries whose factors and d+1 intermediates fit in 32 KB
 * (d=3 n<=8, d=4 n<=5, d=5 n<=3, d=6 n=2); otherwise one CTA per entry.
 * _ex with opt->engine = KMX_ENGINE_PER_MODE takes the CTA-per-entry kernel
 * for every shape. */
int kmx_kronmult_batched_grad_f64(int d, int n, const double* A, const double* X,
                                  const double* G, double* Y, double* dX, double* dA,
                                  double* W, size_t Wcapacity_bytes, int batchCount,
                                  kmx_stream_t stream);
int kmx_kronmult_batched_grad_f64_ex(int d, int n, const double* A, const double* X,
                                     const double* G, double* Y, double* dX, double* dA,
                                     double* W, size_t Wcapacity_bytes, int batchCount,
                                     const kmx_options* opt, kmx_stream_t stream);
int kmx_kronmult_batched_grad_f32(int d, int n, const float* A, const float* X, const float* G,
                                  float* Y, float* dX, float* dA, float* W,
                                  size_t Wcapacity_bytes, int batchCount, kmx_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Mixed shapes in one call (no counterpart in the reference, whose        */
/* vbatched takes one shape per call, kronmult_vbatched.hpp:19-248).       */
/* ---------------------------------------------------------------------- */

/* Instance i (0 <= i < count) has dims[2i] = d_i and dims[2i+1] = n_i (square
 * n_i x n_i factors, leading dimension n_i), factors Aarray[a_off[i] + l] for
 * l < d_i, and blocks pX[i], pY[i]; dims, Aarray, a_off, pX, pY are device
 * arrays.  classes is a HOST array of nclasses (d, n) pairs (<= 64) covering
 * every instance; instances of other shapes are skipped and flagged in the
 * device status word.  Instances are grouped by class on the device and each
 * class runs its tuned kernel, in the order of the class list, without a host
 * synchronisation (the call can be captured in a CUDA graph after one warm-up
 * call).  W (Wcapacity_bytes) is needed only by classes whose entries exceed
 * on-chip memory (slots of 2*n^d elements).  With deterministic accumulation
 * every class runs a generic kernel over one set of Y segments (slower than
 * the tuned kernels, bitwise reproducible). */
int kmx_kronmult_mixed_f64(int count, const int* dims, const double* const* Aarray,
                           const long long* a_off, double* const* pX, double* const* pY,
                           double* W, size_t Wcapacity_bytes, const int* classes, int nclasses,
                           const kmx_options* opt, kmx_stream_t stream);
int kmx_kronmult_mixed_f32(int count, const int* dims, const float* const* Aarray,
                           const long long* a_off, float* const* pX, float* const* pY, float* W,
                           size_t Wcapacity_bytes, const int* classes, int nclasses,
                           const kmx_options* opt, kmx_stream_t stream);

/* Rectangular shapes mixed in one call (the reference needs one
 * kronmult{d}_vbatched call per shape, kronmult_vbatched.hpp:19-248).  Class c
 * (nclasses <= 64) is the HOST record classes[13c .. 13c+12] =
 * (d, m_1..m_6, n_1..n_6), entries past d ignored: factor l is m_l x n_l with
 * leading dimension m_l, as in vbatched.  Instance i belongs to class cls[i]
 * (device array); its factors are Aarray[a_off[i] + l], its blocks pX[i]
 * (prod n_l elements) and pY[i] (prod m_l), accumulated into with atomics (pY
 * may repeat).  Instances with a class id outside [0, nclasses) are skipped
 * and flagged in the device status word.  Grouping, launch order and graph
 * capture as for kmx_kronmult_mixed_*; W slots of twice the class's largest
 * intermediate, for classes whose entries exceed on-chip memory.  Atomic or
 * deterministic accumulation (kmx_options.accumulate). */
int kmx_kronmult_vmixed_f64(int count, const int* cls, const double* const* Aarray,
                            const long long* a_off, double* const* pX, double* const* pY,
                            double* W, size_t Wcapacity_bytes, const int* classes, int nclasses,
                            const kmx_options* opt, kmx_stream_t stream);
int kmx_kronmult_vmixed_f32(int count, const int* cls, const float* const* Aarray,
                            const long long* a_off, float* const* pX, float* const* pY, float* W,
                            size_t Wcapacity_bytes, const int* classes, int nclasses,
                            const kmx_options* opt, kmx_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Library state and diagnostics.                                          */
/* ---------------------------------------------------------------------- */

/* Default options used by the drop-in entry points (process-wide). */
void kmx_set_default_options(const kmx_options* opt);
void kmx_get_default_options(kmx_options* opt);

/* Deterministic xbatched (FP64, automatic form) that allocates nothing, for
 * callers that cannot allocate device memory.  No counterpart in the
 * reference.  Its sort and segment scratch is a fixed 16 MiB array in the
 * library's device image (per GPU, held until exit); batches whose scratch
 * exceeds it return KMX_ERR_WORKSPACE before any launch.  Shapes: any square
 * shape whose entry fits in on-chip memory; one that would need a global
 * workspace for its intermediate (n = 8 with d >= 5, for example) returns
 * KMX_ERR_UNSUPPORTED, also before any launch.  The first call on a device
 * looks the array up (cudaGetSymbolAddress) and keeps the address for the
 * life of the device's primary context: make that call before any stream
 * capture, and do not use the library across cudaDeviceReset.  All calls
 * share the array, so calls overlapping on the GPU race. */
int kmx_kronmult_xbatched_f64_noalloc(int d, int n, const double* const* Aarray, int lda,
                                      double* const* pX, double* const* pY, int batchCount,
                                      kmx_stream_t stream);

/* Device workspace the deterministic mode needs for batchCount entries. */
size_t kmx_deterministic_workspace_bytes(int batchCount);

/* Bytes the library currently holds in its cached workspaces on the current
 * device (see kmx_release_workspace); 0 when none was ever needed. */
size_t kmx_cached_workspace_bytes(void);

/* Frees the library's cached deterministic-mode workspace of the current
 * device (stream-ordered on the given stream).
 *
 * Besides that workspace the library keeps two more per device: the grouping
 * arrays of kmx_kronmult_mixed_* / kmx_kronmult_vmixed_* and the digits form's
 * list of entries handed back to the double-float pass.  All three are shared
 * by every call on the device and reallocated (stream-ordered) when a larger
 * one is needed, so calls that use them must be ordered on the GPU (one
 * stream, or streams joined by events); deterministic calls that overlap can
 * pass their own kmx_options.workspace instead. */
int kmx_release_workspace(kmx_stream_t stream);

/* Reads and clears the current device's status word, written by kernels
 * that met a NULL pointer inside a pointer array or a wait that ran out.
 * Synchronises the stream.  Returns KMX_OK or KMX_ERR_DEVICE; *flags gets
 * the raw bits (may be NULL). */
int kmx_check_device_status(kmx_stream_t stream, int* flags);

/* Reads and clears the current device's diagnostic counters (no counterpart
 * in the reference).  counts[0]: entries of the double-float forms that the
 * cancellation guard recomputed in plain FP64 (an entry whose
 * rho_F = ||KX|| sqrt(prod n_l) / (prod_l ||A_l||_F ||X||) falls below 1/4,
 * where double-float's ~2^-48 relative to |K||X| would lose more accuracy than
 * FP64); counts[1]: entries the digits form handed to the double-float pass.
 * The cluster kernels (double-float entries beyond one SM's shared memory)
 * decide per block of n^(d-2) outputs and count blocks.  Synchronises the
 * stream; counts may be NULL (then only cleared). */
int kmx_read_redo_counters(kmx_stream_t stream, unsigned long long* counts);

/* The last CUDA error code seen by the library on this thread. */
int kmx_last_cuda_error(void);

/* Human-readable name of a kmx_status. */
const char* kmx_status_string(int status);

/* Flops of one entry, 2 * sum over the recursion levels (kroncommon.hpp:204-234). */
double kmx_kron_flops(int d, const int* m, const int* n);

/* Measured fused multiply-add rate of the current device (FP64 when fp64 is
 * nonzero, else FP32), in FMA per second, from a timed register-only loop.
 * Used as the denominator of the compute roofline.  Synchronises the device. */
int kmx_probe_fma_rate(int fp64, double* fma_per_second);

/* Version string of the library. */
const char* kmx_version(void);

#ifdef __cplusplus
}
#endif

#endif /* KRONMULT_GB300_H */
