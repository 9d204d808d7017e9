// Per-form launchers, one translation unit each (compiled in parallel).
#pragma once
#include <cuda_runtime.h>

namespace kmx {
struct Problem;
struct LaunchHint;
cudaError_t launch_f64_plain(Problem& p, const LaunchHint& h, cudaStream_t s);
cudaError_t launch_f64_split(Problem& p, const LaunchHint& h, cudaStream_t s);
cudaError_t launch_f32_plain(Problem& p, const LaunchHint& h, cudaStream_t s);
// Whether the FP64 forward of p needs a global workspace (an entry beyond
// shared memory), decided as the launchers decide (seg: deterministic mode).
bool needs_workspace_f64_plain(const Problem& p, bool seg, int engine);
bool needs_workspace_f64_split(const Problem& p, bool seg, int engine);
// Class shapes of a persistent mixed-shape launch, passed in the kernel's
// parameters: per class the applied factors' shapes (m_l x n_l, leading
// dimension ld_l) and the X, Y and largest intermediate lengths.
constexpr int PERSIST_MAXD = 6;
constexpr int PERSIST_MAX_CLASSES = 64;
struct PersistClass {
  int d;
  int m[PERSIST_MAXD], n[PERSIST_MAXD], ld[PERSIST_MAXD];
  long long Nx, Ny, sxw;
};
struct PersistClasses {
  int count;
  PersistClass c[PERSIST_MAX_CLASSES];
};
// Whether every class fits the persistent kernel, and the largest
// intermediate (elements) of the classes that need the workspace (0: none).
bool persistent_fits(const PersistClasses& pc, long long* ws_elems);
// One persistent launch over every instance of a mixed-shape FP64 call
// (kmx_persist.cu): p.order = instances grouped by class, keys = class of
// each instance, queue zeroed.
cudaError_t launch_mixed_persistent(Problem& p, const PersistClasses& pc, const int* keys,
                                    int* queue, cudaStream_t s);
// The xbatched FP64 problem the C ABI would run for (d, n, lda) and the form
// it would pick for `form` (KMX_FORM_*); KMX_OK or a kmx_status.
int xbatched_f64_plan(int d, int n, int lda, int form, int accumulate, bool* needs_ws);
// FP32 data, dot products rounded once (the reference's float kernels)
cudaError_t launch_f32_ref(Problem& p, const LaunchHint& h, cudaStream_t s);
cudaError_t launch_wide_f32(Problem& p, const LaunchHint& h, cudaStream_t s);
cudaError_t launch_wide_bf16(Problem& p, const LaunchHint& h, cudaStream_t s);
// FP64 digits form on the FP16 tensor cores: redo (p.count ints) and
// redo_count are device scratch for the entries handed to the double-float pass.
bool digits_supported(const Problem& p);
cudaError_t launch_f64_digits(Problem& p, const LaunchHint& h, int* redo, int* redo_count,
                              cudaStream_t s);
// Tensor-core (3xTF32) forms; cudaErrorNotSupported for shapes without a kernel.
cudaError_t launch_tc_f32(Problem& p, cudaStream_t s);
cudaError_t launch_tc_wide_f32(Problem& p, cudaStream_t s);
cudaError_t launch_tc_wide_bf16(Problem& p, cudaStream_t s);
}  // namespace kmx
