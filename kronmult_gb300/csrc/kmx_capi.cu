// kmx_capi.cu -- the C ABI (include/kronmult_gb300.h): argument validation,
// problem set-up and dispatch to the per-form launchers.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "../../include/kronmult_gb300.h"
#include "kmx_forms.h"
#include "kmx_launch.cuh"
#include "kmx_mixed.h"
#include "kmx_segments.h"
#include "kmx_tune_table.h"

namespace kmx {

// Device status word written by kernels (NULL pointer met inside a pointer
// array, a bounded wait that ran out).  Read and cleared by
// kmx_check_device_status.
__device__ int g_status_word;

// Diagnostic counters (kmx_read_redo_counters): [0] double-float entries the
// cancellation guard recomputed in FP64, [1] digits-form entries handed to the
// double-float pass.
__device__ unsigned long long g_redo_words[2];

namespace {

constexpr int MAX_DEVICES = 64;
thread_local int t_last_cuda_error = 0;

std::mutex g_mu;
DeviceInfo g_dev[MAX_DEVICES];
bool g_dev_ok[MAX_DEVICES];
int* g_status_ptr[MAX_DEVICES];
unsigned long long* g_redo_ptr[MAX_DEVICES];
std::unordered_map<const void*, size_t> g_smem_set[MAX_DEVICES];

kmx_options g_default = {KMX_FORM_AUTO, KMX_ACC_ATOMIC, 0, KMX_ENGINE_TUNED, nullptr, 0, 0, 0, 0};

// Library-owned workspaces, stream ordered, one per device and purpose
// (0: deterministic segments, 1: mixed-shape grouping, 2: digits-form redo list).
constexpr int WS_SLOTS = 3;
void* g_ws_ptr[WS_SLOTS][MAX_DEVICES];
size_t g_ws_bytes[WS_SLOTS][MAX_DEVICES];
bool g_default_init = false;

void init_defaults_locked() {
  if (g_default_init) return;
  g_default_init = true;
  const char* f = std::getenv("KMX_FORM");
  if (f) {
    if (!std::strcmp(f, "plain")) g_default.form = KMX_FORM_PLAIN;
    else if (!std::strcmp(f, "split")) g_default.form = KMX_FORM_SPLIT;
    else if (!std::strcmp(f, "auto")) g_default.form = KMX_FORM_AUTO;
  }
}

kmx_options resolve_options(const kmx_options* opt) {
  if (opt) return *opt;
  std::lock_guard<std::mutex> lk(g_mu);
  init_defaults_locked();
  return g_default;
}

int cuda_fail(cudaError_t e) {
  t_last_cuda_error = (int)e;
  return KMX_ERR_CUDA;
}

int status_ptr(int** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e);
  if (dev < 0 || dev >= MAX_DEVICES) return KMX_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_status_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_status_word);
    if (e != cudaSuccess) return cuda_fail(e);
    g_status_ptr[dev] = static_cast<int*>(p);
  }
  *out = g_status_ptr[dev];
  return KMX_OK;
}

int redo_ptr(unsigned long long** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e);
  if (dev < 0 || dev >= MAX_DEVICES) return KMX_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_redo_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_redo_words);
    if (e != cudaSuccess) return cuda_fail(e);
    g_redo_ptr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_redo_ptr[dev];
  return KMX_OK;
}

bool ipow_checked(int n, int d, long long* out) {
  long long r = 1;
  for (int i = 0; i < d; ++i) {
    r *= n;
    if (r > (1LL << 31) - 1) return false;
  }
  *out = r;
  return true;
}

int cached_workspace(int slot, size_t need, cudaStream_t s, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e);
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_ws_bytes[slot][dev] < need) {
    if (g_ws_ptr[slot][dev]) {
      e = cudaFreeAsync(g_ws_ptr[slot][dev], s);
      if (e != cudaSuccess) return cuda_fail(e);
      g_ws_ptr[slot][dev] = nullptr;
      g_ws_bytes[slot][dev] = 0;
    }
    void* p = nullptr;
    e = cudaMallocAsync(&p, need, s);
    if (e != cudaSuccess) return cuda_fail(e);
    g_ws_ptr[slot][dev] = p;
    g_ws_bytes[slot][dev] = need;
  }
  *out = g_ws_ptr[slot][dev];
  return KMX_OK;
}

}  // namespace

int device_status_ptr(int** out) { return status_ptr(out); }

DeviceInfo device_info(int dev) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev >= 0 && dev < MAX_DEVICES && g_dev_ok[dev]) return g_dev[dev];
  DeviceInfo di;
  cudaDeviceGetAttribute(&di.sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&di.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&di.max_threads_per_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  if (dev >= 0 && dev < MAX_DEVICES) {
    g_dev[dev] = di;
    g_dev_ok[dev] = true;
  }
  return di;
}

cudaError_t ensure_smem(const void* func, int dev, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  std::lock_guard<std::mutex> lk(g_mu);
  auto& m = g_smem_set[dev];
  auto it = m.find(func);
  if (it != m.end() && it->second >= bytes) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) m[func] = bytes;
  return e;
}

// Tuning-table row for (form code, layout class, d, n), layout class 0 for
// the batched layout (disjoint Y blocks), 1 for the pointer layouts (Y blocks
// may be shared, atomic accumulation); the other layout's row when the table
// has none for this one; nullptr when it has neither.
static const TuneRow* tuned_row(int form, int layout, int d, int n) {
  const TuneRow* other = nullptr;
  for (int i = 0; i < kTuneRows; ++i) {
    const TuneRow& r = kTuneTable[i];
    if (r.form != form || r.d != d || r.n != n) continue;
    if (r.layout == layout) return &r;
    other = &r;
  }
  return other;
}

static int layout_class(const Problem& p) { return p.layout == L_BATCHED ? 0 : 1; }

// The launch hint of a TUNED call: the row's engine and launch shape where
// the caller left them at 0.
static void apply_tuned(LaunchHint& h, const Problem& p, int form, const kmx_options& o) {
  if (!is_square(p)) return;
  const TuneRow* r = tuned_row(form, layout_class(p), p.d, p.n[0]);
  if (!r) return;
  h.engine = r->engine;
  if (o.group_threads == 0) h.group_threads = r->group_threads;
  if (o.groups_per_cta == 0) h.groups_per_cta = r->groups_per_cta;
  if (o.ctas_per_sm == 0) h.ctas_per_sm = r->ctas_per_sm;
}

// Tuned automatic FP64 form for (d, n): 0 when the table has no row.
static int tuned_form(int d, int n) {
  for (int i = 0; i < kAutoRows; ++i)
    if (kAutoTable[i].d == d && kAutoTable[i].n == n) return kAutoTable[i].form;
  return 0;
}

// The FP64 form a call runs: SPLIT_RAW is SPLIT without the guard; AUTO
// takes the tuning table's choice for square shapes, else double-float once
// an X or Y block has 512 elements (below that its per-entry scaling costs
// more than FP64 does).
static int resolve_f64_form(const Problem& p, int form) {
  if (form == KMX_FORM_SPLIT_RAW) return KMX_FORM_SPLIT;
  if (form != KMX_FORM_AUTO) return form;
  const bool sq = is_square(p);
  const bool spec_n = (p.n[0] >= 2 && p.n[0] <= 8) || p.n[0] == 16;
  const int t = sq ? tuned_form(p.d, p.n[0]) : 0;
  const bool gen_split = p.Nx >= 512 || p.Ny >= 512;
  return t ? t : (((sq && spec_n) || gen_split) ? KMX_FORM_SPLIT : KMX_FORM_PLAIN);
}

// Tuning-table form code of an FP64 form.
static int f64_tune_form(int form) {
  return (form == KMX_FORM_SPLIT || form == KMX_FORM_DIGITS) ? 2 : 1;
}

// The tuned engine for an FP64 form on square shapes (0 = choose).
static int f64_engine(const Problem& p, int form, int engine) {
  if (engine || !is_square(p)) return engine;
  const TuneRow* r = tuned_row(f64_tune_form(form), layout_class(p), p.d, p.n[0]);
  return r ? r->engine : 0;
}

// ---------------------------------------------------------------------------
// Common driver: validated Problem -> launcher of the requested form.
// ---------------------------------------------------------------------------
static int run_problem(Problem& p, bool is_f64, const kmx_options& o, cudaStream_t s,
                       int wide_in = 0) {
  if (o.accumulate != KMX_ACC_ATOMIC && o.accumulate != KMX_ACC_DETERMINISTIC)
    return KMX_ERR_INVALID_ARG;
  // Deterministic mode groups entries by Y block.  The contiguous batched
  // layout has one contribution per Y block and is deterministic already.
  const bool det = o.accumulate == KMX_ACC_DETERMINISTIC && p.layout != L_BATCHED;
  // The generic kernel keeps one fiber of a square middle mode in a local
  // array of GEN_MAXN elements; larger n has no code path.
  const bool spec_n = (p.n[0] >= 2 && p.n[0] <= 8) || p.n[0] == 16;
  if (!(is_square(p) && spec_n)) {
    for (int k = 1; k < p.d - 1; ++k)
      if (p.m[k] == p.n[k] && p.n[k] > GEN_MAXN) return KMX_ERR_UNSUPPORTED;
  }
  int rc = status_ptr(&p.status);
  if (rc != KMX_OK) return rc;
  rc = redo_ptr(&p.redo_ctr);
  if (rc != KMX_OK) return rc;
  // Test hook: KMX_TEST_EXPIRE_WAITS=1 makes the register-tiled kernels'
  // first wait on a staged X block report a timeout (the copy is drained and
  // DF_WAIT_TIMEOUT set, as when a wait really runs out).  Read on every call.
  {
    const char* w = std::getenv("KMX_TEST_EXPIRE_WAITS");
    p.wait_expire = (w && w[0] == '1') ? 1 : 0;
  }
  if (det && p.seg_entries) {
    p.y_exclusive = 1;  // segments prepared by the caller (mixed shapes)
  } else if (det) {
    // FP32/BF16-stored inputs with FP64 Y: register-tiled segment kernels only
    if (wide_in && (!is_square(p) || !spec_n || p.d < 3)) return KMX_ERR_UNSUPPORTED;
    const size_t need = seg_workspace_bytes(p.count);
    void* ws = o.workspace;
    size_t wsb = o.workspace_bytes;
    if (ws == nullptr) {
      rc = cached_workspace(0, need, s, &ws);
      if (rc != KMX_OK) return rc;
      wsb = need;
    } else if (wsb < need) {
      return KMX_ERR_WORKSPACE;
    }
    SegArrays sa;
    cudaError_t se = seg_prepare(reinterpret_cast<void* const*>(p.Y), p.count,
                                 p.Ny * ((is_f64 || wide_in) ? 8 : 4), ws, wsb, p.status, s, &sa);
    if (se != cudaSuccess) return cuda_fail(se);
    p.seg_entries = sa.entries;
    p.seg_offset = sa.offset;
    p.seg_count = sa.count;
    p.seg_order = sa.order;
    p.seg_num = sa.num;
    p.seg_queue = sa.queue;
    p.y_exclusive = 1;  // a segment's Y block belongs to one group
  }
  LaunchHint h = {};
  h.group_threads = o.group_threads;
  h.groups_per_cta = o.groups_per_cta;
  h.ctas_per_sm = o.ctas_per_sm;
  static const int engine_env = [] {
    const char* e = std::getenv("KMX_ENGINE");
    return e ? std::atoi(e) : 0;
  }();
  h.engine = o.engine ? o.engine : engine_env;
  if (h.engine == KMX_ENGINE_PERSISTENT) h.engine = 0;  // mixed-shape calls only
  if (h.engine == KMX_ENGINE_CLUSTER && !is_f64) h.engine = 0;
  cudaError_t e;
  const bool sq = is_square(p);
  if (wide_in) {
    e = cudaErrorNotSupported;
    if (o.form == KMX_FORM_TF32X3)
      e = wide_in == KMX_IN_BF16 ? launch_tc_wide_bf16(p, s) : launch_tc_wide_f32(p, s);
    if (e == cudaErrorNotSupported)
      e = wide_in == KMX_IN_BF16 ? launch_wide_bf16(p, h, s) : launch_wide_f32(p, h, s);
  } else if (!is_f64) {
    // FP32 data.  AUTO / SPLIT: the reference's float semantics (each dot
    // product accumulated exactly enough and rounded once, stage by stage in
    // its mode order); PLAIN: FP32 fused multiply-add (fastest); TF32X3:
    // tensor cores where a kernel exists, else PLAIN.
    e = cudaErrorNotSupported;
    if (o.form == KMX_FORM_TF32X3) e = launch_tc_f32(p, s);
    if (e == cudaErrorNotSupported) {
      if (o.form == KMX_FORM_AUTO || o.form == KMX_FORM_SPLIT) {
        e = launch_f32_ref(p, h, s);
      } else if (o.form == KMX_FORM_PLAIN || o.form == KMX_FORM_TF32X3) {
        if (h.engine == 0) apply_tuned(h, p, 3, o);
        e = launch_f32_plain(p, h, s);
      } else {
        return KMX_ERR_INVALID_ARG;
      }
    }
  } else {
    if (o.form == KMX_FORM_SPLIT_RAW) p.guard_off = 1;
    int form = resolve_f64_form(p, o.form);
    // the cluster engine exists for double-float entries beyond one SM's
    // shared memory (square d=5 n=8, d=6 n=6..8); elsewhere it is TUNED
    if (h.engine == KMX_ENGINE_CLUSTER &&
        !(sq && form == KMX_FORM_SPLIT &&
          ((p.d == 5 && p.n[0] == 8) || (p.d == 6 && p.n[0] >= 6 && p.n[0] <= 8))))
      h.engine = 0;
    if (h.engine == 0) apply_tuned(h, p, f64_tune_form(form), o);
    if (form == KMX_FORM_DIGITS) {
      e = cudaErrorNotSupported;
      if (digits_supported(p)) {
        void* ws = nullptr;
        rc = cached_workspace(2, ((size_t)p.count + 64) * sizeof(int), s, &ws);
        if (rc != KMX_OK) return rc;
        int* redo_count = static_cast<int*>(ws);
        e = launch_f64_digits(p, h, redo_count + 64, redo_count, s);
      }
      if (e == cudaErrorNotSupported) form = KMX_FORM_SPLIT;
    }
    if (form == KMX_FORM_DIGITS) {
      // launched above
    } else if (form == KMX_FORM_SPLIT) {
      e = launch_f64_split(p, h, s);
      if (e == cudaErrorNotSupported) e = launch_f64_plain(p, h, s);
    } else if (form == KMX_FORM_PLAIN) {
      e = launch_f64_plain(p, h, s);
    } else {
      return KMX_ERR_INVALID_ARG;
    }
  }
  if (e == cudaErrorInvalidValue) return KMX_ERR_WORKSPACE;
  if (e == cudaErrorNotSupported) return KMX_ERR_UNSUPPORTED;
  if (e != cudaSuccess) return cuda_fail(e);
  return KMX_OK;
}

static void base_square(Problem& p, int layout, int d, int n, int ld, long long N);

int xbatched_f64_plan(int d, int n, int lda, int form, int accumulate, bool* needs_ws) {
  if (d < 1 || d > MAXD || n < 1) return KMX_ERR_INVALID_ARG;
  if (lda == 0) lda = n;
  if (lda < n) return KMX_ERR_INVALID_ARG;
  long long N;
  if (!ipow_checked(n, d, &N)) return KMX_ERR_UNSUPPORTED;
  Problem p;
  base_square(p, L_XBATCHED, d, n, lda, N);
  const int f = resolve_f64_form(p, form);
  const bool seg = accumulate == KMX_ACC_DETERMINISTIC;
  const int engine = f64_engine(p, f, 0);
  *needs_ws = (f == KMX_FORM_PLAIN) ? needs_workspace_f64_plain(p, seg, engine)
                                    : needs_workspace_f64_split(p, seg, engine);
  return KMX_OK;
}

static void base_square(Problem& p, int layout, int d, int n, int ld, long long N) {
  std::memset(&p, 0, sizeof(p));
  p.layout = layout;
  p.d = d;
  for (int l = 0; l < MAXD; ++l) {
    p.m[l] = (l < d) ? n : 1;
    p.n[l] = (l < d) ? n : 1;
    p.ld[l] = (l < d) ? ld : 1;
  }
  p.Nx = p.Ny = p.sxw = N;
}

template <typename T>
static int batched_impl(int d, int n, const T* A, T* X, T* Y, T* W, int batch, const kmx_options* opt,
                        cudaStream_t s) {
  if (d < 1 || d > MAXD || n < 1 || batch < 0) return KMX_ERR_INVALID_ARG;
  if (batch == 0) return KMX_OK;
  if (!A || !X || !Y) return KMX_ERR_NULL_POINTER;
  long long N;
  if (!ipow_checked(n, d, &N)) return KMX_ERR_UNSUPPORTED;
  kmx_options o = resolve_options(opt);
  Problem p;
  base_square(p, L_BATCHED, d, n, n, N);
  p.count = batch;
  p.A = A;
  p.X = X;
  p.Y = Y;
  p.trans = o.transpose;
  p.y_exclusive = 1;  // Y(:,k) are disjoint columns
  if (W) {
    p.wmode = 3;
    p.Wbase = W;
    p.w_stride = N;
    p.nslots = batch;
  }
  return run_problem(p, sizeof(T) == 8, o, s);
}

template <typename T>
static int pbatched_impl(int d, int n, const T* A, T* const* pX, T* const* pY, T* const* pW, int batch,
                         const kmx_options* opt, cudaStream_t s) {
  if (d < 1 || d > MAXD || n < 1 || batch < 0) return KMX_ERR_INVALID_ARG;
  if (batch == 0) return KMX_OK;
  if (!A || !pX || !pY) return KMX_ERR_NULL_POINTER;
  long long N;
  if (!ipow_checked(n, d, &N)) return KMX_ERR_UNSUPPORTED;
  kmx_options o = resolve_options(opt);
  Problem p;
  base_square(p, L_PBATCHED, d, n, n, N);
  p.count = batch;
  p.A = A;
  p.X = pX;
  p.Y = const_cast<T**>(pY);
  p.trans = o.transpose;
  if (pW) {
    p.wmode = 1;
    p.pW = reinterpret_cast<void* const*>(pW);
    p.nslots = batch;
  }
  return run_problem(p, sizeof(T) == 8, o, s);
}

template <typename T>
static int xbatched_impl(int d, int n, const T* const* Aarray, int lda, T* const* pX, T* const* pY,
                         T* const* pW, int batch, int sub, const kmx_options* opt, cudaStream_t s) {
  if (d < 1 || d > MAXD || n < 1 || batch < 0 || sub < 0) return KMX_ERR_INVALID_ARG;
  if (lda == 0) lda = n;
  if (lda < n) return KMX_ERR_INVALID_ARG;
  if (batch == 0) return KMX_OK;
  if (!Aarray || !pX || !pY) return KMX_ERR_NULL_POINTER;
  long long N;
  if (!ipow_checked(n, d, &N)) return KMX_ERR_UNSUPPORTED;
  kmx_options o = resolve_options(opt);
  Problem p;
  base_square(p, L_XBATCHED, d, n, lda, N);
  p.count = batch;
  p.A = Aarray;
  p.X = pX;
  p.Y = const_cast<T**>(pY);
  p.trans = o.transpose;
  if (pW) {
    // Workspace slots exactly as the reference lays them out
    // (kronmult_xbatched.hpp:121-126): pairs pW[2*iz], pW[2*iz+1] for
    // iz < subbatchCount when batch > 1; pW[0] when batch == 1.
    if (sub == 0) sub = (batch / 2 > 1) ? batch / 2 : 1;
    if (batch > 1) {
      p.wmode = 2;
      p.nslots = sub;
    } else {
      p.wmode = 1;
      p.nslots = 1;
    }
    p.pW = reinterpret_cast<void* const*>(pW);
  }
  return run_problem(p, sizeof(T) == 8, o, s);
}

// Rectangular shape of one call or class: applied operator A_l (m_l x n_l),
// or A_l^T (n_l x m_l) when transposed, stored with ld = m_l (the reference's
// vbatched convention, kronmult_vbatched.hpp:206-211).
static int rect_problem(Problem& p, int layout, int d, const int* m, const int* n,
                        const kmx_options& o) {
  if (d < 1 || d > MAXD || !m || !n) return KMX_ERR_INVALID_ARG;
  for (int l = 0; l < d; ++l)
    if (m[l] < 1 || n[l] < 1) return KMX_ERR_INVALID_ARG;
  std::memset(&p, 0, sizeof(p));
  p.layout = layout;
  p.d = d;
  for (int l = 0; l < MAXD; ++l) {
    const int ml = (l < d) ? m[l] : 1, nl = (l < d) ? n[l] : 1;
    p.m[l] = o.transpose ? nl : ml;
    p.n[l] = o.transpose ? ml : nl;
    p.ld[l] = ml;
  }
  long long Nx = 1, Ny = 1, sxw = 0;
  for (int l = 0; l < d; ++l) {
    Nx *= p.n[l];
    Ny *= p.m[l];
    if (Nx > (1LL << 31) - 1 || Ny > (1LL << 31) - 1) return KMX_ERR_UNSUPPORTED;
  }
  // largest intermediate m1..mk * n(k+1)..nd (kronmult_vbatched.hpp:136-153)
  sxw = Nx;
  for (int k = 1; k <= d; ++k) {
    long long sz = 1;
    for (int l = 0; l < k; ++l) sz *= p.m[l];
    for (int l = k; l < d; ++l) sz *= p.n[l];
    if (sz > sxw) sxw = sz;
  }
  p.Nx = Nx;
  p.Ny = Ny;
  p.sxw = sxw;
  p.trans = o.transpose;
  bool square = true;
  for (int l = 0; l < d; ++l) square = square && (p.m[l] == p.n[0] && p.n[l] == p.n[0]);
  if (!square) {
    for (int l = 0; l < d; ++l)
      if (p.m[l] == p.n[l] && p.n[l] > GEN_MAXN) return KMX_ERR_UNSUPPORTED;
  }
  return KMX_OK;
}

// The caller's workspace W (Wcap bytes) as slots of two sxw buffers.
template <typename T>
static void rect_workspace(Problem& p, T* W, size_t Wcap, int count) {
  if (W && Wcap > 0) {
    const size_t slot_bytes = 2 * (size_t)p.sxw * sizeof(T);
    p.wmode = 3;
    p.Wbase = W;
    p.w_stride = 2 * p.sxw;
    p.nslots = (int)((Wcap / slot_bytes) < (size_t)count ? (Wcap / slot_bytes) : (size_t)count);
  }
}

template <typename T>
static int vbatched_impl(int d, const int* m, const int* n, const T* const* Aarray, T* const* pX,
                         T* const* pY, T* W, size_t Wcap, int batch, const kmx_options* opt,
                         cudaStream_t s) {
  if (d < 1 || d > MAXD || batch < 0 || !m || !n) return KMX_ERR_INVALID_ARG;
  for (int l = 0; l < d; ++l)
    if (m[l] < 1 || n[l] < 1) return KMX_ERR_INVALID_ARG;
  if (batch == 0) return KMX_OK;
  if (!Aarray || !pX || !pY) return KMX_ERR_NULL_POINTER;
  kmx_options o = resolve_options(opt);
  Problem p;
  int rc = rect_problem(p, L_VBATCHED, d, m, n, o);
  if (rc != KMX_OK) return rc;
  p.count = batch;
  p.A = Aarray;
  p.X = pX;
  p.Y = const_cast<T**>(pY);
  rect_workspace(p, W, Wcap, batch);
  return run_problem(p, sizeof(T) == 8, o, s);
}

// xbatched with FP32/BF16 inputs and an FP64 Y (register-tiled shapes).
static int xbatched_wide_impl(int in_type, int d, int n, const void* const* Aarray, int lda,
                              const void* const* pX, double* const* pY, int batch,
                              const kmx_options* opt, cudaStream_t s) {
  if (in_type != KMX_IN_F32 && in_type != KMX_IN_BF16) return KMX_ERR_INVALID_ARG;
  if (d < 1 || d > MAXD || n < 1 || batch < 0) return KMX_ERR_INVALID_ARG;
  if (lda == 0) lda = n;
  if (lda < n) return KMX_ERR_INVALID_ARG;
  if (batch == 0) return KMX_OK;
  if (!Aarray || !pX || !pY) return KMX_ERR_NULL_POINTER;
  long long N;
  if (!ipow_checked(n, d, &N)) return KMX_ERR_UNSUPPORTED;
  kmx_options o = resolve_options(opt);
  Problem p;
  base_square(p, L_XBATCHED, d, n, lda, N);
  p.count = batch;
  p.A = Aarray;
  p.X = pX;
  p.Y = const_cast<double**>(pY);
  p.trans = o.transpose;
  return run_problem(p, false, o, s, in_type);
}

// The persistent engine (kmx_persist.cu) for a mixed-shape call, FP64 only:
// KMX_OK or an error, or PERSIST_SKIP when a class does not fit its kernel
// (the caller then launches class by class).
constexpr int PERSIST_SKIP = -1;

static void persist_class(const Problem& q, PersistClass* c) {
  c->d = q.d;
  for (int l = 0; l < MAXD; ++l) {
    c->m[l] = q.m[l];
    c->n[l] = q.n[l];
    c->ld[l] = q.ld[l];
  }
  c->Nx = q.Nx;
  c->Ny = q.Ny;
  c->sxw = q.sxw;
}

template <typename T>
static int run_persistent(const PersistClasses& pc, int count, const MixedArrays& ma,
                          const long long* a_off, const T* const* Aarray, T* const* pX,
                          T* const* pY, T* W, size_t Wcap, const kmx_options& o, int* status,
                          cudaStream_t s) {
  long long ws_elems = 0;
  if (!persistent_fits(pc, &ws_elems)) return PERSIST_SKIP;
  Problem p;
  base_square(p, L_MIXED, 1, 2, 2, 2);
  p.count = count;
  p.order = ma.order;
  p.a_off = a_off;
  p.A = Aarray;
  p.X = pX;
  p.Y = const_cast<T**>(pY);
  p.trans = o.transpose;
  p.status = status;
  int rc = redo_ptr(&p.redo_ctr);
  if (rc != KMX_OK) return rc;
  if (ws_elems > 0 && W && Wcap > 0) {
    p.Wbase = W;
    p.w_stride = 2 * ws_elems;
    const size_t slots = Wcap / (2 * (size_t)ws_elems * sizeof(T));
    p.nslots = (int)(slots < (size_t)count ? slots : (size_t)count);
  }
  const cudaError_t e = launch_mixed_persistent(p, pc, ma.keys, ma.queue, s);
  if (e == cudaErrorInvalidValue) return KMX_ERR_WORKSPACE;
  if (e == cudaErrorNotSupported) return PERSIST_SKIP;
  return e == cudaSuccess ? KMX_OK : cuda_fail(e);
}

// Deterministic mixed-shape calls: one set of segments over every instance,
// Y blocks of ybytes[c] bytes for class c, handed to each class's launch
// (which takes only its own entries, EntryStream).
template <typename T>
static int mixed_segments(int count, T* const* pY, const MixedArrays& ma, const long long* ybytes,
                          int nclasses, const kmx_options& o, int* status, cudaStream_t s,
                          SegArrays* sa) {
  const size_t need = seg_workspace_bytes(count);
  void* ws = o.workspace;
  size_t wsb = o.workspace_bytes;
  if (ws == nullptr) {
    const int rc = cached_workspace(0, need, s, &ws);
    if (rc != KMX_OK) return rc;
    wsb = need;
  } else if (wsb < need) {
    return KMX_ERR_WORKSPACE;
  }
  SegClassBytes cb{};
  for (int c = 0; c < nclasses && c < 64; ++c) cb.bytes[c] = ybytes[c];
  const cudaError_t e = seg_prepare(reinterpret_cast<void* const*>(pY), count, 0, ws, wsb, status,
                                    s, sa, ma.keys, &cb);
  return e == cudaSuccess ? KMX_OK : cuda_fail(e);
}

static void use_segments(Problem& p, const SegArrays& sa, const MixedArrays& ma, int c) {
  p.seg_entries = sa.entries;
  p.seg_offset = sa.offset;
  p.seg_count = sa.count;
  p.seg_order = sa.order;
  p.seg_num = sa.num;
  p.seg_queue = sa.queue;
  p.seg_key = ma.keys;
  p.seg_class = c;
}

// One call over instances of mixed (d, n): group by class on the device,
// then one tuned launch per class reading its range from device memory.
template <typename T>
static int mixed_impl(int count, const int* dims, const T* const* Aarray, const long long* a_off,
                      T* const* pX, T* const* pY, T* W, size_t Wcap, const int* classes,
                      int nclasses, const kmx_options* opt, cudaStream_t s) {
  if (count < 0 || nclasses < 1 || nclasses > KMX_MAX_CLASSES || !classes)
    return KMX_ERR_INVALID_ARG;
  if (count == 0) return KMX_OK;
  if (!dims || !Aarray || !a_off || !pX || !pY) return KMX_ERR_NULL_POINTER;
  for (int c = 0; c < nclasses; ++c) {
    const int d = classes[2 * c], n = classes[2 * c + 1];
    long long N;
    if (d < 1 || d > MAXD || n < 1) return KMX_ERR_INVALID_ARG;
    if (!ipow_checked(n, d, &N)) return KMX_ERR_UNSUPPORTED;
  }
  kmx_options o = resolve_options(opt);
  if (o.accumulate != KMX_ACC_ATOMIC && o.accumulate != KMX_ACC_DETERMINISTIC)
    return KMX_ERR_INVALID_ARG;
  const bool det = o.accumulate == KMX_ACC_DETERMINISTIC;
  int* status = nullptr;
  int rc = status_ptr(&status);
  if (rc != KMX_OK) return rc;
  void* ws = nullptr;
  const size_t need = mixed_workspace_bytes(count);
  rc = cached_workspace(1, need, s, &ws);
  if (rc != KMX_OK) return rc;
  MixedArrays ma;
  cudaError_t e = mixed_prepare(count, dims, nullptr, classes, nclasses, ws, need, status, s, &ma);
  if (e != cudaSuccess) return cuda_fail(e);
  if (o.engine == KMX_ENGINE_PERSISTENT && sizeof(T) == 8 && !det &&
      (o.form == KMX_FORM_AUTO || o.form == KMX_FORM_SPLIT)) {
    PersistClasses pc;
    pc.count = nclasses;
    for (int c = 0; c < nclasses; ++c) {
      Problem q;
      long long N = 0;
      ipow_checked(classes[2 * c + 1], classes[2 * c], &N);  // checked above
      base_square(q, L_MIXED, classes[2 * c], classes[2 * c + 1], classes[2 * c + 1], N);
      persist_class(q, &pc.c[c]);
    }
    rc = run_persistent(pc, count, ma, a_off, Aarray, pX, pY, W, Wcap, o, status, s);
    if (rc != PERSIST_SKIP) return rc;
  }
  SegArrays sa{};
  if (det) {
    long long yb[KMX_MAX_CLASSES];
    for (int c = 0; c < nclasses; ++c) {
      long long N = 0;
      ipow_checked(classes[2 * c + 1], classes[2 * c], &N);
      yb[c] = N * (long long)sizeof(T);
    }
    rc = mixed_segments(count, pY, ma, yb, nclasses, o, status, s, &sa);
    if (rc != KMX_OK) return rc;
  }
  for (int c = 0; c < nclasses; ++c) {
    const int d = classes[2 * c], n = classes[2 * c + 1];
    long long N = 0;
    ipow_checked(n, d, &N);  // checked for every class above
    Problem p;
    base_square(p, L_MIXED, d, n, n, N);
    if (det) use_segments(p, sa, ma, c);
    p.count = count;  // upper bound for the grid; the kernels read the class count
    p.count_dev = ma.counts + c;
    p.order = ma.order;
    p.order_base = ma.offsets + c;
    p.a_off = a_off;
    p.A = Aarray;
    p.X = pX;
    p.Y = const_cast<T**>(pY);
    p.trans = o.transpose;
    if (W && Wcap > 0) {
      const size_t slot_bytes = 2 * (size_t)N * sizeof(T);
      p.wmode = 3;
      p.Wbase = W;
      p.w_stride = 2 * N;
      p.sxw = N;
      const size_t slots = Wcap / slot_bytes;
      p.nslots = (int)(slots < (size_t)count ? slots : (size_t)count);
    }
    rc = run_problem(p, sizeof(T) == 8, o, s);
    if (rc != KMX_OK) return rc;
  }
  return KMX_OK;
}

// One call over instances of mixed rectangular shapes: instance i belongs to
// class cls[i]; class c is the host record classes[13c..13c+12] =
// (d, m_1..m_6, n_1..n_6).  Grouped on the device like mixed_impl, then one
// launch per class.
template <typename T>
static int vmixed_impl(int count, const int* cls, const T* const* Aarray, const long long* a_off,
                       T* const* pX, T* const* pY, T* W, size_t Wcap, const int* classes,
                       int nclasses, const kmx_options* opt, cudaStream_t s) {
  if (count < 0 || nclasses < 1 || nclasses > KMX_MAX_CLASSES || !classes)
    return KMX_ERR_INVALID_ARG;
  kmx_options o = resolve_options(opt);
  for (int c = 0; c < nclasses; ++c) {
    Problem p;
    const int* r = classes + 13 * c;
    const int rc = rect_problem(p, L_MIXED, r[0], r + 1, r + 7, o);
    if (rc != KMX_OK) return rc;
  }
  if (count == 0) return KMX_OK;
  if (!cls || !Aarray || !a_off || !pX || !pY) return KMX_ERR_NULL_POINTER;
  if (o.accumulate != KMX_ACC_ATOMIC && o.accumulate != KMX_ACC_DETERMINISTIC)
    return KMX_ERR_INVALID_ARG;
  const bool det = o.accumulate == KMX_ACC_DETERMINISTIC;
  int* status = nullptr;
  int rc = status_ptr(&status);
  if (rc != KMX_OK) return rc;
  void* ws = nullptr;
  const size_t need = mixed_workspace_bytes(count);
  rc = cached_workspace(1, need, s, &ws);
  if (rc != KMX_OK) return rc;
  MixedArrays ma;
  cudaError_t e = mixed_prepare(count, nullptr, cls, nullptr, nclasses, ws, need, status, s, &ma);
  if (e != cudaSuccess) return cuda_fail(e);
  if (o.engine == KMX_ENGINE_PERSISTENT && sizeof(T) == 8 && !det &&
      (o.form == KMX_FORM_AUTO || o.form == KMX_FORM_SPLIT)) {
    PersistClasses pc;
    pc.count = nclasses;
    for (int c = 0; c < nclasses; ++c) {
      Problem q;
      const int* r = classes + 13 * c;
      rect_problem(q, L_MIXED, r[0], r + 1, r + 7, o);  // checked above
      persist_class(q, &pc.c[c]);
    }
    rc = run_persistent(pc, count, ma, a_off, Aarray, pX, pY, W, Wcap, o, status, s);
    if (rc != PERSIST_SKIP) return rc;
  }
  SegArrays sa{};
  if (det) {
    long long yb[KMX_MAX_CLASSES];
    for (int c = 0; c < nclasses; ++c) {
      Problem q;
      const int* r = classes + 13 * c;
      rect_problem(q, L_MIXED, r[0], r + 1, r + 7, o);
      yb[c] = q.Ny * (long long)sizeof(T);
    }
    rc = mixed_segments(count, pY, ma, yb, nclasses, o, status, s, &sa);
    if (rc != KMX_OK) return rc;
  }
  for (int c = 0; c < nclasses; ++c) {
    const int* r = classes + 13 * c;
    Problem p;
    rect_problem(p, L_MIXED, r[0], r + 1, r + 7, o);
    if (det) use_segments(p, sa, ma, c);
    p.count = count;  // upper bound for the grid; the kernels read the class count
    p.count_dev = ma.counts + c;
    p.order = ma.order;
    p.order_base = ma.offsets + c;
    p.a_off = a_off;
    p.A = Aarray;
    p.X = pX;
    p.Y = const_cast<T**>(pY);
    rect_workspace(p, W, Wcap, count);
    rc = run_problem(p, sizeof(T) == 8, o, s);
    if (rc != KMX_OK) return rc;
  }
  return KMX_OK;
}

}  // namespace kmx

using namespace kmx;

#define KMX_STREAM(s) reinterpret_cast<cudaStream_t>(s)

extern "C" {

int kmx_kronmult_batched_f64(int d, int n, const double* A, double* X, double* Y, double* W,
                             int batchCount, kmx_stream_t stream) {
  return batched_impl<double>(d, n, A, X, Y, W, batchCount, nullptr, KMX_STREAM(stream));
}
int kmx_kronmult_batched_f64_ex(int d, int n, const double* A, double* X, double* Y, double* W,
                                int batchCount, const kmx_options* opt, kmx_stream_t stream) {
  return batched_impl<double>(d, n, A, X, Y, W, batchCount, opt, KMX_STREAM(stream));
}
int kmx_kronmult_batched_f32(int d, int n, const float* A, float* X, float* Y, float* W,
                             int batchCount, kmx_stream_t stream) {
  return batched_impl<float>(d, n, A, X, Y, W, batchCount, nullptr, KMX_STREAM(stream));
}

int kmx_kronmult_batched_f32_ex(int d, int n, const float* A, float* X, float* Y, float* W,
                                int batchCount, const kmx_options* opt, kmx_stream_t stream) {
  return batched_impl<float>(d, n, A, X, Y, W, batchCount, opt, KMX_STREAM(stream));
}

int kmx_kronmult_pbatched_f64(int d, int n, const double* A, double* const* pX, double* const* pY,
                              double* const* pW, int batchCount, kmx_stream_t stream) {
  return pbatched_impl<double>(d, n, A, pX, pY, pW, batchCount, nullptr, KMX_STREAM(stream));
}
int kmx_kronmult_pbatched_f64_ex(int d, int n, const double* A, double* const* pX,
                                 double* const* pY, double* const* pW, int batchCount,
                                 const kmx_options* opt, kmx_stream_t stream) {
  return pbatched_impl<double>(d, n, A, pX, pY, pW, batchCount, opt, KMX_STREAM(stream));
}
int kmx_kronmult_pbatched_f32(int d, int n, const float* A, float* const* pX, float* const* pY,
                              float* const* pW, int batchCount, kmx_stream_t stream) {
  return pbatched_impl<float>(d, n, A, pX, pY, pW, batchCount, nullptr, KMX_STREAM(stream));
}

int kmx_kronmult_pbatched_f32_ex(int d, int n, const float* A, float* const* pX, float* const* pY,
                                 float* const* pW, int batchCount, const kmx_options* opt,
                                 kmx_stream_t stream) {
  return pbatched_impl<float>(d, n, A, pX, pY, pW, batchCount, opt, KMX_STREAM(stream));
}

int kmx_kronmult_xbatched_f64(int d, int n, const double* const* Aarray, int lda,
                              double* const* pX, double* const* pY, double* const* pW,
                              int batchCount, int subbatchCount, kmx_stream_t stream) {
  return xbatched_impl<double>(d, n, Aarray, lda, pX, pY, pW, batchCount, subbatchCount, nullptr,
                               KMX_STREAM(stream));
}
int kmx_kronmult_xbatched_f64_ex(int d, int n, const double* const* Aarray, int lda,
                                 double* const* pX, double* const* pY, double* const* pW,
                                 int batchCount, int subbatchCount, const kmx_options* opt,
                                 kmx_stream_t stream) {
  return xbatched_impl<double>(d, n, Aarray, lda, pX, pY, pW, batchCount, subbatchCount, opt,
                               KMX_STREAM(stream));
}
int kmx_kronmult_xbatched_f32(int d, int n, const float* const* Aarray, int lda, float* const* pX,
                              float* const* pY, float* const* pW, int batchCount, int subbatchCount,
                              kmx_stream_t stream) {
  return xbatched_impl<float>(d, n, Aarray, lda, pX, pY, pW, batchCount, subbatchCount, nullptr,
                              KMX_STREAM(stream));
}

int kmx_kronmult_xbatched_f32_ex(int d, int n, const float* const* Aarray, int lda,
                                 float* const* pX, float* const* pY, float* const* pW,
                                 int batchCount, int subbatchCount, const kmx_options* opt,
                                 kmx_stream_t stream) {
  return xbatched_impl<float>(d, n, Aarray, lda, pX, pY, pW, batchCount, subbatchCount, opt,
                              KMX_STREAM(stream));
}

int kmx_kronmult_vbatched_f64(int d, const int* m, const int* n, const double* const* Aarray,
                              double* const* pX, double* const* pY, double* W,
                              size_t Wcapacity_bytes, int batchCount, kmx_stream_t stream) {
  return vbatched_impl<double>(d, m, n, Aarray, pX, pY, W, Wcapacity_bytes, batchCount, nullptr,
                               KMX_STREAM(stream));
}
int kmx_kronmult_vbatched_f64_ex(int d, const int* m, const int* n, const double* const* Aarray,
                                 double* const* pX, double* const* pY, double* W,
                                 size_t Wcapacity_bytes, int batchCount, const kmx_options* opt,
                                 kmx_stream_t stream) {
  return vbatched_impl<double>(d, m, n, Aarray, pX, pY, W, Wcapacity_bytes, batchCount, opt,
                               KMX_STREAM(stream));
}
int kmx_kronmult_vbatched_f32(int d, const int* m, const int* n, const float* const* Aarray,
                              float* const* pX, float* const* pY, float* W, size_t Wcapacity_bytes,
                              int batchCount, kmx_stream_t stream) {
  return vbatched_impl<float>(d, m, n, Aarray, pX, pY, W, Wcapacity_bytes, batchCount, nullptr,
                              KMX_STREAM(stream));
}

int kmx_kronmult_vbatched_f32_ex(int d, const int* m, const int* n, const float* const* Aarray,
                                 float* const* pX, float* const* pY, float* W,
                                 size_t Wcapacity_bytes, int batchCount, const kmx_options* opt,
                                 kmx_stream_t stream) {
  return vbatched_impl<float>(d, m, n, Aarray, pX, pY, W, Wcapacity_bytes, batchCount, opt,
                              KMX_STREAM(stream));
}

int kmx_kronmult_mixed_f64(int count, const int* dims, const double* const* Aarray,
                           const long long* a_off, double* const* pX, double* const* pY,
                           double* W, size_t Wcapacity_bytes, const int* classes, int nclasses,
                           const kmx_options* opt, kmx_stream_t stream) {
  return mixed_impl<double>(count, dims, Aarray, a_off, pX, pY, W, Wcapacity_bytes, classes,
                            nclasses, opt, KMX_STREAM(stream));
}

int kmx_kronmult_mixed_f32(int count, const int* dims, const float* const* Aarray,
                           const long long* a_off, float* const* pX, float* const* pY, float* W,
                           size_t Wcapacity_bytes, const int* classes, int nclasses,
                           const kmx_options* opt, kmx_stream_t stream) {
  return mixed_impl<float>(count, dims, Aarray, a_off, pX, pY, W, Wcapacity_bytes, classes,
                           nclasses, opt, KMX_STREAM(stream));
}

int kmx_kronmult_vmixed_f64(int count, const int* cls, const double* const* Aarray,
                            const long long* a_off, double* const* pX, double* const* pY,
                            double* W, size_t Wcapacity_bytes, const int* classes, int nclasses,
                            const kmx_options* opt, kmx_stream_t stream) {
  return vmixed_impl<double>(count, cls, Aarray, a_off, pX, pY, W, Wcapacity_bytes, classes,
                             nclasses, opt, KMX_STREAM(stream));
}

int kmx_kronmult_vmixed_f32(int count, const int* cls, const float* const* Aarray,
                            const long long* a_off, float* const* pX, float* const* pY, float* W,
                            size_t Wcapacity_bytes, const int* classes, int nclasses,
                            const kmx_options* opt, kmx_stream_t stream) {
  return vmixed_impl<float>(count, cls, Aarray, a_off, pX, pY, W, Wcapacity_bytes, classes,
                            nclasses, opt, KMX_STREAM(stream));
}

int kmx_kronmult_xbatched_wide(int in_type, int d, int n, const void* const* Aarray, int lda,
                               const void* const* pX, double* const* pY, int batchCount,
                               const kmx_options* opt, kmx_stream_t stream) {
  return xbatched_wide_impl(in_type, d, n, Aarray, lda, pX, pY, batchCount, opt,
                            KMX_STREAM(stream));
}

size_t kmx_deterministic_workspace_bytes(int batchCount) {
  return batchCount > 0 ? seg_workspace_bytes(batchCount) : 0;
}

size_t kmx_cached_workspace_bytes(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return 0;
  std::lock_guard<std::mutex> lk(g_mu);
  size_t total = 0;
  for (int slot = 0; slot < WS_SLOTS; ++slot) total += g_ws_bytes[slot][dev];
  return total;
}

int kmx_release_workspace(kmx_stream_t stream) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e);
  std::lock_guard<std::mutex> lk(g_mu);
  for (int slot = 0; slot < WS_SLOTS; ++slot) {
    if (g_ws_ptr[slot][dev]) {
      e = cudaFreeAsync(g_ws_ptr[slot][dev], KMX_STREAM(stream));
      g_ws_ptr[slot][dev] = nullptr;
      g_ws_bytes[slot][dev] = 0;
      if (e != cudaSuccess) return cuda_fail(e);
    }
  }
  return KMX_OK;
}

void kmx_set_default_options(const kmx_options* opt) {
  if (!opt) return;
  std::lock_guard<std::mutex> lk(g_mu);
  init_defaults_locked();
  g_default = *opt;
}

void kmx_get_default_options(kmx_options* opt) {
  if (!opt) return;
  std::lock_guard<std::mutex> lk(g_mu);
  init_defaults_locked();
  *opt = g_default;
}

int kmx_check_device_status(kmx_stream_t stream, int* flags) {
  int* sp = nullptr;
  int rc = status_ptr(&sp);
  if (rc != KMX_OK) return rc;
  int host = 0;
  cudaError_t e = cudaMemcpyAsync(&host, sp, sizeof(int), cudaMemcpyDeviceToHost, KMX_STREAM(stream));
  if (e == cudaSuccess) e = cudaStreamSynchronize(KMX_STREAM(stream));
  if (e != cudaSuccess) return cuda_fail(e);
  if (host != 0) {
    const int zero = 0;
    e = cudaMemcpyAsync(sp, &zero, sizeof(int), cudaMemcpyHostToDevice, KMX_STREAM(stream));
    if (e == cudaSuccess) e = cudaStreamSynchronize(KMX_STREAM(stream));
    if (e != cudaSuccess) return cuda_fail(e);
  }
  if (flags) *flags = host;
  return host ? KMX_ERR_DEVICE : KMX_OK;
}

int kmx_read_redo_counters(kmx_stream_t stream, unsigned long long* counts) {
  unsigned long long* dp = nullptr;
  int rc = redo_ptr(&dp);
  if (rc != KMX_OK) return rc;
  unsigned long long host[2] = {0, 0};
  cudaError_t e =
      cudaMemcpyAsync(host, dp, sizeof(host), cudaMemcpyDeviceToHost, KMX_STREAM(stream));
  if (e == cudaSuccess) e = cudaStreamSynchronize(KMX_STREAM(stream));
  if (e != cudaSuccess) return cuda_fail(e);
  e = cudaMemsetAsync(dp, 0, sizeof(host), KMX_STREAM(stream));
  if (e == cudaSuccess) e = cudaStreamSynchronize(KMX_STREAM(stream));
  if (e != cudaSuccess) return cuda_fail(e);
  if (counts) {
    counts[0] = host[0];
    counts[1] = host[1];
  }
  return KMX_OK;
}

int kmx_last_cuda_error(void) { return t_last_cuda_error; }

const char* kmx_status_string(int status) {
  switch (status) {
    case KMX_OK: return "KMX_OK";
    case KMX_ERR_INVALID_ARG: return "KMX_ERR_INVALID_ARG";
    case KMX_ERR_NULL_POINTER: return "KMX_ERR_NULL_POINTER";
    case KMX_ERR_WORKSPACE: return "KMX_ERR_WORKSPACE";
    case KMX_ERR_UNSUPPORTED: return "KMX_ERR_UNSUPPORTED";
    case KMX_ERR_CUDA: return "KMX_ERR_CUDA";
    case KMX_ERR_DEVICE: return "KMX_ERR_DEVICE";
    case KMX_ERR_OVERLAP: return "KMX_ERR_OVERLAP";
    default: return "KMX_UNKNOWN_STATUS";
  }
}

double kmx_kron_flops(int d, const int* m, const int* n) {
  // kroncommon.hpp:204-234: level 1 costs 2*n2..nd*n1*m1, then m1 vectors recurse
  if (d <= 0 || !m || !n) return 0.0;
  if (d == 1) return 2.0 * m[0] * n[0];
  double rest = 1.0;
  for (int l = 1; l < d; ++l) rest *= n[l];
  return 2.0 * rest * n[0] * m[0] + kmx_kron_flops(d - 1, m + 1, n + 1) * m[0];
}

const char* kmx_version(void) { return "kronmult-gb300 0.1 (sm_103a)"; }

}  // extern "C"
