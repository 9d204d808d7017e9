// kmx_launch.cuh -- host-side launch logic shared by the per-form translation
// units: picks the kernel for a shape, sizes shared memory and the grid.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <type_traits>
#include <unordered_map>

#include "kmx_cluster.cuh"
#include "kmx_engine.cuh"
#include "kmx_lane.cuh"
#include "kmx_small.cuh"
#include "kmx_tile.cuh"

namespace kmx {

// FORM_REF32: FP32 data, each dot product rounded once (the reference's float
// semantics), per-mode kernels only (they apply the modes in the reference's
// order, A1 first, rounding each stage to FP32 as it does).
enum Form : int { FORM_PLAIN = 1, FORM_SPLIT = 2, FORM_WIDE = 3, FORM_REF32 = 4 };

// Execution shape requested by the caller (0 = choose).
struct LaunchHint {
  int group_threads;   // per-mode kernels: threads per entry group (0 = default)
  int groups_per_cta;  // entry groups per CTA (0 = default)
  int max_ctas;        // cap on the grid (0 = fill the GPU)
  int engine;          // 0 choose, 1 per-mode, 2 register-tiled, 3 small-entry, 5 cluster,
                       // 6 one entry per thread
  int ctas_per_sm;     // cap on the resident CTAs per SM the grid is sized for (0 = occupancy)
};

struct DeviceInfo {
  int sms = 0;
  int max_smem_optin = 0;
  int max_threads_per_sm = 0;
};

DeviceInfo device_info(int dev);
// Device address of the library's status word on the current device (KMX_OK or an error).
int device_status_ptr(int** out);
// Raise a kernel's dynamic shared-memory limit once per (kernel, device).
cudaError_t ensure_smem(const void* func, int dev, size_t bytes);

inline size_t align16(size_t x) { return (x + 15) / 16 * 16; }

inline bool is_square(const Problem& p) {
  for (int l = 0; l < p.d; ++l)
    if (p.m[l] != p.n[0] || p.n[l] != p.n[0]) return false;
  return true;
}

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// Threads per entry: about four work items per lane in the widest mode.
inline int default_group_threads(long long N, int nn) {
  long long items = N / (nn > 0 ? nn : 1);
  long long g = (items + 3) / 4;
  if (g < 32) g = 32;
  if (g > 256) g = (N >= 16384) ? 512 : 256;
  return round_up((int)g, 32);
}

template <typename T, int FORM, int NN, bool GB>
const void* sq_kernel() {
  if constexpr (FORM == FORM_SPLIT) {
    return reinterpret_cast<const void*>(&sq_split_kernel<NN, GB>);
  } else if constexpr (FORM == FORM_REF32) {
    return reinterpret_cast<const void*>(&sq_plain_kernel<T, NN, GB, true>);
  } else {
    return reinterpret_cast<const void*>(&sq_plain_kernel<T, NN, GB>);
  }
}

template <typename T, int FORM, bool GB>
const void* pick_sq(int nn) {
  switch (nn) {
    case 2: return sq_kernel<T, FORM, 2, GB>();
    case 3: return sq_kernel<T, FORM, 3, GB>();
    case 4: return sq_kernel<T, FORM, 4, GB>();
    case 5: return sq_kernel<T, FORM, 5, GB>();
    case 6: return sq_kernel<T, FORM, 6, GB>();
    case 7: return sq_kernel<T, FORM, 7, GB>();
    case 8: return sq_kernel<T, FORM, 8, GB>();
    case 16: return sq_kernel<T, FORM, 16, GB>();
    default: return nullptr;
  }
}

// ---------------------------------------------------------------------------
// Register-tiled kernels (kmx_tile.cuh) for square NN in 2..8, d in 3..6,
// where one entry's intermediate fits in shared memory.
// ---------------------------------------------------------------------------
template <typename T, int FORM, int NN, int D>
struct TilePol {
  using type = tile::PlainPolicy<T>;
};
// Double-float on packed FP32 pairs where it measured faster on GB300 (same
// box, same build, batched layout): even n <= 8 with one tile per thread in
// the first phase, e.g. d=6 n=4 +10 %, d=3 n=8 +19 %, d=4 n=6 +11 %.  Odd n
// pads a zero row to every row pair (a third more arithmetic for n = 3:
// d=5 n=3 -16 %), and with several tiles per thread the packed operands
// spill (d=5 n=7 -16 %, d=5 n=5 -11 %): those keep the scalar form, as does
// n = 16, whose broadcast operands would not fit in registers.
template <typename T, int NN, int D>
struct TilePol<T, FORM_SPLIT, NN, D> {
  using type = typename std::conditional<tile::packed_pays(NN, D), tile::PackedSplitPolicy,
                                         tile::SplitPolicy>::type;
};
// FP32 / BF16 storage, FP32 arithmetic, FP64 Y (T is the storage type)
template <typename T, int NN, int D>
struct TilePol<T, FORM_WIDE, NN, D> {
  using type = tile::WidePolicy<T>;
};

struct TileKernel {
  const void* func = nullptr;
  int group_threads = 0;
  int group_smem = 0;
  int cta_threads = 0;  // the kernel's launch bound: groups_per_cta * group_threads <= this
};

template <typename T, int FORM, int NN, int D, bool SEG>
TileKernel tile_entry() {
  using Pol = typename TilePol<T, FORM, NN, D>::type;
  TileKernel k;
  constexpr int bytes = tile::group_smem_bytes<Pol, NN, D, SEG>();
  if constexpr (bytes <= 227 * 1024) {
    k.func = reinterpret_cast<const void*>(&tile::tile_kernel<Pol, NN, D, SEG>);
    k.group_threads = tile::group_threads(NN, D);
    k.group_smem = bytes;
    k.cta_threads = tile::cta_threads(NN, D);
  }
  return k;
}

template <typename T, int FORM, int NN, bool SEG>
TileKernel tile_for_d(int d) {
  switch (d) {
    case 3: return tile_entry<T, FORM, NN, 3, SEG>();
    case 4: return tile_entry<T, FORM, NN, 4, SEG>();
    case 5: return tile_entry<T, FORM, NN, 5, SEG>();
    case 6: return tile_entry<T, FORM, NN, 6, SEG>();
    default: return TileKernel();
  }
}

// Register-tiled kernel for (nn, d); SEG selects the deterministic
// segment-queue variant.  func == nullptr when none exists.
template <typename T, int FORM, bool SEG = false>
TileKernel pick_tile(int nn, int d) {
  switch (nn) {
    case 2: return tile_for_d<T, FORM, 2, SEG>(d);
    case 3: return tile_for_d<T, FORM, 3, SEG>(d);
    case 4: return tile_for_d<T, FORM, 4, SEG>(d);
    case 5: return tile_for_d<T, FORM, 5, SEG>(d);
    case 6: return tile_for_d<T, FORM, 6, SEG>(d);
    case 7: return tile_for_d<T, FORM, 7, SEG>(d);
    case 8: return tile_for_d<T, FORM, 8, SEG>(d);
    case 16: return d == 3 ? tile_entry<T, FORM, 16, 3, SEG>() : TileKernel();
    default: return TileKernel();
  }
}

// Launch a register-tiled kernel; grid fills the GPU by occupancy.
inline cudaError_t launch_tile(Problem& p, const TileKernel& k, const LaunchHint& hint,
                               cudaStream_t stream) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  const DeviceInfo di = device_info(dev);
  const int G = k.group_threads;
  int E = hint.groups_per_cta > 0 ? hint.groups_per_cta : (G >= 256 ? 1 : 256 / G);
  while (E > 1 && (size_t)E * k.group_smem > (size_t)di.max_smem_optin) --E;
  while (E > 1 && E * G > k.cta_threads) --E;
  if (E > p.count) E = p.count;
  const size_t smem = (size_t)E * k.group_smem;
  err = ensure_smem(k.func, dev, smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.func, E * G, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (hint.ctas_per_sm > 0 && per_sm > hint.ctas_per_sm) per_sm = hint.ctas_per_sm;
  const long long want = ((long long)p.count + E - 1) / E;
  long long cap = (long long)di.sms * per_sm;
  if (hint.max_ctas > 0 && cap > hint.max_ctas) cap = hint.max_ctas;
  const int grid = (int)(want < cap ? want : cap);
  p.group_threads = G;
  p.groups_per_cta = E;
  p.group_smem = k.group_smem;
  void* args[] = {&p};
  return cudaLaunchKernel(k.func, dim3(grid), dim3(E * G), args, smem, stream);
}

// ---------------------------------------------------------------------------
// Small-entry kernels (kmx_small.cuh): d <= 3, n^d <= 256, many entries per CTA.
// ---------------------------------------------------------------------------
template <typename T, int FORM>
struct SmallPol {
  using type = small::SmallPlain<T, false>;
};
template <typename T>
struct SmallPol<T, FORM_SPLIT> {
  using type = small::SmallSplit;
};
template <typename T>
struct SmallPol<T, FORM_REF32> {
  using type = small::SmallPlain<T, true>;
};

struct SmallKernel {
  const void* func = nullptr;
  int smem = 0;
};

template <typename T, int FORM, int NN, int D>
SmallKernel small_entry() {
  SmallKernel k;
  if constexpr (small::supported(NN, D)) {
    using Pol = typename SmallPol<T, FORM>::type;
    k.func = reinterpret_cast<const void*>(&small::small_kernel<Pol, NN, D>);
    k.smem = small::Layout<Pol, NN, D>::BYTES;
  }
  return k;
}

template <typename T, int FORM, int NN>
SmallKernel small_for_d(int d) {
  switch (d) {
    case 1: return small_entry<T, FORM, NN, 1>();
    case 2: return small_entry<T, FORM, NN, 2>();
    case 3: return small_entry<T, FORM, NN, 3>();
    default: return SmallKernel();
  }
}

template <typename T, int FORM>
SmallKernel pick_small(int nn, int d) {
  if constexpr (FORM == FORM_WIDE) {
    return SmallKernel();
  } else {
    switch (nn) {
      case 2: return small_for_d<T, FORM, 2>(d);
      case 3: return small_for_d<T, FORM, 3>(d);
      case 4: return small_for_d<T, FORM, 4>(d);
      case 5: return small_for_d<T, FORM, 5>(d);
      case 6: return small_for_d<T, FORM, 6>(d);
      case 7: return small_for_d<T, FORM, 7>(d);
      case 8: return small_for_d<T, FORM, 8>(d);
      case 16: return small_for_d<T, FORM, 16>(d);
      default: return SmallKernel();
    }
  }
}

inline cudaError_t launch_small(Problem& p, const SmallKernel& k, const LaunchHint& hint,
                                cudaStream_t stream) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  const DeviceInfo di = device_info(dev);
  err = ensure_smem(k.func, dev, k.smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.func, small::THREADS, k.smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (hint.ctas_per_sm > 0 && per_sm > hint.ctas_per_sm) per_sm = hint.ctas_per_sm;
  long long cap = (long long)di.sms * per_sm;
  if (hint.max_ctas > 0 && cap > hint.max_ctas) cap = hint.max_ctas;
  // chunks of the launch: an upper bound when the count is on the device
  const int grid = (int)(cap < (long long)p.count ? cap : (p.count > 0 ? p.count : 1));
  void* args[] = {&p};
  return cudaLaunchKernel(k.func, dim3(grid), dim3(small::THREADS), args, k.smem, stream);
}

// ---------------------------------------------------------------------------
// The lane engine (kmx_lane.cuh): one entry per thread for n^2 <= 16,
// n^d <= 16; one group of n lanes per entry for d = 2 with n = 5..8; one
// group of n^(d-1) <= 32 lanes per entry (a fiber per lane) for d >= 3.
// ---------------------------------------------------------------------------
template <typename T, int FORM>
struct LanePol {
  using type = lane::LanePlain<T, false>;
};
template <typename T>
struct LanePol<T, FORM_SPLIT> {
  using type = lane::LaneSplit;
};
template <typename T>
struct LanePol<T, FORM_REF32> {
  using type = lane::LanePlain<T, true>;
};

struct LaneKernel {
  const void* func = nullptr;
  int threads = 0;
  int per_cta = 0;  // entries one CTA takes at a time
};

template <typename T, int FORM, int NN, int D>
LaneKernel lane_entry() {
  LaneKernel k;
  if constexpr (FORM != FORM_WIDE && (FORM != FORM_SPLIT || std::is_same<T, double>::value)) {
    using Pol = typename LanePol<T, FORM>::type;
    if constexpr (lane::supported(NN, D)) {
      k.func = reinterpret_cast<const void*>(&lane::lane_kernel<Pol, NN, D>);
      k.threads = lane::THREADS;
      k.per_cta = lane::THREADS;
    } else if constexpr (lane::group::supported(NN, D)) {
      k.func = reinterpret_cast<const void*>(&lane::group::group_kernel<Pol, NN>);
      k.threads = lane::group::THREADS;
      k.per_cta = lane::group::WARPS * lane::group::Layout<Pol, NN>::GPW;
    } else if constexpr (lane::fiber::supported(NN, D)) {
      k.func = reinterpret_cast<const void*>(&lane::fiber::fiber_kernel<Pol, NN, D>);
      k.threads = lane::fiber::THREADS;
      k.per_cta = lane::fiber::WARPS * lane::fiber::Layout<Pol, NN, D>::GPW;
    }
  }
  return k;
}

template <typename T, int FORM>
LaneKernel pick_lane(int nn, int d) {
  switch (nn * 10 + d) {
    case 21: return lane_entry<T, FORM, 2, 1>();
    case 31: return lane_entry<T, FORM, 3, 1>();
    case 41: return lane_entry<T, FORM, 4, 1>();
    case 22: return lane_entry<T, FORM, 2, 2>();
    case 32: return lane_entry<T, FORM, 3, 2>();
    case 42: return lane_entry<T, FORM, 4, 2>();
    case 52: return lane_entry<T, FORM, 5, 2>();
    case 62: return lane_entry<T, FORM, 6, 2>();
    case 72: return lane_entry<T, FORM, 7, 2>();
    case 82: return lane_entry<T, FORM, 8, 2>();
    case 23: return lane_entry<T, FORM, 2, 3>();
    case 33: return lane_entry<T, FORM, 3, 3>();
    case 43: return lane_entry<T, FORM, 4, 3>();
    case 53: return lane_entry<T, FORM, 5, 3>();
    case 24: return lane_entry<T, FORM, 2, 4>();
    case 34: return lane_entry<T, FORM, 3, 4>();
    case 25: return lane_entry<T, FORM, 2, 5>();
    case 26: return lane_entry<T, FORM, 2, 6>();
    default: return LaneKernel();
  }
}

inline cudaError_t launch_lane(Problem& p, const LaneKernel& k, const LaunchHint& hint,
                               cudaStream_t stream) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  const DeviceInfo di = device_info(dev);
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.func, k.threads, 0);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (hint.ctas_per_sm > 0 && per_sm > hint.ctas_per_sm) per_sm = hint.ctas_per_sm;
  long long cap = (long long)di.sms * per_sm;
  if (hint.max_ctas > 0 && cap > hint.max_ctas) cap = hint.max_ctas;
  // CTAs of per_cta entries (an upper bound when the count is on the device)
  const long long want = p.count > 0 ? ((long long)p.count + k.per_cta - 1) / k.per_cta : 1;
  const int grid = (int)(cap < want ? cap : want);
  void* args[] = {&p};
  return cudaLaunchKernel(k.func, dim3(grid), dim3(k.threads), args, 0, stream);
}

// ---------------------------------------------------------------------------
// Cluster kernels (kmx_cluster.cuh): double-float entries beyond one SM's
// shared memory, n CTAs per (entry, i1) sharing mode 2 through distributed
// shared memory.
// ---------------------------------------------------------------------------
struct ClusterKernel {
  const void* func = nullptr;
  int smem = 0;
  int threads = 0;
  int cluster = 0;
};

template <int NN, int D>
ClusterKernel cluster_entry() {
  ClusterKernel k;
  if constexpr (clus::supported(NN, D)) {
    k.func = reinterpret_cast<const void*>(&clus::cluster_kernel<NN, D>);
    k.smem = clus::Layout<NN, D>::BYTES;
    k.threads = clus::cta_threads(NN, D);
    k.cluster = NN;
  }
  return k;
}

// The cluster kernel for (nn, d): the shapes whose entries exceed the
// register-tiled kernel's shared memory.
inline ClusterKernel pick_cluster(int nn, int d) {
  switch (nn * 10 + d) {
    case 85: return cluster_entry<8, 5>();
    case 66: return cluster_entry<6, 6>();
    case 76: return cluster_entry<7, 6>();
    case 86: return cluster_entry<8, 6>();
    default: return ClusterKernel();
  }
}

inline cudaError_t launch_cluster(Problem& p, const ClusterKernel& k, const LaunchHint& hint,
                                  cudaStream_t stream) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  err = ensure_smem(k.func, dev, k.smem);
  if (err != cudaSuccess) return err;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)k.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)k.cluster);
  cfg.blockDim = dim3((unsigned)k.threads);
  cfg.dynamicSmemBytes = (size_t)k.smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int active = 0;
  err = cudaOccupancyMaxActiveClusters(&active, k.func, &cfg);
  if (err != cudaSuccess) return err;
  if (active < 1) return cudaErrorInvalidConfiguration;
  const long long want = (long long)p.count * k.cluster;  // (entry, i1) items
  long long nclusters = active;
  if (hint.max_ctas > 0 && nclusters * k.cluster > hint.max_ctas)
    nclusters = hint.max_ctas / k.cluster > 0 ? hint.max_ctas / k.cluster : 1;
  if (nclusters > want) nclusters = want;
  cfg.gridDim = dim3((unsigned)(nclusters * k.cluster));
  void* args[] = {&p};
  return cudaLaunchKernelExC(&cfg, k.func, args);
}

// Bytes of shared memory one group needs (on-chip intermediate included).
template <typename T, int FORM>
size_t sq_group_smem(const Problem& p, bool gbuf) {
  const int nn = p.n[0];
  size_t head = (FORM == FORM_SPLIT) ? sq_split_head(nn) : align16(MAXD * nn * nn * sizeof(T));
  size_t buf = (p.d >= 2 && !gbuf) ? align16((size_t)p.Nx * (FORM == FORM_SPLIT ? 8 : sizeof(T))) : 0;
  return head + buf;
}

template <typename T>
size_t gen_group_smem(const Problem& p, bool gbuf) {
  size_t fac = 0;
  for (int l = 0; l < p.d; ++l) fac += (size_t)p.m[l] * p.n[l];
  size_t head = align16(fac * sizeof(T));
  if (gbuf || p.d < 2) return head;
  // square modes work in place: one buffer; rectangular ones ping-pong: two
  return head + (is_square(p) ? 1 : 2) * align16((size_t)p.sxw * sizeof(T));
}

// Generic split kernel.  Rows per lane and buffers, as measured on GB300
// (d = 2..6, n = 3..32): entries of 4096 or more elements take four rows per
// lane and, where every mode but the last is square with n <= 16 and one
// buffer fits, work in place (the fiber a lane holds is reused for four
// rows); smaller entries take two rows per lane and ping-pong between two
// buffers.
inline bool gen_split_wide(const Problem& p) { return p.Nx >= 4096 || p.Ny >= 4096; }

// [factors as pairs][exponents and guard sums, GEN_SPLIT_HDR bytes][one or
// two buffers].  X itself is split into the first buffer, so d = 1 needs one too.
inline size_t gen_split_group_smem(const Problem& p, bool gbuf, size_t limit) {
  size_t fac = 0;
  for (int l = 0; l < p.d; ++l) fac += (size_t)p.m[l] * p.n[l];
  const size_t head = align16(fac * 8) + GEN_SPLIT_HDR;
  if (gbuf) return head;
  const size_t b = align16((size_t)p.sxw * 8);
  bool one_ok = true;
  for (int k = 0; k + 1 < p.d; ++k) one_ok = one_ok && gen_split_in_place(p.m[k], p.n[k]);
  if (one_ok && (gen_split_wide(p) || head + 2 * b > limit)) return head + b;
  return head + 2 * b;
}

// Whether launch_forward would need a global workspace for p (an entry too
// large for shared memory), decided as it decides, without launching.  seg:
// the deterministic (segment) mode; engine: the LaunchHint engine.
template <typename T, int FORM>
bool needs_workspace(const Problem& p, bool seg, int engine) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return true;
  const DeviceInfo di = device_info(dev);
  const bool square = is_square(p);
  const int nn = p.n[0];
  if constexpr (FORM != FORM_REF32) {
    if (seg && square && !p.seg_key && pick_tile<T, FORM, true>(nn, p.d).func) return false;
    if (!seg && square && engine != 1 && pick_tile<T, FORM>(nn, p.d).func) return false;
  }
  if constexpr (FORM == FORM_SPLIT) {
    if (!seg && square && pick_cluster(nn, p.d).func) return false;
  }
  if constexpr (FORM == FORM_WIDE) {
    return false;
  } else {
    const bool spec = !seg && square && pick_sq<T, FORM, false>(nn) != nullptr;
    size_t gsm;
    if (spec) {
      gsm = sq_group_smem<T, FORM>(p, false);
    } else if constexpr (FORM == FORM_SPLIT) {
      gsm = gen_split_group_smem(p, false, di.max_smem_optin);
    } else {
      gsm = gen_group_smem<T>(p, false);
    }
    return gsm > (size_t)di.max_smem_optin;
  }
}

// Launch one forward pass over p.count entries.  Returns cudaSuccess, or the
// CUDA error of the launch; cudaErrorInvalidValue when the shape needs a
// global workspace that p does not provide.
template <typename T, int FORM>
cudaError_t launch_forward(Problem& p, const LaunchHint& hint, cudaStream_t stream) {
  if (p.count <= 0) return cudaSuccess;
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  const DeviceInfo di = device_info(dev);
  const bool square = is_square(p);
  const int nn = p.n[0];
  const bool seg = p.seg_entries != nullptr;
  if (!seg && square && hint.engine == 3) {
    const SmallKernel sk = pick_small<T, FORM>(nn, p.d);
    if (sk.func) return launch_small(p, sk, hint, stream);
  }
  if (!seg && square && hint.engine == 6) {
    const LaneKernel lk = pick_lane<T, FORM>(nn, p.d);
    if (lk.func) return launch_lane(p, lk, hint, stream);
  }
  if constexpr (FORM != FORM_REF32) {
    if (seg) {
      // deterministic mode: the register-tiled segment kernels where they
      // exist, else the generic kernels walking whole segments (EntryStream)
      // (class-filtered segments of mixed-shape calls: generic kernels only)
      const TileKernel tk = square && !p.seg_key ? pick_tile<T, FORM, true>(nn, p.d) : TileKernel();
      if (tk.func) return launch_tile(p, tk, hint, stream);
    }
    if (!seg && square) {
      const TileKernel tk = hint.engine != 1 ? pick_tile<T, FORM>(nn, p.d) : TileKernel();
      if (tk.func) return launch_tile(p, tk, hint, stream);
      if constexpr (FORM == FORM_SPLIT) {
        // entries beyond one SM's shared memory: a cluster per (entry, i1)
        // when no workspace is given (or the cluster engine is asked for);
        // with a workspace the per-mode kernels below run faster
        const bool no_ws = p.wmode == 0 || p.nslots <= 0;
        const ClusterKernel ck = (no_ws || hint.engine == 5) ? pick_cluster(nn, p.d) : ClusterKernel();
        if (ck.func) return launch_cluster(p, ck, hint, stream);
      }
    }
  }
  if constexpr (FORM == FORM_WIDE) {
    return cudaErrorNotSupported;  // register-tiled shapes only (handled above)
  } else {
  // the square per-mode kernels take entries grid-stride only
  const bool spec = !seg && square && pick_sq<T, FORM, false>(nn) != nullptr;
  auto group_smem = [&](bool gb) -> size_t {
    if (spec) return sq_group_smem<T, FORM>(p, gb);
    if constexpr (FORM == FORM_SPLIT) return gen_split_group_smem(p, gb, di.max_smem_optin);
    return gen_group_smem<T>(p, gb);
  };
  bool gbuf = false;
  size_t gsm = group_smem(false);
  if (gsm > (size_t)di.max_smem_optin) {
    gbuf = true;
    gsm = group_smem(true);
    if (p.wmode == 0 || p.nslots <= 0) return cudaErrorInvalidValue;
  }
  const void* func = nullptr;
  if (spec) {
    func = gbuf ? pick_sq<T, FORM, true>(nn) : pick_sq<T, FORM, false>(nn);
  } else if constexpr (FORM == FORM_SPLIT) {
    if (gen_split_wide(p)) {
      func = gbuf ? reinterpret_cast<const void*>(&gen_split_kernel<true, 4>)
                  : reinterpret_cast<const void*>(&gen_split_kernel<false, 4>);
    } else {
      func = gbuf ? reinterpret_cast<const void*>(&gen_split_kernel<true, 2>)
                  : reinterpret_cast<const void*>(&gen_split_kernel<false, 2>);
    }
  } else if constexpr (FORM == FORM_REF32) {
    func = gbuf ? reinterpret_cast<const void*>(&gen_plain_kernel<T, true, true>)
                : reinterpret_cast<const void*>(&gen_plain_kernel<T, false, true>);
  } else {
    func = gbuf ? reinterpret_cast<const void*>(&gen_plain_kernel<T, true>)
                : reinterpret_cast<const void*>(&gen_plain_kernel<T, false>);
  }

  int G = hint.group_threads > 0 ? hint.group_threads : default_group_threads(p.Nx > p.Ny ? p.Nx : p.Ny, spec ? nn : 1);
  // a generic split entry that holds more than half of the shared memory runs
  // alone on its SM: give it every thread
  if (FORM == FORM_SPLIT && !spec && hint.group_threads <= 0 && 2 * gsm > (size_t)di.max_smem_optin)
    G = MAX_THREADS;
  // small generic split entries: two 128-thread groups per CTA, each on its
  // own barrier, so that one group's barriers overlap the other's work
  // (measured on GB300 against one 256-thread group: +8 to +23 % on the
  // rectangular shapes; four 64-thread groups lose, shared memory then
  // holding half the threads per SM)
  if (FORM == FORM_SPLIT && !spec && hint.group_threads <= 0 && !gen_split_wide(p) && G > 128)
    G = 128;
  if (G > MAX_THREADS) G = MAX_THREADS;
  G = round_up(G, 32);
  int E = hint.groups_per_cta > 0 ? hint.groups_per_cta : (256 / G > 0 ? 256 / G : 1);
  if (gbuf) E = 1;
  while (E > 1 && (size_t)E * gsm > (size_t)di.max_smem_optin) --E;
  while (E > 1 && E * G > MAX_THREADS) --E;
  // never more groups per CTA than entries
  if (E > p.count) E = p.count;
  const size_t smem = (size_t)E * gsm;
  err = ensure_smem(func, dev, smem);
  if (err != cudaSuccess) return err;

  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, E * G, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) per_sm = 1;
  if (hint.ctas_per_sm > 0 && per_sm > hint.ctas_per_sm) per_sm = hint.ctas_per_sm;
  long long want = ((long long)p.count + E - 1) / E;
  long long cap = (long long)di.sms * per_sm;
  if (hint.max_ctas > 0 && cap > hint.max_ctas) cap = hint.max_ctas;
  if (gbuf) {
    long long slot_cap = p.nslots / E;
    if (slot_cap < 1) return cudaErrorInvalidValue;
    if (cap > slot_cap) cap = slot_cap;
  }
  const int grid = (int)(want < cap ? want : cap);

  p.group_threads = G;
  p.groups_per_cta = E;
  p.group_smem = (int)gsm;
  void* args[] = {&p};
  return cudaLaunchKernel(func, dim3(grid), dim3(E * G), args, smem, stream);
  }
}

}  // namespace kmx
