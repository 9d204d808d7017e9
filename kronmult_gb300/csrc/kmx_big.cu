// kmx_big.cu -- entries beyond one SM (square n = 8, d = 5, 6: 256 KB and
// 2 MB per FP64 block) in two register-tiled passes instead of d per-mode
// passes over a global intermediate.
//
// With a = d - 3 leading modes and 3 trailing modes, an X block is a
// (8^a x 512) row-major matrix Xm and
//   Y += (A_0 x .. x A_{a-1}) Xm (A_a x A_{a+1} x A_{a+2})^T.
// Pass 1: every row r of Xm (512 contiguous values) is a 3-mode problem with
//   the trailing factors; its 512 outputs go to a scratch block W in a
//   column-blocked layout W[c / 8][r][c % 8] (blocked Y layout of the tiled
//   kernel: inner 8, outer stride 8^a * 8).
// Pass 2: every block of 8 columns of W (8^a * 8 contiguous values) is an
//   (a + 1)-mode problem with the leading factors and the 8 x 8 identity as
//   its last factor; its outputs land in Y rows of 8 contiguous values
//   (blocked Y layout: inner 8, outer stride 512).
// Both passes run the double-float tiled kernels (3 and a + 1 modes fit on
// chip).  The identity mode adds 17-20 % flops; each W element receives one
// contribution (exact), Y is accumulated into as usual.  Entries are taken in
// chunks so that W stays within a bounded workspace.
#include <cuda_runtime.h>

#include "../../include/kronmult_gb300.h"
#include "kmx_forms.h"
#include "kmx_launch.cuh"
#include "kmx_tile.cuh"

namespace kmx {
namespace {

constexpr int BN = 8;                  // n of the shapes this path takes
constexpr long long ROW = 512;         // 8^3: one row of Xm
constexpr size_t W_BUDGET = 512ull << 20;  // bytes of W per chunk

struct BigPtrs {
  const double** a1;  // pass 1: 3 factors per sub-entry
  const double** x1;
  double** y1;
  const double** a2;  // pass 2: a + 1 factors per sub-entry
  const double** x2;
  double** y2;
  double* ident;      // 8 x 8 identity
};

// One thread per pass-1 sub-entry (row) of the chunk; rows 0 of each entry
// also write that entry's pass-2 sub-entries.
__global__ void big_build_kernel(const Problem p, int a, long long e0, int cnt, double* W,
                                 long long wstride, BigPtrs b) {
  const long long rows = 1LL << (3 * a);  // 8^a
  const long long total = (long long)cnt * rows;
  if (blockIdx.x == 0 && threadIdx.x < BN * BN)
    b.ident[threadIdx.x] = (threadIdx.x % BN) == (threadIdx.x / BN) ? 1.0 : 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long el = i / rows, r = i - el * rows;
    const long long ent = tile::entry_index(p, e0 + el);
    const double* xp = tile::x_ptr<double>(p, ent);
    double* wb = W + el * wstride;
    b.x1[i] = xp ? xp + r * ROW : nullptr;
    b.y1[i] = wb + r * BN;
    for (int j = 0; j < 3; ++j) b.a1[i * 3 + j] = tile::a_ptr<double>(p, ent, a + j);
    if (r < ROW / BN) {
      // pass-2 sub-entry: column block r of this entry
      const long long s2 = el * (ROW / BN) + r;
      double* yp = tile::y_ptr<double>(p, ent);
      b.x2[s2] = wb + r * rows * BN;
      b.y2[s2] = yp ? yp + r * BN : nullptr;
      for (int j = 0; j < a; ++j) b.a2[s2 * (a + 1) + j] = tile::a_ptr<double>(p, ent, j);
      b.a2[s2 * (a + 1) + a] = b.ident;
    }
  }
}

inline size_t al256(size_t x) { return (x + 255) / 256 * 256; }

struct BigLayout {
  long long chunk;  // entries per chunk
  size_t w, a1, x1, y1, a2, x2, y2, ident, total;
};

BigLayout big_layout(int d, int count) {
  BigLayout L;
  const int a = d - 3;
  const long long N = 1LL << (3 * d);
  const long long rows = 1LL << (3 * a);
  long long chunk = (long long)(W_BUDGET / ((size_t)N * 8));
  if (chunk < 1) chunk = 1;
  if (chunk > count) chunk = count;
  L.chunk = chunk;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += al256(bytes);
    return at;
  };
  L.w = take((size_t)chunk * N * 8);
  L.a1 = take((size_t)chunk * rows * 3 * 8);
  L.x1 = take((size_t)chunk * rows * 8);
  L.y1 = take((size_t)chunk * rows * 8);
  L.a2 = take((size_t)chunk * (ROW / BN) * (a + 1) * 8);
  L.x2 = take((size_t)chunk * (ROW / BN) * 8);
  L.y2 = take((size_t)chunk * (ROW / BN) * 8);
  L.ident = take(BN * BN * 8);
  L.total = o;
  return L;
}

}  // namespace

bool big_supported(const Problem& p) {
  return is_square(p) && p.n[0] == BN && (p.d == 5 || p.d == 6) && !p.seg_entries &&
         !p.count_dev && p.y_inner == 0;
}

size_t big_workspace_bytes(int d, int count) { return big_layout(d, count).total; }

cudaError_t launch_big_split(Problem& p, const LaunchHint& h2, const LaunchHint& h1, void* ws,
                             size_t ws_bytes, cudaStream_t s) {
  if (!big_supported(p)) return cudaErrorNotSupported;
  const BigLayout L = big_layout(p.d, p.count);
  if (ws == nullptr || ws_bytes < L.total) return cudaErrorInvalidValue;
  const int a = p.d - 3;
  const long long N = 1LL << (3 * p.d);
  const long long rows = 1LL << (3 * a);
  unsigned char* w = static_cast<unsigned char*>(ws);
  double* W = reinterpret_cast<double*>(w + L.w);
  BigPtrs b;
  b.a1 = reinterpret_cast<const double**>(w + L.a1);
  b.x1 = reinterpret_cast<const double**>(w + L.x1);
  b.y1 = reinterpret_cast<double**>(w + L.y1);
  b.a2 = reinterpret_cast<const double**>(w + L.a2);
  b.x2 = reinterpret_cast<const double**>(w + L.x2);
  b.y2 = reinterpret_cast<double**>(w + L.y2);
  b.ident = reinterpret_cast<double*>(w + L.ident);
  for (long long e0 = 0; e0 < p.count; e0 += L.chunk) {
    const int cnt = (int)((p.count - e0) < L.chunk ? (p.count - e0) : L.chunk);
    cudaError_t e = cudaMemsetAsync(W, 0, (size_t)cnt * N * 8, s);
    if (e != cudaSuccess) return e;
    const long long total = (long long)cnt * rows;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    big_build_kernel<<<blocks, 256, 0, s>>>(p, a, e0, cnt, W, N, b);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // pass 1: rows, trailing three modes, into W (column-blocked)
    Problem q1 = p;
    q1.layout = L_XBATCHED;
    q1.d = 3;
    for (int j = 0; j < 3; ++j) {
      q1.m[j] = q1.n[j] = BN;
      q1.ld[j] = p.ld[a + j];
    }
    for (int j = 3; j < MAXD; ++j) q1.m[j] = q1.n[j] = q1.ld[j] = 1;
    q1.Nx = q1.Ny = ROW;
    q1.sxw = ROW;
    q1.count = (int)total;
    q1.entry_offset = 0;
    q1.order = nullptr;
    q1.a_off = nullptr;
    q1.A = b.a1;
    q1.X = b.x1;
    q1.Y = b.y1;
    q1.y_exclusive = 1;
    q1.wmode = 0;
    q1.y_inner = BN;
    q1.y_ostride = rows * BN;
    e = launch_f64_split(q1, h1, s);
    if (e != cudaSuccess) return e;
    // pass 2: column blocks, leading modes and the identity, into Y
    Problem q2 = q1;
    q2.d = a + 1;
    for (int j = 0; j < a; ++j) {
      q2.m[j] = q2.n[j] = BN;
      q2.ld[j] = p.ld[j];
    }
    q2.m[a] = q2.n[a] = BN;
    q2.ld[a] = BN;
    for (int j = a + 1; j < MAXD; ++j) q2.m[j] = q2.n[j] = q2.ld[j] = 1;
    q2.Nx = q2.Ny = rows * BN;
    q2.sxw = rows * BN;
    q2.count = cnt * (int)(ROW / BN);
    q2.A = b.a2;
    q2.X = b.x2;
    q2.Y = b.y2;
    q2.y_exclusive = p.y_exclusive;
    q2.y_inner = BN;
    q2.y_ostride = ROW;
    e = launch_f64_split(q2, h2, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace kmx
