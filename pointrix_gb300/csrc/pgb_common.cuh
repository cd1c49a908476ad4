// Shared helpers for the pointrix_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pointrix_gb300.h"

namespace pgb {

constexpr int kTile = 16;            // 16x16 pixel tiles
constexpr int kNumSMs = 152;         // GB300: 2 dies x 76 SMs

// Streaming per-Gaussian kernels: 256 threads, grid a multiple of the SM
// count (grid-stride loop beyond that).
constexpr int kStreamThreads = 256;

// True when p is not a multiple of `bytes`: the entry points refuse buffers
// that a kernel would access with wider loads or stores than their start allows.
inline bool misaligned(const void* p, uintptr_t bytes) {
  return (reinterpret_cast<uintptr_t>(p) & (bytes - 1)) != 0;
}

inline int stream_grid(int64_t n, int threads = kStreamThreads, int per_sm = 8) {
  int64_t need = (n + threads - 1) / threads;
  int64_t cap = (int64_t)kNumSMs * per_sm;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PGB_OK : PGB_ERR_CUDA;
}

__host__ __device__ inline int grid_x(int w) { return (w + kTile - 1) / kTile; }
__host__ __device__ inline int grid_y(int h) { return (h + kTile - 1) / kTile; }

// Tile rectangle of a disc of radius r centred at (u, v), clipped to the
// grid.  Every step is a single IEEE-rounded float operation (the files that
// use it are compiled without FMA contraction), so the integer result is
// reproducible on any IEEE host.
__device__ inline void tile_rect(float u, float v, float r, int gx, int gy, int& xmin, int& xmax,
                                 int& ymin, int& ymax) {
  const float t = 16.0f, c = 15.0f;
  xmin = (int)fminf((float)gx, fmaxf(0.0f, (u - r) / t));
  xmax = (int)fminf((float)gx, fmaxf(0.0f, (u + r + c) / t));
  ymin = (int)fminf((float)gy, fmaxf(0.0f, (v - r) / t));
  ymax = (int)fminf((float)gy, fmaxf(0.0f, (v + r + c) / t));
}

// The same for tiles 16 pixels wide and th (16 or 32) high; th = 16 is
// tile_rect operation for operation.
__device__ inline void tile_rect_h(float u, float v, float r, int th, int gx, int gy, int& xmin,
                                   int& xmax, int& ymin, int& ymax) {
  const float t = 16.0f, c = 15.0f, ty = (float)th, cy = (float)(th - 1);
  xmin = (int)fminf((float)gx, fmaxf(0.0f, (u - r) / t));
  xmax = (int)fminf((float)gx, fmaxf(0.0f, (u + r + c) / t));
  ymin = (int)fminf((float)gy, fmaxf(0.0f, (v - r) / ty));
  ymax = (int)fminf((float)gy, fmaxf(0.0f, (v + r + cy) / ty));
}

__host__ __device__ inline int grid_y_h(int h, int th) { return (h + th - 1) / th; }

// Where the tiles and pixels of a launch live, passed by value in kernel
// parameters: one image (nviews == 0, size W x H) or a batch of up to
// kMaxViews views.  In a batch the views own consecutive ranges of one global
// 16x16 tile index space (view v's first tile is tile_base[v]), per-pixel
// arrays hold the views one after another (view v's first pixel is
// pixel_base[v]), and element g of the per-Gaussian arrays belongs to view
// g / n_per_view.
constexpr int kMaxViews = 64;

// One image may also be processed in bands of tile rows [band0, band1):
// the sort then emits only the entries of those rows, with tile ids local to
// the band (row r of the band is tile row band0 + r of the image), and a
// blend launch covers only the band's tiles, reading band-local tile ranges
// and writing the image's own pixels.  single_view covers every row.
struct ViewTable {
  int nviews;
  int W, H;
  int band0, band1;
  int th;  // a batch of views: tile height in pixels (16, or 32 for 16x32 tiles)
  int64_t n_per_view;
  int32_t w[kMaxViews], h[kMaxViews], tile_base[kMaxViews];
  int64_t pixel_base[kMaxViews];
};

inline ViewTable single_view(int W, int H) {
  ViewTable vt{};
  vt.nviews = 0;
  vt.W = W;
  vt.H = H;
  vt.band0 = 0;
  vt.band1 = grid_y(H);
  return vt;
}

// One image restricted to tile rows [row0, row1); false when the rows are
// not a non-empty range of the image's tile rows.
inline bool band_view(int W, int H, int row0, int row1, ViewTable& vt) {
  if (W <= 0 || H <= 0 || row0 < 0 || row1 <= row0 || row1 > grid_y(H)) return false;
  vt = single_view(W, H);
  vt.band0 = row0;
  vt.band1 = row1;
  return true;
}

// A batch from host (width, height) pairs; fills the bases and returns the
// total tile and pixel counts, or false when a size is invalid.
inline bool make_views(const int32_t* sizes, int nviews, int64_t n_per_view, ViewTable& vt,
                       uint32_t& tiles, int64_t& pixels, int th = 16) {
  if (!sizes || nviews < 1 || nviews > kMaxViews || n_per_view < 0) return false;
  if (th != 16 && th != 32) return false;
  vt = ViewTable{};
  vt.nviews = nviews;
  vt.th = th;
  vt.n_per_view = n_per_view;
  uint64_t t = 0;
  int64_t p = 0;
  for (int v = 0; v < nviews; ++v) {
    const int W = sizes[2 * v], H = sizes[2 * v + 1];
    if (W <= 0 || H <= 0 || grid_x(W) > 65535 || grid_y(H) > 65535) return false;
    vt.w[v] = W;
    vt.h[v] = H;
    vt.tile_base[v] = (int32_t)t;
    vt.pixel_base[v] = p;
    t += (uint64_t)grid_x(W) * grid_y_h(H, th);
    p += (int64_t)W * H;
    if (t > (1u << 24)) return false;
  }
  tiles = (uint32_t)t;
  pixels = p;
  return true;
}

// Tile grid and first global tile of the view that owns element g.
__device__ inline void element_view(const ViewTable& vt, uint32_t g, int& gx, int& gy,
                                    uint32_t& tile_base) {
  if (vt.nviews == 0) {
    gx = grid_x(vt.W);
    gy = grid_y(vt.H);
    tile_base = 0;
    return;
  }
  int v = (int)((int64_t)g / vt.n_per_view);
  v = v < vt.nviews - 1 ? v : vt.nviews - 1;
  gx = grid_x(vt.w[v]);
  gy = grid_y_h(vt.h[v], vt.th);
  tile_base = (uint32_t)vt.tile_base[v];
}

// The view that owns global tile `tile`: its size, tile grid width, the tile's
// index within the view and the view's first pixel in per-pixel arrays.
__device__ inline void tile_view(const ViewTable& vt, int tile, int& W, int& H, int& gx,
                                 int& local, int64_t& pixel_base) {
  if (vt.nviews == 0) {
    W = vt.W;
    H = vt.H;
    gx = grid_x(W);
    local = tile + vt.band0 * gx;  // the band's tiles are launched from 0
    pixel_base = 0;
    return;
  }
  int v = 0;
  for (int i = 1; i < vt.nviews; ++i)
    if (vt.tile_base[i] <= tile) v = i;
  W = vt.w[v];
  H = vt.h[v];
  gx = grid_x(W);
  local = tile - vt.tile_base[v];
  pixel_base = vt.pixel_base[v];
}

__device__ inline uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 16-byte asynchronous global -> shared copy (cp.async, L1 bypass), and the
// group commit / wait that orders it; the wait is a hardware wait for this
// thread's own copies, it cannot spin.
__device__ inline void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ inline void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Deterministic sum over rows b < nrows of v[b * stride + col] for NCOL
// columns, run by one CTA of NCOL * TPC threads: thread j of a column sums
// rows j, j + TPC, ... in order (groups of eight rows pairwise in T, each
// group's sum added in double), then a fixed shared-memory tree adds the
// TPC partial sums.  Returns the column's total in the column's
// thread j == 0 (others: unspecified).  `s` holds NCOL * TPC doubles.
template <int NCOL, int TPC, typename T>
__device__ inline double column_sum(const T* __restrict__ v, int nrows, int stride, double* s) {
  static_assert((TPC & (TPC - 1)) == 0, "TPC must be a power of two");
  const int col = threadIdx.x / TPC, j = threadIdx.x % TPC;
  double acc = 0.0;
  if (col < NCOL) {
    // eight rows' loads in flight at a time, added in row order
    int b = j;
    for (; b + 7 * TPC < nrows; b += 8 * TPC) {
      T x[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) x[u] = v[(size_t)(b + u * TPC) * stride + col];
      // eight rows summed pairwise in T, then one double add: FP64 is a
      // slow pipe on this part, and the finish runs on one SM
      const T s01 = x[0] + x[1], s23 = x[2] + x[3], s45 = x[4] + x[5], s67 = x[6] + x[7];
      acc += (double)((s01 + s23) + (s45 + s67));
    }
    for (; b < nrows; b += TPC) acc += (double)v[(size_t)b * stride + col];
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int h = TPC / 2; h > 0; h >>= 1) {
    if (j < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  return s[threadIdx.x];
}

__device__ inline float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace pgb
