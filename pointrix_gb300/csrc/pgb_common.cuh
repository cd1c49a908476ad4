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

__device__ inline float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace pgb
