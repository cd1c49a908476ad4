// SSIM of a rendered image against a target, forward and backward.
//
// The reference (pointrix/model/loss.py:71-125, ssim / _ssim / create_window)
// convolves x, y, x^2, y^2 and x y per channel with an 11 x 11 Gaussian
// window (sigma 1.5, the outer product of the normalised 1-D window; zero
// padding 5), forms
//   S = (2 mu1 mu2 + C1)(2 s12 + C2) / ((mu1^2 + mu2^2 + C1)(s11 + s22 + C2)),
//   s11 = E[x^2] - mu1^2, s22 = E[y^2] - mu2^2, s12 = E[xy] - mu1 mu2,
// C1 = 0.01^2, C2 = 0.03^2, and returns the mean of S: five convolutions and
// a dozen elementwise kernels forward, more backward.
//
// Here one CTA computes a 32 x 32 output tile of one image plane.  Forward:
// the tile and a 5-pixel halo of x and y are staged in shared memory (zeros
// outside the image), the five moments are convolved separably (11 taps
// along rows into shared memory, then 11 down columns), and the CTA adds its
// sum of S to a per-CTA partial (summed in a fixed order by a one-CTA
// finish).  Backward (x only; y is the target): with dL/dS = g / count,
//   dS/dmu1 = S (2 mu2 / A - 2 mu2 / B - 2 mu1 / C + 2 mu1 / D),
//   dS/dE[x^2] = -S / D,  dS/dE[xy] = 2 S / B,
// (A..D the four factors above) and dx = W * dmu1 + 2 x W * dExx + y W * dExy
// with W the same symmetric window (the transpose of a zero-padded
// correlation).  The CTA recomputes the moments on the tile plus a 5-pixel
// halo (inputs on a 10-pixel halo), forms the three maps there (zero outside
// the image), convolves them separably and writes dx for its tile.
#include <algorithm>
#include <cmath>

#include "pgb_common.cuh"

namespace pgb {

constexpr int kSsimTile = 32;
constexpr int kSsimR = 5;  // window radius
constexpr int kSsimThreads = 256;
constexpr float kSsimC1 = 0.0001f;  // 0.01^2
constexpr float kSsimC2 = 0.0009f;  // 0.03^2

// The normalised 1-D window exp(-(k-5)^2 / (2 * 1.5^2)) / sum, k = 0..10,
// passed by value in the kernel parameters.
struct SsimWindow {
  float w[11];
};

inline SsimWindow ssim_window() {
  SsimWindow win;
  double e[11], s = 0.0;
  for (int k = 0; k < 11; ++k) {
    const double d = k - 5;
    e[k] = exp(-d * d / (2.0 * 1.5 * 1.5));
    s += e[k];
  }
  for (int k = 0; k < 11; ++k) win.w[k] = (float)(e[k] / s);
  return win;
}

// ---------------------------------------------------------------- forward
constexpr int kFwdIn = kSsimTile + 2 * kSsimR;  // 42

__global__ void __launch_bounds__(kSsimThreads) ssim_fwd_kernel(
    const float* __restrict__ x, const float* __restrict__ y, int H, int W, SsimWindow win,
    double* __restrict__ partial) {
  __shared__ float sx[kFwdIn][kFwdIn + 1], sy[kFwdIn][kFwdIn + 1];
  __shared__ float hm[5][kFwdIn][kSsimTile + 1];
  __shared__ double s_red[kSsimThreads / 32];
  const int plane = blockIdx.z;
  const int ox = blockIdx.x * kSsimTile, oy = blockIdx.y * kSsimTile;
  const float* xp = x + (int64_t)plane * H * W;
  const float* yp = y + (int64_t)plane * H * W;
  for (int i = threadIdx.x; i < kFwdIn * kFwdIn; i += kSsimThreads) {
    const int r = i / kFwdIn, c = i % kFwdIn;
    const int gy = oy - kSsimR + r, gx = ox - kSsimR + c;
    const bool in = gy >= 0 && gy < H && gx >= 0 && gx < W;
    sx[r][c] = in ? xp[(int64_t)gy * W + gx] : 0.f;
    sy[r][c] = in ? yp[(int64_t)gy * W + gx] : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kFwdIn * kSsimTile; i += kSsimThreads) {
    const int r = i / kSsimTile, c = i % kSsimTile;
    float m1 = 0.f, m2 = 0.f, e11 = 0.f, e22 = 0.f, e12 = 0.f;
#pragma unroll
    for (int k = 0; k < 11; ++k) {
      const float w = win.w[k], a = sx[r][c + k], b = sy[r][c + k];
      m1 = fmaf(w, a, m1);
      m2 = fmaf(w, b, m2);
      e11 = fmaf(w, a * a, e11);
      e22 = fmaf(w, b * b, e22);
      e12 = fmaf(w, a * b, e12);
    }
    hm[0][r][c] = m1;
    hm[1][r][c] = m2;
    hm[2][r][c] = e11;
    hm[3][r][c] = e22;
    hm[4][r][c] = e12;
  }
  __syncthreads();
  double acc = 0.0;
  for (int i = threadIdx.x; i < kSsimTile * kSsimTile; i += kSsimThreads) {
    const int r = i / kSsimTile, c = i % kSsimTile;
    if (oy + r >= H || ox + c >= W) continue;
    float mu1 = 0.f, mu2 = 0.f, e11 = 0.f, e22 = 0.f, e12 = 0.f;
#pragma unroll
    for (int k = 0; k < 11; ++k) {
      const float w = win.w[k];
      mu1 = fmaf(w, hm[0][r + k][c], mu1);
      mu2 = fmaf(w, hm[1][r + k][c], mu2);
      e11 = fmaf(w, hm[2][r + k][c], e11);
      e22 = fmaf(w, hm[3][r + k][c], e22);
      e12 = fmaf(w, hm[4][r + k][c], e12);
    }
    const float m12 = mu1 * mu2, m11 = mu1 * mu1, m22 = mu2 * mu2;
    const float A = 2.f * m12 + kSsimC1, B = 2.f * (e12 - m12) + kSsimC2;
    const float C = m11 + m22 + kSsimC1, D = (e11 - m11) + (e22 - m22) + kSsimC2;
    acc += (double)((A * B) / (C * D));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) s_red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kSsimThreads / 32; ++w) t += s_red[w];
    const int64_t b = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    partial[b] = t;
  }
}

constexpr int kSsimFinishTPC = 512;

__global__ void __launch_bounds__(kSsimFinishTPC) ssim_finish_kernel(
    const double* __restrict__ partial, int blocks, int64_t count, float* __restrict__ out) {
  __shared__ double s[kSsimFinishTPC];
  column_sum<1, kSsimFinishTPC>(partial, blocks, 1, s);
  if (threadIdx.x == 0) out[0] = (float)(s[0] / (double)count);
}

// --------------------------------------------------------------- backward
constexpr int kBwdIn = kSsimTile + 4 * kSsimR;   // 52: inputs
constexpr int kBwdMid = kSsimTile + 2 * kSsimR;  // 42: moments and maps

__global__ void __launch_bounds__(kSsimThreads) ssim_bwd_kernel(
    const float* __restrict__ x, const float* __restrict__ y, int H, int W, SsimWindow win,
    const float* __restrict__ d_out, int64_t count, float* __restrict__ dx) {
  extern __shared__ __align__(16) float sm[];
  float* sx = sm;                                  // [52][53]
  float* sy = sx + kBwdIn * (kBwdIn + 1);          // [52][53]
  float* hm = sy + kBwdIn * (kBwdIn + 1);          // 5 x [52][43] row-convolved moments
  float* gm = hm + 5 * kBwdIn * (kBwdMid + 1);     // 3 x [42][43] maps
  float* hg = gm + 3 * kBwdMid * (kBwdMid + 1);    // 3 x [42][33] row-convolved maps
  constexpr int PI = kBwdIn + 1, PH = kBwdMid + 1, PG = kSsimTile + 1;
  const int plane = blockIdx.z;
  const int ox = blockIdx.x * kSsimTile, oy = blockIdx.y * kSsimTile;
  const float* xp = x + (int64_t)plane * H * W;
  const float* yp = y + (int64_t)plane * H * W;
  const float gscale = d_out[0] / (float)count;
  // inputs on the tile + 10-pixel halo
  for (int i = threadIdx.x; i < kBwdIn * kBwdIn; i += kSsimThreads) {
    const int r = i / kBwdIn, c = i % kBwdIn;
    const int gy = oy - 2 * kSsimR + r, gx = ox - 2 * kSsimR + c;
    const bool in = gy >= 0 && gy < H && gx >= 0 && gx < W;
    sx[r * PI + c] = in ? xp[(int64_t)gy * W + gx] : 0.f;
    sy[r * PI + c] = in ? yp[(int64_t)gy * W + gx] : 0.f;
  }
  __syncthreads();
  // moments along rows: 52 rows x 42 columns
  for (int i = threadIdx.x; i < kBwdIn * kBwdMid; i += kSsimThreads) {
    const int r = i / kBwdMid, c = i % kBwdMid;
    float m1 = 0.f, m2 = 0.f, e11 = 0.f, e22 = 0.f, e12 = 0.f;
#pragma unroll
    for (int k = 0; k < 11; ++k) {
      const float w = win.w[k], a = sx[r * PI + c + k], b = sy[r * PI + c + k];
      m1 = fmaf(w, a, m1);
      m2 = fmaf(w, b, m2);
      e11 = fmaf(w, a * a, e11);
      e22 = fmaf(w, b * b, e22);
      e12 = fmaf(w, a * b, e12);
    }
    const int o = r * PH + c, st = kBwdIn * PH;
    hm[o] = m1;
    hm[st + o] = m2;
    hm[2 * st + o] = e11;
    hm[3 * st + o] = e22;
    hm[4 * st + o] = e12;
  }
  __syncthreads();
  // moments down columns and the three maps on the tile + 5-pixel halo
  for (int i = threadIdx.x; i < kBwdMid * kBwdMid; i += kSsimThreads) {
    const int r = i / kBwdMid, c = i % kBwdMid;
    const int gy = oy - kSsimR + r, gx = ox - kSsimR + c;
    float g1 = 0.f, g11 = 0.f, g12 = 0.f;
    if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
      const int st = kBwdIn * PH;
      float mu1 = 0.f, mu2 = 0.f, e11 = 0.f, e22 = 0.f, e12 = 0.f;
#pragma unroll
      for (int k = 0; k < 11; ++k) {
        const float w = win.w[k];
        const int o = (r + k) * PH + c;
        mu1 = fmaf(w, hm[o], mu1);
        mu2 = fmaf(w, hm[st + o], mu2);
        e11 = fmaf(w, hm[2 * st + o], e11);
        e22 = fmaf(w, hm[3 * st + o], e22);
        e12 = fmaf(w, hm[4 * st + o], e12);
      }
      const float m12 = mu1 * mu2, m11 = mu1 * mu1, m22 = mu2 * mu2;
      const float A = 2.f * m12 + kSsimC1, B = 2.f * (e12 - m12) + kSsimC2;
      const float C = m11 + m22 + kSsimC1, D = (e11 - m11) + (e22 - m22) + kSsimC2;
      const float S = (A * B) / (C * D);
      const float gS = gscale * S;
      g1 = gS * (2.f * mu2 / A - 2.f * mu2 / B - 2.f * mu1 / C + 2.f * mu1 / D);
      g11 = -gS / D;
      g12 = 2.f * gS / B;
    }
    const int o = r * PH + c, st = kBwdMid * PH;
    gm[o] = g1;
    gm[st + o] = g11;
    gm[2 * st + o] = g12;
  }
  __syncthreads();
  // maps along rows: 42 rows x 32 columns
  for (int i = threadIdx.x; i < kBwdMid * kSsimTile; i += kSsimThreads) {
    const int r = i / kSsimTile, c = i % kSsimTile;
    const int st = kBwdMid * PH;
    float a = 0.f, b = 0.f, d = 0.f;
#pragma unroll
    for (int k = 0; k < 11; ++k) {
      const float w = win.w[k];
      const int o = r * PH + c + k;
      a = fmaf(w, gm[o], a);
      b = fmaf(w, gm[st + o], b);
      d = fmaf(w, gm[2 * st + o], d);
    }
    const int o = r * PG + c, sg = kBwdMid * PG;
    hg[o] = a;
    hg[sg + o] = b;
    hg[2 * sg + o] = d;
  }
  __syncthreads();
  // down columns and dx on the tile
  float* dxp = dx + (int64_t)plane * H * W;
  for (int i = threadIdx.x; i < kSsimTile * kSsimTile; i += kSsimThreads) {
    const int r = i / kSsimTile, c = i % kSsimTile;
    const int gy = oy + r, gx = ox + c;
    if (gy >= H || gx >= W) continue;
    const int sg = kBwdMid * PG;
    float a = 0.f, b = 0.f, d = 0.f;
#pragma unroll
    for (int k = 0; k < 11; ++k) {
      const float w = win.w[k];
      const int o = (r + k) * PG + c;
      a = fmaf(w, hg[o], a);
      b = fmaf(w, hg[sg + o], b);
      d = fmaf(w, hg[2 * sg + o], d);
    }
    const float xv = sx[(r + 2 * kSsimR) * PI + c + 2 * kSsimR];
    const float yv = sy[(r + 2 * kSsimR) * PI + c + 2 * kSsimR];
    dxp[(int64_t)gy * W + gx] = a + 2.f * xv * b + yv * d;
  }
}

constexpr size_t kSsimBwdSmem =
    (2 * (size_t)kBwdIn * (kBwdIn + 1) + 5 * (size_t)kBwdIn * (kBwdMid + 1) +
     3 * (size_t)kBwdMid * (kBwdMid + 1) + 3 * (size_t)kBwdMid * (kSsimTile + 1)) *
    sizeof(float);

inline dim3 ssim_grid(int planes, int H, int W) {
  return dim3((W + kSsimTile - 1) / kSsimTile, (H + kSsimTile - 1) / kSsimTile, planes);
}

}  // namespace pgb

using namespace pgb;

extern "C" {

int64_t pgb_ssim_scratch_doubles(int planes, int height, int width) {
  if (planes <= 0 || height <= 0 || width <= 0) return 0;
  const dim3 g = ssim_grid(planes, height, width);
  return (int64_t)g.x * g.y * g.z;
}

int pgb_ssim_forward(const float* x, const float* y, int planes, int height, int width,
                     double* scratch, int64_t scratch_doubles, float* ssim_out, void* stream) {
  if (planes <= 0 || height <= 0 || width <= 0 || !x || !y || !scratch || !ssim_out)
    return PGB_ERR_INVALID;
  const dim3 g = ssim_grid(planes, height, width);
  const int64_t blocks = (int64_t)g.x * g.y * g.z;
  if (scratch_doubles < blocks || blocks > INT32_MAX || g.z > 65535) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  ssim_fwd_kernel<<<g, kSsimThreads, 0, s>>>(x, y, height, width, ssim_window(), scratch);
  ssim_finish_kernel<<<1, kSsimFinishTPC, 0, s>>>(scratch, (int)blocks,
                                                  (int64_t)planes * height * width, ssim_out);
  return launch_status();
}

int pgb_ssim_backward(const float* x, const float* y, int planes, int height, int width,
                      const float* d_out, float* d_x, void* stream) {
  if (planes <= 0 || height <= 0 || width <= 0 || !x || !y || !d_out || !d_x)
    return PGB_ERR_INVALID;
  const dim3 g = ssim_grid(planes, height, width);
  if (g.z > 65535) return PGB_ERR_INVALID;
  if (cudaFuncSetAttribute(ssim_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kSsimBwdSmem) != cudaSuccess)
    return PGB_ERR_CUDA;
  ssim_bwd_kernel<<<g, kSsimThreads, kSsimBwdSmem, as_stream(stream)>>>(
      x, y, height, width, ssim_window(), d_out, (int64_t)planes * height * width, d_x);
  return launch_status();
}

}  // extern "C"
