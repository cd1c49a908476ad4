// Photometric loss L = mean|x - t| + w * mean((x - t)^2) and its gradient.
//
// The training step's loss (the L1 term of pointrix/model/loss.py:27-33 with
// a weighted L2 term, as torch's l1_loss + w * mse_loss) is a handful of
// elementwise and reduction kernels forward and backward over the rendered
// [C,H,W] image.  Here the forward is one pass that reads x and t once and
// writes per-block partial sums (double), summed in block order by a
// one-block finish (deterministic); the backward is one pass that reads x,
// t and dL from the device and writes
//   dx = sign(x - t) * (dL / n) + ((2 / n) * (x - t)) * (w * dL),
// the same expression torch's l1 and mse backward formulas sum.  A training
// step's forward can also write dx for dL = 1 in its own pass (the loss is
// the step's output, so dL is 1 unless scaled); the backward then returns
// at once when dL is 1, and rewrites dx otherwise.
#include <algorithm>

#include "pgb_common.cuh"

namespace pgb {

constexpr int kLossThreads = 256;
constexpr int kLossBlocksMax = kNumSMs * 8;

inline int loss_grid(int64_t n) {
  const int64_t need = (n / 4 + kLossThreads - 1) / kLossThreads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(need, kLossBlocksMax));
}

__device__ inline double block_sum_double(double v, double* s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kLossThreads / 32; ++w) t += s_red[w];
  __syncthreads();
  return t;
}

__device__ inline float l1l2_grad(float x, float t, float a, float b, float inv2n) {
  const float d = x - t;
  const float sg = d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f);
  return sg * a + (inv2n * d) * b;
}

__device__ inline float4 l1l2_grad4(float4 x, float4 t, float a, float b, float inv2n) {
  return make_float4(l1l2_grad(x.x, t.x, a, b, inv2n), l1l2_grad(x.y, t.y, a, b, inv2n),
                     l1l2_grad(x.z, t.z, a, b, inv2n), l1l2_grad(x.w, t.w, a, b, inv2n));
}

// x and t 16-byte aligned: float4 body, scalar tail handled by block 0.
// With GRAD, the same pass also writes dx = the backward for dL = 1 (the
// backward kernel's expression with g = 1, so bit for bit its values).
template <bool GRAD>
__global__ void __launch_bounds__(kLossThreads) l1l2_partial_kernel(
    const float* __restrict__ x, const float* __restrict__ t, int64_t n, float w,
    double* __restrict__ partial, float* __restrict__ dx) {
  __shared__ double s_red[kLossThreads / 32];
  // per-thread sums in float over at most a few dozen float4 (four loads in
  // flight per iteration), then double across threads and blocks
  float f1 = 0.f, f2 = 0.f;
  const int64_t n4 = n / 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const float nf = (float)n;
  const float ga = 1.f / nf, gb = w, inv2n = 2.f / nf;  // l1l2_bwd_kernel's a, b at g = 1
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; q + stride < n4; q += 2 * stride) {
    const float4 xa = reinterpret_cast<const float4*>(x)[q];
    const float4 ta = reinterpret_cast<const float4*>(t)[q];
    const float4 xb = reinterpret_cast<const float4*>(x)[q + stride];
    const float4 tb = reinterpret_cast<const float4*>(t)[q + stride];
    if constexpr (GRAD) {
      reinterpret_cast<float4*>(dx)[q] = l1l2_grad4(xa, ta, ga, gb, inv2n);
      reinterpret_cast<float4*>(dx)[q + stride] = l1l2_grad4(xb, tb, ga, gb, inv2n);
    }
    const float d[8] = {xa.x - ta.x, xa.y - ta.y, xa.z - ta.z, xa.w - ta.w,
                        xb.x - tb.x, xb.y - tb.y, xb.z - tb.z, xb.w - tb.w};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      f1 += fabsf(d[c]);
      f2 += d[c] * d[c];
    }
  }
  if (q < n4) {
    const float4 xv = reinterpret_cast<const float4*>(x)[q];
    const float4 tv = reinterpret_cast<const float4*>(t)[q];
    if constexpr (GRAD) reinterpret_cast<float4*>(dx)[q] = l1l2_grad4(xv, tv, ga, gb, inv2n);
    const float d[4] = {xv.x - tv.x, xv.y - tv.y, xv.z - tv.z, xv.w - tv.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      f1 += fabsf(d[c]);
      f2 += d[c] * d[c];
    }
  }
  double a1 = f1, a2 = f2;
  if (blockIdx.x == 0)
    for (int64_t i = 4 * n4 + threadIdx.x; i < n; i += blockDim.x) {
      const float d = x[i] - t[i];
      a1 += fabsf(d);
      a2 += d * d;
      if constexpr (GRAD) dx[i] = l1l2_grad(x[i], t[i], ga, gb, inv2n);
    }
  const double b1 = block_sum_double(a1, s_red);
  const double b2 = block_sum_double(a2, s_red);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = b1;
    partial[2 * blockIdx.x + 1] = b2;
  }
}

constexpr int kFinishTPC = 256;  // threads per summed column

__global__ void __launch_bounds__(2 * kFinishTPC) l1l2_finish_kernel(
    const double* __restrict__ partial, int blocks, int64_t n, float w, float* __restrict__ loss) {
  __shared__ double s[2 * kFinishTPC];
  column_sum<2, kFinishTPC>(partial, blocks, 2, s);
  if (threadIdx.x == 0) {
    const double s1 = s[0], s2 = s[kFinishTPC];
    loss[0] = (float)(s1 / (double)n + (double)w * (s2 / (double)n));
  }
}

// UNIT: dx already holds the backward for dL = 1 (l1l2_partial_kernel<true>);
// it is left as it is when dL is 1 and rewritten otherwise.
template <bool UNIT>
__global__ void __launch_bounds__(kLossThreads) l1l2_bwd_kernel(
    const float* __restrict__ x, const float* __restrict__ t, int64_t n, float w,
    const float* __restrict__ d_loss, float* __restrict__ dx) {
  const float g = d_loss[0];
  if (UNIT && g == 1.f) return;
  const float nf = (float)n;
  const float a = g / nf;        // dL / n (the mean's backward)
  const float b = w * g;         // the weighted L2 term's incoming gradient
  const float inv2n = 2.f / nf;  // mse backward's 2 / n
  const int64_t n4 = n / 4;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4;
       q += (int64_t)gridDim.x * blockDim.x) {
    const float4 xv = reinterpret_cast<const float4*>(x)[q];
    const float4 tv = reinterpret_cast<const float4*>(t)[q];
    reinterpret_cast<float4*>(dx)[q] = l1l2_grad4(xv, tv, a, b, inv2n);
  }
  if (blockIdx.x == 0)
    for (int64_t i = 4 * n4 + threadIdx.x; i < n; i += blockDim.x)
      dx[i] = l1l2_grad(x[i], t[i], a, b, inv2n);
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_l1_l2_loss_scratch_doubles(int64_t n) { return 2 * loss_grid(n); }

int pgb_l1_l2_loss_forward(const float* x, const float* target, int64_t n, float w,
                           double* scratch, int64_t scratch_doubles, float* loss, void* stream) {
  if (n <= 0 || !x || !target || !loss || !scratch) return PGB_ERR_INVALID;
  const int grid = loss_grid(n);
  if (scratch_doubles < 2 * grid || !aligned16(x) || !aligned16(target)) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  l1l2_partial_kernel<false><<<grid, kLossThreads, 0, s>>>(x, target, n, w, scratch, nullptr);
  l1l2_finish_kernel<<<1, 2 * kFinishTPC, 0, s>>>(scratch, grid, n, w, loss);
  return launch_status();
}

int pgb_l1_l2_loss_forward_grad(const float* x, const float* target, int64_t n, float w,
                                double* scratch, int64_t scratch_doubles, float* loss,
                                float* d_x_unit, void* stream) {
  if (n <= 0 || !x || !target || !loss || !scratch || !d_x_unit) return PGB_ERR_INVALID;
  const int grid = loss_grid(n);
  if (scratch_doubles < 2 * grid || !aligned16(x) || !aligned16(target) || !aligned16(d_x_unit))
    return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  l1l2_partial_kernel<true><<<grid, kLossThreads, 0, s>>>(x, target, n, w, scratch, d_x_unit);
  l1l2_finish_kernel<<<1, 2 * kFinishTPC, 0, s>>>(scratch, grid, n, w, loss);
  return launch_status();
}

int pgb_l1_l2_loss_backward(const float* x, const float* target, int64_t n, float w,
                            const float* d_loss, float* d_x, void* stream) {
  if (n <= 0 || !x || !target || !d_loss || !d_x) return PGB_ERR_INVALID;
  if (!aligned16(x) || !aligned16(target) || !aligned16(d_x)) return PGB_ERR_INVALID;
  l1l2_bwd_kernel<false><<<loss_grid(n), kLossThreads, 0, as_stream(stream)>>>(x, target, n, w,
                                                                                d_loss, d_x);
  return launch_status();
}

int pgb_l1_l2_loss_backward_unit(const float* x, const float* target, int64_t n, float w,
                                 const float* d_loss, float* d_x, void* stream) {
  if (n <= 0 || !x || !target || !d_loss || !d_x) return PGB_ERR_INVALID;
  if (!aligned16(x) || !aligned16(target) || !aligned16(d_x)) return PGB_ERR_INVALID;
  l1l2_bwd_kernel<true><<<loss_grid(n), kLossThreads, 0, as_stream(stream)>>>(x, target, n, w,
                                                                               d_loss, d_x);
  return launch_status();
}

}  // extern "C"
