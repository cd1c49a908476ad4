// Densification statistics of a training step, in one pass over the Gaussians.
//
// After the backward, the reference's DensificationController.preprocess
// (pointrix/controller/gs.py:318-333, with accumulate_viewspace_grad at
// gs.py:260-284) updates, for the points visible in the step:
//   max_radii  = max(max_radii, radii)
//   grad_accum += |(ndc.grad.x * sx, ndc.grad.y * sy)|     (sx = W/2, sy = H/2
//                                                           with normalize_grad,
//                                                           else 1)
//   acc_steps  += 1
// where the screen-space gradient is summed over the views of the batch and
// "visible" is radius > 0 (render_batch: any view; radii: max over views).
// The torch form indexes with the boolean mask three times (each a host
// synchronisation and a compaction); here one thread per Gaussian reads
// the gradient and the radius once and updates the three statistics in place.
#include "pgb_common.cuh"

namespace pgb {

__global__ void __launch_bounds__(kStreamThreads) densify_accumulate_kernel(
    const float* __restrict__ d_uv, int64_t n, const int32_t* __restrict__ radius, float sx,
    float sy, float* __restrict__ grad_accum, float* __restrict__ acc_steps,
    float* __restrict__ max_radii) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = radius[i];
    if (r <= 0) continue;
    const float2 g = reinterpret_cast<const float2*>(d_uv)[i];
    const float gx = g.x * sx, gy = g.y * sy;
    grad_accum[i] += sqrtf(gx * gx + gy * gy);
    acc_steps[i] += 1.f;
    max_radii[i] = fmaxf(max_radii[i], (float)r);
  }
}

}  // namespace pgb

using namespace pgb;

extern "C" int pgb_densify_accumulate(const float* d_uv, int64_t n, const int32_t* radius, float sx,
                                      float sy, float* grad_accum, float* acc_steps,
                                      float* max_radii, void* stream) {
  if (n < 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!d_uv || !radius || !grad_accum || !acc_steps || !max_radii ||
      (reinterpret_cast<uintptr_t>(d_uv) & 7))
    return PGB_ERR_INVALID;
  densify_accumulate_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(
      d_uv, n, radius, sx, sy, grad_accum, acc_steps, max_radii);
  return launch_status();
}
