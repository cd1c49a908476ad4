// Adam over the Gaussian (and camera) parameters in one launch.
//
// The training step of Pointrix updates every parameter group with torch's
// Adam (pointrix/optimizer/optimizer.py:128-140; an apex FusedAdam hook at
// pointrix/optimizer/__init__.py:56-59).  Here all groups are one segment
// table and one launch; each element is read once (param, grad, both moments)
// and written once (param, both moments): 28 bytes per element, an HBM
// stream.  The update is torch.optim.Adam's (no weight decay, no amsgrad):
//   m = b1 m + (1 - b1) g;  v = b2 v + (1 - b2) g^2
//   p -= (lr / bc1) * m / (sqrt(v) / sqrt(bc2) + eps)
// with the bias corrections bc1 = 1 - b1^t, bc2 = 1 - b2^t of each segment's
// own step count t (a tensor skipped in a step keeps its count, as in torch).
#include "pgb_common.cuh"

namespace pgb {

constexpr int kAdamThreads = 256;
constexpr int kMaxAdamSegments = 32;

struct AdamTable {
  pgb_adam_segment seg[kMaxAdamSegments];
  int64_t start4[kMaxAdamSegments + 1];  // prefix of ceil(n / 4) over segments
  int nseg;
};

__device__ __forceinline__ void adam_one(float& p, float g, float& m, float& v, float b1, float b2,
                                         float eps, float step_size, float inv_sqrt_bc2) {
  m = b1 * m + (1.f - b1) * g;
  v = b2 * v + (1.f - b2) * g * g;
  p -= step_size * m / (sqrtf(v) * inv_sqrt_bc2 + eps);
}

// Step counts on the device (graph-captured steps): every segment's count
// goes up by one, and its bias corrections 1 - beta^t are formed once for
// the update to read.  beta^t is the double product of t factors, by binary
// powering over the bits of t (a few multiplies, not a pow per step).
__device__ inline double pow_int(double b, int t) {
  double r = 1.0;
  while (t > 0) {
    if (t & 1) r *= b;
    b *= b;
    t >>= 1;
  }
  return r;
}

__global__ void adam_tick_kernel(int32_t* __restrict__ steps, float* __restrict__ bc, int nseg,
                                 double b1d, double b2d) {
  const int s = threadIdx.x;
  if (s < nseg) {
    const int t = steps[s] + 1;
    steps[s] = t;
    bc[2 * s] = (float)(1.0 - pow_int(b1d, t));
    bc[2 * s + 1] = (float)(1.0 - pow_int(b2d, t));
  }
}

// bc == nullptr: the table's bias corrections; else those the tick formed.
__global__ void __launch_bounds__(kAdamThreads) adam_kernel(AdamTable t, float b1, float b2,
                                                            float eps,
                                                            const float* __restrict__ bc) {
  const int64_t total = t.start4[t.nseg];
  int s = 0;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    while (q >= t.start4[s + 1]) ++s;  // q only grows for a thread
    const pgb_adam_segment& sg = t.seg[s];
    const int64_t i = (q - t.start4[s]) * 4;
    const float bc1 = bc ? bc[2 * s] : sg.bias_correction1;
    const float bc2 = bc ? bc[2 * s + 1] : sg.bias_correction2;
    const float step_size = sg.lr / bc1;
    const float inv_sqrt_bc2 = 1.0f / sqrtf(bc2);
    if (i + 4 <= sg.n && (((uintptr_t)sg.param | (uintptr_t)sg.grad | (uintptr_t)sg.exp_avg |
                           (uintptr_t)sg.exp_avg_sq) & 15) == 0) {
      float4 p = reinterpret_cast<float4*>(sg.param)[i / 4];
      const float4 g = reinterpret_cast<const float4*>(sg.grad)[i / 4];
      float4 m = reinterpret_cast<float4*>(sg.exp_avg)[i / 4];
      float4 v = reinterpret_cast<float4*>(sg.exp_avg_sq)[i / 4];
      adam_one(p.x, g.x, m.x, v.x, b1, b2, eps, step_size, inv_sqrt_bc2);
      adam_one(p.y, g.y, m.y, v.y, b1, b2, eps, step_size, inv_sqrt_bc2);
      adam_one(p.z, g.z, m.z, v.z, b1, b2, eps, step_size, inv_sqrt_bc2);
      adam_one(p.w, g.w, m.w, v.w, b1, b2, eps, step_size, inv_sqrt_bc2);
      reinterpret_cast<float4*>(sg.param)[i / 4] = p;
      reinterpret_cast<float4*>(sg.exp_avg)[i / 4] = m;
      reinterpret_cast<float4*>(sg.exp_avg_sq)[i / 4] = v;
    } else {
      for (int64_t j = i; j < i + 4 && j < sg.n; ++j)
        adam_one(sg.param[j], sg.grad[j], sg.exp_avg[j], sg.exp_avg_sq[j], b1, b2, eps, step_size,
                 inv_sqrt_bc2);
    }
  }
}

static int adam_launch(const pgb_adam_segment* segments, int nsegments, float beta1, float beta2,
                       float eps, int32_t* steps, float* bc, double b1d, double b2d,
                       cudaStream_t st) {
  if (nsegments < 0 || nsegments > kMaxAdamSegments || (nsegments > 0 && !segments))
    return PGB_ERR_INVALID;
  AdamTable t;
  t.nseg = nsegments;
  t.start4[0] = 0;
  for (int i = 0; i < nsegments; ++i) {
    const pgb_adam_segment& s = segments[i];
    if (s.n < 0 || (s.n > 0 && (!s.param || !s.grad || !s.exp_avg || !s.exp_avg_sq)))
      return PGB_ERR_INVALID;
    if (!steps && (!(s.bias_correction1 > 0.f) || !(s.bias_correction2 > 0.f)))
      return PGB_ERR_INVALID;
    t.seg[i] = s;
    t.start4[i + 1] = t.start4[i] + (s.n + 3) / 4;
  }
  if (steps) adam_tick_kernel<<<1, 32, 0, st>>>(steps, bc, nsegments, b1d, b2d);
  const int64_t total = t.start4[nsegments];
  if (total > 0)
    adam_kernel<<<stream_grid(total, kAdamThreads, 8), kAdamThreads, 0, st>>>(t, beta1, beta2, eps,
                                                                              steps ? bc : nullptr);
  return launch_status();
}

}  // namespace pgb

extern "C" int pgb_adam_step(const pgb_adam_segment* segments, int nsegments, float beta1,
                             float beta2, float eps, void* stream) {
  return pgb::adam_launch(segments, nsegments, beta1, beta2, eps, nullptr, nullptr, 0.0, 0.0,
                          pgb::as_stream(stream));
}

extern "C" int pgb_adam_step_device(const pgb_adam_segment* segments, int nsegments, double beta1,
                                    double beta2, float eps, int32_t* step_counts,
                                    float* bias_corrections, void* stream) {
  if ((!step_counts || !bias_corrections) && nsegments > 0) return PGB_ERR_INVALID;
  return pgb::adam_launch(segments, nsegments, (float)beta1, (float)beta2, eps, step_counts,
                          bias_corrections, beta1, beta2, pgb::as_stream(stream));
}
