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

// One float4 group q of the table: segment s (found by walking forward from
// the caller's s, since a thread's q only grows), element offset i, and
// whether the group is a whole aligned float4 of the segment.
struct AdamGroup {
  const pgb_adam_segment* sg;
  int64_t i;
  float step_size, inv_sqrt_bc2;
  bool vec;
};

__device__ __forceinline__ AdamGroup adam_group(const AdamTable& t, const float* bc, int64_t q,
                                                int& s) {
  while (q >= t.start4[s + 1]) ++s;
  AdamGroup gr;
  gr.sg = &t.seg[s];
  gr.i = (q - t.start4[s]) * 4;
  const float bc1 = bc ? bc[2 * s] : gr.sg->bias_correction1;
  const float bc2 = bc ? bc[2 * s + 1] : gr.sg->bias_correction2;
  gr.step_size = gr.sg->lr / bc1;
  gr.inv_sqrt_bc2 = 1.0f / sqrtf(bc2);
  gr.vec = gr.i + 4 <= gr.sg->n &&
           (((uintptr_t)gr.sg->param | (uintptr_t)gr.sg->grad | (uintptr_t)gr.sg->exp_avg |
             (uintptr_t)gr.sg->exp_avg_sq) & 15) == 0;
  return gr;
}

__device__ __forceinline__ void adam_scalar(const AdamGroup& gr, float b1, float b2, float eps) {
  const pgb_adam_segment& sg = *gr.sg;
  for (int64_t j = gr.i; j < gr.i + 4 && j < sg.n; ++j)
    adam_one(sg.param[j], sg.grad[j], sg.exp_avg[j], sg.exp_avg_sq[j], b1, b2, eps, gr.step_size,
             gr.inv_sqrt_bc2);
}

__device__ __forceinline__ void adam_vec4(float4& p, const float4& g, float4& m, float4& v, float b1,
                                          float b2, float eps, const AdamGroup& gr) {
  adam_one(p.x, g.x, m.x, v.x, b1, b2, eps, gr.step_size, gr.inv_sqrt_bc2);
  adam_one(p.y, g.y, m.y, v.y, b1, b2, eps, gr.step_size, gr.inv_sqrt_bc2);
  adam_one(p.z, g.z, m.z, v.z, b1, b2, eps, gr.step_size, gr.inv_sqrt_bc2);
  adam_one(p.w, g.w, m.w, v.w, b1, b2, eps, gr.step_size, gr.inv_sqrt_bc2);
}

// bc == nullptr: the table's bias corrections; else those the tick formed.
// Each thread takes two float4 groups per iteration (q and q + stride) and
// issues all eight loads before the arithmetic, so twice the bytes are in
// flight per thread.
__global__ void __launch_bounds__(kAdamThreads) adam_kernel(AdamTable t, float b1, float b2,
                                                            float eps,
                                                            const float* __restrict__ bc) {
  const int64_t total = t.start4[t.nseg];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int s = 0;
  for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q0 < total;
       q0 += 2 * stride) {
    const int64_t q1 = q0 + stride;
    const bool has1 = q1 < total;
    const AdamGroup g0 = adam_group(t, bc, q0, s);
    int s1 = s;
    const AdamGroup g1 = has1 ? adam_group(t, bc, q1, s1) : g0;
    if (g0.vec && (!has1 || g1.vec)) {
      float4 p0 = reinterpret_cast<float4*>(g0.sg->param)[g0.i / 4];
      const float4 gg0 = reinterpret_cast<const float4*>(g0.sg->grad)[g0.i / 4];
      float4 m0 = reinterpret_cast<float4*>(g0.sg->exp_avg)[g0.i / 4];
      float4 v0 = reinterpret_cast<float4*>(g0.sg->exp_avg_sq)[g0.i / 4];
      float4 p1, gg1, m1, v1;
      if (has1) {
        p1 = reinterpret_cast<float4*>(g1.sg->param)[g1.i / 4];
        gg1 = reinterpret_cast<const float4*>(g1.sg->grad)[g1.i / 4];
        m1 = reinterpret_cast<float4*>(g1.sg->exp_avg)[g1.i / 4];
        v1 = reinterpret_cast<float4*>(g1.sg->exp_avg_sq)[g1.i / 4];
      }
      adam_vec4(p0, gg0, m0, v0, b1, b2, eps, g0);
      reinterpret_cast<float4*>(g0.sg->param)[g0.i / 4] = p0;
      reinterpret_cast<float4*>(g0.sg->exp_avg)[g0.i / 4] = m0;
      reinterpret_cast<float4*>(g0.sg->exp_avg_sq)[g0.i / 4] = v0;
      if (has1) {
        adam_vec4(p1, gg1, m1, v1, b1, b2, eps, g1);
        reinterpret_cast<float4*>(g1.sg->param)[g1.i / 4] = p1;
        reinterpret_cast<float4*>(g1.sg->exp_avg)[g1.i / 4] = m1;
        reinterpret_cast<float4*>(g1.sg->exp_avg_sq)[g1.i / 4] = v1;
      }
    } else {
      adam_scalar(g0, b1, b2, eps);
      if (has1) adam_scalar(g1, b1, b2, eps);
    }
    s = s1;
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
