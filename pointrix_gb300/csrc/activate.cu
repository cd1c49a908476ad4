// Parameter activations of the Gaussian point cloud and the normal feature,
// forward and backward, in one pass over the Gaussians.
//
// The reference evaluates these in torch before every render:
//   scaling  = exp(log_scale)               gaussian_points.py:74-76
//   opacity  = sigmoid(logit)               gaussian_points.py:70-72
//   rotation = q / max(|q|, 1e-12)          gaussian_points.py:78-80 (F.normalize)
//   normal   = normalize(R(rotation) e_a),  a = argmin(log_scale)
//              examples/supervise/model.py:50-62, R from the unit-quaternion
//              formula of pointrix/utils/pose.py:40-84 (wxyz storage)
// which is a dozen kernels forward and as many backward over [N,*] tensors.
// Here one thread per Gaussian reads the 8 stored floats once and writes the
// 11 activated ones (forward), or reads the stored floats and the incoming
// gradients and writes the 8 parameter gradients (backward, recomputing the
// forward values).  The argmin takes the first minimum, like torch.argmin.
#include "pgb_common.cuh"

namespace pgb {

constexpr float kNormEps = 1e-12f;  // F.normalize's eps

// Column a of the rotation matrix of unit quaternion (w, x, y, z).
__device__ inline void rot_column(float w, float x, float y, float z, int a, float& c0, float& c1,
                                  float& c2) {
  const float x2 = x * x, y2 = y * y, z2 = z * z, w2 = w * w;
  if (a == 0) {
    c0 = x2 - y2 - z2 + w2;
    c1 = 2.f * (x * y + z * w);
    c2 = 2.f * (x * z - y * w);
  } else if (a == 1) {
    c0 = 2.f * (x * y - z * w);
    c1 = -x2 + y2 - z2 + w2;
    c2 = 2.f * (y * z + x * w);
  } else {
    c0 = 2.f * (x * z + y * w);
    c1 = 2.f * (y * z - x * w);
    c2 = -x2 - y2 + z2 + w2;
  }
}

// Gradient of column a with respect to (w, x, y, z), contracted with g.
__device__ inline void rot_column_grad(float w, float x, float y, float z, int a, float g0, float g1,
                                       float g2, float& dw, float& dx, float& dy, float& dz) {
  if (a == 0) {  // (x2-y2-z2+w2, 2(xy+zw), 2(xz-yw))
    dw = 2.f * (w * g0 + z * g1 - y * g2);
    dx = 2.f * (x * g0 + y * g1 + z * g2);
    dy = 2.f * (-y * g0 + x * g1 - w * g2);
    dz = 2.f * (-z * g0 + w * g1 + x * g2);
  } else if (a == 1) {  // (2(xy-zw), -x2+y2-z2+w2, 2(yz+xw))
    dw = 2.f * (-z * g0 + w * g1 + x * g2);
    dx = 2.f * (y * g0 - x * g1 + w * g2);
    dy = 2.f * (x * g0 + y * g1 + z * g2);
    dz = 2.f * (-w * g0 - z * g1 + y * g2);
  } else {  // (2(xz+yw), 2(yz-xw), -x2-y2+z2+w2)
    dw = 2.f * (y * g0 - x * g1 + w * g2);
    dx = 2.f * (z * g0 - w * g1 - x * g2);
    dy = 2.f * (w * g0 + z * g1 - y * g2);
    dz = 2.f * (x * g0 + y * g1 + z * g2);
  }
}

__device__ inline int argmin3(float a, float b, float c) {
  int i = 0;
  float m = a;
  if (b < m) { i = 1; m = b; }
  if (c < m) i = 2;
  return i;
}

struct Activated {
  float s[3], q[4], o, nrm_q, nraw[3], nrm_n;
  int axis;
};

__device__ inline Activated activate_one(const float* __restrict__ log_scale,
                                         const float* __restrict__ quat,
                                         const float* __restrict__ logit, int64_t i) {
  Activated A;
  const float l0 = log_scale[3 * i], l1 = log_scale[3 * i + 1], l2 = log_scale[3 * i + 2];
  A.s[0] = expf(l0);
  A.s[1] = expf(l1);
  A.s[2] = expf(l2);
  A.o = 1.f / (1.f + expf(-logit[i]));
  const float4 q = reinterpret_cast<const float4*>(quat)[i];
  A.nrm_q = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  const float dq = fmaxf(A.nrm_q, kNormEps);
  A.q[0] = q.x / dq;
  A.q[1] = q.y / dq;
  A.q[2] = q.z / dq;
  A.q[3] = q.w / dq;
  A.axis = argmin3(l0, l1, l2);
  rot_column(A.q[0], A.q[1], A.q[2], A.q[3], A.axis, A.nraw[0], A.nraw[1], A.nraw[2]);
  A.nrm_n = sqrtf(A.nraw[0] * A.nraw[0] + A.nraw[1] * A.nraw[1] + A.nraw[2] * A.nraw[2]);
  return A;
}

__global__ void __launch_bounds__(kStreamThreads) activate_fwd_kernel(
    const float* __restrict__ log_scale, const float* __restrict__ quat,
    const float* __restrict__ logit, int64_t n, float* __restrict__ scaling,
    float* __restrict__ rotation, float* __restrict__ opacity, float* __restrict__ normal) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Activated A = activate_one(log_scale, quat, logit, i);
    scaling[3 * i] = A.s[0];
    scaling[3 * i + 1] = A.s[1];
    scaling[3 * i + 2] = A.s[2];
    reinterpret_cast<float4*>(rotation)[i] = make_float4(A.q[0], A.q[1], A.q[2], A.q[3]);
    opacity[i] = A.o;
    if (normal) {
      const float dn = fmaxf(A.nrm_n, kNormEps);
      normal[3 * i] = A.nraw[0] / dn;
      normal[3 * i + 1] = A.nraw[1] / dn;
      normal[3 * i + 2] = A.nraw[2] / dn;
    }
  }
}

// d(v / max(|v|, eps)) for v of norm `nrm`: (g - u (u . g)) / |v| above eps,
// g / eps below (where the clamp is active the norm has no gradient).
template <int D>
__device__ inline void normalize_grad(const float* v, float nrm, const float* g, float* dv) {
  if (nrm > kNormEps) {
    float u[D], dot = 0.f;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      u[j] = v[j] / nrm;
      dot += u[j] * g[j];
    }
#pragma unroll
    for (int j = 0; j < D; ++j) dv[j] = (g[j] - u[j] * dot) / nrm;
  } else {
#pragma unroll
    for (int j = 0; j < D; ++j) dv[j] = g[j] / kNormEps;
  }
}

__global__ void __launch_bounds__(kStreamThreads) activate_bwd_kernel(
    const float* __restrict__ log_scale, const float* __restrict__ quat,
    const float* __restrict__ logit, int64_t n, const float* __restrict__ d_scaling,
    const float* __restrict__ d_rotation, const float* __restrict__ d_opacity,
    const float* __restrict__ d_normal, float* __restrict__ d_log_scale,
    float* __restrict__ d_quat, float* __restrict__ d_logit) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Activated A = activate_one(log_scale, quat, logit, i);
#pragma unroll
    for (int j = 0; j < 3; ++j) d_log_scale[3 * i + j] = d_scaling ? d_scaling[3 * i + j] * A.s[j] : 0.f;
    d_logit[i] = d_opacity ? d_opacity[i] * (A.o * (1.f - A.o)) : 0.f;
    float dr[4] = {0.f, 0.f, 0.f, 0.f};
    if (d_rotation) {
      const float4 g = reinterpret_cast<const float4*>(d_rotation)[i];
      dr[0] = g.x;
      dr[1] = g.y;
      dr[2] = g.z;
      dr[3] = g.w;
    }
    if (d_normal) {
      const float gn[3] = {d_normal[3 * i], d_normal[3 * i + 1], d_normal[3 * i + 2]};
      float dnr[3];
      normalize_grad<3>(A.nraw, A.nrm_n, gn, dnr);
      float dw, dx, dy, dz;
      rot_column_grad(A.q[0], A.q[1], A.q[2], A.q[3], A.axis, dnr[0], dnr[1], dnr[2], dw, dx, dy, dz);
      dr[0] += dw;
      dr[1] += dx;
      dr[2] += dy;
      dr[3] += dz;
    }
    const float4 q = reinterpret_cast<const float4*>(quat)[i];
    const float qv[4] = {q.x, q.y, q.z, q.w};
    float dq[4];
    normalize_grad<4>(qv, A.nrm_q, dr, dq);
    reinterpret_cast<float4*>(d_quat)[i] = make_float4(dq[0], dq[1], dq[2], dq[3]);
  }
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_gaussian_activate_forward(const float* log_scale, const float* quat,
                                  const float* opacity_logit, int64_t n, float* scaling,
                                  float* rotation, float* opacity, float* normal, void* stream) {
  if (n < 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!log_scale || !quat || !opacity_logit || !scaling || !rotation || !opacity)
    return PGB_ERR_INVALID;
  if (!aligned16(quat) || !aligned16(rotation)) return PGB_ERR_INVALID;
  activate_fwd_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(
      log_scale, quat, opacity_logit, n, scaling, rotation, opacity, normal);
  return launch_status();
}

int pgb_gaussian_activate_backward(const float* log_scale, const float* quat,
                                   const float* opacity_logit, int64_t n, const float* d_scaling,
                                   const float* d_rotation, const float* d_opacity,
                                   const float* d_normal, float* d_log_scale, float* d_quat,
                                   float* d_opacity_logit, void* stream) {
  if (n < 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!log_scale || !quat || !opacity_logit || !d_log_scale || !d_quat || !d_opacity_logit)
    return PGB_ERR_INVALID;
  if (!aligned16(quat) || !aligned16(d_quat) || (d_rotation && !aligned16(d_rotation)))
    return PGB_ERR_INVALID;
  activate_bwd_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(
      log_scale, quat, opacity_logit, n, d_scaling, d_rotation, d_opacity, d_normal, d_log_scale,
      d_quat, d_opacity_logit);
  return launch_status();
}

}  // extern "C"
