// Camera pose of a differentiable camera, forward and backward, in one
// single-block launch each way.
//
// Pointrix optimises camera poses stored as a wxyz quaternion and a
// translation; the rotation is the homogeneous unit-quaternion formula of
// pointrix/utils/pose.py:40-84 applied to q / |q|, the world->camera matrix
// is [R t; 0 0 0 1] and the camera centre is -R^T t.  In torch that is a
// dozen tiny kernels forward and as many backward per step; here:
//   forward:  q [4], t [3] -> E [4,4] (row-major), centre [3]
//   backward: dE [4,4] (or NULL), dcentre [3] (or NULL) -> dq [4], dt [3]
// The arithmetic is float, in the order of the torch composition (rotation
// entries from the products of the unit quaternion's components).
#include "pgb_common.cuh"

namespace pgb {

// Rotation of unit quaternion u = (w, x, y, z), row-major.
__device__ inline void quat_rotation(const float u[4], float R[9]) {
  const float w = u[0], x = u[1], y = u[2], z = u[3];
  R[0] = w * w + x * x - y * y - z * z;
  R[1] = 2.f * (x * y) - 2.f * (w * z);
  R[2] = 2.f * (x * z) + 2.f * (w * y);
  R[3] = 2.f * (x * y) + 2.f * (w * z);
  R[4] = w * w - x * x + y * y - z * z;
  R[5] = 2.f * (y * z) - 2.f * (w * x);
  R[6] = 2.f * (x * z) - 2.f * (w * y);
  R[7] = 2.f * (y * z) + 2.f * (w * x);
  R[8] = w * w - x * x - y * y + z * z;
}

__global__ void camera_pose_fwd_kernel(const float* __restrict__ q, const float* __restrict__ t,
                                       float* __restrict__ E, float* __restrict__ centre) {
  if (threadIdx.x != 0) return;
  const float nq = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const float u[4] = {q[0] / nq, q[1] / nq, q[2] / nq, q[3] / nq};
  float R[9];
  quat_rotation(u, R);
  const float tv[3] = {t[0], t[1], t[2]};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    E[4 * i] = R[3 * i];
    E[4 * i + 1] = R[3 * i + 1];
    E[4 * i + 2] = R[3 * i + 2];
    E[4 * i + 3] = tv[i];
  }
  E[12] = 0.f;
  E[13] = 0.f;
  E[14] = 0.f;
  E[15] = 1.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) centre[i] = -(R[i] * tv[0] + R[3 + i] * tv[1] + R[6 + i] * tv[2]);
}

__global__ void camera_pose_bwd_kernel(const float* __restrict__ q, const float* __restrict__ t,
                                       const float* __restrict__ dE,
                                       const float* __restrict__ dcentre, float* __restrict__ dq,
                                       float* __restrict__ dt) {
  if (threadIdx.x != 0) return;
  const float nq = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const float u[4] = {q[0] / nq, q[1] / nq, q[2] / nq, q[3] / nq};
  float R[9];
  quat_rotation(u, R);
  const float tv[3] = {t[0], t[1], t[2]};
  float dR[9], dtv[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) dR[3 * i + j] = dE ? dE[4 * i + j] : 0.f;
    dtv[i] = dE ? dE[4 * i + 3] : 0.f;
  }
  if (dcentre) {  // c_j = -sum_i R_ij t_i
    const float dc[3] = {dcentre[0], dcentre[1], dcentre[2]};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = 0; j < 3; ++j) dR[3 * i + j] -= tv[i] * dc[j];
      dtv[i] -= R[3 * i] * dc[0] + R[3 * i + 1] * dc[1] + R[3 * i + 2] * dc[2];
    }
  }
  // d(rotation entries)/d(unit quaternion), contracted with dR
  const float w = u[0], x = u[1], y = u[2], z = u[3];
  const float du[4] = {
      2.f * (w * (dR[0] + dR[4] + dR[8]) - z * dR[1] + y * dR[2] + z * dR[3] - x * dR[5] -
             y * dR[6] + x * dR[7]),
      2.f * (x * (dR[0] - dR[4] - dR[8]) + y * dR[1] + z * dR[2] + y * dR[3] - w * dR[5] +
             z * dR[6] + w * dR[7]),
      2.f * (y * (-dR[0] + dR[4] - dR[8]) + x * dR[1] + w * dR[2] + x * dR[3] + z * dR[5] -
             w * dR[6] + z * dR[7]),
      2.f * (z * (-dR[0] - dR[4] + dR[8]) - w * dR[1] + x * dR[2] + w * dR[3] + y * dR[5] +
             x * dR[6] + y * dR[7])};
  // u = q / |q|: dq = (du - u (u . du)) / |q|
  const float dot = u[0] * du[0] + u[1] * du[1] + u[2] * du[2] + u[3] * du[3];
#pragma unroll
  for (int k = 0; k < 4; ++k) dq[k] = (du[k] - u[k] * dot) / nq;
#pragma unroll
  for (int i = 0; i < 3; ++i) dt[i] = dtv[i];
}

}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_camera_pose_forward(const float* quat, const float* translation, float* world_to_camera,
                            float* centre, void* stream) {
  if (!quat || !translation || !world_to_camera || !centre) return PGB_ERR_INVALID;
  camera_pose_fwd_kernel<<<1, 32, 0, as_stream(stream)>>>(quat, translation, world_to_camera,
                                                          centre);
  return launch_status();
}

int pgb_camera_pose_backward(const float* quat, const float* translation,
                             const float* d_world_to_camera, const float* d_centre, float* d_quat,
                             float* d_translation, void* stream) {
  if (!quat || !translation || !d_quat || !d_translation) return PGB_ERR_INVALID;
  camera_pose_bwd_kernel<<<1, 32, 0, as_stream(stream)>>>(quat, translation, d_world_to_camera,
                                                          d_centre, d_quat, d_translation);
  return launch_status();
}

}  // extern "C"
