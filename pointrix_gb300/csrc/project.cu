// Per-Gaussian projection operators: project_point, compute_cov3d,
// ewa_project (forward and backward), and the camera-gradient reduction.
//
// This translation unit is compiled with -fmad=false: every float step is a
// separately rounded IEEE operation in source order, so radius and
// tiles_touched (integers derived from float arithmetic) are reproduced bit
// for bit by a float32 CPU rendition that performs the same steps.  These
// kernels are HBM streams (24-65 algorithmic bytes per Gaussian), so giving
// up FMA costs nothing measurable.
//
// Operator contracts: pointrix/model/renderer/msplat.py:109-130 (call
// sites); the mathematics is EWA splatting (Zwicker et al. 2001) as used by
// 3D Gaussian Splatting (Kerbl et al. 2023).
#include "pgb_common.cuh"

namespace pgb {

constexpr float kFovClamp = 1.3f;
constexpr float kDilation = 0.3f;
constexpr float kEigFloor = 0.1f;
constexpr float kRadiusCap = 1048576.0f;

struct Cam {
  float e[12];  // world->camera [3,4]
  float fx, fy, cx, cy;
};

__device__ inline Cam load_cam(const float* __restrict__ intr, const float* __restrict__ extr) {
  Cam c;
#pragma unroll
  for (int i = 0; i < 12; ++i) c.e[i] = __ldg(extr + i);
  c.fx = __ldg(intr + 0);
  c.fy = __ldg(intr + 1);
  c.cx = __ldg(intr + 2);
  c.cy = __ldg(intr + 3);
  return c;
}

__device__ inline void cam_point(const Cam& c, float x, float y, float z, float& px, float& py,
                                 float& pz) {
  px = c.e[0] * x + c.e[1] * y + c.e[2] * z + c.e[3];
  py = c.e[4] * x + c.e[5] * y + c.e[6] * z + c.e[7];
  pz = c.e[8] * x + c.e[9] * y + c.e[10] * z + c.e[11];
}

// Projection with the visibility test of project_point.
__device__ inline bool project_visible(const Cam& c, float px, float py, float pz, int W, int H,
                                       float nearest, float extent, float& u, float& v) {
  if (!(pz > nearest)) return false;
  u = c.fx * px / pz + c.cx;
  v = c.fy * py / pz + c.cy;
  const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;
  return fabsf(u - hw) < extent * hw && fabsf(v - hh) < extent * hh;
}

// ---------------------------------------------------------------------------
// Camera-gradient reduction: every block of a backward kernel writes its 16
// partial sums (d_intr[4], d_extr[12]); one block then sums the partials in
// block order, so the result does not depend on scheduling.
// ---------------------------------------------------------------------------
constexpr int kCamGradBlocksMax = kNumSMs * 8;

__device__ inline void block_write_partials(float (&acc)[16], float* __restrict__ partials) {
  __shared__ float red[kStreamThreads / 32][16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    float s = warp_sum(acc[i]);
    if (lane == 0) red[warp][i] = s;
  }
  __syncthreads();
  if (threadIdx.x < 16) {
    float s = 0.f;
    for (int w = 0; w < kStreamThreads / 32; ++w) s += red[w][threadIdx.x];
    partials[blockIdx.x * 16 + threadIdx.x] = s;
  }
}

// 16 columns x 64 threads: column c sums partials[b * 16 + c] over blocks in
// a fixed order (in double).
constexpr int kCamTPC = 64;

__global__ void __launch_bounds__(16 * kCamTPC) cam_grad_finish_kernel(
    const float* __restrict__ partials, int nblocks, float* __restrict__ d_intr,
    float* __restrict__ d_extr) {
  __shared__ double s[16 * kCamTPC];
  const double t = column_sum<16, kCamTPC>(partials, nblocks, 16, s);
  if (threadIdx.x % kCamTPC == 0) {
    const int col = threadIdx.x / kCamTPC;
    if (col < 4)
      d_intr[col] = (float)t;
    else
      d_extr[col - 4] = (float)t;
  }
}

// ---------------------------------------------------------------------------
// project_point
// ---------------------------------------------------------------------------
__global__ void project_point_fwd_kernel(const float* __restrict__ xyz, int64_t n,
                                         const float* __restrict__ intr,
                                         const float* __restrict__ extr, int W, int H,
                                         float nearest, float extent, float* __restrict__ uv,
                                         float* __restrict__ depth) {
  const Cam c = load_cam(intr, extr);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    float px, py, pz, u, v;
    cam_point(c, x, y, z, px, py, pz);
    const bool vis = project_visible(c, px, py, pz, W, H, nearest, extent, u, v);
    reinterpret_cast<float2*>(uv)[i] = vis ? make_float2(u, v) : make_float2(0.f, 0.f);
    depth[i] = vis ? pz : 0.f;
  }
}

// Backward of project_point for one visible Gaussian (camera point p):
// d xyz and the camera accumulators from d uv and d depth.
__device__ inline void project_bwd_one(const Cam& c, float x, float y, float z, float px, float py,
                                       float pz, float2 du, float dd, float& gx, float& gy,
                                       float& gz, float (&acc)[16]) {
  const float iz = 1.0f / pz;
  const float gpx = du.x * c.fx * iz;
  const float gpy = du.y * c.fy * iz;
  const float gpz = dd - (du.x * c.fx * px + du.y * c.fy * py) * iz * iz;
  gx = c.e[0] * gpx + c.e[4] * gpy + c.e[8] * gpz;
  gy = c.e[1] * gpx + c.e[5] * gpy + c.e[9] * gpz;
  gz = c.e[2] * gpx + c.e[6] * gpy + c.e[10] * gpz;
  acc[0] += du.x * px * iz;
  acc[1] += du.y * py * iz;
  acc[2] += du.x;
  acc[3] += du.y;
  const float gp[3] = {gpx, gpy, gpz};
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    acc[4 + 4 * r + 0] += gp[r] * x;
    acc[4 + 4 * r + 1] += gp[r] * y;
    acc[4 + 4 * r + 2] += gp[r] * z;
    acc[4 + 4 * r + 3] += gp[r];
  }
}

__global__ void project_point_bwd_kernel(const float* __restrict__ xyz, int64_t n,
                                         const float* __restrict__ intr,
                                         const float* __restrict__ extr, int W, int H,
                                         float nearest, float extent,
                                         const float* __restrict__ d_uv,
                                         const float* __restrict__ d_depth,
                                         float* __restrict__ d_xyz, float* __restrict__ partials) {
  const Cam c = load_cam(intr, extr);
  float acc[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i] = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    float px, py, pz, u, v;
    cam_point(c, x, y, z, px, py, pz);
    float gx = 0.f, gy = 0.f, gz = 0.f;
    if (project_visible(c, px, py, pz, W, H, nearest, extent, u, v))
      project_bwd_one(c, x, y, z, px, py, pz, reinterpret_cast<const float2*>(d_uv)[i], d_depth[i],
                      gx, gy, gz, acc);
    d_xyz[3 * i] = gx;
    d_xyz[3 * i + 1] = gy;
    d_xyz[3 * i + 2] = gz;
  }
  block_write_partials(acc, partials);
}

// ---------------------------------------------------------------------------
// compute_cov3d
// ---------------------------------------------------------------------------
struct Rot {
  float r[3][3];
};

__device__ inline Rot quat_rot(float w, float x, float y, float z) {
  const float xx = x * x, yy = y * y, zz = z * z;
  const float xy = x * y, xz = x * z, yz = y * z;
  const float wx = w * x, wy = w * y, wz = w * z;
  Rot R;
  R.r[0][0] = 1.f - 2.f * (yy + zz);
  R.r[0][1] = 2.f * (xy - wz);
  R.r[0][2] = 2.f * (xz + wy);
  R.r[1][0] = 2.f * (xy + wz);
  R.r[1][1] = 1.f - 2.f * (xx + zz);
  R.r[1][2] = 2.f * (yz - wx);
  R.r[2][0] = 2.f * (xz - wy);
  R.r[2][1] = 2.f * (yz + wx);
  R.r[2][2] = 1.f - 2.f * (xx + yy);
  return R;
}

// Sigma = (R S)(R S)^T, upper triangle, of Gaussian i.
__device__ inline void cov3d_one(const float* __restrict__ scales, const float* __restrict__ q,
                                 int64_t i, float (&out)[6]) {
  const float4 qq = reinterpret_cast<const float4*>(q)[i];
  const float s[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
  const Rot R = quat_rot(qq.x, qq.y, qq.z, qq.w);
  float M[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) M[a][b] = R.r[a][b] * s[b];
  auto sig = [&](int a, int b) {
    return M[a][0] * M[b][0] + M[a][1] * M[b][1] + M[a][2] * M[b][2];
  };
  out[0] = sig(0, 0);
  out[1] = sig(0, 1);
  out[2] = sig(0, 2);
  out[3] = sig(1, 1);
  out[4] = sig(1, 2);
  out[5] = sig(2, 2);
}

__global__ void cov3d_fwd_kernel(const float* __restrict__ scales, const float* __restrict__ q,
                                 const uint8_t* __restrict__ visible, int64_t n,
                                 float* __restrict__ cov) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float out[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (visible[i]) cov3d_one(scales, q, i, out);
    float2* o = reinterpret_cast<float2*>(cov + 6 * i);
    o[0] = make_float2(out[0], out[1]);
    o[1] = make_float2(out[2], out[3]);
    o[2] = make_float2(out[4], out[5]);
  }
}

// d scales and d quaternion of Gaussian i from the stored gradient g[6] of
// its covariance (upper triangle).
__device__ inline void cov3d_grad_one(const float* __restrict__ scales,
                                      const float* __restrict__ q, int64_t i, const float* g,
                                      float (&ds)[3], float4& dq) {
  const float4 qq = reinterpret_cast<const float4*>(q)[i];
  const float w = qq.x, x = qq.y, y = qq.z, z = qq.w;
  const float s[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
  const Rot R = quat_rot(w, x, y, z);
  float M[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) M[a][b] = R.r[a][b] * s[b];
  // Symmetric full gradient: off-diagonal stored entries feed both
  // halves of Sigma.
  float G[3][3];
  G[0][0] = g[0];
  G[1][1] = g[3];
  G[2][2] = g[5];
  G[0][1] = G[1][0] = 0.5f * g[1];
  G[0][2] = G[2][0] = 0.5f * g[2];
  G[1][2] = G[2][1] = 0.5f * g[4];
  float dM[3][3];  // dL/dM = 2 G M
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      dM[a][b] = 2.f * (G[a][0] * M[0][b] + G[a][1] * M[1][b] + G[a][2] * M[2][b]);
  float dR[3][3];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    ds[b] = dM[0][b] * R.r[0][b] + dM[1][b] * R.r[1][b] + dM[2][b] * R.r[2][b];
#pragma unroll
    for (int a = 0; a < 3; ++a) dR[a][b] = dM[a][b] * s[b];
  }
  dq.x = 2.f * (-z * dR[0][1] + y * dR[0][2] + z * dR[1][0] - x * dR[1][2] - y * dR[2][0] +
                x * dR[2][1]);
  dq.y = 2.f * (y * dR[0][1] + z * dR[0][2] + y * dR[1][0] - 2.f * x * dR[1][1] -
                w * dR[1][2] + z * dR[2][0] + w * dR[2][1] - 2.f * x * dR[2][2]);
  dq.z = 2.f * (-2.f * y * dR[0][0] + x * dR[0][1] + w * dR[0][2] + x * dR[1][0] +
                z * dR[1][2] - w * dR[2][0] + z * dR[2][1] - 2.f * y * dR[2][2]);
  dq.w = 2.f * (-2.f * z * dR[0][0] - w * dR[0][1] + x * dR[0][2] + w * dR[1][0] -
                2.f * z * dR[1][1] + y * dR[1][2] + x * dR[2][0] + y * dR[2][1]);
}

__global__ void cov3d_bwd_kernel(const float* __restrict__ scales, const float* __restrict__ q,
                                 const uint8_t* __restrict__ visible, int64_t n,
                                 const float* __restrict__ d_cov, float* __restrict__ d_scales,
                                 float* __restrict__ d_q) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float ds[3] = {0.f, 0.f, 0.f};
    float4 dq = make_float4(0.f, 0.f, 0.f, 0.f);
    if (visible[i]) cov3d_grad_one(scales, q, i, d_cov + 6 * i, ds, dq);
    d_scales[3 * i] = ds[0];
    d_scales[3 * i + 1] = ds[1];
    d_scales[3 * i + 2] = ds[2];
    reinterpret_cast<float4*>(d_q)[i] = dq;
  }
}

// ---------------------------------------------------------------------------
// ewa_project
// ---------------------------------------------------------------------------
struct Ewa {
  float pz, tx, ty, limx, limy, txtz, tytz, px, py;
  float J00, J02, J11, J12;
  float T0[3], T1[3];
  float a, b, c, det;
};

__device__ inline void ewa_core(const Cam& cm, int W, int H, float x, float y, float z,
                                const float* __restrict__ s6, Ewa& E) {
  cam_point(cm, x, y, z, E.px, E.py, E.pz);
  const float pz = E.pz;
  E.limx = kFovClamp * ((0.5f * (float)W) / cm.fx);
  E.limy = kFovClamp * ((0.5f * (float)H) / cm.fy);
  E.txtz = E.px / pz;
  E.tytz = E.py / pz;
  E.tx = fminf(fmaxf(E.txtz, -E.limx), E.limx) * pz;
  E.ty = fminf(fmaxf(E.tytz, -E.limy), E.limy) * pz;
  const float pz2 = pz * pz;
  E.J00 = cm.fx / pz;
  E.J02 = -(cm.fx * E.tx) / pz2;
  E.J11 = cm.fy / pz;
  E.J12 = -(cm.fy * E.ty) / pz2;
  const float* e = cm.e;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    E.T0[k] = E.J00 * e[k] + E.J02 * e[8 + k];
    E.T1[k] = E.J11 * e[4 + k] + E.J12 * e[8 + k];
  }
  const float s00 = s6[0], s01 = s6[1], s02 = s6[2], s11 = s6[3], s12 = s6[4], s22 = s6[5];
  const float* T0 = E.T0;
  const float* T1 = E.T1;
  const float V00 = s00 * T0[0] + s01 * T0[1] + s02 * T0[2];
  const float V01 = s01 * T0[0] + s11 * T0[1] + s12 * T0[2];
  const float V02 = s02 * T0[0] + s12 * T0[1] + s22 * T0[2];
  const float V10 = s00 * T1[0] + s01 * T1[1] + s02 * T1[2];
  const float V11 = s01 * T1[0] + s11 * T1[1] + s12 * T1[2];
  const float V12 = s02 * T1[0] + s12 * T1[1] + s22 * T1[2];
  E.a = T0[0] * V00 + T0[1] * V01 + T0[2] * V02 + kDilation;
  E.b = T1[0] * V00 + T1[1] * V01 + T1[2] * V02;
  E.c = T1[0] * V10 + T1[1] * V11 + T1[2] * V12 + kDilation;
  E.det = E.a * E.c - E.b * E.b;
}

// Conic, radius and tiles touched of one visible Gaussian (uv p).
__device__ inline void ewa_fwd_one(const Cam& cm, int W, int H, int gx, int gy, float x, float y,
                                   float z, const float* s6, float2 p, float& c0, float& c1,
                                   float& c2, int& rad, int& nt) {
  Ewa E;
  ewa_core(cm, W, H, x, y, z, s6, E);
  if (E.det > 0.f) {
    const float mid = 0.5f * (E.a + E.c);
    const float disc = fmaxf(kEigFloor, mid * mid - E.det);
    const float lam = mid + sqrtf(disc);
    const float rf = fminf(ceilf(3.0f * sqrtf(lam)), kRadiusCap);
    int x0, x1, y0, y1;
    tile_rect(p.x, p.y, rf, gx, gy, x0, x1, y0, y1);
    const int cnt = (x1 - x0) * (y1 - y0);
    if (cnt > 0) {
      const float inv = 1.0f / E.det;
      c0 = E.c * inv;
      c1 = -E.b * inv;
      c2 = E.a * inv;
      rad = (int)rf;
      nt = cnt;
    }
  }
}

__global__ void ewa_fwd_kernel(const float* __restrict__ xyz, const float* __restrict__ cov,
                               const float* __restrict__ intr, const float* __restrict__ extr,
                               const float* __restrict__ uv, const uint8_t* __restrict__ visible,
                               int64_t n, int W, int H, float* __restrict__ conic,
                               int32_t* __restrict__ radius, int32_t* __restrict__ tiles) {
  const Cam cm = load_cam(intr, extr);
  const int gx = grid_x(W), gy = grid_y(H);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
    int rad = 0, nt = 0;
    if (visible[i]) {
      float s6[6];
      const float2* cv = reinterpret_cast<const float2*>(cov + 6 * i);
      const float2 q0 = cv[0], q1 = cv[1], q2 = cv[2];
      s6[0] = q0.x; s6[1] = q0.y; s6[2] = q1.x; s6[3] = q1.y; s6[4] = q2.x; s6[5] = q2.y;
      ewa_fwd_one(cm, W, H, gx, gy, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], s6,
                  reinterpret_cast<const float2*>(uv)[i], c0, c1, c2, rad, nt);
    }
    conic[3 * i] = c0;
    conic[3 * i + 1] = c1;
    conic[3 * i + 2] = c2;
    radius[i] = rad;
    tiles[i] = nt;
  }
}

// Backward of ewa_project for one Gaussian with radius > 0: d xyz
// (gxw, gyw, gzw), d cov3d (dS) and the camera accumulators acc
// (d_intr[4], d_extr[12]) from the conic gradient (g0, g1, g2).
__device__ inline void ewa_bwd_one(const Cam& cm, int W, int H, float x, float y, float z,
                                   const float* s6, float g0, float g1, float g2, float& gxw,
                                   float& gyw, float& gzw, float (&dS)[6], float (&acc)[16]) {
  Ewa E;
  ewa_core(cm, W, H, x, y, z, s6, E);
  const float a = E.a, b = E.b, c = E.c;
  const float id = 1.0f / E.det;
  const float id2 = id * id;
  // conic = (c, -b, a) / det, det = a c - b^2
  const float da = -g0 * c * c * id2 + g1 * b * c * id2 + g2 * (id - a * c * id2);
  const float dc = g0 * (id - a * c * id2) + g1 * a * b * id2 - g2 * a * a * id2;
  const float db = 2.f * g0 * b * c * id2 + g1 * (-id - 2.f * b * b * id2) + 2.f * g2 * a * b * id2;
  // symmetric 2x2 gradient G2 = [[da, db/2], [db/2, dc]]
  const float G00 = da, G01 = 0.5f * db, G11 = dc;
  const float* T0 = E.T0;
  const float* T1 = E.T1;
  // dSigma_full = T^T G2 T; stored off-diagonals take both halves
  float U0[3], U1[3];  // (G2 T) rows
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    U0[k] = G00 * T0[k] + G01 * T1[k];
    U1[k] = G01 * T0[k] + G11 * T1[k];
  }
  auto full = [&](int p, int q) { return T0[p] * U0[q] + T1[p] * U1[q]; };
  dS[0] = full(0, 0);
  dS[1] = full(0, 1) + full(1, 0);
  dS[2] = full(0, 2) + full(2, 0);
  dS[3] = full(1, 1);
  dS[4] = full(1, 2) + full(2, 1);
  dS[5] = full(2, 2);
  // dT = 2 G2 T Sigma
  float S[3][3];
  S[0][0] = s6[0]; S[0][1] = S[1][0] = s6[1]; S[0][2] = S[2][0] = s6[2];
  S[1][1] = s6[3]; S[1][2] = S[2][1] = s6[4]; S[2][2] = s6[5];
  float dT0[3], dT1[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dT0[k] = 2.f * (U0[0] * S[0][k] + U0[1] * S[1][k] + U0[2] * S[2][k]);
    dT1[k] = 2.f * (U1[0] * S[0][k] + U1[1] * S[1][k] + U1[2] * S[2][k]);
  }
  const float* e = cm.e;
  const float dJ00 = dT0[0] * e[0] + dT0[1] * e[1] + dT0[2] * e[2];
  const float dJ02 = dT0[0] * e[8] + dT0[1] * e[9] + dT0[2] * e[10];
  const float dJ11 = dT1[0] * e[4] + dT1[1] * e[5] + dT1[2] * e[6];
  const float dJ12 = dT1[0] * e[8] + dT1[1] * e[9] + dT1[2] * e[10];
  // W = R part of the extrinsic: dW0 = J00 dT0, dW1 = J11 dT1, dW2 = J02 dT0 + J12 dT1
  float dR[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dR[0][k] = E.J00 * dT0[k];
    dR[1][k] = E.J11 * dT1[k];
    dR[2][k] = E.J02 * dT0[k] + E.J12 * dT1[k];
  }
  const float pz = E.pz, iz = 1.0f / pz, iz2 = iz * iz, iz3 = iz2 * iz;
  const float fx = cm.fx, fy = cm.fy;
  float dpz = -fx * iz2 * dJ00 - fy * iz2 * dJ11 + 2.f * fx * E.tx * iz3 * dJ02 +
              2.f * fy * E.ty * iz3 * dJ12;
  const float dtx = -fx * iz2 * dJ02;
  const float dty = -fy * iz2 * dJ12;
  float dfx = dJ00 * iz - E.tx * iz2 * dJ02;
  float dfy = dJ11 * iz - E.ty * iz2 * dJ12;
  float dpx = 0.f, dpy = 0.f;
  if (E.txtz < -E.limx) {
    dpz += -E.limx * dtx;
    dfx += (-pz * dtx) * (-E.limx / fx);
  } else if (E.txtz > E.limx) {
    dpz += E.limx * dtx;
    dfx += (pz * dtx) * (-E.limx / fx);
  } else {
    dpx = dtx;
  }
  if (E.tytz < -E.limy) {
    dpz += -E.limy * dty;
    dfy += (-pz * dty) * (-E.limy / fy);
  } else if (E.tytz > E.limy) {
    dpz += E.limy * dty;
    dfy += (pz * dty) * (-E.limy / fy);
  } else {
    dpy = dty;
  }
  // p = R x + t
  gxw = e[0] * dpx + e[4] * dpy + e[8] * dpz;
  gyw = e[1] * dpx + e[5] * dpy + e[9] * dpz;
  gzw = e[2] * dpx + e[6] * dpy + e[10] * dpz;
  const float dp[3] = {dpx, dpy, dpz};
  const float xw[3] = {x, y, z};
  acc[0] += dfx;
  acc[1] += dfy;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[4 + 4 * r + k] += dR[r][k] + dp[r] * xw[k];
    acc[4 + 4 * r + 3] += dp[r];
  }
}

__global__ void ewa_bwd_kernel(const float* __restrict__ xyz, const float* __restrict__ cov,
                               const float* __restrict__ intr, const float* __restrict__ extr,
                               const int32_t* __restrict__ radius, int64_t n, int W, int H,
                               const float* __restrict__ d_conic, float* __restrict__ d_xyz,
                               float* __restrict__ d_cov, float* __restrict__ partials) {
  const Cam cm = load_cam(intr, extr);
  float acc[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i] = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float gxw = 0.f, gyw = 0.f, gzw = 0.f;
    float dS[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (radius[i] > 0) {
      float s6[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) s6[k] = cov[6 * i + k];
      ewa_bwd_one(cm, W, H, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], s6, d_conic[3 * i],
                  d_conic[3 * i + 1], d_conic[3 * i + 2], gxw, gyw, gzw, dS, acc);
    }
    d_xyz[3 * i] = gxw;
    d_xyz[3 * i + 1] = gyw;
    d_xyz[3 * i + 2] = gzw;
#pragma unroll
    for (int k = 0; k < 6; ++k) d_cov[6 * i + k] = dS[k];
  }
  block_write_partials(acc, partials);
}

// ---------------------------------------------------------------------------
// Fused preprocessing: project_point + compute_cov3d + ewa_project of the
// renderer, in one pass forward and one backward.  The per-Gaussian
// arithmetic is the same device code as the three operators' (this unit is
// FMA-free), so every output is bit-identical to the three calls; cov3d is
// recomputed in the backward instead of stored, the two position and camera
// gradients are added before they are written.
// ---------------------------------------------------------------------------
__global__ void preprocess_fwd_kernel(const float* __restrict__ xyz, const float* __restrict__ scales,
                                      const float* __restrict__ q, int64_t n,
                                      const float* __restrict__ intr,
                                      const float* __restrict__ extr, int W, int H, float nearest,
                                      float extent, float* __restrict__ uv,
                                      float* __restrict__ depth, float* __restrict__ conic,
                                      int32_t* __restrict__ radius, int32_t* __restrict__ tiles) {
  const Cam cm = load_cam(intr, extr);
  const int gx = grid_x(W), gy = grid_y(H);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    float px, py, pz, u, v;
    cam_point(cm, x, y, z, px, py, pz);
    const bool vis = project_visible(cm, px, py, pz, W, H, nearest, extent, u, v);
    const float2 p = vis ? make_float2(u, v) : make_float2(0.f, 0.f);
    reinterpret_cast<float2*>(uv)[i] = p;
    depth[i] = vis ? pz : 0.f;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
    int rad = 0, nt = 0;
    if (vis) {
      float s6[6];
      cov3d_one(scales, q, i, s6);
      ewa_fwd_one(cm, W, H, gx, gy, x, y, z, s6, p, c0, c1, c2, rad, nt);
    }
    conic[3 * i] = c0;
    conic[3 * i + 1] = c1;
    conic[3 * i + 2] = c2;
    radius[i] = rad;
    tiles[i] = nt;
  }
}

__global__ void preprocess_bwd_kernel(
    const float* __restrict__ xyz, const float* __restrict__ scales, const float* __restrict__ q,
    int64_t n, const float* __restrict__ intr, const float* __restrict__ extr, int W, int H,
    float nearest, float extent, const int32_t* __restrict__ radius,
    const float* __restrict__ d_uv, const float* __restrict__ d_depth,
    const float* __restrict__ d_conic, float* __restrict__ d_xyz, float* __restrict__ d_scales,
    float* __restrict__ d_q, float* __restrict__ partials) {
  const Cam cm = load_cam(intr, extr);
  float acc[16];  // camera-gradient partials of the projection and the EWA terms
#pragma unroll
  for (int k = 0; k < 16; ++k) acc[k] = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    float px, py, pz, u, v;
    cam_point(cm, x, y, z, px, py, pz);
    float gx = 0.f, gy = 0.f, gz = 0.f;
    float ds[3] = {0.f, 0.f, 0.f};
    float4 dq = make_float4(0.f, 0.f, 0.f, 0.f);
    if (project_visible(cm, px, py, pz, W, H, nearest, extent, u, v)) {
      project_bwd_one(cm, x, y, z, px, py, pz, reinterpret_cast<const float2*>(d_uv)[i],
                      d_depth[i], gx, gy, gz, acc);
      if (radius[i] > 0) {
        float s6[6];
        cov3d_one(scales, q, i, s6);
        float ex = 0.f, ey = 0.f, ez = 0.f;
        float dS[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        ewa_bwd_one(cm, W, H, x, y, z, s6, d_conic[3 * i], d_conic[3 * i + 1], d_conic[3 * i + 2],
                    ex, ey, ez, dS, acc);
        gx = gx + ex;
        gy = gy + ey;
        gz = gz + ez;
        cov3d_grad_one(scales, q, i, dS, ds, dq);
      }
    }
    d_xyz[3 * i] = gx;
    d_xyz[3 * i + 1] = gy;
    d_xyz[3 * i + 2] = gz;
    d_scales[3 * i] = ds[0];
    d_scales[3 * i + 1] = ds[1];
    d_scales[3 * i + 2] = ds[2];
    reinterpret_cast<float4*>(d_q)[i] = dq;
  }
  block_write_partials(acc, partials);
}

// ---------------------------------------------------------------------------
// Fused preprocessing of V views of the same Gaussians (the batched
// multi-view path): view v's camera is intrs[4v..], extrs[12v..], its image
// size sizes[2v], sizes[2v + 1]; outputs are view-major (element v N + i).
// The forward is the single-view arithmetic per (Gaussian, view), so every
// output equals the single-view call's bit for bit.  The backward loops the
// views in order inside one thread per Gaussian, so the Gaussian gradients
// are summed over views in registers and written once per view pass
// (read-modify-write by the thread that owns the Gaussian: deterministic),
// and each view's camera partials are reduced per block as in the
// single-view kernel.
// ---------------------------------------------------------------------------
struct ViewSizes {
  int nviews;
  int w[kMaxViews], h[kMaxViews];
};

__global__ void preprocess_views_fwd_kernel(
    const float* __restrict__ xyz, const float* __restrict__ scales, const float* __restrict__ q,
    int64_t n, const float* __restrict__ intrs, const float* __restrict__ extrs,
    const ViewSizes vs, float nearest, float extent, float* __restrict__ uv,
    float* __restrict__ depth, float* __restrict__ conic, int32_t* __restrict__ radius,
    int32_t* __restrict__ tiles) {
  const int v = blockIdx.y;
  const Cam cm = load_cam(intrs + 4 * v, extrs + 12 * v);
  const int W = vs.w[v], H = vs.h[v];
  const int gx = grid_x(W), gy = grid_y(H);
  const int64_t o = (int64_t)v * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    float px, py, pz, u, vv;
    cam_point(cm, x, y, z, px, py, pz);
    const bool vis = project_visible(cm, px, py, pz, W, H, nearest, extent, u, vv);
    const float2 p = vis ? make_float2(u, vv) : make_float2(0.f, 0.f);
    const int64_t e = o + i;
    reinterpret_cast<float2*>(uv)[e] = p;
    depth[e] = vis ? pz : 0.f;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
    int rad = 0, nt = 0;
    if (vis) {
      float s6[6];
      cov3d_one(scales, q, i, s6);
      ewa_fwd_one(cm, W, H, gx, gy, x, y, z, s6, p, c0, c1, c2, rad, nt);
    }
    conic[3 * e] = c0;
    conic[3 * e + 1] = c1;
    conic[3 * e + 2] = c2;
    radius[e] = rad;
    tiles[e] = nt;
  }
}

// Views inside the per-Gaussian loop: a thread reads its Gaussian's
// parameters once, adds the views' gradients in view order in registers and
// writes each parameter gradient once (the views-outer form re-read and
// re-wrote them per view: ~5.7 GB of traffic for 16 views of 3M Gaussians
// against ~1.6 GB).  A view's camera-gradient sums are reduced across the
// warp right away (reduce-scatter: lane 2c ends with component c) and added
// by their owner lanes to the warp's own row of a shared table, so the order
// is fixed; the block then writes, per view, the sum of its warps' rows in
// warp order -- the partials the finish kernel adds over blocks.
__device__ __forceinline__ float warp_reduce_scatter16(float (&v)[16]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 16, m = 8; m >= 1; off >>= 1, m >>= 1) {
    const bool upper = (lane & off) != 0;
#pragma unroll
    for (int i = 0; i < m; ++i) {
      const float send = upper ? v[i] : v[i + m];
      const float keep = upper ? v[i + m] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

__global__ void __launch_bounds__(kStreamThreads) preprocess_views_bwd_kernel(
    const float* __restrict__ xyz, const float* __restrict__ scales, const float* __restrict__ q,
    int64_t n, const float* __restrict__ intrs, const float* __restrict__ extrs,
    const ViewSizes vs, float nearest, float extent, const int32_t* __restrict__ radius,
    const float* __restrict__ d_uv, const float* __restrict__ d_depth,
    const float* __restrict__ d_conic, float* __restrict__ d_xyz, float* __restrict__ d_scales,
    float* __restrict__ d_q, float* __restrict__ partials) {
  constexpr int NW = kStreamThreads / 32;
  extern __shared__ float s_cam[];  // [NW][nviews][16]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int V = vs.nviews;
  for (int j = threadIdx.x; j < NW * V * 16; j += blockDim.x) s_cam[j] = 0.f;
  __syncthreads();
  float* my_cam = s_cam + warp * V * 16;
  // whole warps iterate together (the reduction needs every lane)
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + warp * 32; base < n; base += stride) {
    const int64_t i = base + lane;
    const bool in = i < n;
    float x = 0.f, y = 0.f, z = 0.f;
    if (in) {
      x = xyz[3 * i];
      y = xyz[3 * i + 1];
      z = xyz[3 * i + 2];
    }
    float gx = 0.f, gy = 0.f, gz = 0.f;
    float ds[3] = {0.f, 0.f, 0.f};
    float4 dq = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int v = 0; v < V; ++v) {
      const Cam cm = load_cam(intrs + 4 * v, extrs + 12 * v);
      const int W = vs.w[v], H = vs.h[v];
      const int64_t e = (int64_t)v * n + i;
      float acc[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) acc[k] = 0.f;
      float px, py, pz, u, uy;
      cam_point(cm, x, y, z, px, py, pz);
      float vx = 0.f, vy = 0.f, vz = 0.f;
      float vds[3] = {0.f, 0.f, 0.f};
      float4 vdq = make_float4(0.f, 0.f, 0.f, 0.f);
      if (in && project_visible(cm, px, py, pz, W, H, nearest, extent, u, uy)) {
        project_bwd_one(cm, x, y, z, px, py, pz, reinterpret_cast<const float2*>(d_uv)[e],
                        d_depth[e], vx, vy, vz, acc);
        if (radius[e] > 0) {
          float s6[6];
          cov3d_one(scales, q, i, s6);
          float ex = 0.f, ey = 0.f, ez = 0.f;
          float dS[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
          ewa_bwd_one(cm, W, H, x, y, z, s6, d_conic[3 * e], d_conic[3 * e + 1],
                      d_conic[3 * e + 2], ex, ey, ez, dS, acc);
          vx = vx + ex;
          vy = vy + ey;
          vz = vz + ez;
          cov3d_grad_one(scales, q, i, dS, vds, vdq);
        }
      }
      // the sums over views, in view order (as the views-outer form added them)
      gx = gx + vx;
      gy = gy + vy;
      gz = gz + vz;
      ds[0] = ds[0] + vds[0];
      ds[1] = ds[1] + vds[1];
      ds[2] = ds[2] + vds[2];
      dq = make_float4(dq.x + vdq.x, dq.y + vdq.y, dq.z + vdq.z, dq.w + vdq.w);
      const float sum = warp_reduce_scatter16(acc);
      if ((lane & 1) == 0) my_cam[v * 16 + (lane >> 1)] += sum;
    }
    if (in) {
      d_xyz[3 * i] = gx;
      d_xyz[3 * i + 1] = gy;
      d_xyz[3 * i + 2] = gz;
      d_scales[3 * i] = ds[0];
      d_scales[3 * i + 1] = ds[1];
      d_scales[3 * i + 2] = ds[2];
      reinterpret_cast<float4*>(d_q)[i] = dq;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < V * 16; j += blockDim.x) {
    float t = 0.f;
    for (int w = 0; w < NW; ++w) t += s_cam[w * V * 16 + j];
    partials[((size_t)(j >> 4) * gridDim.x + blockIdx.x) * 16 + (j & 15)] = t;
  }
}

// One block per view: view v's camera gradient from its block partials.
__global__ void __launch_bounds__(16 * kCamTPC) cam_grad_views_finish_kernel(
    const float* __restrict__ partials, int nblocks, float* __restrict__ d_intrs,
    float* __restrict__ d_extrs) {
  __shared__ double s[16 * kCamTPC];
  const int v = blockIdx.x;
  const double t = column_sum<16, kCamTPC>(partials + (size_t)v * nblocks * 16, nblocks, 16, s);
  if (threadIdx.x % kCamTPC == 0) {
    const int col = threadIdx.x / kCamTPC;
    if (col < 4)
      d_intrs[4 * v + col] = (float)t;
    else
      d_extrs[12 * v + col - 4] = (float)t;
  }
}

}  // namespace pgb

using namespace pgb;

extern "C" {

size_t pgb_camera_grad_scratch_bytes(void) { return (size_t)kCamGradBlocksMax * 16 * sizeof(float); }

int pgb_project_point_forward(const float* xyz, int64_t n, const float* intr, const float* extr,
                              int width, int height, float nearest, float extent, float* uv,
                              float* depth, void* stream) {
  if (n < 0 || width <= 0 || height <= 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!xyz || !intr || !extr || !uv || !depth || misaligned(uv, 8)) return PGB_ERR_INVALID;
  project_point_fwd_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(
      xyz, n, intr, extr, width, height, nearest, extent, uv, depth);
  return launch_status();
}

int pgb_project_point_backward(const float* xyz, int64_t n, const float* intr, const float* extr,
                               int width, int height, float nearest, float extent,
                               const float* d_uv, const float* d_depth, float* d_xyz,
                               float* d_intr, float* d_extr, void* scratch, size_t scratch_bytes,
                               void* stream) {
  if (n < 0 || width <= 0 || height <= 0) return PGB_ERR_INVALID;
  if (scratch_bytes < pgb_camera_grad_scratch_bytes() || !scratch || !intr || !extr || !d_intr ||
      !d_extr)
    return PGB_ERR_INVALID;
  if (n > 0 && (!xyz || !d_uv || !d_depth || !d_xyz || misaligned(d_uv, 8))) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  const int grid = stream_grid(n);
  float* partials = static_cast<float*>(scratch);
  project_point_bwd_kernel<<<grid, kStreamThreads, 0, s>>>(xyz, n, intr, extr, width, height,
                                                           nearest, extent, d_uv, d_depth, d_xyz,
                                                           partials);
  cam_grad_finish_kernel<<<1, 16 * kCamTPC, 0, s>>>(partials, grid, d_intr, d_extr);
  return launch_status();
}

int pgb_compute_cov3d_forward(const float* scales, const float* uquats, const uint8_t* visible,
                              int64_t n, float* cov3d, void* stream) {
  if (n < 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!scales || !uquats || !visible || !cov3d || misaligned(uquats, 16) || misaligned(cov3d, 8))
    return PGB_ERR_INVALID;
  cov3d_fwd_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(scales, uquats,
                                                                             visible, n, cov3d);
  return launch_status();
}

int pgb_compute_cov3d_backward(const float* scales, const float* uquats, const uint8_t* visible,
                               int64_t n, const float* d_cov3d, float* d_scales, float* d_uquats,
                               void* stream) {
  if (n < 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!scales || !uquats || !visible || !d_cov3d || !d_scales || !d_uquats ||
      misaligned(uquats, 16) || misaligned(d_uquats, 16))
    return PGB_ERR_INVALID;
  cov3d_bwd_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(
      scales, uquats, visible, n, d_cov3d, d_scales, d_uquats);
  return launch_status();
}

int pgb_ewa_project_forward(const float* xyz, const float* cov3d, const float* intr,
                            const float* extr, const float* uv, const uint8_t* visible, int64_t n,
                            int width, int height, float* conic, int32_t* radius,
                            int32_t* tiles_touched, void* stream) {
  if (n < 0 || width <= 0 || height <= 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!xyz || !cov3d || !intr || !extr || !uv || !visible || !conic || !radius || !tiles_touched ||
      misaligned(cov3d, 8) || misaligned(uv, 8))
    return PGB_ERR_INVALID;
  ewa_fwd_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(
      xyz, cov3d, intr, extr, uv, visible, n, width, height, conic, radius, tiles_touched);
  return launch_status();
}

int pgb_ewa_project_backward(const float* xyz, const float* cov3d, const float* intr,
                             const float* extr, const int32_t* radius, int64_t n, int width,
                             int height, const float* d_conic, float* d_xyz, float* d_cov3d,
                             float* d_intr, float* d_extr, void* scratch, size_t scratch_bytes,
                             void* stream) {
  if (n < 0 || width <= 0 || height <= 0) return PGB_ERR_INVALID;
  if (scratch_bytes < pgb_camera_grad_scratch_bytes() || !scratch || !intr || !extr || !d_intr ||
      !d_extr)
    return PGB_ERR_INVALID;
  if (n > 0 && (!xyz || !cov3d || !radius || !d_conic || !d_xyz || !d_cov3d))
    return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  const int grid = stream_grid(n);
  float* partials = static_cast<float*>(scratch);
  ewa_bwd_kernel<<<grid, kStreamThreads, 0, s>>>(xyz, cov3d, intr, extr, radius, n, width, height,
                                                 d_conic, d_xyz, d_cov3d, partials);
  cam_grad_finish_kernel<<<1, 16 * kCamTPC, 0, s>>>(partials, grid, d_intr, d_extr);
  return launch_status();
}

int pgb_preprocess_forward(const float* xyz, const float* scales, const float* uquats, int64_t n,
                           const float* intr, const float* extr, int width, int height,
                           float nearest, float extent, float* uv, float* depth, float* conic,
                           int32_t* radius, int32_t* tiles_touched, void* stream) {
  if (n < 0 || width <= 0 || height <= 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!xyz || !scales || !uquats || !intr || !extr || !uv || !depth || !conic || !radius ||
      !tiles_touched || misaligned(uquats, 16) || misaligned(uv, 8))
    return PGB_ERR_INVALID;
  preprocess_fwd_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(
      xyz, scales, uquats, n, intr, extr, width, height, nearest, extent, uv, depth, conic, radius,
      tiles_touched);
  return launch_status();
}

int pgb_preprocess_backward(const float* xyz, const float* scales, const float* uquats, int64_t n,
                            const float* intr, const float* extr, int width, int height,
                            float nearest, float extent, const int32_t* radius, const float* d_uv,
                            const float* d_depth, const float* d_conic, float* d_xyz,
                            float* d_scales, float* d_uquats, float* d_intr, float* d_extr,
                            void* scratch, size_t scratch_bytes, void* stream) {
  if (n < 0 || width <= 0 || height <= 0) return PGB_ERR_INVALID;
  if (scratch_bytes < pgb_camera_grad_scratch_bytes() || !scratch || !d_intr || !d_extr)
    return PGB_ERR_INVALID;
  if (n > 0 && (!xyz || !scales || !uquats || !intr || !extr || !radius || !d_uv || !d_depth ||
                !d_conic || !d_xyz || !d_scales || !d_uquats || misaligned(uquats, 16) ||
                misaligned(d_uquats, 16) || misaligned(d_uv, 8)))
    return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  const int grid = stream_grid(n);
  float* partials = static_cast<float*>(scratch);
  preprocess_bwd_kernel<<<grid, kStreamThreads, 0, s>>>(
      xyz, scales, uquats, n, intr, extr, width, height, nearest, extent, radius, d_uv, d_depth,
      d_conic, d_xyz, d_scales, d_uquats, partials);
  cam_grad_finish_kernel<<<1, 16 * kCamTPC, 0, s>>>(partials, grid, d_intr, d_extr);
  return launch_status();
}

static bool view_sizes(const int32_t* sizes, int nviews, ViewSizes& vs) {
  if (!sizes || nviews < 1 || nviews > kMaxViews) return false;
  vs.nviews = nviews;
  for (int v = 0; v < nviews; ++v) {
    vs.w[v] = sizes[2 * v];
    vs.h[v] = sizes[2 * v + 1];
    if (vs.w[v] <= 0 || vs.h[v] <= 0) return false;
  }
  return true;
}

size_t pgb_camera_grad_views_scratch_bytes(int nviews) {
  return (size_t)(nviews > 0 ? nviews : 0) * kCamGradBlocksMax * 16 * sizeof(float);
}

int pgb_preprocess_views_forward(const float* xyz, const float* scales, const float* uquats,
                                 int64_t n, const float* intrs, const float* extrs,
                                 const int32_t* sizes, int nviews, float nearest, float extent,
                                 float* uv, float* depth, float* conic, int32_t* radius,
                                 int32_t* tiles_touched, void* stream) {
  ViewSizes vs;
  if (n < 0 || !view_sizes(sizes, nviews, vs)) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!xyz || !scales || !uquats || !intrs || !extrs || !uv || !depth || !conic || !radius ||
      !tiles_touched || misaligned(uquats, 16) || misaligned(uv, 8))
    return PGB_ERR_INVALID;
  const dim3 grid(stream_grid(n), nviews);
  preprocess_views_fwd_kernel<<<grid, kStreamThreads, 0, as_stream(stream)>>>(
      xyz, scales, uquats, n, intrs, extrs, vs, nearest, extent, uv, depth, conic, radius,
      tiles_touched);
  return launch_status();
}

int pgb_preprocess_views_backward(const float* xyz, const float* scales, const float* uquats,
                                  int64_t n, const float* intrs, const float* extrs,
                                  const int32_t* sizes, int nviews, float nearest, float extent,
                                  const int32_t* radius, const float* d_uv, const float* d_depth,
                                  const float* d_conic, float* d_xyz, float* d_scales,
                                  float* d_uquats, float* d_intrs, float* d_extrs, void* scratch,
                                  size_t scratch_bytes, void* stream) {
  ViewSizes vs;
  if (n < 0 || !view_sizes(sizes, nviews, vs)) return PGB_ERR_INVALID;
  if (scratch_bytes < pgb_camera_grad_views_scratch_bytes(nviews) || !scratch || !d_intrs ||
      !d_extrs)
    return PGB_ERR_INVALID;
  if (n > 0 && (!xyz || !scales || !uquats || !intrs || !extrs || !radius || !d_uv || !d_depth ||
                !d_conic || !d_xyz || !d_scales || !d_uquats || misaligned(uquats, 16) ||
                misaligned(d_uquats, 16) || misaligned(d_uv, 8)))
    return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  const int grid = stream_grid(n);
  float* partials = static_cast<float*>(scratch);
  const int smem = (kStreamThreads / 32) * nviews * 16 * (int)sizeof(float);
  preprocess_views_bwd_kernel<<<grid, kStreamThreads, smem, s>>>(
      xyz, scales, uquats, n, intrs, extrs, vs, nearest, extent, radius, d_uv, d_depth, d_conic,
      d_xyz, d_scales, d_uquats, partials);
  cam_grad_views_finish_kernel<<<nviews, 16 * kCamTPC, 0, s>>>(partials, grid, d_intrs, d_extrs);
  return launch_status();
}

}  // extern "C"
