// compute_sh: real spherical-harmonic colour, forward and backward.
//
// Contract: pointrix/model/renderer/msplat.py:99-105 passes the [N,3,K]
// permuted view of get_shs' [N,K,3] storage (element strides 3K,1,3) and
// unit view directions; the op returns the raw sum sum_k c_k Y_k(d) (the
// caller adds 0.5 and clamps).  The basis is the real SH basis up to degree
// 3 with the sign convention of the 3D Gaussian Splatting renderer; the
// constants are the normalisation factors sqrt((2l+1)/(4 pi) ...) written
// out to double precision.
//
// One thread per Gaussian.  For the two dense layouts ([N,K,3] storage seen
// through the permute, or a contiguous [N,3,K]) the 3K coefficients of a
// Gaussian are one contiguous, 16-byte aligned block and are moved with
// float4 loads and stores; any other stride pattern takes a scalar path.
#include <algorithm>

#include "pgb_common.cuh"

namespace pgb {

constexpr float C0 = 0.28209479177387814f;
constexpr float C1 = 0.4886025119029199f;
constexpr float C2_0 = 1.0925484305920792f;
constexpr float C2_1 = -1.0925484305920792f;
constexpr float C2_2 = 0.31539156525252005f;
constexpr float C2_3 = -1.0925484305920792f;
constexpr float C2_4 = 0.5462742152960396f;
constexpr float C3_0 = -0.5900435899266435f;
constexpr float C3_1 = 2.890611442640554f;
constexpr float C3_2 = -0.4570457994644658f;
constexpr float C3_3 = 0.3731763325901154f;
constexpr float C3_4 = -0.4570457994644658f;
constexpr float C3_5 = 1.445305721320277f;
constexpr float C3_6 = -0.5900435899266435f;

template <int K>
__device__ inline void sh_basis(float x, float y, float z, float (&Y)[K]) {
  Y[0] = C0;
  if constexpr (K > 1) {
    Y[1] = -C1 * y;
    Y[2] = C1 * z;
    Y[3] = -C1 * x;
  }
  if constexpr (K > 4) {
    const float xx = x * x, yy = y * y, zz = z * z;
    Y[4] = C2_0 * (x * y);
    Y[5] = C2_1 * (y * z);
    Y[6] = C2_2 * (2.f * zz - xx - yy);
    Y[7] = C2_3 * (x * z);
    Y[8] = C2_4 * (xx - yy);
    if constexpr (K > 9) {
      Y[9] = C3_0 * y * (3.f * xx - yy);
      Y[10] = C3_1 * (x * y) * z;
      Y[11] = C3_2 * y * (4.f * zz - xx - yy);
      Y[12] = C3_3 * z * (2.f * zz - 3.f * xx - 3.f * yy);
      Y[13] = C3_4 * x * (4.f * zz - xx - yy);
      Y[14] = C3_5 * z * (xx - yy);
      Y[15] = C3_6 * x * (xx - 3.f * yy);
    }
  }
}

// d(sum_k G_k Y_k)/d(x,y,z) for given per-basis weights G.
template <int K>
__device__ inline void sh_basis_grad(float x, float y, float z, const float (&G)[K], float& gx,
                                     float& gy, float& gz) {
  gx = gy = gz = 0.f;
  if constexpr (K > 1) {
    gy += -C1 * G[1];
    gz += C1 * G[2];
    gx += -C1 * G[3];
  }
  if constexpr (K > 4) {
    const float xx = x * x, yy = y * y, zz = z * z;
    gx += C2_0 * y * G[4];
    gy += C2_0 * x * G[4];
    gy += C2_1 * z * G[5];
    gz += C2_1 * y * G[5];
    gx += -2.f * C2_2 * x * G[6];
    gy += -2.f * C2_2 * y * G[6];
    gz += 4.f * C2_2 * z * G[6];
    gx += C2_3 * z * G[7];
    gz += C2_3 * x * G[7];
    gx += 2.f * C2_4 * x * G[8];
    gy += -2.f * C2_4 * y * G[8];
    if constexpr (K > 9) {
      gx += 6.f * C3_0 * x * y * G[9];
      gy += C3_0 * (3.f * xx - 3.f * yy) * G[9];
      gx += C3_1 * y * z * G[10];
      gy += C3_1 * x * z * G[10];
      gz += C3_1 * x * y * G[10];
      gx += -2.f * C3_2 * x * y * G[11];
      gy += C3_2 * (4.f * zz - xx - 3.f * yy) * G[11];
      gz += 8.f * C3_2 * y * z * G[11];
      gx += -6.f * C3_3 * x * z * G[12];
      gy += -6.f * C3_3 * y * z * G[12];
      gz += C3_3 * (6.f * zz - 3.f * xx - 3.f * yy) * G[12];
      gx += C3_4 * (4.f * zz - 3.f * xx - yy) * G[13];
      gy += -2.f * C3_4 * x * y * G[13];
      gz += 8.f * C3_4 * x * z * G[13];
      gx += 2.f * C3_5 * x * z * G[14];
      gy += -2.f * C3_5 * y * z * G[14];
      gz += C3_5 * (xx - yy) * G[14];
      gx += C3_6 * (3.f * xx - 3.f * yy) * G[15];
      gy += -6.f * C3_6 * x * y * G[15];
    }
  }
}

// Layouts of the 3K coefficients of one Gaussian.
enum Layout { kKC = 0, kCK = 1, kStrided = 2 };  // kKC: [K][3] block, kCK: [3][K] block

template <int K, int L>
__device__ inline void load_coeffs(const float* __restrict__ sh, int64_t i, int64_t sn, int64_t sc,
                                   int64_t sk, float (&c)[3][K]) {
  if constexpr (L == kStrided) {
    const float* p = sh + i * sn;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
#pragma unroll
      for (int k = 0; k < K; ++k) c[ch][k] = p[ch * sc + k * sk];
  } else {
    float buf[3 * K];
    const float* p = sh + i * (3 * K);
    if constexpr ((3 * K) % 4 == 0) {
#pragma unroll
      for (int j = 0; j < 3 * K / 4; ++j) {
        const float4 v = reinterpret_cast<const float4*>(p)[j];
        buf[4 * j] = v.x; buf[4 * j + 1] = v.y; buf[4 * j + 2] = v.z; buf[4 * j + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 3 * K; ++j) buf[j] = p[j];
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
#pragma unroll
      for (int k = 0; k < K; ++k) c[ch][k] = (L == kKC) ? buf[k * 3 + ch] : buf[ch * K + k];
  }
}

template <int K, int L>
__device__ inline void store_coeffs(float* __restrict__ out, int64_t i, int64_t sn, int64_t sc,
                                    int64_t sk, const float (&c)[3][K]) {
  if constexpr (L == kStrided) {
    float* p = out + i * sn;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
#pragma unroll
      for (int k = 0; k < K; ++k) p[ch * sc + k * sk] = c[ch][k];
  } else {
    float buf[3 * K];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
#pragma unroll
      for (int k = 0; k < K; ++k) buf[(L == kKC) ? (k * 3 + ch) : (ch * K + k)] = c[ch][k];
    float* p = out + i * (3 * K);
    if constexpr ((3 * K) % 4 == 0) {
#pragma unroll
      for (int j = 0; j < 3 * K / 4; ++j)
        reinterpret_cast<float4*>(p)[j] =
            make_float4(buf[4 * j], buf[4 * j + 1], buf[4 * j + 2], buf[4 * j + 3]);
    } else {
#pragma unroll
      for (int j = 0; j < 3 * K; ++j) p[j] = buf[j];
    }
  }
}

template <int K, int L>
__global__ void __launch_bounds__(kStreamThreads) sh_fwd_kernel(
    const float* __restrict__ sh, int64_t n, int64_t sn, int64_t sc, int64_t sk,
    const float* __restrict__ dirs, float* __restrict__ rgb) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float c[3][K];
    load_coeffs<K, L>(sh, i, sn, sc, sk, c);
    float Y[K];
    sh_basis<K>(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], Y);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < K; ++k) s += c[ch][k] * Y[k];
      rgb[3 * i + ch] = s;
    }
  }
}

template <int K, int L>
__global__ void __launch_bounds__(kStreamThreads) sh_bwd_kernel(
    const float* __restrict__ sh, int64_t n, int64_t sn, int64_t sc, int64_t sk,
    const float* __restrict__ dirs, const float* __restrict__ d_rgb, float* __restrict__ d_sh,
    float* __restrict__ d_dirs) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float x = dirs[3 * i], y = dirs[3 * i + 1], z = dirs[3 * i + 2];
    const float g[3] = {d_rgb[3 * i], d_rgb[3 * i + 1], d_rgb[3 * i + 2]};
    float Y[K];
    sh_basis<K>(x, y, z, Y);
    float dc[3][K];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
#pragma unroll
      for (int k = 0; k < K; ++k) dc[ch][k] = g[ch] * Y[k];
    store_coeffs<K, L>(d_sh, i, sn, sc, sk, dc);
    float gx = 0.f, gy = 0.f, gz = 0.f;
    if constexpr (K > 1) {
      float c[3][K];
      load_coeffs<K, L>(sh, i, sn, sc, sk, c);
      float G[K];
#pragma unroll
      for (int k = 0; k < K; ++k) G[k] = g[0] * c[0][k] + g[1] * c[1][k] + g[2] * c[2][k];
      sh_basis_grad<K>(x, y, z, G, gx, gy, gz);
    }
    d_dirs[3 * i] = gx;
    d_dirs[3 * i + 1] = gy;
    d_dirs[3 * i + 2] = gz;
  }
}

static int layout_of(int k, int64_t sn, int64_t sc, int64_t sk, const void* p, const void* q) {
  const bool aligned = ((reinterpret_cast<uintptr_t>(p) | reinterpret_cast<uintptr_t>(q)) & 15) == 0;
  if (sn == 3 * k && aligned) {
    if (sc == 1 && sk == 3) return kKC;
    if (sc == k && sk == 1) return kCK;
  }
  return kStrided;
}

template <int K>
static void launch_fwd(int L, const float* sh, int64_t n, int64_t sn, int64_t sc, int64_t sk,
                       const float* dirs, float* rgb, cudaStream_t s) {
  const int grid = stream_grid(n);
  if (L == kKC)
    sh_fwd_kernel<K, kKC><<<grid, kStreamThreads, 0, s>>>(sh, n, sn, sc, sk, dirs, rgb);
  else if (L == kCK)
    sh_fwd_kernel<K, kCK><<<grid, kStreamThreads, 0, s>>>(sh, n, sn, sc, sk, dirs, rgb);
  else
    sh_fwd_kernel<K, kStrided><<<grid, kStreamThreads, 0, s>>>(sh, n, sn, sc, sk, dirs, rgb);
}

template <int K>
static void launch_bwd(int L, const float* sh, int64_t n, int64_t sn, int64_t sc, int64_t sk,
                       const float* dirs, const float* d_rgb, float* d_sh, float* d_dirs,
                       cudaStream_t s) {
  const int grid = stream_grid(n);
  if (L == kKC)
    sh_bwd_kernel<K, kKC><<<grid, kStreamThreads, 0, s>>>(sh, n, sn, sc, sk, dirs, d_rgb, d_sh, d_dirs);
  else if (L == kCK)
    sh_bwd_kernel<K, kCK><<<grid, kStreamThreads, 0, s>>>(sh, n, sn, sc, sk, dirs, d_rgb, d_sh, d_dirs);
  else
    sh_bwd_kernel<K, kStrided><<<grid, kStreamThreads, 0, s>>>(sh, n, sn, sc, sk, dirs, d_rgb, d_sh,
                                                               d_dirs);
}

// ---------------------------------------------------------------------------
// Fused view colour: rgb = clamp(sum_{k < active} c_k Y_k(d) + 0.5, min 0)
// with d = (xyz - center) / |xyz - center|, the glue of msplat.py:94-105
// around compute_sh (view direction, SH mask, offset and clamp) in one pass.
// Coefficients are the dense [N,K,3] storage (kKC).  Each warp moves the
// 32 * 3K coefficients of its 32 Gaussians between global memory and a
// per-warp shared stage with 16-byte coalesced accesses; a lane then reads
// its own 3K floats at an odd stride (no bank conflicts).
// ---------------------------------------------------------------------------
constexpr int kShWarps = 4;

template <int K>
struct ShStage {
  static constexpr int F = 3 * K;                     // floats per Gaussian
  static constexpr int P = (F % 2 == 1) ? F : F + 1;  // per-lane stride in the stage
};

template <int K>
__device__ inline void stage_in(const float* __restrict__ src, int64_t g0, int cnt,
                                float* __restrict__ stage, int lane) {
  constexpr int F = ShStage<K>::F, P = ShStage<K>::P;
  const float* p = src + g0 * F;
  if (cnt == 32) {  // 32 * F floats: a multiple of 4, 16-byte aligned
    for (int q = lane; q < 8 * F; q += 32) {
      const float4 v = reinterpret_cast<const float4*>(p)[q];
      const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int f = 4 * q + c;
        stage[(f / F) * P + f % F] = vv[c];
      }
    }
  } else {
    for (int f = lane; f < cnt * F; f += 32) stage[(f / F) * P + f % F] = p[f];
  }
  __syncwarp();
}

template <int K>
__device__ inline void stage_out(float* __restrict__ dst, int64_t g0, int cnt,
                                 const float* __restrict__ stage, int lane) {
  constexpr int F = ShStage<K>::F, P = ShStage<K>::P;
  __syncwarp();
  float* p = dst + g0 * F;
  if (cnt == 32) {
    for (int q = lane; q < 8 * F; q += 32) {
      float vv[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int f = 4 * q + c;
        vv[c] = stage[(f / F) * P + f % F];
      }
      reinterpret_cast<float4*>(p)[q] = make_float4(vv[0], vv[1], vv[2], vv[3]);
    }
  } else {
    for (int f = lane; f < cnt * F; f += 32) p[f] = stage[(f / F) * P + f % F];
  }
}

// Unit view direction of Gaussian i (no epsilon, like the torch division).
__device__ inline void view_dir(const float* __restrict__ xyz, int64_t i, float cx, float cy,
                                float cz, float& dx, float& dy, float& dz, float& nrm) {
  const float vx = xyz[3 * i] - cx, vy = xyz[3 * i + 1] - cy, vz = xyz[3 * i + 2] - cz;
  nrm = sqrtf(vx * vx + vy * vy + vz * vz);
  dx = vx / nrm;
  dy = vy / nrm;
  dz = vz / nrm;
}

template <int K>
__device__ inline float sh_channel(const float* __restrict__ c, const float (&Y)[K], int ch,
                                   int active) {
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (k < active) s += c[k * 3 + ch] * Y[k];
  return s;
}

template <int K>
__global__ void __launch_bounds__(kShWarps * 32) sh_rgb_fwd_kernel(
    const float* __restrict__ sh, int64_t n, int active, const float* __restrict__ xyz,
    const float* __restrict__ center, float* __restrict__ rgb) {
  __shared__ float stage_all[kShWarps][32 * ShStage<K>::P];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* stage = stage_all[warp];
  const float cx = center[0], cy = center[1], cz = center[2];
  const int64_t nblocks = (n + 31) / 32;
  for (int64_t wb = (int64_t)blockIdx.x * kShWarps + warp; wb < nblocks;
       wb += (int64_t)gridDim.x * kShWarps) {
    const int64_t g0 = wb * 32;
    const int cnt = n - g0 < 32 ? (int)(n - g0) : 32;
    __syncwarp();
    stage_in<K>(sh, g0, cnt, stage, lane);
    if (lane < cnt) {
      const int64_t i = g0 + lane;
      float dx, dy, dz, nrm;
      view_dir(xyz, i, cx, cy, cz, dx, dy, dz, nrm);
      float Y[K];
      sh_basis<K>(dx, dy, dz, Y);
      const float* c = stage + lane * ShStage<K>::P;
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        const float x = sh_channel<K>(c, Y, ch, active) + 0.5f;
        rgb[3 * i + ch] = x < 0.f ? 0.f : x;  // NaN passes, as torch.clamp
      }
    }
  }
}

// Backward: d_sh (zero for k >= active), d_xyz, and per-block partial sums
// of -d(xyz - center) for the centre's gradient.
template <int K>
__global__ void __launch_bounds__(kShWarps * 32) sh_rgb_bwd_kernel(
    const float* __restrict__ sh, int64_t n, int active, const float* __restrict__ xyz,
    const float* __restrict__ center, const float* __restrict__ d_rgb, float* __restrict__ d_sh,
    float* __restrict__ d_xyz, float* __restrict__ partial) {
  __shared__ float stage_all[kShWarps][32 * ShStage<K>::P];
  __shared__ float s_red[kShWarps][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* stage = stage_all[warp];
  const float cx = center[0], cy = center[1], cz = center[2];
  float ax = 0.f, ay = 0.f, az = 0.f;
  const int64_t nblocks = (n + 31) / 32;
  for (int64_t wb = (int64_t)blockIdx.x * kShWarps + warp; wb < nblocks;
       wb += (int64_t)gridDim.x * kShWarps) {
    const int64_t g0 = wb * 32;
    const int cnt = n - g0 < 32 ? (int)(n - g0) : 32;
    __syncwarp();
    stage_in<K>(sh, g0, cnt, stage, lane);
    if (lane < cnt) {
      const int64_t i = g0 + lane;
      float dx, dy, dz, nrm;
      view_dir(xyz, i, cx, cy, cz, dx, dy, dz, nrm);
      float Y[K];
      sh_basis<K>(dx, dy, dz, Y);
      float* c = stage + lane * ShStage<K>::P;
      float g[3];
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        const float x = sh_channel<K>(c, Y, ch, active) + 0.5f;
        g[ch] = x >= 0.f ? d_rgb[3 * i + ch] : 0.f;  // clamp_min passes where x >= 0
      }
      float G[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const bool on = k < active;
        G[k] = on ? g[0] * c[k * 3] + g[1] * c[k * 3 + 1] + g[2] * c[k * 3 + 2] : 0.f;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) c[k * 3 + ch] = on ? g[ch] * Y[k] : 0.f;
      }
      float gx, gy, gz;
      sh_basis_grad<K>(dx, dy, dz, G, gx, gy, gz);
      const float dot = dx * gx + dy * gy + dz * gz;
      const float vx = (gx - dx * dot) / nrm, vy = (gy - dy * dot) / nrm,
                  vz = (gz - dz * dot) / nrm;
      d_xyz[3 * i] = vx;
      d_xyz[3 * i + 1] = vy;
      d_xyz[3 * i + 2] = vz;
      ax += vx;
      ay += vy;
      az += vz;
    }
    stage_out<K>(d_sh, g0, cnt, stage, lane);
  }
  ax = warp_sum(ax);
  ay = warp_sum(ay);
  az = warp_sum(az);
  if (lane == 0) {
    s_red[warp][0] = ax;
    s_red[warp][1] = ay;
    s_red[warp][2] = az;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    float t = 0.f;
    for (int w = 0; w < kShWarps; ++w) t += s_red[w][threadIdx.x];
    partial[3 * blockIdx.x + threadIdx.x] = -t;
  }
}

// d_center[c] = sum over blocks of partial[b][c] (fixed order).
constexpr int kCenterTPC = 128;

__global__ void __launch_bounds__(4 * kCenterTPC) sh_center_finish_kernel(
    const float* __restrict__ partial, int blocks, float* __restrict__ d_center) {
  __shared__ double s[4 * kCenterTPC];
  const double t = column_sum<3, kCenterTPC>(partial, blocks, 3, s);
  if (threadIdx.x % kCenterTPC == 0 && threadIdx.x / kCenterTPC < 3)
    d_center[threadIdx.x / kCenterTPC] = (float)t;
}

constexpr int kShRgbBlocksMax = kNumSMs * 8;

inline int sh_rgb_grid(int64_t n) {
  const int64_t need = ((n + 31) / 32 + kShWarps - 1) / kShWarps;
  return (int)std::max<int64_t>(1, std::min<int64_t>(need, kShRgbBlocksMax));
}

// ---------------------------------------------------------------------------
// The fused view colour of V cameras in one pass over the coefficients
// (batches of views): each warp stages its 32 Gaussians' coefficients once
// and evaluates every view's direction, basis and colour; the backward
// accumulates d_sh and d_xyz over the views in registers and writes them
// once, and each view's centre gradient through per-block partials.
// rgb and d_rgb are [V][N][3], the centres [V][3] on the device; the view
// count is at most kMaxViews.
// ---------------------------------------------------------------------------

template <int K>
__global__ void __launch_bounds__(kShWarps * 32) sh_rgb_views_fwd_kernel(
    const float* __restrict__ sh, int64_t n, int active, const float* __restrict__ xyz,
    const float* __restrict__ centres, int nviews, float* __restrict__ rgb) {
  __shared__ float stage_all[kShWarps][32 * ShStage<K>::P];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* stage = stage_all[warp];
  const int64_t nblocks = (n + 31) / 32;
  for (int64_t wb = (int64_t)blockIdx.x * kShWarps + warp; wb < nblocks;
       wb += (int64_t)gridDim.x * kShWarps) {
    const int64_t g0 = wb * 32;
    const int cnt = n - g0 < 32 ? (int)(n - g0) : 32;
    __syncwarp();
    stage_in<K>(sh, g0, cnt, stage, lane);
    if (lane < cnt) {
      const int64_t i = g0 + lane;
      const float* c = stage + lane * ShStage<K>::P;
      for (int v = 0; v < nviews; ++v) {
        float dx, dy, dz, nrm;
        view_dir(xyz, i, centres[3 * v], centres[3 * v + 1], centres[3 * v + 2], dx, dy, dz, nrm);
        float Y[K];
        sh_basis<K>(dx, dy, dz, Y);
        float* o = rgb + ((int64_t)v * n + i) * 3;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
          const float x = sh_channel<K>(c, Y, ch, active) + 0.5f;
          o[ch] = x < 0.f ? 0.f : x;
        }
      }
    }
  }
}

template <int K>
__global__ void __launch_bounds__(kShWarps * 32) sh_rgb_views_bwd_kernel(
    const float* __restrict__ sh, int64_t n, int active, const float* __restrict__ xyz,
    const float* __restrict__ centres, int nviews, const float* __restrict__ d_rgb,
    float* __restrict__ d_sh, float* __restrict__ d_xyz, float* __restrict__ partial) {
  __shared__ float stage_all[kShWarps][32 * ShStage<K>::P];
  __shared__ float s_red[kShWarps][kMaxViews * 3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* stage = stage_all[warp];
  for (int j = lane; j < nviews * 3; j += 32) s_red[warp][j] = 0.f;
  const int64_t nblocks = (n + 31) / 32;
  for (int64_t wb = (int64_t)blockIdx.x * kShWarps + warp; wb < nblocks;
       wb += (int64_t)gridDim.x * kShWarps) {
    const int64_t g0 = wb * 32;
    const int cnt = n - g0 < 32 ? (int)(n - g0) : 32;
    __syncwarp();
    stage_in<K>(sh, g0, cnt, stage, lane);
    float dsum[3 * K];
#pragma unroll
    for (int j = 0; j < 3 * K; ++j) dsum[j] = 0.f;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    const int64_t i = g0 + lane;
    float* c = stage + lane * ShStage<K>::P;
    for (int v = 0; v < nviews; ++v) {
      float vx = 0.f, vy = 0.f, vz = 0.f;
      if (lane < cnt) {
        float dx, dy, dz, nrm;
        view_dir(xyz, i, centres[3 * v], centres[3 * v + 1], centres[3 * v + 2], dx, dy, dz, nrm);
        float Y[K];
        sh_basis<K>(dx, dy, dz, Y);
        const float* gr = d_rgb + ((int64_t)v * n + i) * 3;
        float g[3];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
          const float x = sh_channel<K>(c, Y, ch, active) + 0.5f;
          g[ch] = x >= 0.f ? gr[ch] : 0.f;
        }
        float G[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const bool on = k < active;
          G[k] = on ? g[0] * c[k * 3] + g[1] * c[k * 3 + 1] + g[2] * c[k * 3 + 2] : 0.f;
#pragma unroll
          for (int ch = 0; ch < 3; ++ch)
            if (on) dsum[k * 3 + ch] = fmaf(g[ch], Y[k], dsum[k * 3 + ch]);
        }
        float gx, gy, gz;
        sh_basis_grad<K>(dx, dy, dz, G, gx, gy, gz);
        const float dot = dx * gx + dy * gy + dz * gz;
        vx = (gx - dx * dot) / nrm;
        vy = (gy - dy * dot) / nrm;
        vz = (gz - dz * dot) / nrm;
        sx += vx;
        sy += vy;
        sz += vz;
      }
      // this view's centre gradient: -sum of d(xyz - centre) over the warp
      vx = warp_sum(vx);
      vy = warp_sum(vy);
      vz = warp_sum(vz);
      if (lane == 0) {
        s_red[warp][3 * v] -= vx;
        s_red[warp][3 * v + 1] -= vy;
        s_red[warp][3 * v + 2] -= vz;
      }
    }
    if (lane < cnt) {
      d_xyz[3 * i] = sx;
      d_xyz[3 * i + 1] = sy;
      d_xyz[3 * i + 2] = sz;
#pragma unroll
      for (int j = 0; j < 3 * K; ++j) c[j] = dsum[j];
    }
    stage_out<K>(d_sh, g0, cnt, stage, lane);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nviews * 3; j += blockDim.x) {
    float t = 0.f;
    for (int w = 0; w < kShWarps; ++w) t += s_red[w][j];
    partial[(int64_t)blockIdx.x * (kMaxViews * 3) + j] = t;
  }
}

// d_centres[v][c] = sum over blocks of partial[b][3v + c] (fixed order):
// one CTA per (view, axis) column.
__global__ void __launch_bounds__(256) sh_views_centre_finish_kernel(
    const float* __restrict__ partial, int blocks, float* __restrict__ d_centres) {
  __shared__ double s[256];
  const int j = blockIdx.x;
  column_sum<1, 256>(partial + j, blocks, kMaxViews * 3, s);
  if (threadIdx.x == 0) d_centres[j] = (float)s[0];
}

}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_compute_sh_forward(const float* sh, int64_t n, int k, int64_t sn, int64_t sc, int64_t sk,
                           const float* dirs, float* rgb, void* stream) {
  if (n < 0 || !(k == 1 || k == 4 || k == 9 || k == 16)) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!sh || !dirs || !rgb) return PGB_ERR_INVALID;
  const int L = layout_of(k, sn, sc, sk, sh, sh);
  cudaStream_t s = as_stream(stream);
  switch (k) {
    case 1: launch_fwd<1>(L, sh, n, sn, sc, sk, dirs, rgb, s); break;
    case 4: launch_fwd<4>(L, sh, n, sn, sc, sk, dirs, rgb, s); break;
    case 9: launch_fwd<9>(L, sh, n, sn, sc, sk, dirs, rgb, s); break;
    default: launch_fwd<16>(L, sh, n, sn, sc, sk, dirs, rgb, s); break;
  }
  return launch_status();
}

int pgb_compute_sh_backward(const float* sh, int64_t n, int k, int64_t sn, int64_t sc, int64_t sk,
                            const float* dirs, const float* d_rgb, float* d_sh, float* d_dirs,
                            void* stream) {
  if (n < 0 || !(k == 1 || k == 4 || k == 9 || k == 16)) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!sh || !dirs || !d_rgb || !d_sh || !d_dirs) return PGB_ERR_INVALID;
  const int L = layout_of(k, sn, sc, sk, sh, d_sh);
  cudaStream_t s = as_stream(stream);
  switch (k) {
    case 1: launch_bwd<1>(L, sh, n, sn, sc, sk, dirs, d_rgb, d_sh, d_dirs, s); break;
    case 4: launch_bwd<4>(L, sh, n, sn, sc, sk, dirs, d_rgb, d_sh, d_dirs, s); break;
    case 9: launch_bwd<9>(L, sh, n, sn, sc, sk, dirs, d_rgb, d_sh, d_dirs, s); break;
    default: launch_bwd<16>(L, sh, n, sn, sc, sk, dirs, d_rgb, d_sh, d_dirs, s); break;
  }
  return launch_status();
}

int pgb_sh_rgb_scratch_floats(int64_t n) { return 3 * sh_rgb_grid(n); }

int pgb_sh_rgb_forward(const float* sh, int64_t n, int k, int active, const float* xyz,
                       const float* center, float* rgb, void* stream) {
  if (n < 0 || !(k == 1 || k == 4 || k == 9 || k == 16) || active < 0) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!sh || !xyz || !center || !rgb || (reinterpret_cast<uintptr_t>(sh) & 15))
    return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  const int grid = sh_rgb_grid(n);
  switch (k) {
    case 1: sh_rgb_fwd_kernel<1><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, center, rgb); break;
    case 4: sh_rgb_fwd_kernel<4><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, center, rgb); break;
    case 9: sh_rgb_fwd_kernel<9><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, center, rgb); break;
    default: sh_rgb_fwd_kernel<16><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, center, rgb); break;
  }
  return launch_status();
}

int pgb_sh_rgb_backward(const float* sh, int64_t n, int k, int active, const float* xyz,
                        const float* center, const float* d_rgb, float* d_sh, float* d_xyz,
                        float* d_center, float* scratch, int64_t scratch_floats, void* stream) {
  if (n < 0 || !(k == 1 || k == 4 || k == 9 || k == 16) || active < 0) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (n == 0) {
    if (d_center && cudaMemsetAsync(d_center, 0, 3 * sizeof(float), s) != cudaSuccess)
      return PGB_ERR_CUDA;
    return PGB_OK;
  }
  const int grid = sh_rgb_grid(n);
  if (!sh || !xyz || !center || !d_rgb || !d_sh || !d_xyz || !d_center || !scratch ||
      scratch_floats < 3 * grid || ((reinterpret_cast<uintptr_t>(sh) | reinterpret_cast<uintptr_t>(d_sh)) & 15))
    return PGB_ERR_INVALID;
  switch (k) {
    case 1: sh_rgb_bwd_kernel<1><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, center, d_rgb, d_sh, d_xyz, scratch); break;
    case 4: sh_rgb_bwd_kernel<4><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, center, d_rgb, d_sh, d_xyz, scratch); break;
    case 9: sh_rgb_bwd_kernel<9><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, center, d_rgb, d_sh, d_xyz, scratch); break;
    default: sh_rgb_bwd_kernel<16><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, center, d_rgb, d_sh, d_xyz, scratch); break;
  }
  sh_center_finish_kernel<<<1, 4 * kCenterTPC, 0, s>>>(scratch, grid, d_center);
  return launch_status();
}

int pgb_sh_rgb_views_scratch_floats(int64_t n) { return kMaxViews * 3 * sh_rgb_grid(n); }

int pgb_sh_rgb_views_forward(const float* sh, int64_t n, int k, int active, const float* xyz,
                             const float* centres, int nviews, float* rgb, void* stream) {
  if (n < 0 || !(k == 1 || k == 4 || k == 9 || k == 16) || active < 0 || !centres ||
      nviews < 1 || nviews > kMaxViews)
    return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  if (!sh || !xyz || !rgb || (reinterpret_cast<uintptr_t>(sh) & 15)) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  const int grid = sh_rgb_grid(n);
  switch (k) {
    case 1: sh_rgb_views_fwd_kernel<1><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, centres, nviews, rgb); break;
    case 4: sh_rgb_views_fwd_kernel<4><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, centres, nviews, rgb); break;
    case 9: sh_rgb_views_fwd_kernel<9><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, centres, nviews, rgb); break;
    default: sh_rgb_views_fwd_kernel<16><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, centres, nviews, rgb); break;
  }
  return launch_status();
}

int pgb_sh_rgb_views_backward(const float* sh, int64_t n, int k, int active, const float* xyz,
                              const float* centres, int nviews, const float* d_rgb,
                              float* d_sh, float* d_xyz, float* d_centres, float* scratch,
                              int64_t scratch_floats, void* stream) {
  if (n < 0 || !(k == 1 || k == 4 || k == 9 || k == 16) || active < 0 || !centres ||
      nviews < 1 || nviews > kMaxViews || !d_centres)
    return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (n == 0)
    return cudaMemsetAsync(d_centres, 0, 3 * sizeof(float) * nviews, s) == cudaSuccess
               ? PGB_OK
               : PGB_ERR_CUDA;
  const int grid = sh_rgb_grid(n);
  if (!sh || !xyz || !d_rgb || !d_sh || !d_xyz || !scratch ||
      scratch_floats < (int64_t)kMaxViews * 3 * grid ||
      ((reinterpret_cast<uintptr_t>(sh) | reinterpret_cast<uintptr_t>(d_sh)) & 15))
    return PGB_ERR_INVALID;
  switch (k) {
    case 1: sh_rgb_views_bwd_kernel<1><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, centres, nviews, d_rgb, d_sh, d_xyz, scratch); break;
    case 4: sh_rgb_views_bwd_kernel<4><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, centres, nviews, d_rgb, d_sh, d_xyz, scratch); break;
    case 9: sh_rgb_views_bwd_kernel<9><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, centres, nviews, d_rgb, d_sh, d_xyz, scratch); break;
    default: sh_rgb_views_bwd_kernel<16><<<grid, kShWarps * 32, 0, s>>>(sh, n, active, xyz, centres, nviews, d_rgb, d_sh, d_xyz, scratch); break;
  }
  sh_views_centre_finish_kernel<<<nviews * 3, 256, 0, s>>>(scratch, grid, d_centres);
  return launch_status();
}

}  // extern "C"
