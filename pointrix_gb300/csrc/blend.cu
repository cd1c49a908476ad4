// alpha_blending: per-tile front-to-back compositing of N-channel features,
// forward and backward.
//
// Contract (pointrix/model/renderer/msplat.py:141-151, channel packing in
// pointrix/model/renderer/utils/renderer_utils.py:30-71): for each pixel of
// a 16x16 tile, walk the tile's depth-sorted Gaussians; alpha =
// min(0.99, o exp(power)), power = -(a dx^2 + c dy^2)/2 - b dx dy with
// d = uv - pixel (pixel centres on integer coordinates); skip power > 0 or
// alpha < 1/255; stop before the Gaussian that would take the transmittance
// T below 1e-4; out_c = sum f_c alpha T + T_final bg.  The backward is the
// exact gradient of that function (including the background term and the
// 0.99 clamp), replayed back to front from the stored final T and
// last-contributor count.
//
// GB300 design:
//  * pack: one pass writes a record per Gaussian (u, v, scaled conic, o,
//    tau, thr, f_0..f_{C-1}, zero padding: 48 to 144 bytes) so that a splat is
//    one 16-byte aligned contiguous block read with 16-byte loads;
//  * forward/backward: one CTA per tile, two pixels per thread and 8x8
//    warp boxes (the backward also four pixels per thread, 64 threads and
//    8x16 boxes); each warp culls the staged splats of a batch against its
//    box (exact minimum of the conic over the box) into a list, so every
//    per-splat step serves 64 (128) pixels.  The tile's sorted ids are
//    consumed in batches of 32-256 records (the kernel variants, chosen at
//    run time by the caller's autotuner).  Forward: each thread issues a TMA
//    bulk copy (cp.async.bulk, no multicast) of one record into a
//    double-buffered shared-memory stage that completes on an mbarrier, so
//    batch b+1 streams in while batch b is composited; every mbarrier wait
//    is bounded, and on expiry the CTA records PGB_ERR_TIMEOUT, drains its
//    own copies (bounded again) and returns.  Backward: the same stage
//    filled with 16-byte cp.async copies;
//  * the record's conic is pre-scaled by -log2(e) / 2, so a pair's power
//    comes out as a base-2 exponent for one ex2; the alpha test is a
//    comparison of that exponent with a per-splat threshold -log2(255 o),
//    before the exponential;
//  * forward early exit per CTA (__syncthreads_count) and per warp;
//  * backward: per-Gaussian gradients are summed across the warp with a
//    reduce-scatter butterfly (16 shuffles for 16 values instead of 80),
//    then across warps with shared-memory atomics, then flushed once per
//    (tile, Gaussian) with 16-byte vector atomics into a gradient record.
#include "pgb_common.cuh"

namespace pgb {

constexpr uint32_t kWaitLimit = 1u << 22;

// ---------------------------------------------------------------- PTX helpers
__device__ inline void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ inline void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ inline void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ inline bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ inline bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// Global -> shared bulk copy (TMA, non-tensor form): 16-byte aligned
// addresses, size a multiple of 16; completion counted on `bar`.
__device__ inline void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ inline void set_info(int64_t* info, int code) {
  if (info) atomicCAS(reinterpret_cast<unsigned long long*>(info), 0ull, (unsigned long long)code);
}

// Records hold the conic scaled by K = -log2(e) / 2 (A = K a, B = K b,
// C = K c), so that a pair's power comes out as a base-2 exponent:
// p2 = log2(e) power = dx g0 + dy g1 with g0 = A dx + B dy, g1 = B dx + C dy,
// and e^power = 2^p2 is one ex2.  The gradient of the power with respect to
// uv is -(g0, g1) / K, which the backward accumulates as moments and the
// unpack pass rescales once per Gaussian.
constexpr float kConicScale = -0.72134752044448170f;    // -log2(e) / 2
constexpr float kInvConicScale = -1.38629436111989061f;  // 1 / kConicScale = -2 ln 2

// Base-2 power of (pixel, splat) pairs from the scaled conic.  A thread's
// pixels share one column, so dx is fixed per (thread, splat): the
// x-only terms Adx = A dx, Bdx = B dx and A dx^2 are formed once per splat,
// and each pixel's p2 = A dx^2 + dy (2 Bdx + C dy) is two FMAs.  Written with
// explicit rounding intrinsics so that the forward and the backward take
// identical skip/stop decisions whatever the compiler contracts elsewhere.
struct SplatX {
  float Adx, Bdx, Adx2;
};

__device__ __forceinline__ SplatX splat_x(float A, float B, float dx) {
  SplatX sx;
  sx.Adx = __fmul_rn(A, dx);
  sx.Bdx = __fmul_rn(B, dx);
  sx.Adx2 = __fmul_rn(sx.Adx, dx);
  return sx;
}

__device__ __forceinline__ float splat_power2(const SplatX& sx, float C, float dy) {
  return __fmaf_rn(dy, __fmaf_rn(C, dy, __fadd_rn(sx.Bdx, sx.Bdx)), sx.Adx2);
}

// 2^x by the special-function unit (the exponential of the pair's alpha).
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Issue the bulk copies of one batch of B records: thread t fetches the
// record of list entry first + t (+ NT, ...) (if below last) into stage slot
// t.  One arrive per warp carries the warp's byte count (the barrier expects
// NT/32 arrivals per phase).
// Ids outside [0, n) (a corrupt list) are recorded in `info` and their
// copies skipped; the byte count expected on the barrier counts only the
// copies issued, so the phase still completes.
template <int RF, int NT, int B>
__device__ inline void issue_batch(const float* __restrict__ records,
                                   const int32_t* __restrict__ ids, int64_t first, int64_t last,
                                   int64_t n, float* stage, uint64_t* bar, int64_t* info) {
  constexpr int PER = (B + NT - 1) / NT;  // slots per thread (at most one here)
  const int lane = threadIdx.x & 31;
  int32_t g[PER];
  bool ok[PER];
  uint32_t nvalid = 0;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int slot = threadIdx.x + k * NT;
    const int64_t e = first + slot;
    const bool in = slot < B && e < last;
    g[k] = in ? ids[e] : -1;
    ok[k] = in && g[k] >= 0 && (int64_t)g[k] < n;
    if (in && !ok[k]) set_info(info, PGB_ERR_OVERFLOW);
    nvalid += __popc(__ballot_sync(0xffffffffu, ok[k]));
  }
  if (lane == 0) mbar_arrive_expect_tx(bar, nvalid * RF * 4u);
  __syncwarp();
#pragma unroll
  for (int k = 0; k < PER; ++k)
    if (ok[k])
      bulk_g2s(stage + (threadIdx.x + k * NT) * RF, records + (int64_t)g[k] * RF, RF * 4u, bar);
}

// Stage one batch with cp.async: thread t copies the records of slots
// t, t + NT, ... (16 bytes per instruction) and commits one group.
template <int RF, int NT, int B>
__device__ inline void stage_batch(const float* __restrict__ records,
                                   const int32_t* __restrict__ ids, int64_t first, int64_t last,
                                   int64_t n, float* stage, int64_t* info) {
#pragma unroll
  for (int k = 0; k < (B + NT - 1) / NT; ++k) {
    const int slot = threadIdx.x + k * NT;
    const int64_t e = first + slot;
    if (slot < B && e < last) {
      const int32_t g = ids[e];
      if (g < 0 || (int64_t)g >= n) {
        set_info(info, PGB_ERR_OVERFLOW);
        continue;
      }
      const float* src = records + (int64_t)g * RF;
      float* dst = stage + slot * RF;
#pragma unroll
      for (int q = 0; q < RF / 4; ++q) cp_async16(dst + 4 * q, src + 4 * q);
    }
  }
  cp_async_commit();
}

// stage_batch for one warp and 32 records: lane l stages slot l and returns
// its splat id (-1 past the list or for an id out of range).
template <int RF>
__device__ inline int32_t stage_batch_id(const float* __restrict__ records,
                                         const int32_t* __restrict__ ids, int64_t first,
                                         int64_t last, int64_t n, float* stage, int64_t* info) {
  const int slot = threadIdx.x & 31;
  const int64_t e = first + slot;
  int32_t g = -1;
  if (e < last) {
    g = ids[e];
    if (g < 0 || (int64_t)g >= n) {
      set_info(info, PGB_ERR_OVERFLOW);
      g = -1;
    } else {
      const float* src = records + (int64_t)g * RF;
      float* dst = stage + slot * RF;
#pragma unroll
      for (int q = 0; q < RF / 4; ++q) cp_async16(dst + 4 * q, src + 4 * q);
    }
  }
  cp_async_commit();
  return g;
}

// The radii of one batch's splats (16 x 32 tiles only), plain loads into
// s_rad[slot]; read after the barrier that publishes the batch.
template <int NT, int B>
__device__ inline void stage_radius(const int32_t* __restrict__ ids,
                                    const int32_t* __restrict__ radius, int64_t first,
                                    int64_t last, int64_t n, int* s_rad) {
  for (int slot = threadIdx.x; slot < B; slot += NT) {
    const int64_t e = first + slot;
    int r = 0;
    if (e < last) {
      const int32_t g = ids[e];
      if (g >= 0 && (int64_t)g < n) r = radius[g];
    }
    s_rad[slot] = r;
  }
}

// ------------------------------------------------------------------ pack
// Record of one splat: u, v, K a, K b, K c (the conic scaled by
// K = -log2(e) / 2), o, tau, thr = -log2(255 o), f_0..f_{C-1}, zero
// padding to a multiple of 4 floats.  tau bounds the splat's support: alpha >= 1/255
// requires Q(d) = a dx^2 + 2 b dx dy + c dy^2 <= 2 ln(255 o); tau is that
// level plus a small margin, -1 when o < 1/255 (the splat never passes the
// alpha test) and +inf when the conic is not positive definite (no bound).
constexpr int kRecFeat = 8;  // offset of the first feature in a record (16-byte aligned)
__host__ __device__ constexpr int rec_floats(int C) { return kRecFeat + ((C + 3) / 4) * 4; }
__host__ __device__ constexpr int grad_floats(int C) { return 6 + C <= 16 ? 16 : 32; }

// Where feature channel c of Gaussian i lives: src[c][i * stride[c]] (one
// [N,C] tensor: src[c] = feature + c, stride C; or the columns of several
// [N,w] pieces, so that a caller need not concatenate them).  The gradient
// side writes dst[c][i * stride[c]].  Sized for the largest record.
constexpr int kMaxCols = 28;
struct FeatCols {
  const float* src[kMaxCols];
  int stride[kMaxCols];
};
struct FeatGradCols {
  float* dst[kMaxCols];
  int stride[kMaxCols];
};

// Columns of pieces (device pointers, widths) -> table; false when the
// widths are not positive or add up to more than 26.
template <typename T, typename Cols>
inline bool make_cols(T* const* pieces, const int32_t* widths, int npieces, Cols& cols,
                      int& channels, T** (*slot)(Cols&, int)) {
  channels = 0;
  if (!pieces || !widths || npieces < 1) return false;
  for (int p = 0; p < npieces; ++p) {
    const int w = widths[p];
    if (w < 1 || channels + w > 26 || !pieces[p]) return false;
    for (int c = 0; c < w; ++c) {
      *slot(cols, channels) = pieces[p] + c;
      cols.stride[channels] = w;
      ++channels;
    }
  }
  for (int c = channels; c < kMaxCols; ++c) {
    *slot(cols, c) = nullptr;
    cols.stride[c] = 0;
  }
  return true;
}
inline const float** src_slot(FeatCols& c, int k) { return &c.src[k]; }
inline float** dst_slot(FeatGradCols& c, int k) { return &c.dst[k]; }

template <int RF>
__global__ void pack_kernel(const float* __restrict__ uv, const float* __restrict__ conic,
                            const float* __restrict__ opacity, const FeatCols fc, int64_t n, int C,
                            float* __restrict__ records) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float r[RF];
    r[0] = uv[2 * i];
    r[1] = uv[2 * i + 1];
    const float a = conic[3 * i], b = conic[3 * i + 1], c = conic[3 * i + 2];
    const float o = opacity[i];
    r[2] = kConicScale * a;  // scaled: the power comes out base 2
    r[3] = kConicScale * b;
    r[4] = kConicScale * c;
    r[5] = o;
    float tau;
    if (!(isfinite(r[0]) && isfinite(r[1]) && isfinite(o)))
      tau = __int_as_float(0x7f800000);  // keep whatever the per-pixel arithmetic does
    else if (!(o >= 0.999f / 255.0f))
      tau = -1.0f;
    else if (a > 0.f && c > 0.f && a * c - b * b > 0.f && isfinite(a) && isfinite(b) && isfinite(c))
      tau = 2.0f * logf(255.0f * o) * 1.0001f + 1e-3f;
    else
      tau = __int_as_float(0x7f800000);  // +inf: never culled
    r[6] = tau;
    // alpha >= 1/255 <=> p2 >= -log2(255 o): the per-pair test before the
    // exponential (never passes for o <= 0; a NaN opacity keeps NaN, which
    // no comparison rejects, as the alpha test did not)
    r[7] = o > 0.f ? -log2f(255.0f * o) : __int_as_float(0x7f800000);
#pragma unroll
    for (int k = 0; k < RF - kRecFeat; ++k)
      r[kRecFeat + k] = k < C ? fc.src[k][i * fc.stride[k]] : 0.f;
    float4* dst = reinterpret_cast<float4*>(records + i * RF);
#pragma unroll
    for (int q = 0; q < RF / 4; ++q)
      dst[q] = make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
  }
}

// Conservative test: can the splat pass the alpha test at any pixel centre
// of the box [x0, x0 + BW - 1] x [y0, y0 + BH - 1]?  Minimum of the (convex) quadratic
// form over the box -- zero if the centre is inside, else the least of its
// four edge minima -- compared with tau after subtracting a bound on the
// rounding of the per-pixel float evaluation (1e-5 of the largest term
// magnitude over the box, far above the ~2e-7 that evaluation can lose).
template <int BW, int BH>
__device__ __forceinline__ bool splat_may_touch_box(const float* rec, float x0, float y0) {
  // two 16-byte loads (fewer shared-memory wavefronts than six scalar ones
  // at the record stride)
  const float4 h0 = *reinterpret_cast<const float4*>(rec);      // u, v, A, B
  const float4 h1 = *reinterpret_cast<const float4*>(rec + 4);  // C, o, tau, thr
  const float tau = h1.z;
  if (!(tau < 3.0e38f)) return true;
  // the record's conic is scaled by kConicScale
  const float u = h0.x, v = h0.y, a = h0.z * kInvConicScale, b = h0.w * kInvConicScale,
              c = h1.x * kInvConicScale;
  const float dx0 = u - (x0 + (float)(BW - 1)), dx1 = u - x0;
  const float dy0 = v - (y0 + (float)(BH - 1)), dy1 = v - y0;
  if (dx0 <= 0.f && dx1 >= 0.f && dy0 <= 0.f && dy1 >= 0.f) return tau >= 0.f;
  const float ia = 1.0f / a, ic = 1.0f / c;
  float qmin = 3.0e38f;
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const float dx = e ? dx1 : dx0;
    const float dy = fminf(fmaxf(-b * dx * ic, dy0), dy1);
    qmin = fminf(qmin, a * dx * dx + 2.f * b * dx * dy + c * dy * dy);
    const float ey = e ? dy1 : dy0;
    const float ex = fminf(fmaxf(-b * ey * ia, dx0), dx1);
    qmin = fminf(qmin, a * ex * ex + 2.f * b * ex * ey + c * ey * ey);
  }
  const float mx = fmaxf(fabsf(dx0), fabsf(dx1)) + fmaxf(fabsf(dy0), fabsf(dy1));
  const float slack = 1e-5f * (a + c + 2.f * fabsf(b)) * mx * mx + 1e-4f;
  return qmin - slack <= tau;
}

// Builds this warp's list of batch slots (in increasing order) whose splat
// may touch the warp's pixel box; slots >= cnt are ignored.  Returns the
// list length.
// Tiles taller than 16 pixels (16 x 32 for a batch of views) hold the
// splats of both 16 x 16 tiles they cover.  msplat's lists are per 16 x 16
// tile: a splat belongs to a 16 x 16 tile's list when its 16 x 16 tile
// rectangle (tile_rect of its uv and radius) contains the tile.  F16 keeps
// exactly those splats for the warp's box (which lies in one 16 x 16 tile),
// so every pixel composites the same splats, in the same depth order, as
// with 16 x 16 tiles.
struct List16 {
  const int* rad;  // staged radii of the batch's splats
  int tx, ty;      // the box's 16 x 16 tile
  int gx, gy;      // the view's 16 x 16 tile grid
};

__device__ __forceinline__ bool in_list16(const float* rec, int r, const List16& f) {
  int x0, x1, y0, y1;
  tile_rect(rec[0], rec[1], (float)r, f.gx, f.gy, x0, x1, y0, y1);
  return r > 0 && f.tx >= x0 && f.tx < x1 && f.ty >= y0 && f.ty < y1;
}

template <int BW, int BH, int B, bool F16 = false>
__device__ __forceinline__ int warp_cull(const float* stage, int RF, int cnt, float x0, float y0,
                                         uint8_t* list, const List16& f16 = List16{}) {
  static_assert(B % 32 == 0, "the warp tests its batch 32 slots at a time");
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  int n = 0;
#pragma unroll
  for (int k = 0; k < B / 32; ++k) {
    const int j = k * 32 + lane;
    bool keep = j < cnt && splat_may_touch_box<BW, BH>(stage + j * RF, x0, y0);
    if constexpr (F16) keep = keep && in_list16(stage + j * RF, f16.rad[j], f16);
    const uint32_t m = __ballot_sync(0xffffffffu, keep);
    if (keep) list[n + __popc(m & lt)] = (uint8_t)j;
    n += __popc(m);
  }
  __syncwarp();
  return n;
}

// --------------------------------------------------------------- forward
// 128 threads per 16 x 16 tile (256 per 16 x 32 tile), two pixels per
// thread: warp w owns the 8x8 box at
// (8 (w % 2), 8 (w / 2)); lane l owns pixels (l % 8, l / 8) and
// (l % 8, l / 8 + 4), the layout of the backward.  Every culling test,
// list entry and record read serves 64 pixels.  Batches of 128 records,
// one TMA bulk copy per thread per batch.
constexpr int kFwdPix = 2;
constexpr int kFwdBatch = 128;  // default records per batch (64 and 128 are compiled)
// Forward variant code: records per batch, plus kFwdFlat for the form
// without per-pixel branches in the compositing step.
constexpr int kFwdFlat = 2048;

template <int NC, int RF, int B, int TH = 16, bool FLAT = false>
__global__ void __launch_bounds__(64 * (TH / 8)) blend_fwd_kernel(
    const float* __restrict__ records, const int32_t* __restrict__ ids,
    const int2* __restrict__ ranges, int64_t n, float bg, const ViewTable vt, int C,
    float* __restrict__ out, float* __restrict__ final_T, int32_t* __restrict__ n_contrib,
    int64_t* __restrict__ info, const int32_t* __restrict__ radius) {
  constexpr int NT = 64 * (TH / 8);  // 8 x 8 warp boxes over a 16 x TH tile
  constexpr bool F16 = TH != kTile;
  // One bulk copy per thread per phase: the warp's expect_tx and its copies
  // come from the same predicate, and no thread has a second copy to count.
  static_assert(B <= NT, "a batch holds at most one record per thread");
  static_assert(B * RF * 4 < (1 << 20), "a phase's bytes fit the mbarrier tx-count");
  extern __shared__ __align__(128) float smem[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint8_t s_list[NT / 32][B];
  __shared__ int s_rad[F16 ? 2 : 1][F16 ? B : 1];

  const int tile = blockIdx.x;  // global tile (of its view, for a batch)
  int W, H, gx, ltile;
  int64_t pbase;
  tile_view(vt, tile, W, H, gx, ltile, pbase);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bx0 = (ltile % gx) * kTile + 8 * (w & 1);
  const int by0 = (ltile / gx) * TH + 8 * (w >> 1);
  uint8_t* my_list = s_list[w];
  List16 f16{};
  if constexpr (F16) {
    f16.tx = bx0 / kTile;
    f16.ty = by0 / kTile;
    f16.gx = grid_x(W);
    f16.gy = grid_y(H);
  }

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], NT / 32);
    mbar_init(&bars[1], NT / 32);
    fence_mbar_init();
  }
  __syncthreads();

  const int2 rg = ranges[tile];
  const int64_t start = rg.x, end = rg.y;
  const int nb = end > start ? (int)((end - start + B - 1) / B) : 0;

  const int px = bx0 + (lane & 7);
  // colour sums in channel pairs (one fma.rn.f32x2 per pair, each lane a
  // correctly rounded fmaf); an odd NC's last pair carries the record's pad
  constexpr int NP = (NC + 1) / 2;
  static_assert(kRecFeat + 2 * NP <= RF, "channel pairs stay inside the record");
  float pyf[kFwdPix], T[kFwdPix];
  float2 acc[kFwdPix][NP];
  int last[kFwdPix];
  bool done[kFwdPix], inside[kFwdPix];
  const float pxf = (float)px;
#pragma unroll
  for (int q = 0; q < kFwdPix; ++q) {
    const int py = by0 + (lane >> 3) + 4 * q;
    pyf[q] = (float)py;
    inside[q] = px < W && py < H;
    done[q] = !inside[q];
    T[q] = 1.f;
    last[q] = 0;
#pragma unroll
    for (int k = 0; k < NP; ++k) acc[q][k] = make_float2(0.f, 0.f);
  }
  bool timed_out = false;

  if (nb > 0) {
    issue_batch<RF, NT, B>(records, ids, start, end, n, smem, &bars[0], info);
    if constexpr (F16) stage_radius<NT, B>(ids, radius, start, end, n, s_rad[0]);
  }
  for (int b = 0; b < nb; ++b) {
    const int buf = b & 1;
    const int64_t first = start + (int64_t)b * B;
    if (b + 1 < nb) {
      issue_batch<RF, NT, B>(records, ids, first + B, end, n, smem + (buf ^ 1) * B * RF,
                             &bars[buf ^ 1], info);
      if constexpr (F16) stage_radius<NT, B>(ids, radius, first + B, end, n, s_rad[buf ^ 1]);
    }
    // every thread observes the phase (that makes the TMA writes visible to
    // it); the outcome is made block-uniform before any warp collective
    timed_out = __syncthreads_or(!mbar_wait_bounded(&bars[buf], (b >> 1) & 1));
    if (timed_out && threadIdx.x == 0) set_info(info, PGB_ERR_TIMEOUT);
    const int cnt = (int)(end - first < B ? end - first : B);
    const float* st = smem + buf * B * RF;
    bool all_done = true;
#pragma unroll
    for (int q = 0; q < kFwdPix; ++q) all_done &= done[q];
    if (!timed_out && !__all_sync(0xffffffffu, all_done)) {
      if constexpr (F16) f16.rad = s_rad[buf];
      const int nl = warp_cull<8, 8, B, F16>(st, RF, cnt, (float)bx0, (float)by0, my_list, f16);
      const int base = (int)(first - start) + 1;
      for (int t = 0; t < nl; ++t) {
        const int j = my_list[t];
        const float* rec = st + j * RF;
        const float4 r0 = *reinterpret_cast<const float4*>(rec);
        const float4 r1 = *reinterpret_cast<const float4*>(rec + 4);
        const float dx = __fsub_rn(r0.x, pxf);
        const SplatX sx = splat_x(r0.z, r0.w, dx);
        if constexpr (FLAT) {
          // both pixels' steps without per-pixel branches (independent
          // dependency chains): a pixel that skips the splat, has stopped
          // or stops at it composites nothing and keeps T and last
          bool any = false;
          float p2q[kFwdPix];
          bool okq[kFwdPix];
#pragma unroll
          for (int q = 0; q < kFwdPix; ++q) {
            p2q[q] = splat_power2(sx, r1.x, __fsub_rn(r0.y, pyf[q]));
            okq[q] = !done[q] && !(p2q[q] > 0.f || p2q[q] < r1.w);  // alpha >= 1/255
            any |= okq[q];
          }
          if (any) {
            const float2* fp = reinterpret_cast<const float2*>(rec + kRecFeat);
            float2 fr[NP];
#pragma unroll
            for (int k = 0; k < NP; ++k) fr[k] = fp[k];
#pragma unroll
            for (int q = 0; q < kFwdPix; ++q) {
              const float alpha = fminf(0.99f, __fmul_rn(r1.y, ex2_approx(p2q[q])));
              const float test_T = __fmul_rn(T[q], __fsub_rn(1.0f, alpha));
              const bool stop = okq[q] && test_T < 1e-4f;
              done[q] = done[q] || stop;
              if (okq[q] && !stop) {  // short: predicated, not a divergent branch
                const float wgt = alpha * T[q];
                const float2 w2 = make_float2(wgt, wgt);
#pragma unroll
                for (int k = 0; k < NP; ++k) acc[q][k] = __ffma2_rn(fr[k], w2, acc[q][k]);
                T[q] = test_T;
                last[q] = base + j;
              }
            }
          }
          bool all = true;
#pragma unroll
          for (int q = 0; q < kFwdPix; ++q) all &= done[q];
          if (all) break;
          continue;
        }
        bool live = false;
#pragma unroll
        for (int q = 0; q < kFwdPix; ++q) {
          if (done[q]) continue;
          live = true;
          const float dy = __fsub_rn(r0.y, pyf[q]);
          const float p2 = splat_power2(sx, r1.x, dy);
          if (p2 > 0.f || p2 < r1.w) continue;  // alpha < 1/255: no exp needed
          const float alpha = fminf(0.99f, __fmul_rn(r1.y, ex2_approx(p2)));
          const float test_T = __fmul_rn(T[q], __fsub_rn(1.0f, alpha));
          if (test_T < 1e-4f) {
            done[q] = true;
            continue;
          }
          const float wgt = alpha * T[q];
          const float2 w2 = make_float2(wgt, wgt);
          const float2* fp = reinterpret_cast<const float2*>(rec + kRecFeat);
#pragma unroll
          for (int k = 0; k < NP; ++k) acc[q][k] = __ffma2_rn(fp[k], w2, acc[q][k]);
          T[q] = test_T;
          last[q] = base + j;
        }
        if (!live) break;
      }
      __syncwarp();
    }
    bool mine_done = true;
#pragma unroll
    for (int q = 0; q < kFwdPix; ++q) mine_done &= done[q];
    const int ndone = __syncthreads_count(mine_done || timed_out);
    if (ndone == NT || timed_out) {
      // no copy may still be in flight when the CTA exits: its shared memory
      // goes to the next CTA on this SM
      if (b + 1 < nb && !mbar_wait_bounded(&bars[buf ^ 1], ((b + 1) >> 1) & 1))
        set_info(info, PGB_ERR_TIMEOUT);
      if (timed_out) mbar_wait_bounded(&bars[buf], (b >> 1) & 1);
      break;
    }
  }

  const int64_t plane = (int64_t)W * H;
#pragma unroll
  for (int q = 0; q < kFwdPix; ++q) {
    if (!inside[q]) continue;
    const int py = by0 + (lane >> 3) + 4 * q;
    const int64_t pix = (int64_t)py * W + px;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const float a = (c & 1) ? acc[q][c >> 1].y : acc[q][c >> 1].x;
      if (c < C) out[C * pbase + c * plane + pix] = a + T[q] * bg;
    }
    final_T[pbase + pix] = T[q];
    n_contrib[pbase + pix] = last[q];
  }
}

// ------------------------------------------------------------- backward
// Warp reduce-scatter: on return lane L holds the warp sum of value
// (GR == 32 ? L : (L >> 1) & 15) in v[0].
template <int GR>
__device__ __forceinline__ float warp_reduce_scatter(float (&v)[GR]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 16, m = GR / 2; m >= 1; off >>= 1, m >>= 1) {
    const bool upper = (lane & off) != 0;
#pragma unroll
    for (int i = 0; i < m; ++i) {
      const float send = upper ? v[i] : v[i + m];
      const float keep = upper ? v[i + m] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  if constexpr (GR == 16) v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
  return v[0];
}

// Backward: PX pixels per thread, 256 / PX threads per tile.  Warp w owns
// an 8 x BH box (8x8 for PX = 2, 8x16 for PX = 4) at (8 (w % 2), BH (w / 2));
// lane l owns pixels (l % 8, l / 8 + 4q), q < PX, of it, so every per-splat
// warp reduction, record read and culling test serves 32 PX pixels: more
// pixels per thread, fewer reductions per pixel and coarser culling.  (Eight
// pixels per thread, one warp per tile, measured slower than either.)
// 128 splats per batch: the double-buffered stage and the per-splat
// gradient sums stay near 25 KB, so registers, not shared memory, bound the
// CTAs per SM.
constexpr int kBwdBatch = 128;
// Backward variant code: records per batch, plus kBwdPx4 for four pixels
// per thread.
constexpr int kBwdPx4 = 4096;

// Per-pixel replay state.  SB = sum_c dout_c B_c, B_c the colour composited
// behind the current splat (background first): the gradient needs only that
// sum, dalpha = sum_c dout_c (f_c - B_c) = F - SB with F = sum_c dout_c f_c,
// and B_c <- alpha f_c + (1 - alpha) B_c gives SB <- alpha F + (1 - alpha) SB.
template <int NC>
struct BwdPixel {
  float T;
  int nc;
  float pxf, pyf;
  float SB;
  float dout[NC];
};

// Adds one pixel's contribution to the splat's gradient moments v:
// sum g0 dp, sum g1 dp, sum dx^2 dp, sum dx dy dp, sum dy^2 dp (dp the
// gradient of the natural-base power; g0, g1 from the scaled conic), sum
// G dalpha (the opacity gradient), then the feature gradients; the unpack
// pass turns the moments into the uv and conic gradients (-(v0, v1) / K;
// -v2 / 2, -v3, -v4 / 2).  Replays the forward's skip decisions exactly.
template <int NC, int GR>
__device__ __forceinline__ bool bwd_pixel(BwdPixel<NC>& P, int j, const float* rec,
                                          const SplatX& sx, float dx, float (&v)[GR]) {
  if (j >= P.nc) return false;
  const float4 r0 = *reinterpret_cast<const float4*>(rec);
  const float4 r1 = *reinterpret_cast<const float4*>(rec + 4);
  const float dy = __fsub_rn(r0.y, P.pyf);
  const float p2 = splat_power2(sx, r1.x, dy);
  if (p2 > 0.f || p2 < r1.w) return false;  // the forward's skip test
  const float g0 = __fmaf_rn(r0.w, dy, sx.Adx), g1 = __fmaf_rn(r1.x, dy, sx.Bdx);
  const float G = ex2_approx(p2);
  const float araw = __fmul_rn(r1.y, G);
  const float alpha = fminf(0.99f, araw);
  const float om = __fsub_rn(1.0f, alpha);
  P.T = __fdividef(P.T, om);
  const float* f = rec + kRecFeat;
  float F = 0.f;
  const float wT = alpha * P.T;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    F = fmaf(P.dout[c], f[c], F);
    v[6 + c] = fmaf(wT, P.dout[c], v[6 + c]);
  }
  const float dalpha = (F - P.SB) * P.T;
  P.SB = fmaf(alpha, F, om * P.SB);
  if (araw < 0.99f) {
    const float dpow = alpha * dalpha;
    v[5] = fmaf(G, dalpha, v[5]);
    v[0] = fmaf(g0, dpow, v[0]);
    v[1] = fmaf(g1, dpow, v[1]);
    const float tx = dpow * dx;
    v[2] = fmaf(tx, dx, v[2]);
    v[3] = fmaf(tx, dy, v[3]);
    v[4] = fmaf(dpow * dy, dy, v[4]);
  }
  return true;
}

template <int NC, int RF, int GR, int B, int PX, int TH = 16>
__global__ void __launch_bounds__(256 / PX * (TH / 16)) blend_bwd_kernel(
    const float* __restrict__ records, const int32_t* __restrict__ ids,
    const int2* __restrict__ ranges, int64_t n, float bg, const ViewTable vt, int C,
    const float* __restrict__ final_T, const int32_t* __restrict__ n_contrib,
    const float* __restrict__ d_out, float* __restrict__ grad_records,
    int64_t* __restrict__ info, const int32_t* __restrict__ radius) {
  static_assert(GR == 16 || GR == 32, "gradient records are 16 or 32 floats");
  static_assert(PX == 2 || PX == 4, "two or four pixels per thread");
  constexpr int NT = 256 / PX * (TH / 16);
  constexpr bool F16 = TH != kTile;
  constexpr int BW = 8;         // warp box width
  constexpr int RS = 32 / BW;   // box rows per pixel step
  constexpr int BH = RS * PX;   // warp box height
  extern __shared__ __align__(128) float smem[];
  __shared__ int s_max_nc;
  __shared__ uint8_t s_touched[B];
  __shared__ uint8_t s_list[NT / 32][B];
  __shared__ int s_rad[F16 ? 2 : 1][F16 ? B : 1];
  float* gacc = smem + 2 * B * RF;  // [B][GR]

  const int tile = blockIdx.x;  // global tile (of its view, for a batch)
  int W, H, gx, ltile;
  int64_t pbase;
  tile_view(vt, tile, W, H, gx, ltile, pbase);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bx0 = (ltile % gx) * kTile + BW * (w & 1);
  const int by0 = (ltile / gx) * TH + BH * (w >> 1);
  uint8_t* my_list = s_list[w];
  List16 f16{};
  if constexpr (F16) {
    f16.tx = bx0 / kTile;
    f16.ty = by0 / kTile;
    f16.gx = grid_x(W);
    f16.gy = grid_y(H);
  }

  if (threadIdx.x == 0) s_max_nc = 0;
  for (int i = threadIdx.x; i < B * GR; i += NT) gacc[i] = 0.f;
  for (int i = threadIdx.x; i < B; i += NT) s_touched[i] = 0;
  __syncthreads();

  const int64_t plane = (int64_t)W * H;
  BwdPixel<NC> P[PX];
  int my_nc = 0;
#pragma unroll
  for (int q = 0; q < PX; ++q) {
    const int px = bx0 + lane % BW, py = by0 + lane / BW + RS * q;
    P[q].pxf = (float)px;
    P[q].pyf = (float)py;
    P[q].T = 1.f;
    P[q].nc = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) P[q].dout[c] = 0.f;
    if (px < W && py < H) {
      const int64_t pix = (int64_t)py * W + px;
      P[q].T = final_T[pbase + pix];
      P[q].nc = n_contrib[pbase + pix];
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (c < C) P[q].dout[c] = d_out[C * pbase + c * plane + pix];
    }
    float sd = 0.f;
#pragma unroll
    for (int c = 0; c < NC; ++c) sd += P[q].dout[c];
    P[q].SB = bg * sd;
    my_nc = max(my_nc, P[q].nc);
  }
  int warp_nc = my_nc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) warp_nc = max(warp_nc, __shfl_xor_sync(0xffffffffu, warp_nc, o));
  if (lane == 0) atomicMax(&s_max_nc, warp_nc);
  __syncthreads();
  const int2 rg = ranges[tile];
  const int64_t start = rg.x;
  // the replay never reads past the tile's list, whatever n_contrib holds
  const int list_len = max(0, rg.y - rg.x);
  if (s_max_nc > list_len && threadIdx.x == 0) set_info(info, PGB_ERR_OVERFLOW);
  const int max_nc = min(s_max_nc, list_len);
  const int nb = (max_nc + B - 1) / B;

  // batch b covers list positions [hi_b - B, hi_b) with
  // hi_b = max_nc - b*B, clipped at 0; slot t holds position lo_b + t.
  auto lo_of = [&](int b) { return max(0, max_nc - (b + 1) * B); };
  auto hi_of = [&](int b) { return max_nc - b * B; };

  if (nb > 0) {
    stage_batch<RF, NT, B>(records, ids, start + lo_of(0), start + hi_of(0), n, smem, info);
    if constexpr (F16)
      stage_radius<NT, B>(ids, radius, start + lo_of(0), start + hi_of(0), n, s_rad[0]);
  }
  for (int b = 0; b < nb; ++b) {
    const int buf = b & 1;
    const int lo = lo_of(b), hi = hi_of(b);
    if (b + 1 < nb) {
      stage_batch<RF, NT, B>(records, ids, start + lo_of(b + 1), start + hi_of(b + 1), n,
                             smem + (buf ^ 1) * B * RF, info);
      if constexpr (F16)
        stage_radius<NT, B>(ids, radius, start + lo_of(b + 1), start + hi_of(b + 1), n,
                            s_rad[buf ^ 1]);
      cp_async_wait<1>();  // this thread's copies of batch b have landed
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // ... and everyone's
    const float* st = smem + buf * B * RF;
    {
      if constexpr (F16) f16.rad = s_rad[buf];
      const int nl = warp_cull<BW, BH, B, F16>(st, RF, min(hi, warp_nc) - lo, (float)bx0,
                                               (float)by0, my_list, f16);
      for (int t = nl - 1; t >= 0; --t) {
        const int slot = my_list[t];
        const int j = lo + slot;
        const float* rec = st + slot * RF;
        float v[GR];
#pragma unroll
        for (int q = 0; q < GR; ++q) v[q] = 0.f;
        bool contrib = false;
        const float4 r0 = *reinterpret_cast<const float4*>(rec);
        const float dx = __fsub_rn(r0.x, P[0].pxf);  // the thread's pixels share a column
        const SplatX sx = splat_x(r0.z, r0.w, dx);
#pragma unroll
        for (int q = 0; q < PX; ++q) contrib |= bwd_pixel<NC, GR>(P[q], j, rec, sx, dx, v);
        if (__any_sync(0xffffffffu, contrib)) {
          const float sum = warp_reduce_scatter<GR>(v);
          if (GR == 32) {
            if (lane < 6 + NC) atomicAdd(&gacc[slot * GR + lane], sum);
          } else if ((lane & 1) == 0 && (lane >> 1) < 6 + NC) {
            atomicAdd(&gacc[slot * GR + (lane >> 1)], sum);
          }
          if (lane == 0) s_touched[slot] = 1;
        }
      }
      __syncwarp();
    }
    __syncthreads();
    // flush this batch's per-splat sums: one set of vector atomics per splat
    for (int t = threadIdx.x; t < hi - lo; t += NT) {
      if (!s_touched[t]) continue;
      const int32_t g = ids[start + lo + t];
      if (g < 0 || (int64_t)g >= n) {
        set_info(info, PGB_ERR_OVERFLOW);
        continue;
      }
      float4* dst = reinterpret_cast<float4*>(grad_records + (int64_t)g * GR);
      float4* srcv = reinterpret_cast<float4*>(gacc + t * GR);
#pragma unroll
      for (int q = 0; q < (6 + NC + 3) / 4; ++q) {
        atomicAdd(dst + q, srcv[q]);
        srcv[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      s_touched[t] = 0;
    }
    __syncthreads();
  }
}

// Backward, second form: the same replay and reductions as
// blend_bwd_kernel, with fewer registers and fewer instructions per pair.
//  * d_out lives in shared memory (two 16-byte planes per pixel: channels
//    0-3 and 4-7), read only by a pixel that composites the splat, instead
//    of NC registers per pixel; pixel coordinates are formed from the lane.
//    The per-pixel registers are T, SB and the contributor count.
//  * Packed FP32 pairs (fma.rn.f32x2, sm_100 and later) for the channel sums
//    F = sum dout f and the feature gradients (two channels per
//    instruction) and for the moment updates (two moments per instruction).
// The skip decisions use the forward's exact arithmetic (splat_power2).
// Variant codes: kBwdV2 + records per batch (butterfly reduction),
// kBwdV2 + 512 + records (transposed reduction), kBwdV2 + 1024 + records
// (transposed reduction, at most 85 registers: twelve CTAs per SM),
// kBwdV2 + kBwdFlat + records (butterfly reduction, the pixels' replay steps
// without per-pixel branches), kBwdV2 + kBwdFlat + 1024 + records (the same
// at most 102 registers: ten CTAs per SM); four pixels per thread.
constexpr int kBwdV2 = 8192;
constexpr int kBwdFlat = 2048;
// One warp per CTA (blend_bwd_solo_kernel): kBwdSolo + records per batch
// (at most 128 registers), + 1024 + records (102 registers), + 2048 +
// records (85 registers).
constexpr int kBwdSolo = 16384;
// One warp per 16 x 16 tile (blend_bwd_tile_kernel): kBwdTile + records per
// batch.
constexpr int kBwdTile = 32768;

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }

// Transposed per-splat reduction (XRED): each lane stores its GR partial
// sums as a row of a per-warp [32][20] shared table, then lane k < 16 sums
// column k over rows 0-15 and lane 16 + k over rows 16-31 (visited in the
// order r ^ 4, which keeps the two half-warps on distinct banks), and one
// shuffle adds the halves: 4 stores, 16 loads and 16 adds per lane instead
// of the butterfly's 16 shuffles, 16 adds and 32 selects.
constexpr int kRedStride = 20;  // floats per row: 16-byte rows on distinct bank groups

template <int NC, int RF, int GR, int B, int PX, int MINB, bool XRED, bool FLAT = false>
__global__ void __launch_bounds__(256 / PX, MINB) blend_bwd2_kernel(
    const float* __restrict__ records, const int32_t* __restrict__ ids,
    const int2* __restrict__ ranges, int64_t n, float bg, const ViewTable vt, int C,
    const float* __restrict__ final_T, const int32_t* __restrict__ n_contrib,
    const float* __restrict__ d_out, float* __restrict__ grad_records,
    int64_t* __restrict__ info) {
  static_assert(GR == 16 || GR == 32, "gradient records are 16 or 32 floats");
  static_assert(PX == 2 || PX == 4, "two or four pixels per thread");
  static_assert(NC <= 8, "the d_out planes hold eight channels");
  constexpr int NT = 256 / PX;
  constexpr int BW = 8;
  constexpr int RS = 32 / BW;
  constexpr int BH = RS * PX;
  constexpr int NP = (NC + 1) / 2;  // channel pairs
  extern __shared__ __align__(128) float smem[];
  __shared__ int s_max_nc;
  __shared__ uint8_t s_touched[B];
  __shared__ uint8_t s_list[NT / 32][B];
  __shared__ __align__(16) float4 s_dout[2][256];  // [plane][q * NT + thread]
  __shared__ __align__(16) float s_red[XRED ? NT / 32 : 1][XRED ? 32 * kRedStride : 1];
  float* gacc = smem + 2 * B * RF;                  // [B][GR]

  const int tile = blockIdx.x;
  int W, H, gx, ltile;
  int64_t pbase;
  tile_view(vt, tile, W, H, gx, ltile, pbase);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bx0 = (ltile % gx) * kTile + BW * (w & 1);
  const int by0 = (ltile / gx) * kTile + BH * (w >> 1);
  uint8_t* my_list = s_list[w];

  if (threadIdx.x == 0) s_max_nc = 0;
  for (int i = threadIdx.x; i < B * GR; i += NT) gacc[i] = 0.f;
  for (int i = threadIdx.x; i < B; i += NT) s_touched[i] = 0;

  const int64_t plane = (int64_t)W * H;
  const int pxi = bx0 + (lane & (BW - 1));
  const float pxf = (float)pxi;
  const float py0 = (float)(by0 + lane / BW);
  float T[PX], SB[PX];
  int nc[PX];
  int my_nc = 0;
#pragma unroll
  for (int q = 0; q < PX; ++q) {
    const int py = by0 + lane / BW + RS * q;
    float dv[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) dv[c] = 0.f;
    T[q] = 1.f;
    nc[q] = 0;
    if (pxi < W && py < H) {
      const int64_t pix = (int64_t)py * W + pxi;
      T[q] = final_T[pbase + pix];
      nc[q] = n_contrib[pbase + pix];
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (c < C) dv[c] = d_out[C * pbase + c * plane + pix];
    }
    float sd = 0.f;
#pragma unroll
    for (int c = 0; c < NC; ++c) sd += dv[c];
    SB[q] = bg * sd;
    s_dout[0][q * NT + threadIdx.x] = make_float4(dv[0], dv[1], dv[2], dv[3]);
    s_dout[1][q * NT + threadIdx.x] = make_float4(dv[4], dv[5], dv[6], dv[7]);
    my_nc = max(my_nc, nc[q]);
  }
  int warp_nc = my_nc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) warp_nc = max(warp_nc, __shfl_xor_sync(0xffffffffu, warp_nc, o));
  __syncthreads();  // gacc, s_touched and s_max_nc initialised
  if (lane == 0) atomicMax(&s_max_nc, warp_nc);
  __syncthreads();
  const int2 rg = ranges[tile];
  const int64_t start = rg.x;
  const int list_len = max(0, rg.y - rg.x);
  if (s_max_nc > list_len && threadIdx.x == 0) set_info(info, PGB_ERR_OVERFLOW);
  const int max_nc = min(s_max_nc, list_len);
  const int nb = (max_nc + B - 1) / B;
  auto lo_of = [&](int b) { return max(0, max_nc - (b + 1) * B); };
  auto hi_of = [&](int b) { return max_nc - b * B; };

  if (nb > 0)
    stage_batch<RF, NT, B>(records, ids, start + lo_of(0), start + hi_of(0), n, smem, info);
  for (int b = 0; b < nb; ++b) {
    const int buf = b & 1;
    const int lo = lo_of(b), hi = hi_of(b);
    if (b + 1 < nb) {
      stage_batch<RF, NT, B>(records, ids, start + lo_of(b + 1), start + hi_of(b + 1), n,
                             smem + (buf ^ 1) * B * RF, info);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* st = smem + buf * B * RF;
    const int nl = warp_cull<BW, BH, B>(st, RF, min(hi, warp_nc) - lo, (float)bx0, (float)by0,
                                        my_list);
    for (int t = nl - 1; t >= 0; --t) {
      const int slot = my_list[t];
      const int j = lo + slot;
      const float* rec = st + slot * RF;
      const float4 r0 = *reinterpret_cast<const float4*>(rec);  // u, v, A, B
      const float4 r1 = *reinterpret_cast<const float4*>(rec + 4);  // C, o, tau, thr
      const float dx = __fsub_rn(r0.x, pxf);
      const SplatX sx = splat_x(r0.z, r0.w, dx);
      float2 v[GR / 2];
#pragma unroll
      for (int k = 0; k < GR / 2; ++k) v[k] = f2(0.f, 0.f);
      bool contrib = false;
      if constexpr (FLAT) {
        // every pixel's skip test first, then one warp-uniform branch and
        // the pixels' replay steps without per-pixel branches: the PX
        // dependency chains are independent and interleave.  A pixel that
        // skips the splat gets alpha = 0 and keeps T and SB exactly.
        float dyq[PX], p2q[PX];
        bool okq[PX];
#pragma unroll
        for (int q = 0; q < PX; ++q) {
          dyq[q] = __fsub_rn(r0.y, py0 + (float)(RS * q));
          p2q[q] = splat_power2(sx, r1.x, dyq[q]);
          okq[q] = j < nc[q] && !(p2q[q] > 0.f || p2q[q] < r1.w);  // the forward's skip test
          contrib |= okq[q];
        }
        if (!__any_sync(0xffffffffu, contrib)) continue;
        const float2* fp = reinterpret_cast<const float2*>(rec + kRecFeat);
        float2 fr[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) fr[k] = fp[k];
#pragma unroll
        for (int q = 0; q < PX; ++q) {
          const float dy = dyq[q];
          const float g0 = __fmaf_rn(r0.w, dy, sx.Adx), g1 = __fmaf_rn(r1.x, dy, sx.Bdx);
          const float G = ex2_approx(p2q[q]);
          const float araw = __fmul_rn(r1.y, G);
          const float alpha = okq[q] ? fminf(0.99f, araw) : 0.f;
          const float om = __fsub_rn(1.0f, alpha);
          T[q] = okq[q] ? __fdividef(T[q], om) : T[q];
          const float4 dlo = s_dout[0][q * NT + threadIdx.x];
          const float4 dhi = s_dout[1][q * NT + threadIdx.x];
          const float2 dp[4] = {f2(dlo.x, dlo.y), f2(dlo.z, dlo.w), f2(dhi.x, dhi.y),
                                f2(dhi.z, dhi.w)};
          float2 F2 = __fmul2_rn(dp[0], fr[0]);
#pragma unroll
          for (int k = 1; k < NP; ++k) F2 = __ffma2_rn(dp[k], fr[k], F2);
          const float F = F2.x + F2.y;
          const float wT = alpha * T[q];
          const float2 wT2 = f2(wT, wT);
#pragma unroll
          for (int k = 0; k < NP; ++k) v[3 + k] = __ffma2_rn(wT2, dp[k], v[3 + k]);
          const float dalpha = (F - SB[q]) * T[q];
          SB[q] = fmaf(alpha, F, om * SB[q]);
          const bool m = okq[q] && araw < 0.99f;
          const float dpow = m ? alpha * dalpha : 0.f;
          const float Gm = m ? G : 0.f;
          const float tx = dpow * dx;
          v[0] = __ffma2_rn(f2(g0, g1), f2(dpow, dpow), v[0]);
          v[1] = __ffma2_rn(f2(tx, tx), f2(dx, dy), v[1]);
          v[2] = __ffma2_rn(f2(dpow * dy, Gm), f2(dy, dalpha), v[2]);
        }
      } else {
#pragma unroll
      for (int q = 0; q < PX; ++q) {
        if (j >= nc[q]) continue;
        const float dy = __fsub_rn(r0.y, py0 + (float)(RS * q));
        const float p2 = splat_power2(sx, r1.x, dy);
        if (p2 > 0.f || p2 < r1.w) continue;  // the forward's skip test
        contrib = true;
        const float g0 = __fmaf_rn(r0.w, dy, sx.Adx), g1 = __fmaf_rn(r1.x, dy, sx.Bdx);
        const float G = ex2_approx(p2);
        const float araw = __fmul_rn(r1.y, G);
        const float alpha = fminf(0.99f, araw);
        const float om = __fsub_rn(1.0f, alpha);
        T[q] = __fdividef(T[q], om);
        const float4 dlo = s_dout[0][q * NT + threadIdx.x];
        const float4 dhi = s_dout[1][q * NT + threadIdx.x];
        const float2 dp[4] = {f2(dlo.x, dlo.y), f2(dlo.z, dlo.w), f2(dhi.x, dhi.y),
                              f2(dhi.z, dhi.w)};
        const float2* fp = reinterpret_cast<const float2*>(rec + kRecFeat);
        float2 F2 = __fmul2_rn(dp[0], fp[0]);
#pragma unroll
        for (int k = 1; k < NP; ++k) F2 = __ffma2_rn(dp[k], fp[k], F2);
        const float F = F2.x + F2.y;
        const float wT = alpha * T[q];
        const float2 wT2 = f2(wT, wT);
#pragma unroll
        for (int k = 0; k < NP; ++k) v[3 + k] = __ffma2_rn(wT2, dp[k], v[3 + k]);
        const float dalpha = (F - SB[q]) * T[q];
        SB[q] = fmaf(alpha, F, om * SB[q]);
        if (araw < 0.99f) {
          const float dpow = alpha * dalpha;
          const float tx = dpow * dx;
          v[0] = __ffma2_rn(f2(g0, g1), f2(dpow, dpow), v[0]);            // sum g0 dp, g1 dp
          v[1] = __ffma2_rn(f2(tx, tx), f2(dx, dy), v[1]);                // dx^2 dp, dx dy dp
          v[2] = __ffma2_rn(f2(dpow * dy, G), f2(dy, dalpha), v[2]);      // dy^2 dp, G dalpha
        }
      }
      }
      if (FLAT || __any_sync(0xffffffffu, contrib)) {
        if constexpr (XRED && GR == 16) {
          float* tab = s_red[w];
          float4* row = reinterpret_cast<float4*>(tab + lane * kRedStride);
#pragma unroll
          for (int k = 0; k < 4; ++k) row[k] = make_float4(v[2 * k].x, v[2 * k].y, v[2 * k + 1].x, v[2 * k + 1].y);
          __syncwarp();
          const int h = lane >> 4;
          const float* a0 = tab + h * 16 * kRedStride + (lane & 15);
          const float* ap = a0 + h * 4 * kRedStride;   // rows r ^ 4 with bit 2 of r clear
          const float* am = a0 - h * 4 * kRedStride;   // ... and set
          float sum = 0.f;
#pragma unroll
          for (int r = 0; r < 16; ++r) sum += ((r & 4) ? am : ap)[r * kRedStride];
          sum += __shfl_xor_sync(0xffffffffu, sum, 16);
          if (lane < 6 + NC) atomicAdd(&gacc[slot * GR + lane], sum);
          __syncwarp();   // the table is rewritten by the next splat
        } else {
          float vf[GR];
#pragma unroll
          for (int k = 0; k < GR / 2; ++k) {
            vf[2 * k] = v[k].x;
            vf[2 * k + 1] = v[k].y;
          }
          const float sum = warp_reduce_scatter<GR>(vf);
          if (GR == 32) {
            if (lane < 6 + NC) atomicAdd(&gacc[slot * GR + lane], sum);
          } else if ((lane & 1) == 0 && (lane >> 1) < 6 + NC) {
            atomicAdd(&gacc[slot * GR + (lane >> 1)], sum);
          }
        }
        if (lane == 0) s_touched[slot] = 1;
      }
    }
    __syncwarp();
    __syncthreads();
    for (int t = threadIdx.x; t < hi - lo; t += NT) {
      if (!s_touched[t]) continue;
      const int32_t g = ids[start + lo + t];
      if (g < 0 || (int64_t)g >= n) {
        set_info(info, PGB_ERR_OVERFLOW);
        continue;
      }
      float4* dst = reinterpret_cast<float4*>(grad_records + (int64_t)g * GR);
      float4* srcv = reinterpret_cast<float4*>(gacc + t * GR);
#pragma unroll
      for (int q = 0; q < (6 + NC + 3) / 4; ++q) {
        atomicAdd(dst + q, srcv[q]);
        srcv[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      s_touched[t] = 0;
    }
    __syncthreads();
  }
}

// Backward, one warp per CTA: each 8 x 16 half of a 16 x 16 tile is its own
// CTA of 32 threads (CTA 2t + h covers half h of tile t), with its own
// double-buffered record stage, list and per-splat sums.  Nothing is shared
// between the halves, so the kernel has no CTA-wide barrier: a warp waits
// only for its own copies (cp.async groups, __syncwarp), walks only its own
// last-contributor range, and frees its slot on the SM when it finishes.
// A splat's per-batch sums have one owner lane per component, so they
// accumulate with plain shared-memory adds (no atomics); each half flushes
// its own sums with 16-byte vector atomics.  The replay is the flat form of
// blend_bwd2_kernel (four pixels per lane, no per-pixel branches).
template <int NC, int RF, int GR, int B, int MINB>
__global__ void __launch_bounds__(32, MINB) blend_bwd_solo_kernel(
    const float* __restrict__ records, const int32_t* __restrict__ ids,
    const int2* __restrict__ ranges, int64_t n, float bg, const ViewTable vt, int C,
    const float* __restrict__ final_T, const int32_t* __restrict__ n_contrib,
    const float* __restrict__ d_out, float* __restrict__ grad_records,
    int64_t* __restrict__ info) {
  static_assert(GR == 16, "one owner lane per component of a 16-float gradient record");
  static_assert(NC <= 8, "the d_out planes hold eight channels");
  constexpr int PX = 4, BW = 8, RS = 4, BH = 16;
  constexpr int NP = (NC + 1) / 2;
  // 32-record batches: each splat's sums go straight to its gradient record
  // (the tile form's scheme); 64: a shared table flushed once per batch
  constexpr bool DIRECT = B == 32;
  extern __shared__ __align__(128) float smem[];
  __shared__ uint8_t s_touched[DIRECT ? 1 : B];
  __shared__ uint8_t s_list[B];
  __shared__ __align__(16) float4 s_dout[2][PX * 32];  // [plane][q * 32 + lane]
  float* gacc = smem + 2 * B * RF;                     // [B][GR] (not DIRECT)

  const int tile = blockIdx.x >> 1;
  int W, H, gx, ltile;
  int64_t pbase;
  tile_view(vt, tile, W, H, gx, ltile, pbase);
  const int lane = threadIdx.x;
  const int bx0 = (ltile % gx) * kTile + BW * (blockIdx.x & 1);
  const int by0 = (ltile / gx) * kTile;

  if constexpr (!DIRECT) {
    for (int i = lane; i < B * GR; i += 32) gacc[i] = 0.f;
    for (int i = lane; i < B; i += 32) s_touched[i] = 0;
  }

  const int64_t plane = (int64_t)W * H;
  const int pxi = bx0 + (lane & (BW - 1));
  const float pxf = (float)pxi;
  const float py0 = (float)(by0 + lane / BW);
  float T[PX], SB[PX];
  int nc[PX];
  int my_nc = 0;
#pragma unroll
  for (int q = 0; q < PX; ++q) {
    const int py = by0 + lane / BW + RS * q;
    float dv[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) dv[c] = 0.f;
    T[q] = 1.f;
    nc[q] = 0;
    if (pxi < W && py < H) {
      const int64_t pix = (int64_t)py * W + pxi;
      T[q] = final_T[pbase + pix];
      nc[q] = n_contrib[pbase + pix];
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (c < C) dv[c] = d_out[C * pbase + c * plane + pix];
    }
    float sd = 0.f;
#pragma unroll
    for (int c = 0; c < NC; ++c) sd += dv[c];
    SB[q] = bg * sd;
    s_dout[0][q * 32 + lane] = make_float4(dv[0], dv[1], dv[2], dv[3]);
    s_dout[1][q * 32 + lane] = make_float4(dv[4], dv[5], dv[6], dv[7]);
    my_nc = max(my_nc, nc[q]);
  }
  int warp_nc = my_nc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) warp_nc = max(warp_nc, __shfl_xor_sync(0xffffffffu, warp_nc, o));
  const int2 rg = ranges[tile];
  const int64_t start = rg.x;
  const int list_len = max(0, rg.y - rg.x);
  if (warp_nc > list_len && lane == 0) set_info(info, PGB_ERR_OVERFLOW);
  const int max_nc = min(warp_nc, list_len);
  const int nb = (max_nc + B - 1) / B;
  auto lo_of = [&](int b) { return max(0, max_nc - (b + 1) * B); };
  auto hi_of = [&](int b) { return max_nc - b * B; };
  __syncwarp();

  int32_t g_cur = -1, g_nxt = -1;  // DIRECT: the splat id of slot `lane`
  if (nb > 0) {
    if constexpr (DIRECT)
      g_nxt = stage_batch_id<RF>(records, ids, start + lo_of(0), start + hi_of(0), n, smem, info);
    else
      stage_batch<RF, 32, B>(records, ids, start + lo_of(0), start + hi_of(0), n, smem, info);
  }
  for (int b = 0; b < nb; ++b) {
    const int buf = b & 1;
    const int lo = lo_of(b), hi = hi_of(b);
    g_cur = g_nxt;
    if (b + 1 < nb) {
      if constexpr (DIRECT)
        g_nxt = stage_batch_id<RF>(records, ids, start + lo_of(b + 1), start + hi_of(b + 1), n,
                                   smem + (buf ^ 1) * B * RF, info);
      else
        stage_batch<RF, 32, B>(records, ids, start + lo_of(b + 1), start + hi_of(b + 1), n,
                               smem + (buf ^ 1) * B * RF, info);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncwarp();  // every lane's copies of batch b have landed
    const float* st = smem + buf * B * RF;
    const int nl = warp_cull<BW, BH, B>(st, RF, hi - lo, (float)bx0, (float)by0, s_list);
    for (int t = nl - 1; t >= 0; --t) {
      const int slot = s_list[t];
      const int j = lo + slot;
      const float* rec = st + slot * RF;
      const float4 r0 = *reinterpret_cast<const float4*>(rec);      // u, v, A, B
      const float4 r1 = *reinterpret_cast<const float4*>(rec + 4);  // C, o, tau, thr
      const float dx = __fsub_rn(r0.x, pxf);
      const SplatX sx = splat_x(r0.z, r0.w, dx);
      float dyq[PX], p2q[PX];
      bool okq[PX];
      bool contrib = false;
#pragma unroll
      for (int q = 0; q < PX; ++q) {
        dyq[q] = __fsub_rn(r0.y, py0 + (float)(RS * q));
        p2q[q] = splat_power2(sx, r1.x, dyq[q]);
        okq[q] = j < nc[q] && !(p2q[q] > 0.f || p2q[q] < r1.w);  // the forward's skip test
        contrib |= okq[q];
      }
      if (!__any_sync(0xffffffffu, contrib)) continue;
      float2 v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = f2(0.f, 0.f);
      const float2* fp = reinterpret_cast<const float2*>(rec + kRecFeat);
      float2 fr[NP];
#pragma unroll
      for (int k = 0; k < NP; ++k) fr[k] = fp[k];
#pragma unroll
      for (int q = 0; q < PX; ++q) {
        const float dy = dyq[q];
        const float g0 = __fmaf_rn(r0.w, dy, sx.Adx), g1 = __fmaf_rn(r1.x, dy, sx.Bdx);
        const float G = ex2_approx(p2q[q]);
        const float araw = __fmul_rn(r1.y, G);
        const float alpha = okq[q] ? fminf(0.99f, araw) : 0.f;
        const float om = __fsub_rn(1.0f, alpha);
        T[q] = okq[q] ? __fdividef(T[q], om) : T[q];
        const float4 dlo = s_dout[0][q * 32 + lane];
        const float4 dhi = s_dout[1][q * 32 + lane];
        const float2 dp[4] = {f2(dlo.x, dlo.y), f2(dlo.z, dlo.w), f2(dhi.x, dhi.y),
                              f2(dhi.z, dhi.w)};
        float2 F2 = __fmul2_rn(dp[0], fr[0]);
#pragma unroll
        for (int k = 1; k < NP; ++k) F2 = __ffma2_rn(dp[k], fr[k], F2);
        const float F = F2.x + F2.y;
        const float wT = alpha * T[q];
        const float2 wT2 = f2(wT, wT);
#pragma unroll
        for (int k = 0; k < NP; ++k) v[3 + k] = __ffma2_rn(wT2, dp[k], v[3 + k]);
        const float dalpha = (F - SB[q]) * T[q];
        SB[q] = fmaf(alpha, F, om * SB[q]);
        const bool m = okq[q] && araw < 0.99f;
        const float dpow = m ? alpha * dalpha : 0.f;
        const float Gm = m ? G : 0.f;
        const float tx = dpow * dx;
        v[0] = __ffma2_rn(f2(g0, g1), f2(dpow, dpow), v[0]);        // sum g0 dp, g1 dp
        v[1] = __ffma2_rn(f2(tx, tx), f2(dx, dy), v[1]);            // dx^2 dp, dx dy dp
        v[2] = __ffma2_rn(f2(dpow * dy, Gm), f2(dy, dalpha), v[2]);  // dy^2 dp, G dalpha
      }
      float vf[16];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        vf[2 * k] = v[k].x;
        vf[2 * k + 1] = v[k].y;
      }
      const float sum = warp_reduce_scatter<16>(vf);
      // lanes 2k and 2k + 1 both hold component k; the even one owns it
      if constexpr (DIRECT) {
        const int32_t g = __shfl_sync(0xffffffffu, g_cur, slot);
        if (g >= 0 && (lane & 1) == 0 && (lane >> 1) < 6 + NC)
          atomicAdd(grad_records + (int64_t)g * GR + (lane >> 1), sum);
      } else {
        if ((lane & 1) == 0 && (lane >> 1) < 6 + NC) gacc[slot * GR + (lane >> 1)] += sum;
        if (lane == 0) s_touched[slot] = 1;
      }
    }
    if constexpr (!DIRECT) {
      __syncwarp();
      for (int t = lane; t < hi - lo; t += 32) {
        if (!s_touched[t]) continue;
        const int32_t g = ids[start + lo + t];
        if (g < 0 || (int64_t)g >= n) {
          set_info(info, PGB_ERR_OVERFLOW);
          continue;
        }
        float4* dst = reinterpret_cast<float4*>(grad_records + (int64_t)g * GR);
        float4* srcv = reinterpret_cast<float4*>(gacc + t * GR);
#pragma unroll
        for (int q = 0; q < (6 + NC + 3) / 4; ++q) {
          atomicAdd(dst + q, srcv[q]);
          srcv[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        s_touched[t] = 0;
      }
    }
    __syncwarp();  // the stage of batch b is refilled by the next iteration's copies
  }
}

// Backward, one warp per 16 x 16 tile: lane l owns the eight pixels
// (l % 8 + 8 (q & 1), l / 8 + 4 (q >> 1)), q < 8, so one per-splat warp
// reduction serves the whole tile (256 pixels) and every pixel slot q is an
// 8 x 4 block.  The skip tests of all eight slots come first; a slot where
// no lane composites the splat is skipped by a warp-uniform branch, and a
// slot where some lane does runs its replay step without per-pixel branches
// (a lane that skips gets alpha = 0 and keeps T and SB exactly).  No CTA
// barrier (one warp per CTA); each splat's reduced sums are added to its
// gradient record at once by their owner lanes (one warp-wide atomic, no
// shared gradient table: 12.4 KB of shared memory per CTA, so 16 CTAs per
// SM at 121 registers).
template <int NC, int RF, int GR, int B, int MINB, int TH = 16>
__global__ void __launch_bounds__(32, MINB) blend_bwd_tile_kernel(
    const float* __restrict__ records, const int32_t* __restrict__ ids,
    const int2* __restrict__ ranges, int64_t n, float bg, const ViewTable vt, int C,
    const float* __restrict__ final_T, const int32_t* __restrict__ n_contrib,
    const float* __restrict__ d_out, float* __restrict__ grad_records,
    int64_t* __restrict__ info, const int32_t* __restrict__ radius) {
  static_assert(GR == 16, "one owner lane per component of a 16-float gradient record");
  static_assert(NC <= 8, "the d_out planes hold eight channels");
  static_assert(B == 32, "one staged splat id per lane");
  constexpr int PX = 8;
  // 16 x 32 tiles (a batch of views): one warp per 16 x 16 half (CTA
  // 2t + h), the tile's list filtered to the half's msplat list
  constexpr bool F16 = TH != kTile;
  constexpr int NP = (NC + 1) / 2;
  extern __shared__ __align__(128) float smem[];
  __shared__ uint8_t s_list[B];
  __shared__ __align__(16) float4 s_dout[2][PX * 32];  // [plane][q * 32 + lane]
  __shared__ int s_rad[F16 ? 2 : 1][F16 ? B : 1];

  const int tile = F16 ? blockIdx.x >> 1 : blockIdx.x;
  int W, H, gx, ltile;
  int64_t pbase;
  tile_view(vt, tile, W, H, gx, ltile, pbase);
  const int lane = threadIdx.x;
  const int bx0 = (ltile % gx) * kTile;
  const int by0 = (ltile / gx) * TH + (F16 ? kTile * (blockIdx.x & 1) : 0);
  List16 f16{};
  if constexpr (F16) {
    f16.tx = bx0 / kTile;
    f16.ty = by0 / kTile;
    f16.gx = grid_x(W);
    f16.gy = grid_y(H);
  }


  const int64_t plane = (int64_t)W * H;
  const float pxa = (float)(bx0 + (lane & 7)), pxb = pxa + 8.f;
  const float py0 = (float)(by0 + (lane >> 3));
  float T[PX], SB[PX];
  int nc[PX];
  int my_nc = 0;
#pragma unroll
  for (int q = 0; q < PX; ++q) {
    const int px = bx0 + (lane & 7) + 8 * (q & 1), py = by0 + (lane >> 3) + 4 * (q >> 1);
    float dv[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) dv[c] = 0.f;
    T[q] = 1.f;
    nc[q] = 0;
    if (px < W && py < H) {
      const int64_t pix = (int64_t)py * W + px;
      T[q] = final_T[pbase + pix];
      nc[q] = n_contrib[pbase + pix];
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (c < C) dv[c] = d_out[C * pbase + c * plane + pix];
    }
    float sd = 0.f;
#pragma unroll
    for (int c = 0; c < NC; ++c) sd += dv[c];
    SB[q] = bg * sd;
    s_dout[0][q * 32 + lane] = make_float4(dv[0], dv[1], dv[2], dv[3]);
    s_dout[1][q * 32 + lane] = make_float4(dv[4], dv[5], dv[6], dv[7]);
    my_nc = max(my_nc, nc[q]);
  }
  int warp_nc = my_nc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) warp_nc = max(warp_nc, __shfl_xor_sync(0xffffffffu, warp_nc, o));
  const int2 rg = ranges[tile];
  const int64_t start = rg.x;
  const int list_len = max(0, rg.y - rg.x);
  if (warp_nc > list_len && lane == 0) set_info(info, PGB_ERR_OVERFLOW);
  const int max_nc = min(warp_nc, list_len);
  const int nb = (max_nc + B - 1) / B;
  auto lo_of = [&](int b) { return max(0, max_nc - (b + 1) * B); };
  auto hi_of = [&](int b) { return max_nc - b * B; };
  __syncwarp();

  int32_t g_cur = -1, g_nxt = -1;  // the splat id of slot `lane` (current, next batch)
  if (nb > 0) {
    g_nxt = stage_batch_id<RF>(records, ids, start + lo_of(0), start + hi_of(0), n, smem, info);
    if constexpr (F16)
      stage_radius<32, B>(ids, radius, start + lo_of(0), start + hi_of(0), n, s_rad[0]);
  }
  for (int b = 0; b < nb; ++b) {
    const int buf = b & 1;
    const int lo = lo_of(b), hi = hi_of(b);
    g_cur = g_nxt;
    if (b + 1 < nb) {
      g_nxt = stage_batch_id<RF>(records, ids, start + lo_of(b + 1), start + hi_of(b + 1), n,
                                 smem + (buf ^ 1) * B * RF, info);
      if constexpr (F16)
        stage_radius<32, B>(ids, radius, start + lo_of(b + 1), start + hi_of(b + 1), n,
                            s_rad[buf ^ 1]);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncwarp();  // every lane's copies of batch b (and its radii) have landed
    const float* st = smem + buf * B * RF;
    if constexpr (F16) f16.rad = s_rad[buf];
    const int nl = warp_cull<16, 16, B, F16>(st, RF, hi - lo, (float)bx0, (float)by0, s_list, f16);
    for (int t = nl - 1; t >= 0; --t) {
      const int slot = s_list[t];
      const int j = lo + slot;
      const float* rec = st + slot * RF;
      const float4 r0 = *reinterpret_cast<const float4*>(rec);      // u, v, A, B
      const float4 r1 = *reinterpret_cast<const float4*>(rec + 4);  // C, o, tau, thr
      const float dxh[2] = {__fsub_rn(r0.x, pxa), __fsub_rn(r0.x, pxb)};
      const SplatX sxh[2] = {splat_x(r0.z, r0.w, dxh[0]), splat_x(r0.z, r0.w, dxh[1])};
      float p2q[PX];
      bool okq[PX];
      uint32_t mine = 0;  // this lane's compositing slots
#pragma unroll
      for (int q = 0; q < PX; ++q) {
        const float dy = __fsub_rn(r0.y, py0 + (float)(4 * (q >> 1)));
        p2q[q] = splat_power2(sxh[q & 1], r1.x, dy);
        okq[q] = j < nc[q] && !(p2q[q] > 0.f || p2q[q] < r1.w);  // the forward's skip test
        mine |= (uint32_t)okq[q] << q;
      }
      // the slots some lane composites: one reduction, then uniform branches
      const uint32_t slots = __reduce_or_sync(0xffffffffu, mine);
      if (!slots) continue;
      float2 v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = f2(0.f, 0.f);
      const float2* fp = reinterpret_cast<const float2*>(rec + kRecFeat);
      float2 fr[NP];
#pragma unroll
      for (int k = 0; k < NP; ++k) fr[k] = fp[k];
#pragma unroll
      for (int q = 0; q < PX; ++q) {
        if (!(slots & (1u << q))) continue;  // warp-uniform
        const float dx = dxh[q & 1];
        const float dy = __fsub_rn(r0.y, py0 + (float)(4 * (q >> 1)));
        const SplatX& sx = sxh[q & 1];
        const float g0 = __fmaf_rn(r0.w, dy, sx.Adx), g1 = __fmaf_rn(r1.x, dy, sx.Bdx);
        const float G = ex2_approx(p2q[q]);
        const float araw = __fmul_rn(r1.y, G);
        const float alpha = okq[q] ? fminf(0.99f, araw) : 0.f;
        const float om = __fsub_rn(1.0f, alpha);
        T[q] = okq[q] ? __fdividef(T[q], om) : T[q];
        const float4 dlo = s_dout[0][q * 32 + lane];
        const float4 dhi = s_dout[1][q * 32 + lane];
        const float2 dp[4] = {f2(dlo.x, dlo.y), f2(dlo.z, dlo.w), f2(dhi.x, dhi.y),
                              f2(dhi.z, dhi.w)};
        float2 F2 = __fmul2_rn(dp[0], fr[0]);
#pragma unroll
        for (int k = 1; k < NP; ++k) F2 = __ffma2_rn(dp[k], fr[k], F2);
        const float F = F2.x + F2.y;
        const float wT = alpha * T[q];
        const float2 wT2 = f2(wT, wT);
#pragma unroll
        for (int k = 0; k < NP; ++k) v[3 + k] = __ffma2_rn(wT2, dp[k], v[3 + k]);
        const float dalpha = (F - SB[q]) * T[q];
        SB[q] = fmaf(alpha, F, om * SB[q]);
        const bool m = okq[q] && araw < 0.99f;
        const float dpow = m ? alpha * dalpha : 0.f;
        const float Gm = m ? G : 0.f;
        const float tx = dpow * dx;
        v[0] = __ffma2_rn(f2(g0, g1), f2(dpow, dpow), v[0]);        // sum g0 dp, g1 dp
        v[1] = __ffma2_rn(f2(tx, tx), f2(dx, dy), v[1]);            // dx^2 dp, dx dy dp
        v[2] = __ffma2_rn(f2(dpow * dy, Gm), f2(dy, dalpha), v[2]);  // dy^2 dp, G dalpha
      }
      float vf[16];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        vf[2 * k] = v[k].x;
        vf[2 * k + 1] = v[k].y;
      }
      const float sum = warp_reduce_scatter<16>(vf);
      // the splat's sums go straight to its gradient record, one warp-wide
      // reduction: the owner lanes' 6 + NC floats lie in one 64-byte record
      const int32_t g = __shfl_sync(0xffffffffu, g_cur, slot);
      if (g >= 0 && (lane & 1) == 0 && (lane >> 1) < 6 + NC)
        atomicAdd(grad_records + (int64_t)g * GR + (lane >> 1), sum);
    }
    __syncwarp();  // the stage of batch b is refilled by the next iteration's copies
  }
}

// ---------------------------------------------------------------- unpack
template <int RF>
__global__ void unpack_kernel(const float* __restrict__ g, int64_t n, int C,
                              float* __restrict__ d_uv, float* __restrict__ d_conic,
                              float* __restrict__ d_opacity, const FeatGradCols gc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float r[RF];
    const float4* s = reinterpret_cast<const float4*>(g + i * RF);
#pragma unroll
    for (int q = 0; q < RF / 4; ++q) {
      const float4 x = s[q];
      r[4 * q] = x.x; r[4 * q + 1] = x.y; r[4 * q + 2] = x.z; r[4 * q + 3] = x.w;
    }
    // gradient moments -> uv and conic gradients (g0, g1 carried the scale K)
    reinterpret_cast<float2*>(d_uv)[i] =
        make_float2(-r[0] * kInvConicScale, -r[1] * kInvConicScale);
    d_conic[3 * i] = -0.5f * r[2];
    d_conic[3 * i + 1] = -r[3];
    d_conic[3 * i + 2] = -0.5f * r[4];
    d_opacity[i] = r[5];
#pragma unroll
    for (int c = 0; c < RF - 6; ++c)
      if (c < C) gc.dst[c][i * gc.stride[c]] = r[6 + c];
  }
}

// ---------------------------------------------------------------- census
// The work of one blend, counted for the benchmark's roofline (not on the
// training path): per pixel, the list entries up to its last contributor
// (the pairs the backward replays) and, among them, the composited ones
// (the forward's own alpha test on the record, bit for bit).  One thread per
// pixel of a tile; warp sums, then one 64-bit atomic per warp and counter.
template <int RF>
__global__ void __launch_bounds__(256) census_kernel(const float* __restrict__ records,
                                                     const int32_t* __restrict__ ids,
                                                     const int2* __restrict__ ranges, int64_t n,
                                                     const ViewTable vt,
                                                     const int32_t* __restrict__ n_contrib,
                                                     unsigned long long* __restrict__ counts) {
  const int tile = blockIdx.x;
  int W, H, gx, ltile;
  int64_t pbase;
  tile_view(vt, tile, W, H, gx, ltile, pbase);
  const int px = (ltile % gx) * kTile + (threadIdx.x & (kTile - 1));
  const int py = (ltile / gx) * kTile + (threadIdx.x / kTile);
  unsigned long long evaluated = 0, composited = 0;
  if (px < W && py < H) {
    const int2 rg = ranges[tile];
    const int m = min(n_contrib[pbase + (int64_t)py * W + px], max(0, rg.y - rg.x));
    evaluated = (unsigned long long)max(m, 0);
    const float pxf = (float)px, pyf = (float)py;
    for (int j = 0; j < m; ++j) {
      const int32_t g = ids[rg.x + j];
      if (g < 0 || (int64_t)g >= n) continue;
      const float* rec = records + (int64_t)g * RF;
      const SplatX sx = splat_x(rec[2], rec[3], __fsub_rn(rec[0], pxf));
      const float p2 = splat_power2(sx, rec[4], __fsub_rn(rec[1], pyf));
      if (!(p2 > 0.f || p2 < rec[7])) ++composited;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    evaluated += __shfl_xor_sync(0xffffffffu, evaluated, o);
    composited += __shfl_xor_sync(0xffffffffu, composited, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&counts[0], evaluated);
    atomicAdd(&counts[1], composited);
  }
}

// ------------------------------------------------------------- dispatch
// Tiles 16 x 32 (a batch of views with vt.th == 32) are compiled for the
// channel buckets of RGB, RGB + depth and RGB + depth + normal.
template <int NC>
constexpr bool kTall = NC == 3 || NC == 4 || NC == 7;

inline bool tall_tiles(const ViewTable& vt) { return vt.nviews > 0 && vt.th == 32; }

template <int NC, int B, int TH = 16, bool FLAT = false>
static int launch_fwd_b(const float* records, const int32_t* ids, const int2* ranges, int64_t n,
                        float bg, const ViewTable& vt, int tiles, int C, float* out, float* fT,
                        int32_t* ncon, int64_t* info, cudaStream_t s, const int32_t* radius) {
  constexpr int RF = rec_floats(NC);
  const size_t smem = 2 * B * RF * sizeof(float);
  auto kern = blend_fwd_kernel<NC, RF, B, TH, FLAT>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return PGB_ERR_CUDA;
  kern<<<tiles, 64 * (TH / 8), smem, s>>>(records, ids, ranges, n, bg, vt, C, out, fT, ncon, info,
                                          radius);
  return launch_status();
}

// batch: records per batch, 64 or 128 (0: the default); 16 x 32 tiles also
// 256.  Never more records than threads: one TMA bulk copy per thread per
// phase at most.
template <int NC>
static int launch_fwd_nc(const float* records, const int32_t* ids, const int2* ranges, int64_t n,
                         float bg, const ViewTable& vt, int tiles, int C, float* out, float* fT,
                         int32_t* ncon, int64_t* info, cudaStream_t s, int batch,
                         const int32_t* radius) {
#define PGB_FWD(B, TH) \
  launch_fwd_b<NC, B, TH>(records, ids, ranges, n, bg, vt, tiles, C, out, fT, ncon, info, s, radius)
  if (tall_tiles(vt)) {
    if constexpr (kTall<NC>) {
      if (!radius) return PGB_ERR_INVALID;
      switch (batch == 0 ? kFwdBatch : batch) {
        case 64: return PGB_FWD(64, 32);
        case 128: return PGB_FWD(128, 32);
        case 256: return PGB_FWD(256, 32);
        case kFwdFlat + 64:
          return launch_fwd_b<NC, 64, 32, true>(records, ids, ranges, n, bg, vt, tiles, C, out,
                                                fT, ncon, info, s, radius);
        case kFwdFlat + 128:
          return launch_fwd_b<NC, 128, 32, true>(records, ids, ranges, n, bg, vt, tiles, C, out,
                                                 fT, ncon, info, s, radius);
        case kFwdFlat + 256:
          return launch_fwd_b<NC, 256, 32, true>(records, ids, ranges, n, bg, vt, tiles, C, out,
                                                 fT, ncon, info, s, radius);
        default: return PGB_ERR_INVALID;
      }
    }
    return PGB_ERR_INVALID;
  }
  switch (batch == 0 ? kFwdBatch : batch) {
    case 64: return PGB_FWD(64, 16);
    case 128: return PGB_FWD(128, 16);
    case kFwdFlat + 64:
      return launch_fwd_b<NC, 64, 16, true>(records, ids, ranges, n, bg, vt, tiles, C, out, fT,
                                            ncon, info, s, radius);
    case kFwdFlat + 128:
      return launch_fwd_b<NC, 128, 16, true>(records, ids, ranges, n, bg, vt, tiles, C, out, fT,
                                             ncon, info, s, radius);
    default: return PGB_ERR_INVALID;
  }
#undef PGB_FWD
}

template <int NC, int B, int PX, int MINB, bool XRED, bool FLAT = false>
static int launch_bwd2_b(const float* records, const int32_t* ids, const int2* ranges, int64_t n,
                         float bg, const ViewTable& vt, int tiles, int C, const float* fT,
                         const int32_t* ncon, const float* dout, float* grec, int64_t* info,
                         cudaStream_t s) {
  constexpr int RF = rec_floats(NC);
  constexpr int GR = grad_floats(NC);
  const size_t smem = (2 * RF + GR) * B * sizeof(float);
  auto kern = blend_bwd2_kernel<NC, RF, GR, B, PX, MINB, XRED, FLAT>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess ||
      cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared) != cudaSuccess)
    return PGB_ERR_CUDA;
  kern<<<tiles, 256 / PX, smem, s>>>(records, ids, ranges, n, bg, vt, C, fT, ncon, dout, grec,
                                     info);
  return launch_status();
}

template <int NC, int B, int MINB>
static int launch_bwd_solo(const float* records, const int32_t* ids, const int2* ranges,
                           int64_t n, float bg, const ViewTable& vt, int tiles, int C,
                           const float* fT, const int32_t* ncon, const float* dout, float* grec,
                           int64_t* info, cudaStream_t s) {
  constexpr int RF = rec_floats(NC);
  constexpr int GR = grad_floats(NC);
  const size_t smem = (2 * RF + (B == 32 ? 0 : GR)) * B * sizeof(float);  // no table at 32
  auto kern = blend_bwd_solo_kernel<NC, RF, GR, B, MINB>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess ||
      cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared) != cudaSuccess)
    return PGB_ERR_CUDA;
  kern<<<2 * tiles, 32, smem, s>>>(records, ids, ranges, n, bg, vt, C, fT, ncon, dout, grec, info);
  return launch_status();
}

template <int NC, int B, int MINB, int TH = 16>
static int launch_bwd_tile(const float* records, const int32_t* ids, const int2* ranges,
                           int64_t n, float bg, const ViewTable& vt, int tiles, int C,
                           const float* fT, const int32_t* ncon, const float* dout, float* grec,
                           int64_t* info, cudaStream_t s, const int32_t* radius = nullptr) {
  constexpr int RF = rec_floats(NC);
  constexpr int GR = grad_floats(NC);
  const size_t smem = 2 * RF * B * sizeof(float);
  auto kern = blend_bwd_tile_kernel<NC, RF, GR, B, MINB, TH>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess ||
      cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared) != cudaSuccess)
    return PGB_ERR_CUDA;
  kern<<<tiles * (TH / kTile), 32, smem, s>>>(records, ids, ranges, n, bg, vt, C, fT, ncon, dout,
                                               grec, info, radius);
  return launch_status();
}

template <int NC, int B, int PX, int TH = 16>
static int launch_bwd_b(const float* records, const int32_t* ids, const int2* ranges, int64_t n,
                        float bg, const ViewTable& vt, int tiles, int C, const float* fT,
                        const int32_t* ncon, const float* dout, float* grec, int64_t* info,
                        cudaStream_t s, const int32_t* radius) {
  constexpr int RF = rec_floats(NC);
  constexpr int GR = grad_floats(NC);
  const size_t smem = (2 * RF + GR) * B * sizeof(float);
  auto kern = blend_bwd_kernel<NC, RF, GR, B, PX, TH>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return PGB_ERR_CUDA;
  kern<<<tiles, 256 / PX * (TH / 16), smem, s>>>(records, ids, ranges, n, bg, vt, C, fT, ncon,
                                                 dout, grec, info, radius);
  return launch_status();
}

// batch: a backward variant code -- 64, 128 or 256 splats per batch with two
// pixels per thread, kBwdPx4 + 32 / 64 / 128 with four, kBwdV2 + ... the
// second form (0: the default).  16 x 32 tiles take the first form for
// every code.
template <int NC>
static int launch_bwd_nc(const float* records, const int32_t* ids, const int2* ranges, int64_t n,
                         float bg, const ViewTable& vt, int tiles, int C, const float* fT,
                         const int32_t* ncon, const float* dout, float* grec, int64_t* info,
                         cudaStream_t s, int batch, const int32_t* radius) {
#define PGB_BWD_T(B, PX, TH)                                                                      \
  launch_bwd_b<NC, B, PX, TH>(records, ids, ranges, n, bg, vt, tiles, C, fT, ncon, dout, grec, info, \
                              s, radius)
#define PGB_BWD(B, PX) PGB_BWD_T(B, PX, 16)
  if (tall_tiles(vt)) {
    if constexpr (kTall<NC>) {
      if (!radius) return PGB_ERR_INVALID;
      switch (batch == 0 ? kBwdBatch : batch) {
        case 64: return PGB_BWD_T(64, 2, 32);
        case 128: return PGB_BWD_T(128, 2, 32);
        case 256: return PGB_BWD_T(256, 2, 32);
        case kBwdPx4 + 32:
        case kBwdV2 + 512 + 32:
        case kBwdV2 + 1024 + 32:
        case kBwdV2 + kBwdFlat + 32:
        case kBwdV2 + kBwdFlat + 1024 + 32: return PGB_BWD_T(32, 4, 32);
        case kBwdPx4 + 64:
        case kBwdV2 + 64:
        case kBwdV2 + kBwdFlat + 64:
        case kBwdV2 + kBwdFlat + 1024 + 64:
        case kBwdSolo + 64: return PGB_BWD_T(64, 4, 32);
        case kBwdSolo + 32:
        case kBwdSolo + 1024 + 32:
        case kBwdSolo + 2048 + 32: return PGB_BWD_T(32, 4, 32);
        case kBwdTile + 32:
          if constexpr (NC <= 8)
            return launch_bwd_tile<NC, 32, 16, 32>(records, ids, ranges, n, bg, vt, tiles, C, fT,
                                                   ncon, dout, grec, info, s, radius);
          return PGB_BWD_T(32, 4, 32);
        case kBwdPx4 + 128: return PGB_BWD_T(128, 4, 32);
        default: return PGB_ERR_INVALID;
      }
    }
    return PGB_ERR_INVALID;
  }
  switch (batch == 0 ? kBwdBatch : batch) {
    case 64: return PGB_BWD(64, 2);
    case 128: return PGB_BWD(128, 2);
    case 256: return PGB_BWD(256, 2);
    case kBwdPx4 + 32: return PGB_BWD(32, 4);
    case kBwdPx4 + 64: return PGB_BWD(64, 4);
    case kBwdPx4 + 128: return PGB_BWD(128, 4);
    default: break;
  }
  if constexpr (NC <= 8) {
#define PGB_BWD2(B, PX, MINB, XRED, FLAT)                                                     \
  launch_bwd2_b<NC, B, PX, MINB, XRED, FLAT>(records, ids, ranges, n, bg, vt, tiles, C, fT, ncon, \
                                             dout, grec, info, s)
    switch (batch) {
      case kBwdV2 + 64: return PGB_BWD2(64, 4, 1, false, false);
      case kBwdV2 + 512 + 32: return PGB_BWD2(32, 4, 1, true, false);
      case kBwdV2 + 1024 + 32: return PGB_BWD2(32, 4, 12, true, false);
      case kBwdV2 + kBwdFlat + 32: return PGB_BWD2(32, 4, 1, false, true);
      case kBwdV2 + kBwdFlat + 64: return PGB_BWD2(64, 4, 1, false, true);
      case kBwdV2 + kBwdFlat + 1024 + 32: return PGB_BWD2(32, 4, 10, false, true);
      case kBwdV2 + kBwdFlat + 1024 + 64: return PGB_BWD2(64, 4, 10, false, true);
      default: break;
    }
    if constexpr (grad_floats(NC) == 16) {
      switch (batch) {
        case kBwdSolo + 32:
          return launch_bwd_solo<NC, 32, 16>(records, ids, ranges, n, bg, vt, tiles, C, fT, ncon,
                                              dout, grec, info, s);
        case kBwdSolo + 64:
          return launch_bwd_solo<NC, 64, 16>(records, ids, ranges, n, bg, vt, tiles, C, fT, ncon,
                                              dout, grec, info, s);
        case kBwdSolo + 1024 + 32:
          return launch_bwd_solo<NC, 32, 20>(records, ids, ranges, n, bg, vt, tiles, C, fT, ncon,
                                              dout, grec, info, s);
        case kBwdSolo + 2048 + 32:
          return launch_bwd_solo<NC, 32, 24>(records, ids, ranges, n, bg, vt, tiles, C, fT, ncon,
                                              dout, grec, info, s);
        case kBwdTile + 32:
          return launch_bwd_tile<NC, 32, 16>(records, ids, ranges, n, bg, vt, tiles, C, fT, ncon,
                                              dout, grec, info, s);

        default: break;
      }
    }
#undef PGB_BWD2
  } else {
    // the second form keeps eight channels of d_out in shared memory: wider
    // features take the first form's four-pixel kernel with the same batch
    switch (batch) {
      case kBwdV2 + 64:
      case kBwdV2 + kBwdFlat + 64:
      case kBwdV2 + kBwdFlat + 1024 + 64:
      case kBwdSolo + 64: return PGB_BWD(64, 4);
      case kBwdSolo + 32:
      case kBwdSolo + 1024 + 32:
      case kBwdSolo + 2048 + 32:
      case kBwdTile + 32: return PGB_BWD(32, 4);
      case kBwdV2 + 512 + 32:
      case kBwdV2 + 1024 + 32:
      case kBwdV2 + kBwdFlat + 32:
      case kBwdV2 + kBwdFlat + 1024 + 32: return PGB_BWD(32, 4);
      default: break;
    }
  }
#undef PGB_BWD
#undef PGB_BWD_T
  return PGB_ERR_INVALID;
}

// Channel counts with a compiled kernel; other counts round up (extra
// channels are zero in the records and never written out).
#define PGB_FOR_NC(X) X(1) X(3) X(4) X(7) X(8) X(10) X(16) X(26)

inline int nc_bucket(int C) {
  const int b[] = {1, 3, 4, 7, 8, 10, 16, 26};
  for (int x : b)
    if (C <= x) return x;
  return -1;
}

}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_blend_record_floats(int channels) {
  if (channels < 1 || channels > 26) return -1;
  return rec_floats(nc_bucket(channels));
}

int pgb_blend_grad_record_floats(int channels) {
  if (channels < 1 || channels > 26) return -1;
  return grad_floats(nc_bucket(channels));
}

}  // extern "C"

// One [N,C] tensor as a column table.
static FeatCols cols_of(const float* feature, int C) {
  FeatCols fc;
  for (int c = 0; c < kMaxCols; ++c) {
    fc.src[c] = c < C && feature ? feature + c : nullptr;
    fc.stride[c] = C;
  }
  return fc;
}
static FeatGradCols grad_cols_of(float* d_feature, int C) {
  FeatGradCols gc;
  for (int c = 0; c < kMaxCols; ++c) {
    gc.dst[c] = c < C && d_feature ? d_feature + c : nullptr;
    gc.stride[c] = C;
  }
  return gc;
}

static int blend_forward_impl(const float* uv, const float* conic, const float* opacity,
                              const FeatCols& fc, int64_t n, int channels, const int32_t* ids,
                              int64_t k, const int32_t* tile_range, float bg, const ViewTable& vt,
                              int tiles, float* records, float* out, float* final_T,
                              int32_t* n_contrib, int64_t* info, void* stream, int batch,
                              bool pack = true, const int32_t* radius = nullptr) {
  const int nc = nc_bucket(channels);
  if (n < 0 || k < 0 || tiles <= 0 || channels < 1 || nc < 0) return PGB_ERR_INVALID;
  if (!tile_range || !out || !final_T || !n_contrib || (k > 0 && !ids)) return PGB_ERR_INVALID;
  if (n > 0 && (!records || (pack && (!uv || !conic || !opacity || !fc.src[0]))))
    return PGB_ERR_INVALID;
  // records are staged by bulk copies and read as float4; the ranges as int2
  // (info, when given, takes a 64-bit atomic)
  if (misaligned(records, 16) || misaligned(tile_range, 8) || misaligned(info, 8))
    return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  const int2* rg = reinterpret_cast<const int2*>(tile_range);
  switch (nc) {
#define PGB_CASE(N)                                                                             \
  case N:                                                                                       \
    if (n > 0 && pack)                                                                          \
      pack_kernel<rec_floats(N)><<<stream_grid(n), kStreamThreads, 0, s>>>(uv, conic, opacity,  \
                                                                           fc, n, channels,      \
                                                                           records);            \
    return launch_fwd_nc<N>(records, ids, rg, n, bg, vt, tiles, channels, out, final_T,          \
                            n_contrib, info, s, batch, radius);
    PGB_FOR_NC(PGB_CASE)
#undef PGB_CASE
    default:
      return PGB_ERR_INVALID;
  }
}

static int blend_backward_impl(const float* records, int64_t n, int channels, const int32_t* ids,
                               int64_t k, const int32_t* tile_range, float bg, const ViewTable& vt,
                               int tiles, const float* final_T, const int32_t* n_contrib,
                               const float* d_out, float* grad_records, float* d_uv,
                               float* d_conic, float* d_opacity, const FeatGradCols& gc,
                               int64_t* info, void* stream, int batch, bool first = true,
                               bool last = true, const int32_t* radius = nullptr) {
  const int nc = nc_bucket(channels);
  if (n < 0 || k < 0 || tiles <= 0 || channels < 1 || nc < 0) return PGB_ERR_INVALID;
  if (!tile_range || !final_T || !n_contrib || !d_out || (k > 0 && !ids)) return PGB_ERR_INVALID;
  if (n > 0 && (!records || !grad_records ||
                (last && (!d_uv || !d_conic || !d_opacity || !gc.dst[0]))))
    return PGB_ERR_INVALID;
  if (misaligned(records, 16) || misaligned(grad_records, 16) || misaligned(d_uv, 8) ||
      misaligned(tile_range, 8) || misaligned(info, 8))
    return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  cudaStream_t s = as_stream(stream);
  const int GRf = grad_floats(nc);
  if (first && cudaMemsetAsync(grad_records, 0, (size_t)n * GRf * sizeof(float), s) != cudaSuccess)
    return PGB_ERR_CUDA;
  const int2* rg = reinterpret_cast<const int2*>(tile_range);
  int st = PGB_ERR_INVALID;
  switch (nc) {
#define PGB_CASE(N)                                                                          \
  case N:                                                                                    \
    st = launch_bwd_nc<N>(records, ids, rg, n, bg, vt, tiles, channels, final_T, n_contrib,  \
                          d_out, grad_records, info, s, batch, radius);                      \
    break;
    PGB_FOR_NC(PGB_CASE)
#undef PGB_CASE
    default:
      break;
  }
  if (st != PGB_OK) return st;
  if (!last) return PGB_OK;  // later bands add to the same gradient records
  if (GRf == 16)
    unpack_kernel<16><<<stream_grid(n), kStreamThreads, 0, s>>>(grad_records, n, channels, d_uv,
                                                                d_conic, d_opacity, gc);
  else
    unpack_kernel<32><<<stream_grid(n), kStreamThreads, 0, s>>>(grad_records, n, channels, d_uv,
                                                                d_conic, d_opacity, gc);
  return launch_status();
}

extern "C" {

int pgb_alpha_blending_forward_with_batch(const float* uv, const float* conic,
                                          const float* opacity, const float* feature, int64_t n,
                                          int channels, const int32_t* ids, int64_t k,
                                          const int32_t* tile_range, float bg, int width,
                                          int height, float* records, float* out, float* final_T,
                                          int32_t* n_contrib, int64_t* info, void* stream,
                                          int batch) {
  if (width <= 0 || height <= 0) return PGB_ERR_INVALID;
  return blend_forward_impl(uv, conic, opacity, cols_of(feature, channels), n, channels, ids, k,
                            tile_range, bg, single_view(width, height),
                            grid_x(width) * grid_y(height), records, out, final_T, n_contrib, info,
                            stream, batch);
}

int pgb_alpha_blending_forward(const float* uv, const float* conic, const float* opacity,
                               const float* feature, int64_t n, int channels, const int32_t* ids,
                               int64_t k, const int32_t* tile_range, float bg, int width,
                               int height, float* records, float* out, float* final_T,
                               int32_t* n_contrib, int64_t* info, void* stream) {
  return pgb_alpha_blending_forward_with_batch(uv, conic, opacity, feature, n, channels, ids, k,
                                               tile_range, bg, width, height, records, out,
                                               final_T, n_contrib, info, stream, 0);
}

int pgb_alpha_blending_backward_with_batch(const float* records, int64_t n, int channels,
                                           const int32_t* ids, int64_t k,
                                           const int32_t* tile_range, float bg, int width,
                                           int height, const float* final_T,
                                           const int32_t* n_contrib, const float* d_out,
                                           float* grad_records, float* d_uv, float* d_conic,
                                           float* d_opacity, float* d_feature, int64_t* info,
                                           void* stream, int batch) {
  if (width <= 0 || height <= 0) return PGB_ERR_INVALID;
  return blend_backward_impl(records, n, channels, ids, k, tile_range, bg,
                             single_view(width, height), grid_x(width) * grid_y(height), final_T,
                             n_contrib, d_out, grad_records, d_uv, d_conic, d_opacity,
                             grad_cols_of(d_feature, channels), info, stream, batch);
}

int pgb_alpha_blending_backward(const float* records, int64_t n, int channels,
                                const int32_t* ids, int64_t k, const int32_t* tile_range, float bg,
                                int width, int height, const float* final_T,
                                const int32_t* n_contrib, const float* d_out, float* grad_records,
                                float* d_uv, float* d_conic, float* d_opacity, float* d_feature,
                                int64_t* info, void* stream) {
  return pgb_alpha_blending_backward_with_batch(records, n, channels, ids, k, tile_range, bg, width,
                                                height, final_T, n_contrib, d_out, grad_records,
                                                d_uv, d_conic, d_opacity, d_feature, info, stream,
                                                0);
}

int pgb_alpha_blending_forward_views_with_batch(
    const float* uv, const float* conic, const float* opacity, const float* feature,
    int64_t n_per_view, int channels, const int32_t* ids, int64_t k, const int32_t* tile_range,
    float bg, const int32_t* sizes, int nviews, float* records, float* out, float* final_T,
    int32_t* n_contrib, int64_t* info, void* stream, int batch) {
  ViewTable vt;
  uint32_t T = 0;
  int64_t pixels = 0;
  if (!make_views(sizes, nviews, n_per_view, vt, T, pixels)) return PGB_ERR_INVALID;
  return blend_forward_impl(uv, conic, opacity, cols_of(feature, channels), n_per_view * nviews,
                            channels, ids, k, tile_range, bg, vt, (int)T, records, out, final_T,
                            n_contrib, info, stream, batch);
}

int pgb_alpha_blending_forward_views(const float* uv, const float* conic, const float* opacity,
                                     const float* feature, int64_t n_per_view, int channels,
                                     const int32_t* ids, int64_t k, const int32_t* tile_range,
                                     float bg, const int32_t* sizes, int nviews, float* records,
                                     float* out, float* final_T, int32_t* n_contrib,
                                     int64_t* info, void* stream) {
  return pgb_alpha_blending_forward_views_with_batch(uv, conic, opacity, feature, n_per_view,
                                                     channels, ids, k, tile_range, bg, sizes,
                                                     nviews, records, out, final_T, n_contrib,
                                                     info, stream, 0);
}

int pgb_alpha_blending_backward_views_with_batch(
    const float* records, int64_t n_per_view, int channels, const int32_t* ids, int64_t k,
    const int32_t* tile_range, float bg, const int32_t* sizes, int nviews, const float* final_T,
    const int32_t* n_contrib, const float* d_out, float* grad_records, float* d_uv,
    float* d_conic, float* d_opacity, float* d_feature, int64_t* info, void* stream, int batch) {
  ViewTable vt;
  uint32_t T = 0;
  int64_t pixels = 0;
  if (!make_views(sizes, nviews, n_per_view, vt, T, pixels)) return PGB_ERR_INVALID;
  return blend_backward_impl(records, n_per_view * nviews, channels, ids, k, tile_range, bg, vt,
                             (int)T, final_T, n_contrib, d_out, grad_records, d_uv, d_conic,
                             d_opacity, grad_cols_of(d_feature, channels), info, stream, batch);
}

int pgb_alpha_blending_backward_views(const float* records, int64_t n_per_view, int channels,
                                      const int32_t* ids, int64_t k, const int32_t* tile_range,
                                      float bg, const int32_t* sizes, int nviews,
                                      const float* final_T, const int32_t* n_contrib,
                                      const float* d_out, float* grad_records, float* d_uv,
                                      float* d_conic, float* d_opacity, float* d_feature,
                                      int64_t* info, void* stream) {
  return pgb_alpha_blending_backward_views_with_batch(
      records, n_per_view, channels, ids, k, tile_range, bg, sizes, nviews, final_T, n_contrib,
      d_out, grad_records, d_uv, d_conic, d_opacity, d_feature, info, stream, 0);
}

int pgb_alpha_blending_forward_pieces(const float* uv, const float* conic, const float* opacity,
                                      const float* const* pieces, const int32_t* widths,
                                      int npieces, int64_t n, const int32_t* ids, int64_t k,
                                      const int32_t* tile_range, float bg, int width, int height,
                                      float* records, float* out, float* final_T,
                                      int32_t* n_contrib, int64_t* info, void* stream, int batch) {
  if (width <= 0 || height <= 0) return PGB_ERR_INVALID;
  FeatCols fc;
  int channels = 0;
  if (!make_cols<const float, FeatCols>(pieces, widths, npieces, fc, channels, src_slot))
    return PGB_ERR_INVALID;
  return blend_forward_impl(uv, conic, opacity, fc, n, channels, ids, k, tile_range, bg,
                            single_view(width, height), grid_x(width) * grid_y(height), records,
                            out, final_T, n_contrib, info, stream, batch);
}

int pgb_alpha_blending_backward_pieces(const float* records, int64_t n, const int32_t* widths,
                                       int npieces, const int32_t* ids, int64_t k,
                                       const int32_t* tile_range, float bg, int width, int height,
                                       const float* final_T, const int32_t* n_contrib,
                                       const float* d_out, float* grad_records, float* d_uv,
                                       float* d_conic, float* d_opacity, float* const* d_pieces,
                                       int64_t* info, void* stream, int batch) {
  if (width <= 0 || height <= 0) return PGB_ERR_INVALID;
  FeatGradCols gc;
  int channels = 0;
  if (!make_cols<float, FeatGradCols>(d_pieces, widths, npieces, gc, channels, dst_slot))
    return PGB_ERR_INVALID;
  return blend_backward_impl(records, n, channels, ids, k, tile_range, bg,
                             single_view(width, height), grid_x(width) * grid_y(height), final_T,
                             n_contrib, d_out, grad_records, d_uv, d_conic, d_opacity, gc, info,
                             stream, batch);
}

// One band of tile rows [row0, row1) of an image (no msplat counterpart):
// tile_range holds the band's gx * (row1 - row0) tiles with band-local ids
// (pgb_sort_gaussian_finish_band), out/final_T/n_contrib are the whole
// image's and only the band's pixels are written.  pack = 0 reuses the
// records a previous band's call packed.
int pgb_alpha_blending_forward_band(const float* uv, const float* conic, const float* opacity,
                                    const float* feature, int64_t n, int channels,
                                    const int32_t* ids, int64_t k, const int32_t* tile_range,
                                    float bg, int width, int height, int row0, int row1, int pack,
                                    float* records, float* out, float* final_T,
                                    int32_t* n_contrib, int64_t* info, void* stream, int batch) {
  ViewTable vt;
  if (!band_view(width, height, row0, row1, vt)) return PGB_ERR_INVALID;
  return blend_forward_impl(uv, conic, opacity, cols_of(feature, channels), n, channels, ids, k,
                            tile_range, bg, vt, grid_x(width) * (row1 - row0), records, out,
                            final_T, n_contrib, info, stream, batch, pack != 0);
}

// The backward of one band: first != 0 zeroes grad_records first, last != 0
// turns the records summed over every band into d_uv, d_conic, d_opacity
// and d_feature (which may be NULL on the other bands).
int pgb_alpha_blending_backward_band(const float* records, int64_t n, int channels,
                                     const int32_t* ids, int64_t k, const int32_t* tile_range,
                                     float bg, int width, int height, int row0, int row1,
                                     const float* final_T, const int32_t* n_contrib,
                                     const float* d_out, float* grad_records, int first, int last,
                                     float* d_uv, float* d_conic, float* d_opacity,
                                     float* d_feature, int64_t* info, void* stream, int batch) {
  ViewTable vt;
  if (!band_view(width, height, row0, row1, vt)) return PGB_ERR_INVALID;
  return blend_backward_impl(records, n, channels, ids, k, tile_range, bg, vt,
                             grid_x(width) * (row1 - row0), final_T, n_contrib, d_out,
                             grad_records, d_uv, d_conic, d_opacity,
                             grad_cols_of(d_feature, channels), info, stream, batch, first != 0,
                             last != 0);
}

// A batch of views with tiles 16 pixels wide and tile_height (16 or 32)
// high (no msplat counterpart): ids and tile_range from
// pgb_sort_gaussian_finish_views_h with the same tile height; radius [V*N]
// (the elements' radii, as the sort took them) lets 16 x 32 tiles keep, per
// pixel, exactly the splats of msplat's 16 x 16 lists.
int pgb_alpha_blending_forward_views_h(const float* uv, const float* conic, const float* opacity,
                                       const float* feature, int64_t n_per_view, int channels,
                                       const int32_t* ids, int64_t k, const int32_t* tile_range,
                                       float bg, const int32_t* sizes, int nviews,
                                       int tile_height, const int32_t* radius, float* records,
                                       float* out, float* final_T, int32_t* n_contrib,
                                       int64_t* info, void* stream, int batch) {
  ViewTable vt;
  uint32_t T = 0;
  int64_t pixels = 0;
  if (!make_views(sizes, nviews, n_per_view, vt, T, pixels, tile_height)) return PGB_ERR_INVALID;
  return blend_forward_impl(uv, conic, opacity, cols_of(feature, channels), n_per_view * nviews,
                            channels, ids, k, tile_range, bg, vt, (int)T, records, out, final_T,
                            n_contrib, info, stream, batch, true, radius);
}

int pgb_alpha_blending_backward_views_h(const float* records, int64_t n_per_view, int channels,
                                        const int32_t* ids, int64_t k, const int32_t* tile_range,
                                        float bg, const int32_t* sizes, int nviews,
                                        int tile_height, const int32_t* radius,
                                        const float* final_T, const int32_t* n_contrib,
                                        const float* d_out, float* grad_records, float* d_uv,
                                        float* d_conic, float* d_opacity, float* d_feature,
                                        int64_t* info, void* stream, int batch) {
  ViewTable vt;
  uint32_t T = 0;
  int64_t pixels = 0;
  if (!make_views(sizes, nviews, n_per_view, vt, T, pixels, tile_height)) return PGB_ERR_INVALID;
  return blend_backward_impl(records, n_per_view * nviews, channels, ids, k, tile_range, bg, vt,
                             (int)T, final_T, n_contrib, d_out, grad_records, d_uv, d_conic,
                             d_opacity, grad_cols_of(d_feature, channels), info, stream, batch,
                             true, true, radius);
}

// Forward batch sizes compiled for 16 x tile_height tiles (see
// pgb_blend_batches for 16 x 16).
int pgb_blend_batches_h(int backward, int tile_height, int32_t* out) {
  if (tile_height != 32) return pgb_blend_batches(backward, out);
  static const int32_t f[] = {64, 128, 256, kFwdFlat + 128, kFwdFlat + 256};
  if (backward) return pgb_blend_batches(backward, out);
  if (out)
    for (int i = 0; i < 5; ++i) out[i] = f[i];
  return 5;
}

// Pair census of a blend (no msplat counterpart): counts[0] += list entries
// up to each pixel's last contributor, counts[1] += the composited ones.
int pgb_blend_pair_census(const float* records, int channels, int64_t n, const int32_t* ids,
                          int64_t k, const int32_t* tile_range, int width, int height,
                          const int32_t* n_contrib, unsigned long long* counts, void* stream) {
  const int nc = nc_bucket(channels);
  if (width <= 0 || height <= 0 || n < 0 || k < 0 || channels < 1 || nc < 0) return PGB_ERR_INVALID;
  if (!tile_range || !n_contrib || !counts || (k > 0 && !ids) || (n > 0 && !records))
    return PGB_ERR_INVALID;
  if (misaligned(records, 16) || misaligned(tile_range, 8) || misaligned(counts, 8))
    return PGB_ERR_INVALID;
  const ViewTable vt = single_view(width, height);
  const int tiles = grid_x(width) * grid_y(height);
  const int2* rg = reinterpret_cast<const int2*>(tile_range);
  cudaStream_t s = as_stream(stream);
  switch (rec_floats(nc)) {
    case 12: census_kernel<12><<<tiles, 256, 0, s>>>(records, ids, rg, n, vt, n_contrib, counts); break;
    case 16: census_kernel<16><<<tiles, 256, 0, s>>>(records, ids, rg, n, vt, n_contrib, counts); break;
    case 20: census_kernel<20><<<tiles, 256, 0, s>>>(records, ids, rg, n, vt, n_contrib, counts); break;
    case 24: census_kernel<24><<<tiles, 256, 0, s>>>(records, ids, rg, n, vt, n_contrib, counts); break;
    case 36: census_kernel<36><<<tiles, 256, 0, s>>>(records, ids, rg, n, vt, n_contrib, counts); break;
    default: return PGB_ERR_INVALID;
  }
  return launch_status();
}

// Batch sizes compiled for the forward (backward = 0) or the backward (1).
int pgb_blend_batches(int backward, int32_t* out) {
  static const int32_t f[] = {64, 128, kFwdFlat + 64, kFwdFlat + 128},
                       b[] = {64, 128, 256, kBwdPx4 + 32, kBwdPx4 + 64, kBwdPx4 + 128,
                              kBwdV2 + 64, kBwdV2 + 512 + 32, kBwdV2 + 1024 + 32,
                              kBwdV2 + kBwdFlat + 32, kBwdV2 + kBwdFlat + 64,
                              kBwdV2 + kBwdFlat + 1024 + 32, kBwdV2 + kBwdFlat + 1024 + 64,
                              kBwdSolo + 32, kBwdSolo + 64, kBwdSolo + 1024 + 32,
                              kBwdSolo + 2048 + 32, kBwdTile + 32};
  const int32_t* src = backward ? b : f;
  const int cnt = backward ? 18 : 4;
  if (out)
    for (int i = 0; i < cnt; ++i) out[i] = src[i];
  return cnt;
}

}  // extern "C"
