// sort_gaussian: tile binning and depth ordering of the splats.
//
// Contract (pointrix/model/renderer/msplat.py:133-135): for every Gaussian
// with radius > 0, one entry per touched 16x16 tile; entries ordered as a
// stable sort of the 64-bit key (tile_id << 32) | float_bits(depth) over
// entries emitted in Gaussian-id order, i.e. by tile, then depth, then id;
// tile_range[t] = [start, end) of tile t's run.
//
// GB300 design.  Sorting K 64-bit keys with 8-bit digits would take 6 LSD
// passes over 12-byte (key, value) pairs.  Instead:
//   1. sort_prepare: one pass over the N Gaussians builds 32-bit depth keys
//      (0xFFFFFFFF for culled ones) and all four digit histograms at once,
//      and sums tiles_touched into K;
//   2. four onesweep passes sort the N Gaussians by depth (stable, so equal
//      depths stay in id order);
//   3. scan_rect: a single-pass decoupled-look-back scan of tiles_touched in
//      depth order gives each Gaussian its output offset and tile rectangle;
//      emit then writes the (tile id, Gaussian id) pairs chunk by chunk of
//      the output (load-balanced however unevenly the tiles are spread over
//      Gaussians) and accumulates the tile digit histograms;
//   4. ceil(log2(T)/8) stable onesweep passes (one for T <= 256, two up to
//      65,536 tiles) sort the pairs by tile id;
//   5. a range pass marks each tile's [start, end).
// A stable sort by tile of a depth-ordered sequence is exactly the order of
// the 64-bit key sort, with K * 16 bytes of traffic per tile pass instead of
// K * 24 per 64-bit pass.
//
// Onesweep pass: each CTA takes the next 4096-key partition from an atomic
// counter, ranks its keys stably (warp match_any + per-warp histograms),
// publishes per-digit counts, resolves its global per-digit offset by
// decoupled look-back over earlier partitions, stages the keys in shared
// memory in digit order and writes them out in runs.  A CTA only waits on
// partitions handed out before its own, which are resident or done, and
// every wait is bounded: past the limit the CTA records PGB_ERR_TIMEOUT in
// the info word and carries on, so a fault can never hang the GPU.
#include "pgb_common.cuh"

namespace pgb {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kPartKeys = kSortThreads * kSortItems;  // 4096
constexpr int kScanItems = 8;
constexpr int kScanPart = kSortThreads * kScanItems;  // 2048
constexpr int kDepthPasses = 4;
constexpr int kMaxTilePasses = 3;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1;
constexpr uint32_t kSpinLimit = 1u << 20;

__device__ inline void set_error(int64_t* info, int code) {
  atomicCAS(reinterpret_cast<unsigned long long*>(info + 1), 0ull, (unsigned long long)code);
}

__device__ inline uint32_t ld_volatile(const uint32_t* p) {
  return *reinterpret_cast<const volatile uint32_t*>(p);
}
__device__ inline void st_volatile(uint32_t* p, uint32_t v) {
  *reinterpret_cast<volatile uint32_t*>(p) = v;
}

__device__ inline uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Exclusive scan over the NT threads of a CTA; `total` receives the sum.
template <int NT = kSortThreads>
__device__ inline uint32_t block_excl_scan(uint32_t v, uint32_t& total, uint32_t* warp_tot) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < NW ? warp_tot[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < NW) warp_tot[lane] = w;
  }
  __syncthreads();
  const uint32_t prefix = warp > 0 ? warp_tot[warp - 1] : 0u;
  total = warp_tot[NW - 1];
  __syncthreads();
  return prefix + x - v;
}

// Sum of the counts published by partitions [0, part) for one digit (or the
// scan's single value), walking back until an inclusive prefix is found.
// The status words of the next kWindow predecessors are loaded together (a
// walk over partitions still in flight would otherwise be a chain of
// dependent L2 round trips) and consumed in order up to the first one not
// yet published.
constexpr int kWindow = 8;

__device__ inline uint32_t look_back(const uint32_t* status, int part, int stride, int64_t* info) {
  uint32_t excl = 0, spins = 0;
  int p = part - 1;
  while (p >= 0) {
    uint32_t w[kWindow];
#pragma unroll
    for (int k = 0; k < kWindow; ++k)
      w[k] = p - k >= 0 ? ld_volatile(status + (size_t)(p - k) * stride) : kFlagInc;
    int k = 0;
#pragma unroll
    for (; k < kWindow; ++k) {
      const uint32_t flag = w[k] & ~kValMask;
      if (flag == 0) break;
      excl += w[k] & kValMask;
      if (flag == kFlagInc) return excl;
    }
    p -= k;
    if (k == 0) {
      if (++spins > kSpinLimit) {
        set_error(info, PGB_ERR_TIMEOUT);
        break;
      }
      __nanosleep(32);
    }
  }
  return excl;
}

// ---------------------------------------------------------------------------
// 1. depth keys, all four digit histograms, K
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSortThreads) sort_prepare_kernel(
    const float* __restrict__ depth, const int32_t* __restrict__ radius,
    const int32_t* __restrict__ tiles, int64_t n, uint32_t* __restrict__ keys,
    uint32_t* __restrict__ vals, uint32_t* __restrict__ hist, int64_t* __restrict__ info) {
  __shared__ uint32_t h[kDepthPasses][256];
  for (int i = threadIdx.x; i < kDepthPasses * 256; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  unsigned long long ksum = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const bool vis = radius[i] > 0;
    const uint32_t key = vis ? __float_as_uint(depth[i]) : 0xFFFFFFFFu;
    if (vis) ksum += (unsigned long long)max(tiles[i], 0);
    keys[i] = key;
    vals[i] = (uint32_t)i;
#pragma unroll
    for (int p = 0; p < kDepthPasses; ++p) atomicAdd(&h[p][(key >> (8 * p)) & 0xFF], 1u);
  }
  // K: warp sum then one atomic per warp
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ksum += __shfl_xor_sync(0xffffffffu, ksum, o);
  if ((threadIdx.x & 31) == 0 && ksum)
    atomicAdd(reinterpret_cast<unsigned long long*>(info), ksum);
  __syncthreads();
  for (int i = threadIdx.x; i < kDepthPasses * 256; i += blockDim.x) {
    const uint32_t c = (&h[0][0])[i];
    if (c) atomicAdd(hist + i, c);
  }
}

// ---------------------------------------------------------------------------
// 2/4. one stable LSD onesweep pass over 8 bits starting at `shift`
//
// 512 threads x 8 keys = one 4096-key partition per CTA; the first 256
// threads also act as the 256 digits for the cross-warp prefix, the status
// publication and the look-back.
// ---------------------------------------------------------------------------
constexpr int kOsThreads = 512;
constexpr int kOsItems = kPartKeys / kOsThreads;  // 8
constexpr int kOsWarps = kOsThreads / 32;
constexpr size_t kOsSmem = (size_t)kOsWarps * 256 * 4 + 2 * (size_t)kPartKeys * 4;

__global__ void __launch_bounds__(kOsThreads) onesweep_kernel(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int64_t n, int shift,
    const uint32_t* __restrict__ pass_hist, uint32_t* __restrict__ status,
    uint32_t* __restrict__ part_counter, int64_t* __restrict__ info) {
  extern __shared__ __align__(16) uint32_t os_smem[];
  uint32_t (*warp_hist)[256] = reinterpret_cast<uint32_t (*)[256]>(os_smem);
  uint32_t* s_keys = os_smem + kOsWarps * 256;
  uint32_t* s_vals = s_keys + kPartKeys;
  __shared__ uint32_t s_block_excl[256];
  __shared__ uint32_t s_global_base[256];
  __shared__ uint32_t s_warp_tot[kOsWarps];
  __shared__ uint32_t s_part;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_part = atomicAdd(part_counter, 1u);
  for (int i = lane; i < 256; i += 32) warp_hist[warp][i] = 0;
  __syncthreads();
  const int part = (int)s_part;
  const int64_t base = (int64_t)part * kPartKeys + (int64_t)warp * (32 * kOsItems);

  uint32_t key[kOsItems], val[kOsItems], rank[kOsItems];
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int it = 0; it < kOsItems; ++it) {
    const int64_t e = base + it * 32 + lane;
    const bool valid = e < n;
    key[it] = valid ? keys_in[e] : 0u;
    val[it] = valid ? vals_in[e] : 0u;
  }
#pragma unroll
  for (int it = 0; it < kOsItems; ++it) {
    const bool valid = base + it * 32 + lane < n;
    const uint32_t d = (key[it] >> shift) & 0xFFu;  // 0 for invalid lanes
    const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 256u);
    const uint32_t old = warp_hist[warp][d];
    rank[it] = old + __popc(peers & lt);
    __syncwarp();
    if (valid && (peers & lt) == 0) warp_hist[warp][d] = old + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Per digit (threads 0..255): exclusive offsets across warps, partition
  // count, status publication, look-back.
  const int t = threadIdx.x;
  const bool is_digit = t < 256;
  uint32_t count = 0;
  if (is_digit) {
#pragma unroll
    for (int w = 0; w < kOsWarps; ++w) {
      const uint32_t c = warp_hist[w][t];
      warp_hist[w][t] = count;
      count += c;
    }
    uint32_t* my_status = status + (size_t)part * 256 + t;
    st_volatile(my_status, (part == 0 ? kFlagInc : kFlagAgg) | count);
  }
  uint32_t unused;
  const uint32_t digit_start =
      block_excl_scan<kOsThreads>(is_digit ? pass_hist[t] : 0u, unused, s_warp_tot);
  if (is_digit) {
    uint32_t prior = 0;
    if (part > 0) {
      prior = look_back(status + t, part, 256, info);
      st_volatile(status + (size_t)part * 256 + t, kFlagInc | ((prior + count) & kValMask));
    }
    s_global_base[t] = digit_start + prior;
  }
  uint32_t local_total;
  const uint32_t bex = block_excl_scan<kOsThreads>(is_digit ? count : 0u, local_total, s_warp_tot);
  if (is_digit) s_block_excl[t] = bex;
  __syncthreads();

  // Stage in digit order.
#pragma unroll
  for (int it = 0; it < kOsItems; ++it) {
    const int64_t e = base + it * 32 + lane;
    if (e < n) {
      const uint32_t d = (key[it] >> shift) & 0xFFu;
      const uint32_t lp = s_block_excl[d] + warp_hist[warp][d] + rank[it];
      s_keys[lp] = key[it];
      s_vals[lp] = val[it];
    }
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < local_total; j += kOsThreads) {
    const uint32_t k = s_keys[j];
    const uint32_t d = (k >> shift) & 0xFFu;
    const uint32_t dst = s_global_base[d] + (j - s_block_excl[d]);
    if ((int64_t)dst >= n) {  // only if the histogram disagrees with the keys
      set_error(info, PGB_ERR_OVERFLOW);
      continue;
    }
    keys_out[dst] = k;
    vals_out[dst] = s_vals[j];
  }
}

static int onesweep_attr() {
  return cudaFuncSetAttribute(onesweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kOsSmem) == cudaSuccess
             ? PGB_OK
             : PGB_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// 3a. scan of tiles_touched in depth order
//
// For depth-sorted position i (Gaussian g = order[i]) writes its output
// offset offs[i], its tile rectangle rect[i] = (x0 | y0 << 16, w | h << 16),
// and, for every emission chunk boundary b * kEmitChunk that falls inside
// [offs[i], offs[i] + count), chunk_first[b] = i.
// ---------------------------------------------------------------------------
constexpr int kEmitChunk = 1024;
constexpr int kEmitThreads = 256;

__global__ void __launch_bounds__(kSortThreads) scan_rect_kernel(
    const uint32_t* __restrict__ order, int64_t n, const int32_t* __restrict__ tiles,
    const int32_t* __restrict__ radius, const float* __restrict__ uv, ViewTable vt, int64_t K,
    uint32_t* __restrict__ status, uint32_t* __restrict__ part_counter,
    uint32_t* __restrict__ offs, uint2* __restrict__ rect, uint32_t* __restrict__ chunk_first,
    int64_t* __restrict__ info) {
  __shared__ uint32_t s_warp_tot[kSortThreads / 32];
  __shared__ uint32_t s_part, s_prior;
  if (threadIdx.x == 0) s_part = atomicAdd(part_counter, 1u);
  __syncthreads();
  const int part = (int)s_part;
  const int64_t base = (int64_t)part * kScanPart + (int64_t)threadIdx.x * kScanItems;

  uint32_t cnt[kScanItems];
  uint2 rc[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int it = 0; it < kScanItems; ++it) {
    const int64_t e = base + it;
    cnt[it] = 0;
    rc[it] = make_uint2(0u, 0u);
    if (e < n) {
      const uint32_t g = order[e];
      const int r = radius[g];
      if (r > 0) {
        cnt[it] = (uint32_t)max(tiles[g], 0);
        const float2 p = reinterpret_cast<const float2*>(uv)[g];
        int x0, x1, y0, y1;
        int gx, gy;
        uint32_t tile_base;
        element_view(vt, g, gx, gy, tile_base);
        tile_rect(p.x, p.y, (float)r, gx, gy, x0, x1, y0, y1);
        if ((int64_t)(x1 - x0) * (y1 - y0) != (int64_t)cnt[it]) set_error(info, PGB_ERR_MISMATCH);
        rc[it] = make_uint2((uint32_t)x0 | ((uint32_t)y0 << 16),
                            (uint32_t)(x1 - x0) | ((uint32_t)(y1 - y0) << 16));
      }
    }
    sum += cnt[it];
  }
  uint32_t total;
  const uint32_t excl = block_excl_scan(sum, total, s_warp_tot);
  if (threadIdx.x == 0) {
    uint32_t* my = status + part;
    if (part == 0) {
      st_volatile(my, kFlagInc | (total & kValMask));
      s_prior = 0;
    } else {
      st_volatile(my, kFlagAgg | (total & kValMask));
      const uint32_t prior = look_back(status, part, 1, info);
      st_volatile(my, kFlagInc | ((prior + total) & kValMask));
      s_prior = prior;
    }
  }
  __syncthreads();
  int64_t off = (int64_t)s_prior + excl;
#pragma unroll
  for (int it = 0; it < kScanItems; ++it) {
    const int64_t e = base + it;
    if (e < n) {
      const int64_t end = off + cnt[it];
      if (end > K) {
        set_error(info, PGB_ERR_OVERFLOW);
      } else {
        offs[e] = (uint32_t)off;
        rect[e] = rc[it];
        // chunk boundaries owned by this Gaussian, and the owner of the
        // last entry (stored after the last chunk's)
        for (int64_t b = (off + kEmitChunk - 1) / kEmitChunk; b * kEmitChunk < end; ++b)
          chunk_first[b] = (uint32_t)e;
        if (off < K && K <= end) chunk_first[(K + kEmitChunk - 1) / kEmitChunk] = (uint32_t)e;
      }
      off = end;
    }
  }
}

// ---------------------------------------------------------------------------
// 3b. emission of (tile id, Gaussian id) pairs over output chunks
//
// CTA b writes entries [b*kEmitChunk, min(K, (b+1)*kEmitChunk)): it stages
// the offsets, rectangles and ids of the Gaussians that own them in shared
// memory; each thread takes 8 consecutive entries, finds the owner of the
// first by binary search and walks forward; the pairs are staged in shared
// memory and written with 16-byte stores.  Every CTA does the same amount of
// work however unevenly the tiles are spread over Gaussians.
// ---------------------------------------------------------------------------
constexpr int kEmitPer = kEmitChunk / kEmitThreads;  // 4

__global__ void __launch_bounds__(kEmitThreads) emit_kernel(
    const uint32_t* __restrict__ order, const uint32_t* __restrict__ offs,
    const uint2* __restrict__ rect, const uint32_t* __restrict__ chunk_first, int64_t n_sorted,
    int64_t K, ViewTable vt, int tile_passes, uint32_t* __restrict__ tkeys, uint32_t* __restrict__ tvals,
    uint32_t* __restrict__ tile_hist, int64_t* __restrict__ info) {
  constexpr int CAP = kEmitChunk + 1;
  __shared__ uint32_t s_off[CAP];
  __shared__ uint2 s_rect[CAP];
  __shared__ uint32_t s_g[CAP];
  __shared__ __align__(16) uint32_t s_key[kEmitChunk];
  __shared__ __align__(16) uint32_t s_val[kEmitChunk];
  __shared__ uint32_t s_hist[kMaxTilePasses][256];
  const int64_t e0 = (int64_t)blockIdx.x * kEmitChunk;
  const int64_t e1 = min(K, e0 + kEmitChunk);
  // owners of this chunk's first entry and of the next chunk's first entry
  // (for the last chunk: of entry K - 1)
  const int64_t i0 = chunk_first[blockIdx.x];
  const int64_t i1 = chunk_first[blockIdx.x + 1];
  const int64_t m = i1 - i0 + 1;
  for (int i = threadIdx.x; i < kMaxTilePasses * 256; i += kEmitThreads) (&s_hist[0][0])[i] = 0;
  const bool ok_range = i0 <= i1 && i1 < n_sorted;
  if (!ok_range && threadIdx.x == 0) set_error(info, PGB_ERR_OVERFLOW);
  const bool staged = ok_range && m <= CAP;
  if (staged) {
    for (int64_t i = threadIdx.x; i < m; i += kEmitThreads) {
      s_off[i] = offs[i0 + i];
      s_rect[i] = rect[i0 + i];
      s_g[i] = order[i0 + i];
    }
  }
  __syncthreads();
  const int64_t ebeg = e0 + (int64_t)threadIdx.x * kEmitPer;
  if (ok_range && ebeg < e1) {
    auto off_at = [&](int64_t p) -> int64_t { return staged ? s_off[p] : offs[i0 + p]; };
    // owner of ebeg: the last position p in [0, i1 - i0] with offs <= ebeg
    int64_t lo = 0, hi = i1 - i0;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (off_at(mid) <= ebeg) lo = mid; else hi = mid - 1;
    }
    int64_t own = lo;
    int64_t next_off = own < i1 - i0 ? off_at(own + 1) : INT64_MAX;
    for (int j = 0; j < kEmitPer; ++j) {
      const int64_t e = ebeg + j;
      if (e >= e1) break;
      while (e >= next_off) {  // walk to the owner of e (skips zero-count Gaussians)
        ++own;
        next_off = own < i1 - i0 ? off_at(own + 1) : INT64_MAX;
      }
      const uint32_t o = (uint32_t)off_at(own);
      const uint2 rc = staged ? s_rect[own] : rect[i0 + own];
      const uint32_t g = staged ? s_g[own] : order[i0 + own];
      const uint32_t jj = (uint32_t)(e - o);
      const uint32_t w = rc.y & 0xFFFFu, h = rc.y >> 16;
      int gx, gy;
      uint32_t tile_base;
      element_view(vt, g, gx, gy, tile_base);
      uint32_t tid = tile_base;  // a tiles_touched/rectangle mismatch leaves the view's first tile (reported)
      if (w > 0 && jj < w * h)
        tid = tile_base + ((rc.x >> 16) + jj / w) * (uint32_t)gx + (rc.x & 0xFFFFu) + jj % w;
      s_key[threadIdx.x * kEmitPer + j] = tid;
      s_val[threadIdx.x * kEmitPer + j] = g;
    }
  }
  __syncthreads();
  // coalesced write-out and tile digit histograms (digits of consecutive
  // keys read by consecutive lanes)
  const int cnt = ok_range ? (int)(e1 - e0) : 0;
  if (cnt == kEmitChunk) {
    for (int q = threadIdx.x; q < kEmitChunk / 4; q += kEmitThreads) {
      reinterpret_cast<uint4*>(tkeys + e0)[q] = reinterpret_cast<const uint4*>(s_key)[q];
      reinterpret_cast<uint4*>(tvals + e0)[q] = reinterpret_cast<const uint4*>(s_val)[q];
    }
  } else {
    for (int q = threadIdx.x; q < cnt; q += kEmitThreads) {
      tkeys[e0 + q] = s_key[q];
      tvals[e0 + q] = s_val[q];
    }
  }
  const uint32_t lane = threadIdx.x & 31;
  for (int q0 = 0; q0 < kEmitChunk; q0 += kEmitThreads) {
    const int q = q0 + threadIdx.x;
    const bool valid = q < cnt;
    const uint32_t tid = valid ? s_key[q] : 0u;
    for (int p = 0; p < tile_passes; ++p) {
      const uint32_t d = (tid >> (8 * p)) & 0xFFu;
      const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 256u + lane);
      if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&s_hist[p][d], (uint32_t)__popc(peers));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < tile_passes * 256; i += kEmitThreads) {
    const uint32_t v = (&s_hist[0][0])[i];
    if (v) atomicAdd(tile_hist + i, v);
  }
}

// ---------------------------------------------------------------------------
// 5. tile ranges from the sorted tile keys
// ---------------------------------------------------------------------------
__global__ void tile_range_kernel(const uint32_t* __restrict__ keys, int64_t K, uint32_t T,
                                  int2* __restrict__ range, int64_t* __restrict__ info) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < K;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t k = keys[i];
    if (k >= T) {
      set_error(info, PGB_ERR_OVERFLOW);
      continue;
    }
    if (i == 0 || keys[i - 1] != k) range[k].x = (int)i;
    if (i == K - 1 || keys[i + 1] != k) range[k].y = (int)(i + 1);
  }
}

// ---------------------------------------------------------------------------
// scratch layout
// ---------------------------------------------------------------------------
inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct ScratchN {
  size_t counters, depth_hist, tile_hist, depth_status, scan_status, zero_bytes;
  size_t dk0, dv0, dk1, dv1, offs, rect, total;
  int parts, scan_parts;
};

inline ScratchN layout_n(int64_t n) {
  ScratchN L;
  L.parts = (int)((n + kPartKeys - 1) / kPartKeys);
  L.scan_parts = (int)((n + kScanPart - 1) / kScanPart);
  size_t o = 0;
  L.counters = o; o += align256(16 * sizeof(uint32_t));
  L.depth_hist = o; o += align256(kDepthPasses * 256 * sizeof(uint32_t));
  L.tile_hist = o; o += align256(kMaxTilePasses * 256 * sizeof(uint32_t));
  L.depth_status = o; o += align256((size_t)kDepthPasses * L.parts * 256 * sizeof(uint32_t));
  L.scan_status = o; o += align256((size_t)L.scan_parts * sizeof(uint32_t));
  L.zero_bytes = o;
  const size_t nb = align256((size_t)n * sizeof(uint32_t));
  L.dk0 = o; o += nb;
  L.dv0 = o; o += nb;
  L.dk1 = o; o += nb;
  L.dv1 = o; o += nb;
  L.offs = o; o += nb;
  L.rect = o; o += align256((size_t)n * sizeof(uint2));
  L.total = o;
  return L;
}

struct ScratchK {
  size_t tk0, tv0, tk1, tv1, status, chunk_first, total;
  int parts;
  int64_t chunks;
};

inline ScratchK layout_k(int64_t k) {
  ScratchK L;
  L.parts = (int)((k + kPartKeys - 1) / kPartKeys);
  size_t o = 0;
  const size_t kb = align256((size_t)k * sizeof(uint32_t));
  L.tk0 = o; o += kb;
  L.tv0 = o; o += kb;
  L.tk1 = o; o += kb;
  L.tv1 = o; o += kb;
  L.status = o; o += align256((size_t)kMaxTilePasses * L.parts * 256 * sizeof(uint32_t));
  L.chunks = (k + kEmitChunk - 1) / kEmitChunk;
  L.chunk_first = o; o += align256((size_t)(L.chunks + 2) * sizeof(uint32_t));
  L.total = o;
  return L;
}

inline int tile_passes_for(uint32_t T) {
  int bits = 0;
  while (bits < 32 && (T - 1) >> bits) ++bits;
  return bits <= 8 ? 1 : (bits + 7) / 8;
}

template <typename P>
inline P* at(void* base, size_t off) {
  return reinterpret_cast<P*>(static_cast<char*>(base) + off);
}

}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_sort_scratch_bytes(int64_t n, int64_t k, int width, int height, size_t* bytes_n,
                           size_t* bytes_k) {
  if (n < 0 || k < 0 || width <= 0 || height <= 0) return PGB_ERR_INVALID;
  if (bytes_n) *bytes_n = layout_n(n).total;
  if (bytes_k) *bytes_k = layout_k(k).total;
  return PGB_OK;
}

int pgb_sort_gaussian_begin(const float* depth, const int32_t* radius,
                            const int32_t* tiles_touched, int64_t n, int width, int height,
                            void* scratch_n, size_t bytes_n, int64_t* info, void* stream) {
  if (n < 0 || width <= 0 || height <= 0 || !info) return PGB_ERR_INVALID;
  if (n >= (int64_t)kValMask) return PGB_ERR_OVERFLOW;
  const ScratchN L = layout_n(n);
  if (!scratch_n || bytes_n < L.total) return PGB_ERR_INVALID;
  const uint32_t T = (uint32_t)grid_x(width) * (uint32_t)grid_y(height);
  if (T > (1u << (8 * kMaxTilePasses))) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(info, 0, 2 * sizeof(int64_t), s) != cudaSuccess) return PGB_ERR_CUDA;
  if (cudaMemsetAsync(scratch_n, 0, L.zero_bytes, s) != cudaSuccess) return PGB_ERR_CUDA;
  if (n == 0) return PGB_OK;
  if (onesweep_attr() != PGB_OK) return PGB_ERR_CUDA;
  uint32_t* counters = at<uint32_t>(scratch_n, L.counters);
  uint32_t* hist = at<uint32_t>(scratch_n, L.depth_hist);
  uint32_t* status = at<uint32_t>(scratch_n, L.depth_status);
  uint32_t* k0 = at<uint32_t>(scratch_n, L.dk0);
  uint32_t* v0 = at<uint32_t>(scratch_n, L.dv0);
  uint32_t* k1 = at<uint32_t>(scratch_n, L.dk1);
  uint32_t* v1 = at<uint32_t>(scratch_n, L.dv1);
  sort_prepare_kernel<<<stream_grid(n, kSortThreads, 4), kSortThreads, 0, s>>>(
      depth, radius, tiles_touched, n, k0, v0, hist, info);
  for (int p = 0; p < kDepthPasses; ++p) {
    const uint32_t* ki = (p & 1) ? k1 : k0;
    const uint32_t* vi = (p & 1) ? v1 : v0;
    uint32_t* ko = (p & 1) ? k0 : k1;
    uint32_t* vo = (p & 1) ? v0 : v1;
    onesweep_kernel<<<L.parts, kOsThreads, kOsSmem, s>>>(ki, vi, ko, vo, n, 8 * p, hist + 256 * p,
                                                         status + (size_t)p * L.parts * 256,
                                                         counters + p, info);
  }
  // four passes: the depth order ends in (k0, v0)
  return launch_status();
}

}  // extern "C"

// Phase two for one image or a batch of views (vt), over T global tiles.
static int sort_finish_impl(const float* uv, const int32_t* radius, const int32_t* tiles_touched,
                            int64_t n, const ViewTable& vt, uint32_t T, int64_t k, void* scratch_n,
                            size_t bytes_n, void* scratch_k, size_t bytes_k, int64_t* info,
                            int32_t* ids_out, int32_t* tile_range_out, void* stream) {
  if (n < 0 || k < 0 || !info || !tile_range_out) return PGB_ERR_INVALID;
  if (k >= (int64_t)kValMask) return PGB_ERR_OVERFLOW;
  const ScratchN LN = layout_n(n);
  const ScratchK LK = layout_k(k);
  if (!scratch_n || bytes_n < LN.total) return PGB_ERR_INVALID;
  if (k > 0 && (!scratch_k || bytes_k < LK.total || !ids_out)) return PGB_ERR_INVALID;
  if (T == 0 || T > (1u << (8 * kMaxTilePasses))) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(tile_range_out, 0, (size_t)T * 2 * sizeof(int32_t), s) != cudaSuccess)
    return PGB_ERR_CUDA;
  if (k == 0 || n == 0) return PGB_OK;
  const int passes = tile_passes_for(T);
  if (cudaMemsetAsync(at<char>(scratch_k, LK.status), 0,
                      (size_t)kMaxTilePasses * LK.parts * 256 * sizeof(uint32_t), s) != cudaSuccess)
    return PGB_ERR_CUDA;
  if (onesweep_attr() != PGB_OK) return PGB_ERR_CUDA;
  uint32_t* counters = at<uint32_t>(scratch_n, LN.counters);
  uint32_t* thist = at<uint32_t>(scratch_n, LN.tile_hist);
  const uint32_t* order = at<uint32_t>(scratch_n, LN.dv0);
  uint32_t* bufk[2] = {at<uint32_t>(scratch_k, LK.tk0), at<uint32_t>(scratch_k, LK.tk1)};
  uint32_t* bufv[2] = {at<uint32_t>(scratch_k, LK.tv0), at<uint32_t>(scratch_k, LK.tv1)};
  uint32_t* status = at<uint32_t>(scratch_k, LK.status);
  uint32_t* offs = at<uint32_t>(scratch_n, LN.offs);
  uint2* rect = at<uint2>(scratch_n, LN.rect);
  uint32_t* chunk_first = at<uint32_t>(scratch_k, LK.chunk_first);
  scan_rect_kernel<<<LN.scan_parts, kSortThreads, 0, s>>>(
      order, n, tiles_touched, radius, uv, vt, k, at<uint32_t>(scratch_n, LN.scan_status),
      counters + 4, offs, rect, chunk_first, info);
  emit_kernel<<<(unsigned)LK.chunks, kEmitThreads, 0, s>>>(order, offs, rect, chunk_first, n, k, vt,
                                                           passes, bufk[0], bufv[0], thist, info);
  int cur = 0;
  for (int p = 0; p < passes; ++p) {
    const bool last = p == passes - 1;
    uint32_t* vo = last ? reinterpret_cast<uint32_t*>(ids_out) : bufv[cur ^ 1];
    onesweep_kernel<<<LK.parts, kOsThreads, kOsSmem, s>>>(
        bufk[cur], bufv[cur], bufk[cur ^ 1], vo, k, 8 * p, thist + 256 * p,
        status + (size_t)p * LK.parts * 256, counters + 5 + p, info);
    cur ^= 1;
  }
  tile_range_kernel<<<stream_grid(k), kStreamThreads, 0, s>>>(
      bufk[cur], k, T, reinterpret_cast<int2*>(tile_range_out), info);
  return launch_status();
}

extern "C" {

int pgb_sort_gaussian_finish(const float* uv, const int32_t* radius, const int32_t* tiles_touched,
                             int64_t n, int width, int height, int64_t k, void* scratch_n,
                             size_t bytes_n, void* scratch_k, size_t bytes_k, int64_t* info,
                             int32_t* ids_out, int32_t* tile_range_out, void* stream) {
  if (width <= 0 || height <= 0 || grid_x(width) > 65535 || grid_y(height) > 65535)
    return PGB_ERR_INVALID;
  const uint32_t T = (uint32_t)grid_x(width) * (uint32_t)grid_y(height);
  return sort_finish_impl(uv, radius, tiles_touched, n, single_view(width, height), T, k, scratch_n,
                          bytes_n, scratch_k, bytes_k, info, ids_out, tile_range_out, stream);
}

int pgb_sort_gaussian_finish_views(const float* uv, const int32_t* radius,
                                   const int32_t* tiles_touched, int64_t n_per_view,
                                   const int32_t* sizes, int nviews, int64_t k, void* scratch_n,
                                   size_t bytes_n, void* scratch_k, size_t bytes_k, int64_t* info,
                                   int32_t* ids_out, int32_t* tile_range_out, void* stream) {
  ViewTable vt;
  uint32_t T = 0;
  int64_t pixels = 0;
  if (!make_views(sizes, nviews, n_per_view, vt, T, pixels)) return PGB_ERR_INVALID;
  return sort_finish_impl(uv, radius, tiles_touched, n_per_view * nviews, vt, T, k, scratch_n,
                          bytes_n, scratch_k, bytes_k, info, ids_out, tile_range_out, stream);
}

}  // extern "C"
