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
//      depths stay in id order); a batch of views adds a fifth, by view, so
//      the order is view-major;
//   3. rect: each Gaussian's tile rectangle and entry count (coalesced, in
//      id order), and the tile digit histograms of all its entries (one
//      update per rectangle row); scan_rect: a single-pass decoupled-look-back
//      scan of the counts in depth order gives each Gaussian its output
//      offset (its emission record);
//   4. one stable onesweep pass for T <= 256 tiles, two 8-bit passes up to
//      65,536 tiles, two 9-bit passes up to 2^18, else three, sort the
//      (tile id, Gaussian id) pairs by tile id (a batch of views sorts
//      view-local tile ids with the plan of its largest view).  The first
//      pass generates its partition's pairs from the emission records
//      (load-balanced: every partition is 6144 pairs however unevenly the
//      tiles are spread over Gaussians): the partition's owners are staged
//      in shared memory, each marks the rectangle rows it starts inside the
//      partition, and a running maximum over the marks gives every entry its
//      owner and row.  The
//      depth-ordered pair sequence is never written out; the last pass
//      writes only the ids and records each tile's [start, end) as it goes;
//   5. tiles that no entry reached get [0, 0).
// A stable sort by tile of a depth-ordered sequence is exactly the order of
// the 64-bit key sort, with K * 16 bytes of traffic per tile pass instead of
// K * 24 per 64-bit pass.
//
// Onesweep pass: each CTA takes the next 6144-key partition from an atomic
// counter, ranks its keys stably (warp ballots + per-warp histograms),
// publishes per-digit counts, resolves its global per-digit offset by
// decoupled look-back over earlier partitions, stages the keys in shared
// memory in digit order and writes them out in runs.  A CTA only waits on
// partitions handed out before its own, which are resident or done, and
// every wait is bounded: past the limit the CTA records PGB_ERR_TIMEOUT in
// the info word and carries on, so a fault can never hang the GPU.
//
// Phase two can also run without the host knowing K (capacity mode): the
// K-sized grids cover a capacity, and every kernel reads K from the info
// word that phase one left on the device.
#include <algorithm>

#include "pgb_common.cuh"

namespace pgb {

constexpr int kSortThreads = 256;
constexpr int kPartKeys = 6144;  // keys per onesweep partition (tile passes)
// The depth passes sort N keys.  When 6,144-key partitions would not fill
// one wave of two CTAs per SM (N below ~1.9M; 163 partitions at the 1M
// training workload, half the CTA slots empty and each pass one long
// partition's latency), they use partitions of 512 x 7 keys (280 at 1M);
// larger N keep the large partitions (fewer look-backs: at 48M keys the
// small ones cost 14 % more).
constexpr int kDepthIT = 7;
constexpr int kDepthPartKeys = 512 * kDepthIT;
inline bool small_depth_parts(int64_t n) { return n <= (int64_t)2 * kNumSMs * kPartKeys; }
inline int depth_part_keys(int64_t n) { return small_depth_parts(n) ? kDepthPartKeys : kPartKeys; }
constexpr int kScanItems = 8;
constexpr int kScanPart = kSortThreads * kScanItems;  // 2048
// Chunk of the tile-entry sequence whose first owner the scan records; a
// onesweep partition is kPartKeys / kEmitChunk chunks.
constexpr int kEmitChunk = 1024;
constexpr int kDepthPasses = 4;
// A batch of views adds one pass over the view index after the depth
// passes, so that the emission is view-major (depth order within a view).
constexpr int kViewPass = kDepthPasses;
// counter word where phase one records its view count (0: one image)
constexpr int kViewsMark = 12;
constexpr int kMaxTilePasses = 3;
constexpr int kTileHistWords = 1024;  // 3 passes x 256 digits or 2 x 512
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
    uint32_t* __restrict__ vals, uint32_t* __restrict__ hist, int nviews, int64_t n_per_view,
    uint32_t* __restrict__ views_mark, int64_t* __restrict__ info) {
  __shared__ uint32_t h[kDepthPasses][256];
  // phase two checks that phase one sorted the same way (one image or views)
  if (blockIdx.x == 0 && threadIdx.x == 0) *views_mark = (uint32_t)nviews;
  // the view pass's histogram: n_per_view elements in each view
  if (blockIdx.x == 0)
    for (int v = threadIdx.x; v < nviews; v += blockDim.x)
      hist[kViewPass * 256 + v] = (uint32_t)n_per_view;
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
// 2/4. one stable LSD onesweep pass over RB bits starting at `shift`
//
// A partition is NT threads x IT keys (6144: 512 x 12 for 8- and 9-bit
// digits, 32 warps per SM at two CTAs; 384 x 16 measured 1 % slower).
// Keys are ranked in registers (warp-striped: key it of a lane is element
// it * 32 + lane of its warp's slice, so warp order = element order and
// ranks are stable); the partition's values travel global -> shared by
// cp.async meanwhile, so a thread holds only its keys and ranks.  Within a
// warp equal digits are found by OR-ing each lane's bit into a per-warp
// digit mask in shared memory (8-bit digits) or with RB ballots, one per
// digit bit (9-bit digits, whose masks would not fit beside the staging).
// The first R threads also act as the R digits for the cross-warp prefix,
// the status publication and the look-back, which runs while the other
// warps stage the keys in digit order.
//
// `n_dev` (optional) holds the element count on the device -- the tile
// passes of a capacity-sized sort, whose grid covers the capacity `cap` --
// and partitions past that count return at once.  Without KEYS_OUT the keys
// are not written (the last pass).  With RANGES the pass is the last tile
// pass and also records each tile's [start, end): in the output every key
// run is consecutive, so a staged key whose predecessor in shared memory
// differs may start its tile's run (atomicMin of its position) and one whose
// successor differs may end it (atomicMax); the table starts at (INT_MAX, 0)
// and untouched tiles become (0, 0) afterwards.
// ---------------------------------------------------------------------------
template <int RB>
struct OsCfg;
template <>
struct OsCfg<8> {
  static constexpr int NT = 512, IT = 12;
};
template <>
struct OsCfg<9> {
  static constexpr int NT = 512, IT = 12;
};

template <int RB, int ITK = OsCfg<RB>::IT>
struct Os {
  static constexpr int NT = OsCfg<RB>::NT, IT = ITK, NW = NT / 32;
  static constexpr int PART = NT * IT;
  static constexpr int R = 1 << RB;
  // 8-bit digits: equal digits of a warp found by OR-ing lane bits into a
  // per-warp digit mask in shared memory (one atomic and one load per key);
  // 9-bit digits (no room for the masks): RB ballots
  static constexpr bool OR_MATCH = RB == 8;
  static constexpr int HW = (OR_MATCH ? 2 : 1) * NW * R;  // histogram (+ mask) words
  static constexpr size_t SMEM = ((size_t)HW + 3 * (size_t)PART) * sizeof(uint32_t);
  static_assert(ITK != OsCfg<RB>::IT || PART == kPartKeys,
                "one partition size for every digit width of the tile passes");
  static_assert(NT >= R, "one thread per digit");
};

// Exact a / d for a < 2^30 with one 64-bit multiply and shift (Granlund and
// Montgomery's round-up method): s = 32 + ceil(log2 d), m = ceil(2^s / d).
// Then m < 2^34, a * m < 2^64, and m d - 2^s < d keeps the error of
// a m / 2^s below a / 2^32 < 1 / d, so the floor is exact.
struct FastDiv {
  uint64_t m;
  int s;
};

inline FastDiv fast_div(uint32_t d) {
  int L = 0;
  while ((1ull << L) < (uint64_t)d) ++L;
  const int s = 32 + L;
  return FastDiv{((1ull << s) + d - 1) / d, s};
}

__device__ __forceinline__ uint32_t fdiv(uint32_t a, const FastDiv& f) {
  return (uint32_t)(((uint64_t)a * f.m) >> f.s);
}

// What a pass knows of a batch of views (nviews == 0: one image).  Element
// ids are v * n_per_view + g; `vdiv` divides by n_per_view.  key_from_val:
// the keys written are the views of the values (the depth pass before the
// view pass).  With nviews > 0 the tile passes sort local tile ids, and the
// last one records the range of view v's local tile t as global tile
// tile_base[v] + t.
struct PassViews {
  FastDiv vdiv;
  int key_from_val;
  int nviews;
  uint32_t tile_base[kMaxViews];
};

// Element count of a pass: the host value, or the device count when it
// fits the capacity (a count past the capacity is reported by scan_rect and
// makes every pass empty).
__device__ inline int64_t pass_count(const int64_t* n_dev, int64_t cap) {
  if (!n_dev) return cap;
  const int64_t k = *n_dev;
  return (k >= 0 && k <= cap) ? k : 0;
}

// Lanes of the warp whose RB-bit digit equals this lane's (among `valid`
// lanes); digit bits from `live` on are zero in every key of the pass.
template <int RB>
__device__ inline uint32_t match_digit(uint32_t d, bool valid, int live) {
  uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int b = 0; b < RB; ++b) {
    if (b < live) {  // uniform
      const bool bit = (d >> b) & 1u;
      const uint32_t bb = __ballot_sync(0xffffffffu, bit);
      peers &= bit ? bb : ~bb;
    }
  }
  return peers;
}

// q = a / b, r = a % b for b >= 1: a float estimate (exact to +-1 below
// 2^22: the reciprocal and the product each carry one rounding) corrected
// once; larger a takes the integer division.
__device__ inline void divmod_u32(uint32_t a, uint32_t b, uint32_t& q, uint32_t& r) {
  if (a < (1u << 22)) {
    uint32_t q0 = __float2uint_rz(__uint2float_rn(a) * __frcp_rn(__uint2float_rn(b)));
    int r0 = (int)a - (int)(q0 * b);
    if (r0 < 0) {
      --q0;
      r0 += (int)b;
    } else if (r0 >= (int)b) {
      ++q0;
      r0 -= (int)b;
    }
    q = q0;
    r = (uint32_t)r0;
  } else {
    q = a / b;
    r = a - q * b;
  }
}

// The owner records (first tile, w | gx << 16, g, offset) of a partition's
// entries: positions [i0, i1] of the depth order, staged in shared memory
// (STAGED) when they fit, else read from global memory.
template <bool STAGED>
struct OwnerView {
  const uint4* g;
  const uint4* s;
  uint32_t i0;
  __device__ uint4 rec(uint32_t i) const { return STAGED ? s[i - i0] : g[i]; }
  __device__ uint32_t off(uint32_t i) const { return STAGED ? s[i - i0].w : g[i].w; }
};

// Last position in [lo, hi] whose offset is <= e (offset(lo) <= e).
template <bool STAGED>
__device__ inline uint32_t owner_search(const OwnerView<STAGED>& ov, uint32_t lo, uint32_t hi,
                                        uint32_t e) {
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo + 1) >> 1);
    if (ov.off(mid) <= e) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Fallback generation, for a partition with more owners than fit in shared
// memory (Gaussians of one or two tiles each).  Tile entries e0 + lane (e0
// uniform over the warp) of the depth-ordered emission: entry j of Gaussian
// g (owner record offset o) is tile
// first + (j / w) gx + j % w (one row of `count` tiles when w = 0), value g.
// `p` is a position whose offset is <= e0 (on return: the same for
// e0 + 32).  The 32 owner records p .. p + 31 are read one per lane; a
// lane's owner is the last of them starting at or before its entry.  Their
// starts relative to e0, h (non-decreasing in the window index, 0 for the
// records starting at or before e0), are usually distinct past those: then
// the owner of lane L is the number of records with h = 0 less one plus the
// number of starts in [1, L], one OR-reduce and a popcount.  Records of zero entries repeat a start; a window with
// such a repeat takes a five-step shuffle search instead.  An entry past the
// window (only behind zero-entry owners) is searched in [p + 32, i1].
template <bool STAGED>
__device__ inline void gen_entries(const OwnerView<STAGED>& ov, uint32_t i1, uint32_t& p,
                                   uint32_t e0, int lane, uint32_t& key, uint32_t& val) {
  const uint32_t q = p + (uint32_t)lane;
  const uint4 r = q <= i1 ? ov.rec(q) : make_uint4(0u, 0u, 0u, 0xFFFFFFFFu);
  const uint32_t x32 = p + 32u <= i1 ? ov.off(p + 32u) : 0xFFFFFFFFu;
  // start of record `lane` relative to e0, clamped to [0, 33]
  const uint32_t h = r.w <= e0 ? 0u : min(r.w - e0, 33u);
  const bool inner = h >= 1u && h <= 31u;
  const uint32_t heads = __reduce_or_sync(0xffffffffu, inner ? 1u << h : 0u);
  const uint32_t n_inner = __popc(__ballot_sync(0xffffffffu, inner));
  // records 1 .. z also start at or before e0 (zero-entry owners)
  const int z = __popc(__ballot_sync(0xffffffffu, h == 0u)) - 1;
  int idx;
  if (__popc(heads) == (int)n_inner) {  // distinct starts (warp-uniform)
    idx = z + __popc(heads & (0xFFFFFFFFu >> (31 - lane)));
  } else {
    idx = 0;
#pragma unroll
    for (int st = 16; st >= 1; st >>= 1) {
      const uint32_t hv = __shfl_sync(0xffffffffu, h, idx + st);
      if (hv <= (uint32_t)lane) idx += st;
    }
  }
  uint4 o;
  o.x = __shfl_sync(0xffffffffu, r.x, idx);
  o.y = __shfl_sync(0xffffffffu, r.y, idx);
  o.z = __shfl_sync(0xffffffffu, r.z, idx);
  o.w = __shfl_sync(0xffffffffu, r.w, idx);
  const uint32_t e = e0 + (uint32_t)lane;
  if (x32 <= e) o = ov.rec(owner_search(ov, p + 32u, i1, e));  // behind zero-entry owners
  const uint32_t w = o.y & 0xFFFFu, gx = o.y >> 16;
  const uint32_t jj = e - o.w;
  uint32_t row = 0, col = jj;
  if (w) divmod_u32(jj, w, row, col);
  key = o.x + row * gx + col;
  val = o.z;
  // next window: the last record starting at or before e0 + 32
  const uint32_t in = __popc(__ballot_sync(0xffffffffu, h <= 32u));
  p = x32 <= e0 + 32u ? p + 32u : p + in - 1u;
}

// Keys and values of one warp's IT * 32 entries from ew on (cnt_w of them
// in range), generated into shared memory.
template <bool STAGED, int IT>
__device__ inline void gen_warp(const OwnerView<STAGED>& ov, uint32_t i0, uint32_t i1, uint32_t ew,
                                int cnt_w, int lane, uint32_t* __restrict__ keys,
                                uint32_t* __restrict__ vals) {
  uint32_t pos = owner_search(ov, i0, i1, ew);
#pragma unroll 1
  for (int it = 0; it < IT && it * 32 < cnt_w; ++it) {
    uint32_t k, v;
    gen_entries(ov, i1, pos, ew + (uint32_t)(it * 32), lane, k, v);
    const int j = it * 32 + lane;
    keys[j] = j < cnt_w ? k : 0u;
    vals[j] = v;
  }
}

template <int RB, bool KEYS_OUT, bool RANGES, bool GEN, int ITK = OsCfg<RB>::IT>
__global__ void __launch_bounds__(Os<RB, ITK>::NT, 2) onesweep_kernel(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int64_t cap,
    const int64_t* __restrict__ n_dev, int shift, int live, const uint32_t* __restrict__ pass_hist,
    uint32_t* __restrict__ status, uint32_t* __restrict__ part_counter, int2* __restrict__ range,
    uint32_t T, const uint4* __restrict__ owner, const uint32_t* __restrict__ chunk_first,
    int64_t n_sorted, const PassViews px, int64_t* __restrict__ info) {
  using P = Os<RB, ITK>;
  static_assert(!GEN || ITK == OsCfg<RB>::IT, "generating passes use the tile-pass partitions");
  constexpr int NT = P::NT, IT = P::IT, NW = P::NW, PART = P::PART, R = P::R;
  extern __shared__ __align__(16) uint32_t os_smem[];
  constexpr int HW = P::HW;
  uint32_t* warp_hist = os_smem;       // [NW][R]: per-warp counts, then exclusive offsets
  uint32_t* s_match = os_smem + NW * R;  // [NW][R] digit masks (OR_MATCH)
  uint32_t* s_vin = os_smem + HW;      // the partition's values in input order
  uint32_t* s_keys = s_vin + PART;     // keys in digit order
  uint32_t* s_vals = s_keys + PART;    // values in digit order
  __shared__ uint32_t s_block_excl[R];
  __shared__ uint32_t s_global_base[R];
  __shared__ uint32_t s_warp_tot[NW];
  __shared__ uint32_t s_part;

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int64_t n = pass_count(n_dev, cap);
  if (t == 0) s_part = atomicAdd(part_counter, 1u);
  // (a generating pass holds owner records in warp_hist until it ranks)
  if (!GEN)
    for (int i = t; i < HW; i += NT) warp_hist[i] = 0;
  __syncthreads();
  const int part = (int)s_part;
  const int64_t pbase = (int64_t)part * PART;
  if (pbase >= n) return;  // whole CTA: past the element count
  const int64_t rem = n - pbase;
  const int cnt = rem < (int64_t)PART ? (int)rem : PART;
  const int wofs = warp * 32 * IT;
  uint32_t key[IT], rank[IT];
  const uint32_t lt = lanemask_lt();
  if constexpr (GEN) {
    // keys and values generated from the owner records of the partition's
    // chunks: positions [i0, i1] (i1: the owner of the next partition's first
    // entry, or of entry n - 1)
    static_assert(PART % kEmitChunk == 0, "a partition is whole chunks");
    constexpr uint32_t kOwn = HW / 4;  // owner records that fit in warp_hist (+ masks)
    uint4* s_own = reinterpret_cast<uint4*>(warp_hist);
    const int64_t nchunks = (n + kEmitChunk - 1) / kEmitChunk;
    const int64_t c0 = (int64_t)part * (PART / kEmitChunk);
    const int64_t c1 = min(nchunks, c0 + PART / kEmitChunk);
    const uint32_t i0 = chunk_first[c0], i1 = chunk_first[c1];
    const bool ok = i0 <= i1 && (int64_t)i1 < n_sorted;
    if (!ok && t == 0) set_error(info, PGB_ERR_OVERFLOW);
    const uint32_t m = ok ? i1 - i0 + 1 : 0u;
    const bool staged = m <= kOwn;
    if (staged) {
      for (uint32_t q = t; q < m; q += NT) cp_async16(s_own + q, owner + i0 + q);
      cp_async_commit();
      cp_async_wait<0>();
    }
    __syncthreads();
    if (staged) {
      // Row marks: every row of an owner that starts inside the partition
      // writes (owner + 1) << 16 | row at its start position (s_vals is free
      // until the staging below); position 0 gets the row holding the
      // partition's first entry.  Marks grow with the position, so a running
      // maximum gives every entry its owner and row: no search, no division.
      __shared__ uint32_t s_wmax[NW];
      for (int j = t; j < PART; j += NT) s_vals[j] = 0u;
      __syncthreads();
      if (ok) {
        const uint32_t pb = (uint32_t)pbase, pend = pb + (uint32_t)cnt;
        if (t == 0) {
          const uint4 r0 = s_own[0];
          const uint32_t w0 = r0.y & 0xFFFFu;
          s_vals[0] = (1u << 16) | (w0 ? (pb - r0.w) / w0 : 0u);
        }
        for (uint32_t pl = t; pl < m; pl += NT) {
          const uint4 rec = s_own[pl];
          const uint32_t off = rec.w, w = rec.y & 0xFFFFu;
          const uint32_t off_next = pl + 1 < m ? s_own[pl + 1].w : (uint32_t)n;
          if (off_next <= off) continue;  // no entries
          const uint32_t tag = (pl + 1) << 16;
          if (w == 0) {  // one row of `count` tiles
            if (off >= pb && off < pend) s_vals[off - pb] = tag;
            continue;
          }
          uint32_t r = off < pb ? (pb - off + w - 1) / w : 0u;
          for (uint32_t st = off + r * w; st < off_next && st < pend; st += w, ++r)
            s_vals[st - pb] = tag | r;
        }
      }
      __syncthreads();
      // running maximum in the pass's striped order: per warp over its
      // 32 * IT positions, then across the warps before it
      uint32_t run = 0;
#pragma unroll
      for (int it = 0; it < IT; ++it) {
        uint32_t v = s_vals[wofs + it * 32 + lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
          if (lane >= o) v = max(v, u);
        }
        v = max(v, run);
        run = __shfl_sync(0xffffffffu, v, 31);
        key[it] = v;
      }
      if (lane == 31) s_wmax[warp] = run;
      __syncthreads();
      uint32_t pre = 0;
      for (int w2 = 0; w2 < warp; ++w2) pre = max(pre, s_wmax[w2]);
#pragma unroll
      for (int it = 0; it < IT; ++it) {
        const int j = wofs + it * 32 + lane;
        const uint32_t mk = max(pre, key[it]);
        key[it] = 0u;
        if (ok && j < cnt && mk >= (1u << 16)) {
          const uint4 rec = s_own[(mk >> 16) - 1];
          const uint32_t r = mk & 0xFFFFu, w = rec.y & 0xFFFFu, gx = rec.y >> 16;
          const uint32_t e = (uint32_t)pbase + (uint32_t)j;
          key[it] = rec.x + r * gx + (e - rec.w - r * w);
          s_vin[j] = rec.z;  // read back by this thread only
        }
      }
    } else {
      // more owners than fit in shared memory: the warp-cooperative window
      // search over owner records in global memory, through s_keys
      for (int it = 0; it < IT; ++it) s_keys[wofs + it * 32 + lane] = 0u;
      __syncwarp();
      if (ok && wofs < cnt) {
        const uint32_t ew = (uint32_t)pbase + (uint32_t)wofs;
        const int cnt_w = min(cnt - wofs, 32 * IT);
        gen_warp<false, IT>(OwnerView<false>{owner, s_own, i0}, i0, i1, ew, cnt_w, lane,
                            s_keys + wofs, s_vin + wofs);
      }
      __syncwarp();
#pragma unroll
      for (int it = 0; it < IT; ++it) key[it] = s_keys[wofs + it * 32 + lane];
    }
    __syncthreads();  // every warp is done with the owner records
    for (int i = t; i < HW; i += NT) warp_hist[i] = 0;
    __syncthreads();
  } else {
    if (cnt == PART) {
      for (int q = t; q < PART / 4; q += NT) cp_async16(s_vin + 4 * q, vals_in + pbase + 4 * q);
      cp_async_commit();
    } else {
      for (int q = t; q < cnt; q += NT) s_vin[q] = vals_in[pbase + q];
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const int j = wofs + it * 32 + lane;
      key[it] = j < cnt ? keys_in[pbase + j] : 0u;
    }
  }
  if constexpr (P::OR_MATCH) {
    uint32_t* wm = s_match + warp * R;
    const uint32_t bit = 1u << lane;
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const bool valid = wofs + it * 32 + lane < cnt;
      const uint32_t d = (key[it] >> shift) & (R - 1);
      if (valid) atomicOr(&wm[d], bit);
      __syncwarp();
      const uint32_t peers = valid ? wm[d] : 0u;
      const uint32_t old = warp_hist[warp * R + d];
      rank[it] = old + __popc(peers & lt);
      __syncwarp();
      if (valid && (peers & lt) == 0) {  // the digit's first lane
        warp_hist[warp * R + d] = old + __popc(peers);
        wm[d] = 0u;
      }
      __syncwarp();
    }
  } else {
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const bool valid = wofs + it * 32 + lane < cnt;
      const uint32_t d = (key[it] >> shift) & (R - 1);
      const uint32_t peers = match_digit<RB>(d, valid, live);
      const uint32_t old = warp_hist[warp * R + d];
      rank[it] = old + __popc(peers & lt);
      __syncwarp();
      if (valid && (peers & lt) == 0) warp_hist[warp * R + d] = old + __popc(peers);
      __syncwarp();
    }
  }
  __syncthreads();

  // Per digit: exclusive offsets across warps, partition count, aggregate
  // publication; then the digit's global start and its local start.
  uint32_t count = 0;
  if (t < R) {
#pragma unroll 4
    for (int w = 0; w < NW; ++w) {
      const uint32_t c = warp_hist[w * R + t];
      warp_hist[w * R + t] = count;
      count += c;
    }
    st_volatile(status + (size_t)part * R + t, (part == 0 ? kFlagInc : kFlagAgg) | count);
  }
  uint32_t unused, local_total;
  const uint32_t digit_start =
      block_excl_scan<NT>(t < R ? pass_hist[t] : 0u, unused, s_warp_tot);
  const uint32_t bex = block_excl_scan<NT>(t < R ? count : 0u, local_total, s_warp_tot);
  if (t < R) s_block_excl[t] = bex;
  if (!GEN && cnt == PART) cp_async_wait<0>();
  __syncthreads();

  // Stage in digit order; the digit threads resolve the global bases.
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    const int j = wofs + it * 32 + lane;
    if (j < cnt) {
      const uint32_t d = (key[it] >> shift) & (R - 1);
      const uint32_t lp = s_block_excl[d] + warp_hist[warp * R + d] + rank[it];
      s_keys[lp] = key[it];
      s_vals[lp] = s_vin[j];
    }
  }
  if (t < R) {
    uint32_t prior = 0;
    if (part > 0) {
      prior = look_back(status + t, part, R, info);
      st_volatile(status + (size_t)part * R + t, kFlagInc | ((prior + count) & kValMask));
    }
    s_global_base[t] = digit_start + prior;
  }
  __syncthreads();

  for (int j = t; j < cnt; j += NT) {
    const uint32_t k = s_keys[j];
    const uint32_t d = (k >> shift) & (R - 1);
    const uint32_t dst = s_global_base[d] + (uint32_t)(j - (int)s_block_excl[d]);
    if ((int64_t)dst >= n) {  // only if the histogram disagrees with the keys
      set_error(info, PGB_ERR_OVERFLOW);
      continue;
    }
    const uint32_t val = s_vals[j];
    if (KEYS_OUT) keys_out[dst] = px.key_from_val ? fdiv(val, px.vdiv) : k;
    vals_out[dst] = val;
    if (RANGES) {
      bool first = j == 0 || s_keys[j - 1] != k, last = j + 1 == cnt || s_keys[j + 1] != k;
      uint32_t gt = k;
      if (px.nviews > 0) {  // runs of one local tile hold the views in order
        const uint32_t v = fdiv(val, px.vdiv);
        if (v >= (uint32_t)px.nviews) {
          set_error(info, PGB_ERR_OVERFLOW);
          continue;
        }
        gt = px.tile_base[v] + k;
        if (!first) first = fdiv(s_vals[j - 1], px.vdiv) != v;
        if (!last) last = fdiv(s_vals[j + 1], px.vdiv) != v;
      }
      if (gt >= T) {
        set_error(info, PGB_ERR_OVERFLOW);
        continue;
      }
      if (first) atomicMin(&range[gt].x, (int)dst);
      if (last) atomicMax(&range[gt].y, (int)dst + 1);
    }
  }
}

// Where a generating pass (GEN) reads its entries: the owner records and
// the chunk table of the scan.
struct GenSource {
  const uint4* owner = nullptr;
  const uint32_t* chunk_first = nullptr;
  int64_t n_sorted = 0;
};

// One pass: digit width, whether keys are written, whether ranges are made,
// whether the keys are generated from owner records (ki / vi unused).
template <int RB, bool KEYS_OUT, bool RANGES, bool GEN = false, int ITK = OsCfg<RB>::IT>
static int launch_onesweep(int parts, cudaStream_t s, const uint32_t* ki, const uint32_t* vi,
                           uint32_t* ko, uint32_t* vo, int64_t cap, const int64_t* n_dev,
                           int shift, const uint32_t* hist, uint32_t* status, uint32_t* counter,
                           int2* range, uint32_t T, int64_t* info, const GenSource& src = {},
                           int live = RB, const PassViews& px = PassViews{}) {
  using P = Os<RB, ITK>;
  auto kern = onesweep_kernel<RB, KEYS_OUT, RANGES, GEN, ITK>;
  // the attribute is set on every call: the call is cheap, allowed while a
  // stream is being captured, and per device
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::SMEM) !=
      cudaSuccess)
    return PGB_ERR_CUDA;
  kern<<<parts, P::NT, P::SMEM, s>>>(ki, vi, ko, vo, cap, n_dev, shift, live, hist, status,
                                     counter, range, T, src.owner, src.chunk_first, src.n_sorted,
                                     px, info);
  return PGB_OK;
}

// ---------------------------------------------------------------------------
// 3a. tile rectangles in Gaussian order (coalesced), and the tile-digit
//     histograms of every pair that will be emitted
//
// rect[g] = (first tile, w | h << 16, row stride gx, count): the global id
// of the rectangle's top-left tile (the view's first tile added), its size
// in tiles, the tile-grid width of g's view, and the number of entries g
// emits (tiles_touched when radius > 0, else 0).  A count that disagrees
// with the rectangle is reported as PGB_ERR_MISMATCH.
//
// Emission writes entry j of g as tile first + (j / w) gx + j % w for
// j < count (one row of `count` tiles when w = 0): runs of consecutive tile
// ids, one per rectangle row.  A run [a, a + len) adds to the low digit's
// histogram one range of consecutive digits (mod R) plus len / R full
// cycles -- two or four updates of a shared difference array -- and to a
// higher digit's histogram at most ceil(len / R) + 1 counted digits.  The
// CTA turns its difference array into counts and adds its histograms to
// the global ones once.
// ---------------------------------------------------------------------------
__device__ inline void hist_run(uint32_t a, uint32_t len, int passes, int bits, int R,
                                int* __restrict__ s_diff, uint32_t* __restrict__ s_full,
                                uint32_t* __restrict__ s_hist) {
  if (len == 0) return;
  // low digit: len / R full cycles, then len % R consecutive digits from a's
  const uint32_t full = len >> bits, rem = len & (uint32_t)(R - 1);
  if (full) atomicAdd(s_full, full);
  if (rem) {
    const uint32_t d = a & (uint32_t)(R - 1), e = d + rem;
    atomicAdd(&s_diff[d], 1);
    if (e <= (uint32_t)R) {
      atomicSub(&s_diff[e], 1);
    } else {  // wraps past digit R - 1
      atomicAdd(&s_diff[0], 1);
      atomicSub(&s_diff[e - R], 1);
    }
  }
  for (int p = 1; p < passes; ++p) {
    const int sh = bits * p;
    const uint32_t last = a + len - 1;
    for (uint32_t v = a >> sh; v <= (last >> sh); ++v) {
      const uint32_t lo = max(a, v << sh), hi = min(last, ((v + 1) << sh) - 1);
      atomicAdd(&s_hist[p * R + (v & (uint32_t)(R - 1))], hi - lo + 1);
    }
  }
}

// With `list` (a band's Gaussian list, one image), element i is Gaussian
// list[i] and its entry count is its band-clipped rectangle; otherwise
// element g is Gaussian g with tiles[g] entries (checked against its
// rectangle).
__global__ void __launch_bounds__(kStreamThreads) rect_kernel(
    const float* __restrict__ uv, const int32_t* __restrict__ radius,
    const int32_t* __restrict__ tiles, int64_t n, ViewTable vt, int tile_passes, int digit_bits,
    uint4* __restrict__ rect, uint32_t* __restrict__ tile_hist, int64_t* __restrict__ info,
    const uint32_t* __restrict__ list) {
  constexpr int NW = kStreamThreads / 32;
  __shared__ int s_diff[513];
  __shared__ uint32_t s_hist[kTileHistWords];
  __shared__ uint32_t s_full;
  __shared__ uint32_t s_warp_tot[NW];
  __shared__ uint4 s_rect[NW][32];      // the warp's rectangles
  __shared__ uint32_t s_runs[NW][33];   // exclusive prefix of their run counts
  const int R = 1 << digit_bits;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < 513; i += blockDim.x) s_diff[i] = 0;
  for (int i = threadIdx.x; i < kTileHistWords; i += blockDim.x) s_hist[i] = 0;
  if (threadIdx.x == 0) s_full = 0;
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + warp * 32; base < n; base += stride) {
    const int64_t i = base + lane;
    uint4 out = make_uint4(0u, 0u, 0u, 0u);
    uint32_t runs = 0;
    if (i < n) {
      const int64_t g = list ? (int64_t)list[i] : i;
      const int r = radius[g];
      if (r > 0) {
        const float2 p = reinterpret_cast<const float2*>(uv)[g];
        int gx, gy, x0, x1, y0, y1;
        uint32_t tile_base;
        element_view(vt, (uint32_t)g, gx, gy, tile_base);
        if (vt.nviews == 0)
          tile_rect(p.x, p.y, (float)r, gx, gy, x0, x1, y0, y1);
        else  // a batch of views: 16 x th tiles
          tile_rect_h(p.x, p.y, (float)r, vt.th, gx, gy, x0, x1, y0, y1);
        if (vt.nviews == 0) {  // one image: the rows of its band, band-local
          y0 = max(y0, vt.band0);
          y1 = max(min(y1, vt.band1), y0);
          y0 -= vt.band0;
          y1 -= vt.band0;
        }
        const uint32_t w = (uint32_t)(x1 - x0);
        uint32_t cnt;
        if (list) {
          cnt = w * (uint32_t)(y1 - y0);
        } else {
          cnt = (uint32_t)max(tiles[g], 0);
          if ((int64_t)w * (y1 - y0) != (int64_t)cnt) set_error(info, PGB_ERR_MISMATCH);
        }
        // tile ids local to the element's view: a batch is sorted by local
        // tile over a view-major emission (the last pass adds the bases)
        (void)tile_base;
        const uint32_t first = (uint32_t)y0 * (uint32_t)gx + (uint32_t)x0;
        out = make_uint4(first, w | ((uint32_t)(y1 - y0) << 16), (uint32_t)gx, cnt);
        // runs of consecutive tile ids that emission writes for g
        runs = cnt == 0 ? 0u : (w == 0 ? 1u : cnt / w + (cnt % w ? 1u : 0u));
      }
      rect[g] = out;
    }
    // spread the warp's runs over its lanes
    uint32_t incl = runs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    s_rect[warp][lane] = out;
    s_runs[warp][lane + 1] = incl;
    if (lane == 0) s_runs[warp][0] = 0;
    __syncwarp();
    const uint32_t total = s_runs[warp][32];
    for (uint32_t k = lane; k < total; k += 32) {
      int lo = 0, hi = 31;  // owner: the last lane whose prefix is <= k
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_runs[warp][mid] <= k) lo = mid; else hi = mid - 1;
      }
      const uint4 o = s_rect[warp][lo];
      const uint32_t j = k - s_runs[warp][lo];  // run index within the owner
      const uint32_t w = o.y & 0xFFFFu, cnt = o.w;
      uint32_t a, len;
      if (w == 0) {
        a = o.x;
        len = cnt;
      } else {
        a = o.x + j * o.z;
        len = min(w, cnt - j * w);
      }
      hist_run(a, len, tile_passes, digit_bits, R, s_diff, &s_full, s_hist);
    }
    __syncwarp();
  }
  __syncthreads();
  // low digit: counts = inclusive prefix of the difference array (modular
  // sums of the signed updates) + the full cycles; then one flush
  const uint32_t full = s_full;
  uint32_t carry = 0;
  for (int base = 0; base < R; base += kStreamThreads) {
    const int d = base + threadIdx.x;
    const uint32_t v = (uint32_t)s_diff[d];
    uint32_t total;
    const uint32_t ex = block_excl_scan<kStreamThreads>(v, total, s_warp_tot);
    s_hist[d] = carry + ex + v + full;
    carry += total;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < tile_passes * R; i += blockDim.x) {
    const uint32_t v = s_hist[i];
    if (v) atomicAdd(tile_hist + i, v);
  }
}

// ---------------------------------------------------------------------------
// 3b. scan of the entry counts in depth order
//
// For depth-sorted position i (Gaussian g = order[i]) writes the emission
// record owner[i] = (first tile, w | gx << 16, g, output offset) and, for
// every emission chunk boundary b * kEmitChunk that falls inside
// [offset, offset + count), chunk_first[b] = i.  K is the host value k_cap,
// or the device count k_dev (written by the depth phase) bounded by the
// capacity k_cap.  The grid also sets the tile-range table to (INT_MAX, 0)
// for the last tile pass.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kSortThreads) scan_rect_kernel(
    const uint32_t* __restrict__ order, int64_t n, const uint4* __restrict__ rect, int64_t k_cap,
    const int64_t* __restrict__ k_dev, uint32_t* __restrict__ status,
    uint32_t* __restrict__ part_counter, uint4* __restrict__ owner,
    uint32_t* __restrict__ chunk_first, int2* __restrict__ range, uint32_t T,
    const uint32_t* __restrict__ views_mark, uint32_t nviews, int64_t* __restrict__ info) {
  __shared__ uint32_t s_warp_tot[kSortThreads / 32];
  __shared__ uint32_t s_part, s_prior;
  // the tile-range table starts at (INT_MAX, 0) for the last tile pass
  for (int64_t i = (int64_t)blockIdx.x * kSortThreads + threadIdx.x; i < T;
       i += (int64_t)gridDim.x * kSortThreads)
    range[i] = make_int2(INT_MAX, 0);
  // phase one of a batch (view-major order) must precede phase two of a
  // batch, and the one-image phase one the one-image phase two
  if (*views_mark != nviews) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_error(info, PGB_ERR_INVALID);
    return;
  }
  // a device count past the capacity: reported once, nothing is emitted
  if (k_dev && (*k_dev < 0 || *k_dev > k_cap)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_error(info, PGB_ERR_OVERFLOW);
    return;
  }
  const int64_t K = pass_count(k_dev, k_cap);
  if (threadIdx.x == 0) s_part = atomicAdd(part_counter, 1u);
  __syncthreads();
  const int part = (int)s_part;
  const int64_t base = (int64_t)part * kScanPart + (int64_t)threadIdx.x * kScanItems;

  uint32_t cnt[kScanItems], t0[kScanItems], wg[kScanItems], gid[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int it = 0; it < kScanItems; ++it) {
    const int64_t e = base + it;
    uint4 r = make_uint4(0u, 0u, 0u, 0u);
    gid[it] = 0;
    if (e < n) {
      gid[it] = order[e];
      r = rect[gid[it]];
    }
    t0[it] = r.x;
    wg[it] = (r.y & 0xFFFFu) | (r.z << 16);
    cnt[it] = r.w;
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
        owner[e] = make_uint4(t0[it], wg[it], gid[it], (uint32_t)off);
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
// 5. tiles that no entry reached: (INT_MAX, 0) -> (0, 0)
// ---------------------------------------------------------------------------
__global__ void range_fix_kernel(int2* __restrict__ range, uint32_t T) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < T;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (range[i].x == INT_MAX) range[i] = make_int2(0, 0);
  }
}

// A device count past a capacity that leaves nothing to launch.
__global__ void capacity_check_kernel(const int64_t* __restrict__ k_dev, int64_t k_cap,
                                      int64_t* __restrict__ info) {
  if (threadIdx.x == 0 && (*k_dev < 0 || *k_dev > k_cap)) set_error(info, PGB_ERR_OVERFLOW);
}

// ---------------------------------------------------------------------------
// scratch layout
// ---------------------------------------------------------------------------
inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct ScratchN {
  size_t counters, depth_hist, tile_hist, depth_status, scan_status, zero_bytes;
  size_t dk0, dv0, dk1, dv1, owner, rect, total;
  int parts, scan_parts;
};

inline ScratchN layout_n(int64_t n) {
  ScratchN L;
  L.parts = (int)((n + depth_part_keys(n) - 1) / depth_part_keys(n));
  L.scan_parts = (int)((n + kScanPart - 1) / kScanPart);
  size_t o = 0;
  L.counters = o; o += align256(16 * sizeof(uint32_t));
  L.depth_hist = o; o += align256((kDepthPasses + 1) * 256 * sizeof(uint32_t));
  L.tile_hist = o; o += align256(kTileHistWords * sizeof(uint32_t));
  L.depth_status = o; o += align256((size_t)(kDepthPasses + 1) * L.parts * 256 * sizeof(uint32_t));
  L.scan_status = o; o += align256((size_t)L.scan_parts * sizeof(uint32_t));
  L.zero_bytes = o;
  const size_t nb = align256((size_t)n * sizeof(uint32_t));
  L.dk0 = o; o += nb;
  L.dv0 = o; o += nb;
  L.dk1 = o; o += nb;
  L.dv1 = o; o += nb;
  L.owner = o; o += align256((size_t)n * sizeof(uint4));
  L.rect = o; o += align256((size_t)n * sizeof(uint4));
  L.total = o;
  return L;
}

// Tile passes for T tiles: digit width and count (one 8-bit pass up to 256
// tiles, two up to 2^16, two 9-bit passes up to 2^18, else three 8-bit).
struct TilePlan {
  int passes, bits;
};

inline TilePlan tile_plan(uint64_t T) {
  int b = 0;
  while (b < 32 && ((T - 1) >> b)) ++b;
  if (b <= 8) return {1, 8};
  if (b <= 16) return {2, 8};
  if (b <= 18) return {2, 9};
  return {3, 8};
}

struct ScratchK {
  size_t tk0, tv0, tk1, tv1, status, chunk_first, total;
  int parts;
  int64_t chunks;
};

// K-sized pair buffers: pass 0 generates its pairs and writes pair buffer 1,
// pass 1 reads it and writes buffer 0, pass 2 reads that; the last pass
// writes the ids out.  So one tile pass needs no buffer, two need buffer 1,
// three need both.
inline ScratchK layout_k(int64_t k, int passes) {
  ScratchK L;
  L.parts = (int)((k + kPartKeys - 1) / kPartKeys);
  size_t o = 0;
  const size_t kb = align256((size_t)k * sizeof(uint32_t));
  const size_t kb0 = passes >= 3 ? kb : 0, kb1 = passes >= 2 ? kb : 0;
  L.tk0 = o; o += kb0;
  L.tv0 = o; o += kb0;
  L.tk1 = o; o += kb1;
  L.tv1 = o; o += kb1;
  L.status = o; o += align256((size_t)L.parts * kTileHistWords * sizeof(uint32_t));
  L.chunks = (k + kEmitChunk - 1) / kEmitChunk;
  L.chunk_first = o; o += align256((size_t)(L.chunks + 2) * sizeof(uint32_t));
  L.total = o;
  return L;
}


template <typename P>
inline P* at(void* base, size_t off) {
  return reinterpret_cast<P*>(static_cast<char*>(base) + off);
}

// One tile pass p of `plan` (the last one writes ids and ranges, no keys;
// the first generates its entries from the owner records).
static int tile_pass(const TilePlan& plan, int p, int parts, cudaStream_t s, const uint32_t* ki,
                     const uint32_t* vi, uint32_t* ko, uint32_t* vo, int64_t cap,
                     const int64_t* n_dev, const uint32_t* hist, uint32_t* status,
                     uint32_t* counter, int2* range, uint32_t T, uint32_t T_local, int64_t* info,
                     const GenSource& src, const PassViews& px) {
  const bool last = p == plan.passes - 1;
  const int shift = plan.bits * p;
  const uint32_t* h = hist + (size_t)p * (1u << plan.bits);
  uint32_t* st = status + (size_t)p * parts * (1u << plan.bits);
  // digit bits that some (local) tile id has set in this pass
  int live = 0;
  while (live < plan.bits && ((T_local - 1) >> (shift + live))) ++live;
  live = live < 1 ? 1 : live;
#define PGB_PASS(RB, KO, RG, GN) \
  launch_onesweep<RB, KO, RG, GN>(parts, s, ki, vi, ko, vo, cap, n_dev, shift, h, st, counter, \
                                  range, T, info, src, live, px)
  if (p == 0) {
    if (last) return PGB_PASS(8, false, true, true);  // one pass: at most 256 tiles
    return plan.bits == 9 ? PGB_PASS(9, true, false, true) : PGB_PASS(8, true, false, true);
  }
  if (plan.bits == 9) return last ? PGB_PASS(9, false, true, false) : PGB_PASS(9, true, false, false);
  return last ? PGB_PASS(8, false, true, false) : PGB_PASS(8, true, false, false);
#undef PGB_PASS
}

// ---------------------------------------------------------------------------
// 6. bands of tile rows (one image processed a band at a time)
//
// band_tiles: the entries of each Gaussian inside tile rows [row0, row1) --
// its tile rectangle (tile_rect, as the sort computes it) clipped to the
// band, 0 for radius <= 0.  band_count: the sum of those counts over the
// Gaussians with radius > 0 (the band's K), into info[0].
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kStreamThreads) band_tiles_kernel(
    const float* __restrict__ uv, const int32_t* __restrict__ radius, int64_t n, int gx, int gy,
    int row0, int row1, int32_t* __restrict__ tiles_out) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int r = radius[g];
    int cnt = 0;
    if (r > 0) {
      const float2 p = reinterpret_cast<const float2*>(uv)[g];
      int x0, x1, y0, y1;
      tile_rect(p.x, p.y, (float)r, gx, gy, x0, x1, y0, y1);
      const int rows = min(y1, row1) - max(y0, row0);
      cnt = rows > 0 ? (x1 - x0) * rows : 0;
    }
    tiles_out[g] = cnt;
  }
}

__global__ void __launch_bounds__(kStreamThreads) band_count_kernel(
    const int32_t* __restrict__ radius, const int32_t* __restrict__ tiles, int64_t n,
    int64_t* __restrict__ info) {
  unsigned long long sum = 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x)
    if (radius[g] > 0) sum += (unsigned long long)max(tiles[g], 0);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0 && sum)
    atomicAdd(reinterpret_cast<unsigned long long*>(info), sum);
}

// band_counts: K of every band at once.  bands holds nbands + 1 increasing
// tile rows (band b is rows [bands[b], bands[b + 1])); each Gaussian adds
// its rectangle's entries in every band it crosses.  Per-CTA partial sums
// in shared memory, one 64-bit atomic per band and CTA.
constexpr int kMaxBands = 1024;

__global__ void __launch_bounds__(kStreamThreads) band_counts_kernel(
    const float* __restrict__ uv, const int32_t* __restrict__ radius, int64_t n, int gx, int gy,
    const int32_t* __restrict__ bands, int nbands, unsigned long long* __restrict__ counts) {
  __shared__ unsigned long long s_cnt[kMaxBands];
  __shared__ int s_rows[kMaxBands + 1];
  for (int i = threadIdx.x; i < nbands; i += blockDim.x) s_cnt[i] = 0ull;
  for (int i = threadIdx.x; i <= nbands; i += blockDim.x) s_rows[i] = bands[i];
  __syncthreads();
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int r = radius[g];
    if (r <= 0) continue;
    const float2 p = reinterpret_cast<const float2*>(uv)[g];
    int x0, x1, y0, y1;
    tile_rect(p.x, p.y, (float)r, gx, gy, x0, x1, y0, y1);
    if (x1 <= x0 || y1 <= y0) continue;
    // the first band that reaches row y0 (bands are short lists: linear scan)
    int b = 0;
    while (b < nbands && s_rows[b + 1] <= y0) ++b;
    for (; b < nbands && s_rows[b] < y1; ++b) {
      const int rows = min(y1, s_rows[b + 1]) - max(y0, s_rows[b]);
      if (rows > 0) atomicAdd(&s_cnt[b], (unsigned long long)((x1 - x0) * rows));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbands; i += blockDim.x)
    if (s_cnt[i]) atomicAdd(&counts[i], s_cnt[i]);
}

// ---------------------------------------------------------------------------
// Band lists: for bands of tile rows [rows[b], rows[b + 1]), the Gaussians
// with at least one entry in band b, in the depth order of phase one, so
// that a band's rectangle and scan passes visit only its own Gaussians.
// Three kernels over the depth order: per-block counts per band, a scan of
// each band's block counts (and the bands' offsets), and a stable write
// (warp ballots per band, warps in order within the block).
// ---------------------------------------------------------------------------
constexpr int kListThreads = 256;
constexpr int kListChunk = kListThreads * 16;  // depth positions per block
constexpr int kMaxListBands = 256;

inline int list_blocks(int64_t n) { return (int)((n + kListChunk - 1) / kListChunk); }

// Bands [b0, b1] whose rows meet Gaussian g's tile rectangle (b1 < b0:
// none): the bands where its band-clipped entry count is positive.
__device__ inline void element_bands(const float* __restrict__ uv,
                                     const int32_t* __restrict__ radius, uint32_t g, int gx,
                                     int gy, const int* s_rows, int nbands, int& b0, int& b1) {
  b0 = INT_MAX;
  b1 = -1;
  const int r = radius[g];
  if (r <= 0) return;
  const float2 p = reinterpret_cast<const float2*>(uv)[g];
  int x0, x1, y0, y1;
  tile_rect(p.x, p.y, (float)r, gx, gy, x0, x1, y0, y1);
  if (x1 <= x0 || y1 <= y0) return;
  int lo = 0, hi = nbands;  // the first band ending after row y0
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (s_rows[mid + 1] > y0) hi = mid; else lo = mid + 1;
  }
  const int first = lo;
  hi = nbands;  // the first band starting at or after row y1
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (s_rows[mid] >= y1) hi = mid; else lo = mid + 1;
  }
  if (lo - 1 >= first) {
    b0 = first;
    b1 = lo - 1;
  }
}

__global__ void __launch_bounds__(kListThreads) band_list_count_kernel(
    const uint32_t* __restrict__ order, const float* __restrict__ uv,
    const int32_t* __restrict__ radius, int64_t n, int gx, int gy,
    const int32_t* __restrict__ rows, int nbands, uint32_t* __restrict__ block_counts) {
  __shared__ int s_rows[kMaxListBands + 1];
  __shared__ uint32_t s_cnt[kMaxListBands];
  for (int i = threadIdx.x; i <= nbands; i += kListThreads) s_rows[i] = rows[i];
  for (int i = threadIdx.x; i < nbands; i += kListThreads) s_cnt[i] = 0u;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kListChunk;
  for (int j = threadIdx.x; j < kListChunk; j += kListThreads) {
    const int64_t e = base + j;
    if (e >= n) break;
    int b0, b1;
    element_bands(uv, radius, order[e], gx, gy, s_rows, nbands, b0, b1);
    for (int b = b0; b <= b1; ++b) atomicAdd(&s_cnt[b], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbands; b += kListThreads)
    block_counts[(size_t)b * gridDim.x + blockIdx.x] = s_cnt[b];
}

// One CTA per band: exclusive scan of the band's block counts in place; the
// band's total to offsets[b + 1].
__global__ void __launch_bounds__(kListThreads) band_list_scan_kernel(
    uint32_t* __restrict__ block_counts, int nblocks, int64_t* __restrict__ offsets) {
  __shared__ uint32_t s_warp_tot[kListThreads / 32];
  uint32_t* row = block_counts + (size_t)blockIdx.x * nblocks;
  uint32_t carry = 0;
  for (int base = 0; base < nblocks; base += kListThreads) {
    const int i = base + threadIdx.x;
    const uint32_t v = i < nblocks ? row[i] : 0u;
    uint32_t total;
    const uint32_t ex = block_excl_scan<kListThreads>(v, total, s_warp_tot);
    if (i < nblocks) row[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) offsets[blockIdx.x + 1] = (int64_t)carry;
}

// offsets[0] = 0, offsets[b + 1] = the end of band b's list.
__global__ void band_list_offsets_kernel(int64_t* __restrict__ offsets, int nbands) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int64_t run = 0;
    offsets[0] = 0;
    for (int b = 0; b < nbands; ++b) {
      run += offsets[b + 1];
      offsets[b + 1] = run;
    }
  }
}

__global__ void __launch_bounds__(kListThreads) band_list_write_kernel(
    const uint32_t* __restrict__ order, const float* __restrict__ uv,
    const int32_t* __restrict__ radius, int64_t n, int gx, int gy,
    const int32_t* __restrict__ rows, int nbands, const uint32_t* __restrict__ block_base,
    const int64_t* __restrict__ offsets, uint32_t* __restrict__ lists) {
  constexpr int NW = kListThreads / 32;
  constexpr int PER_WARP = kListChunk / NW;  // consecutive depth positions per warp
  __shared__ int s_rows[kMaxListBands + 1];
  __shared__ uint32_t s_wcnt[NW][kMaxListBands];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = lanemask_lt();
  for (int i = threadIdx.x; i <= nbands; i += kListThreads) s_rows[i] = rows[i];
  for (int i = threadIdx.x; i < NW * kMaxListBands; i += kListThreads) (&s_wcnt[0][0])[i] = 0u;
  __syncthreads();
  const int64_t wbase = (int64_t)blockIdx.x * kListChunk + warp * PER_WARP;
  // per-warp counts per band
  for (int it = 0; it < PER_WARP / 32; ++it) {
    const int64_t e = wbase + it * 32 + lane;
    int b0 = INT_MAX, b1 = -1;
    if (e < n) element_bands(uv, radius, order[e], gx, gy, s_rows, nbands, b0, b1);
    const int lo = __reduce_min_sync(0xffffffffu, b0), hi = __reduce_max_sync(0xffffffffu, b1);
    for (int b = lo; b <= hi; ++b) {
      const uint32_t m = __ballot_sync(0xffffffffu, b >= b0 && b <= b1);
      if (lane == 0) s_wcnt[warp][b] += __popc(m);
    }
  }
  __syncthreads();
  // block-local exclusive prefix per band across the warps, in warp order
  for (int b = threadIdx.x; b < nbands; b += kListThreads) {
    uint32_t run = 0;
    for (int w = 0; w < NW; ++w) {
      const uint32_t c = s_wcnt[w][b];
      s_wcnt[w][b] = run;
      run += c;
    }
  }
  __syncthreads();
  // stable writes: a warp's lanes in lane order, its iterations in order
  for (int it = 0; it < PER_WARP / 32; ++it) {
    const int64_t e = wbase + it * 32 + lane;
    int b0 = INT_MAX, b1 = -1;
    uint32_t g = 0;
    if (e < n) {
      g = order[e];
      element_bands(uv, radius, g, gx, gy, s_rows, nbands, b0, b1);
    }
    const int lo = __reduce_min_sync(0xffffffffu, b0), hi = __reduce_max_sync(0xffffffffu, b1);
    for (int b = lo; b <= hi; ++b) {
      const bool mine = b >= b0 && b <= b1;
      const uint32_t m = __ballot_sync(0xffffffffu, mine);
      if (mine)
        lists[offsets[b] + (int64_t)block_base[(size_t)b * gridDim.x + blockIdx.x] +
              s_wcnt[warp][b] + __popc(m & lt)] = g;
      __syncwarp();
      if (lane == 0) s_wcnt[warp][b] += __popc(m);
      __syncwarp();
    }
  }
}

// Entries of each element of a batch of views for 16 x th tiles (the
// tiles_touched the views' sort then takes): its view's tile rectangle,
// 0 for radius <= 0.
__global__ void __launch_bounds__(kStreamThreads) view_tiles_kernel(
    const float* __restrict__ uv, const int32_t* __restrict__ radius, int64_t n, ViewTable vt,
    int32_t* __restrict__ tiles_out) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int r = radius[g];
    int cnt = 0;
    if (r > 0) {
      int gx, gy, x0, x1, y0, y1;
      uint32_t base;
      element_view(vt, (uint32_t)g, gx, gy, base);
      const float2 p = reinterpret_cast<const float2*>(uv)[g];
      tile_rect_h(p.x, p.y, (float)r, vt.th, gx, gy, x0, x1, y0, y1);
      cnt = (x1 - x0) * (y1 - y0);
    }
    tiles_out[g] = cnt;
  }
}

}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_sort_scratch_bytes(int64_t n, int64_t k, int width, int height, size_t* bytes_n,
                           size_t* bytes_k) {
  if (n < 0 || k < 0 || width <= 0 || height <= 0) return PGB_ERR_INVALID;
  const uint64_t T = (uint64_t)grid_x(width) * (uint64_t)grid_y(height);
  if (bytes_n) *bytes_n = layout_n(n).total;
  if (bytes_k) *bytes_k = layout_k(k, tile_plan(T).passes).total;
  return PGB_OK;
}

}  // extern "C"

// The depth passes (and the view pass of a batch) with ITK keys per thread.
template <int ITK>
static int depth_passes(const ScratchN& L, cudaStream_t s, uint32_t* k0, uint32_t* v0,
                        uint32_t* k1, uint32_t* v1, int64_t n, int nviews, uint32_t* hist,
                        uint32_t* status, uint32_t* counters, int64_t* info, PassViews px) {
  const int passes = kDepthPasses + (nviews > 0 ? 1 : 0);
  for (int p = 0; p < passes; ++p) {
    const uint32_t* ki = (p & 1) ? k1 : k0;
    const uint32_t* vi = (p & 1) ? v1 : v0;
    uint32_t* ko = (p & 1) ? k0 : k1;
    uint32_t* vo = (p & 1) ? v0 : v1;
    uint32_t* st = status + (size_t)p * L.parts * 256;
    int rc;
    if (p == kViewPass) {  // by view (keys: the views the previous pass wrote)
      int live = 1;
      while ((1 << live) < nviews) ++live;
      rc = launch_onesweep<8, false, false, false, ITK>(L.parts, s, ki, vi, ko, vo, n, nullptr, 0,
                                                        hist + 256 * p, st, counters + 8, nullptr,
                                                        0, info, GenSource{}, live);
    } else if (p == kDepthPasses - 1) {
      // the last depth pass: for a batch it writes the views as the next
      // pass's keys; for one image only the order is needed
      px.key_from_val = 1;
      rc = nviews > 0
               ? launch_onesweep<8, true, false, false, ITK>(L.parts, s, ki, vi, ko, vo, n,
                                                             nullptr, 8 * p, hist + 256 * p, st,
                                                             counters + p, nullptr, 0, info,
                                                             GenSource{}, 8, px)
               : launch_onesweep<8, false, false, false, ITK>(L.parts, s, ki, vi, ko, vo, n,
                                                              nullptr, 8 * p, hist + 256 * p, st,
                                                              counters + p, nullptr, 0, info);
    } else {
      rc = launch_onesweep<8, true, false, false, ITK>(L.parts, s, ki, vi, ko, vo, n, nullptr,
                                                       8 * p, hist + 256 * p, st, counters + p,
                                                       nullptr, 0, info);
    }
    if (rc != PGB_OK) return rc;
  }
  return PGB_OK;
}

// Phase one.  nviews == 0: one image, the depth order ends in v0.  A batch
// (nviews views of n_per_view elements): the fourth depth pass writes the
// views of its values as keys and a fifth pass sorts by view, so the order
// (in v1) is by view, then depth, then id.
static int sort_begin_impl(const float* depth, const int32_t* radius, const int32_t* tiles_touched,
                           int64_t n, int nviews, int64_t n_per_view, void* scratch_n,
                           size_t bytes_n, int64_t* info, void* stream) {
  if (n < 0 || !info || misaligned(info, 8)) return PGB_ERR_INVALID;
  if (n > 0 && (!depth || !radius || !tiles_touched)) return PGB_ERR_INVALID;
  if (n >= (int64_t)kValMask) return PGB_ERR_OVERFLOW;
  const ScratchN L = layout_n(n);
  // the scratch holds uint4 arrays at 256-byte offsets from its start
  if (!scratch_n || bytes_n < L.total || misaligned(scratch_n, 16)) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(info, 0, 2 * sizeof(int64_t), s) != cudaSuccess) return PGB_ERR_CUDA;
  if (cudaMemsetAsync(scratch_n, 0, L.zero_bytes, s) != cudaSuccess) return PGB_ERR_CUDA;
  if (n == 0) return PGB_OK;
  uint32_t* counters = at<uint32_t>(scratch_n, L.counters);
  uint32_t* hist = at<uint32_t>(scratch_n, L.depth_hist);
  uint32_t* status = at<uint32_t>(scratch_n, L.depth_status);
  uint32_t* k0 = at<uint32_t>(scratch_n, L.dk0);
  uint32_t* v0 = at<uint32_t>(scratch_n, L.dv0);
  uint32_t* k1 = at<uint32_t>(scratch_n, L.dk1);
  uint32_t* v1 = at<uint32_t>(scratch_n, L.dv1);
  sort_prepare_kernel<<<stream_grid(n, kSortThreads, 4), kSortThreads, 0, s>>>(
      depth, radius, tiles_touched, n, k0, v0, hist, nviews, n_per_view, counters + kViewsMark,
      info);
  PassViews px{};
  if (nviews > 0) px.vdiv = fast_div((uint32_t)n_per_view);
  const int rc = small_depth_parts(n)
                     ? depth_passes<kDepthIT>(L, s, k0, v0, k1, v1, n, nviews, hist, status,
                                              counters, info, px)
                     : depth_passes<OsCfg<8>::IT>(L, s, k0, v0, k1, v1, n, nviews, hist, status,
                                                  counters, info, px);
  if (rc != PGB_OK) return rc;
  return launch_status();
}

extern "C" {

int pgb_sort_gaussian_begin(const float* depth, const int32_t* radius,
                            const int32_t* tiles_touched, int64_t n, int width, int height,
                            void* scratch_n, size_t bytes_n, int64_t* info, void* stream) {
  if (width <= 0 || height <= 0) return PGB_ERR_INVALID;
  const uint64_t T = (uint64_t)grid_x(width) * (uint64_t)grid_y(height);
  if (T > (1u << (8 * kMaxTilePasses))) return PGB_ERR_INVALID;
  return sort_begin_impl(depth, radius, tiles_touched, n, 0, 0, scratch_n, bytes_n, info, stream);
}

int pgb_sort_gaussian_begin_views(const float* depth, const int32_t* radius,
                                  const int32_t* tiles_touched, int64_t n_per_view, int nviews,
                                  void* scratch_n, size_t bytes_n, int64_t* info, void* stream) {
  if (nviews < 1 || nviews > kMaxViews || n_per_view < 0) return PGB_ERR_INVALID;
  return sort_begin_impl(depth, radius, tiles_touched, n_per_view * nviews, nviews, n_per_view,
                         scratch_n, bytes_n, info, stream);
}

}  // extern "C"

// Phase two for one image or a batch of views (vt), over T global tiles.
// K is the host value k, or (device_k) the count the depth phase left in
// info[0], with every K-sized buffer sized for the capacity k.
// With `list` (n_list entries), the passes run over that band list of
// Gaussians (in depth order) instead of all n in the depth order.
static int sort_finish_impl(const float* uv, const int32_t* radius, const int32_t* tiles_touched,
                            int64_t n, const ViewTable& vt, uint32_t T, int64_t k, bool device_k,
                            void* scratch_n, size_t bytes_n, void* scratch_k, size_t bytes_k,
                            int64_t* info, int32_t* ids_out, int32_t* tile_range_out,
                            void* stream, const uint32_t* list = nullptr, int64_t n_list = 0) {
  if (n < 0 || k < 0 || !info || !tile_range_out) return PGB_ERR_INVALID;
  if (list && (n_list < 0 || n_list > n)) return PGB_ERR_INVALID;
  // uv is read as float2 and the ranges written as int2: 8-byte starts
  if (misaligned(uv, 8) || misaligned(tile_range_out, 8) || misaligned(info, 8))
    return PGB_ERR_INVALID;
  if (n > 0 && (!uv || !radius || (!tiles_touched && !list))) return PGB_ERR_INVALID;
  if (k >= (int64_t)kValMask) return PGB_ERR_OVERFLOW;
  const ScratchN LN = layout_n(n);
  const int64_t n_work = list ? n_list : n;  // elements the rectangle and scan passes visit
  // a batch sorts local tile ids: the plan is that of the largest view
  uint32_t T_local = T;
  if (vt.nviews > 0) {
    T_local = 1;
    for (int v = 0; v < vt.nviews; ++v)
      T_local = std::max<uint32_t>(T_local,
                                   (uint32_t)grid_x(vt.w[v]) * (uint32_t)grid_y_h(vt.h[v], vt.th));
  }
  const TilePlan plan = tile_plan(T_local);
  const ScratchK LK = layout_k(k, plan.passes);
  if (!scratch_n || bytes_n < LN.total || misaligned(scratch_n, 16)) return PGB_ERR_INVALID;
  if (k > 0 && (!scratch_k || bytes_k < LK.total || !ids_out || misaligned(scratch_k, 16)))
    return PGB_ERR_INVALID;
  if (T == 0 || T > (1u << (8 * kMaxTilePasses))) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (k == 0 || n_work == 0) {
    // nothing can be emitted (a device count above 0 overflows the capacity)
    if (cudaMemsetAsync(tile_range_out, 0, (size_t)T * 2 * sizeof(int32_t), s) != cudaSuccess)
      return PGB_ERR_CUDA;
    if (device_k) capacity_check_kernel<<<1, 32, 0, s>>>(info, k, info);
    return launch_status();
  }
  if (cudaMemsetAsync(at<char>(scratch_k, LK.status), 0,
                      (size_t)LK.parts * plan.passes * (1u << plan.bits) * sizeof(uint32_t),
                      s) != cudaSuccess)
    return PGB_ERR_CUDA;
  const int64_t* k_dev = device_k ? info : nullptr;
  uint32_t* counters = at<uint32_t>(scratch_n, LN.counters);
  uint32_t* thist = at<uint32_t>(scratch_n, LN.tile_hist);
  // the depth order (view-major for a batch: begin_views ends in v1), or
  // the band's list of it
  const uint32_t* order = list ? list : at<uint32_t>(scratch_n, vt.nviews > 0 ? LN.dv1 : LN.dv0);
  uint32_t* bufk[2] = {at<uint32_t>(scratch_k, LK.tk0), at<uint32_t>(scratch_k, LK.tk1)};
  uint32_t* bufv[2] = {at<uint32_t>(scratch_k, LK.tv0), at<uint32_t>(scratch_k, LK.tv1)};
  uint32_t* status = at<uint32_t>(scratch_k, LK.status);
  uint4* owner = at<uint4>(scratch_n, LN.owner);
  uint4* rect = at<uint4>(scratch_n, LN.rect);
  uint32_t* chunk_first = at<uint32_t>(scratch_k, LK.chunk_first);
  int2* range = reinterpret_cast<int2*>(tile_range_out);
  rect_kernel<<<stream_grid(n_work), kStreamThreads, 0, s>>>(
      uv, radius, tiles_touched, n_work, vt, plan.passes, plan.bits, rect, thist, info, list);
  const int scan_parts = (int)((n_work + kScanPart - 1) / kScanPart);
  scan_rect_kernel<<<scan_parts, kSortThreads, 0, s>>>(
      order, n_work, rect, k, k_dev, at<uint32_t>(scratch_n, LN.scan_status), counters + 4, owner,
      chunk_first, range, T, counters + kViewsMark, (uint32_t)vt.nviews, info);
  GenSource src;
  src.owner = owner;
  src.chunk_first = chunk_first;
  src.n_sorted = n_work;
  PassViews px{};
  if (vt.nviews > 0) {
    px.vdiv = fast_div((uint32_t)vt.n_per_view);
    px.nviews = vt.nviews;
    for (int v = 0; v < vt.nviews; ++v) px.tile_base[v] = (uint32_t)vt.tile_base[v];
  }
  int cur = 0;
  for (int p = 0; p < plan.passes; ++p) {
    const bool last = p == plan.passes - 1;
    uint32_t* vo = last ? reinterpret_cast<uint32_t*>(ids_out) : bufv[cur ^ 1];
    const int rc = tile_pass(plan, p, LK.parts, s, bufk[cur], bufv[cur], bufk[cur ^ 1], vo, k, k_dev,
                             thist, status, counters + 5 + p, range, T, T_local, info, src, px);
    if (rc != PGB_OK) return rc;
    cur ^= 1;
  }
  range_fix_kernel<<<stream_grid(T), kStreamThreads, 0, s>>>(range, T);
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
  return sort_finish_impl(uv, radius, tiles_touched, n, single_view(width, height), T, k, false,
                          scratch_n, bytes_n, scratch_k, bytes_k, info, ids_out, tile_range_out,
                          stream);
}

int pgb_sort_gaussian_finish_capacity(const float* uv, const int32_t* radius,
                                      const int32_t* tiles_touched, int64_t n, int width,
                                      int height, int64_t k_capacity, void* scratch_n,
                                      size_t bytes_n, void* scratch_k, size_t bytes_k,
                                      int64_t* info, int32_t* ids_out, int32_t* tile_range_out,
                                      void* stream) {
  if (width <= 0 || height <= 0 || grid_x(width) > 65535 || grid_y(height) > 65535)
    return PGB_ERR_INVALID;
  const uint32_t T = (uint32_t)grid_x(width) * (uint32_t)grid_y(height);
  return sort_finish_impl(uv, radius, tiles_touched, n, single_view(width, height), T, k_capacity,
                          true, scratch_n, bytes_n, scratch_k, bytes_k, info, ids_out,
                          tile_range_out, stream);
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
  return sort_finish_impl(uv, radius, tiles_touched, n_per_view * nviews, vt, T, k, false,
                          scratch_n, bytes_n, scratch_k, bytes_k, info, ids_out, tile_range_out,
                          stream);
}

int pgb_sort_gaussian_finish_views_capacity(const float* uv, const int32_t* radius,
                                            const int32_t* tiles_touched, int64_t n_per_view,
                                            const int32_t* sizes, int nviews, int64_t k_capacity,
                                            void* scratch_n, size_t bytes_n, void* scratch_k,
                                            size_t bytes_k, int64_t* info, int32_t* ids_out,
                                            int32_t* tile_range_out, void* stream) {
  ViewTable vt;
  uint32_t T = 0;
  int64_t pixels = 0;
  if (!make_views(sizes, nviews, n_per_view, vt, T, pixels)) return PGB_ERR_INVALID;
  return sort_finish_impl(uv, radius, tiles_touched, n_per_view * nviews, vt, T, k_capacity, true,
                          scratch_n, bytes_n, scratch_k, bytes_k, info, ids_out, tile_range_out,
                          stream);
}

}  // extern "C"

extern "C" {

int pgb_band_tiles(const float* uv, const int32_t* radius, int64_t n, int width, int height,
                   int row0, int row1, int32_t* tiles_out, void* stream) {
  ViewTable vt;
  if (n < 0 || !band_view(width, height, row0, row1, vt)) return PGB_ERR_INVALID;
  if (n > 0 && (!uv || !radius || !tiles_out)) return PGB_ERR_INVALID;
  if (misaligned(uv, 8)) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  band_tiles_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(
      uv, radius, n, grid_x(width), grid_y(height), row0, row1, tiles_out);
  return launch_status();
}

int pgb_sort_gaussian_rebegin(const int32_t* radius, const int32_t* tiles_touched, int64_t n,
                              void* scratch_n, size_t bytes_n, int64_t* info, void* stream) {
  if (n < 0 || !info || misaligned(info, 8)) return PGB_ERR_INVALID;
  if (n > 0 && (!radius || !tiles_touched)) return PGB_ERR_INVALID;
  const ScratchN L = layout_n(n);
  if (!scratch_n || bytes_n < L.total || misaligned(scratch_n, 16)) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  // the depth order stays; phase two's counters, tile histograms and scan
  // status start again from zero
  if (cudaMemsetAsync(info, 0, 2 * sizeof(int64_t), s) != cudaSuccess ||
      cudaMemsetAsync(at<char>(scratch_n, L.counters), 0, L.depth_hist - L.counters, s) !=
          cudaSuccess ||
      cudaMemsetAsync(at<char>(scratch_n, L.tile_hist), 0, L.depth_status - L.tile_hist, s) !=
          cudaSuccess ||
      cudaMemsetAsync(at<char>(scratch_n, L.scan_status), 0, L.zero_bytes - L.scan_status, s) !=
          cudaSuccess)
    return PGB_ERR_CUDA;
  if (n == 0) return PGB_OK;
  band_count_kernel<<<stream_grid(n), kStreamThreads, 0, s>>>(radius, tiles_touched, n, info);
  return launch_status();
}

int pgb_sort_gaussian_finish_band(const float* uv, const int32_t* radius,
                                  const int32_t* tiles_touched, int64_t n, int width, int height,
                                  int row0, int row1, int64_t k, void* scratch_n, size_t bytes_n,
                                  void* scratch_k, size_t bytes_k, int64_t* info, int32_t* ids_out,
                                  int32_t* tile_range_out, void* stream) {
  ViewTable vt;
  if (!band_view(width, height, row0, row1, vt)) return PGB_ERR_INVALID;
  const uint32_t T = (uint32_t)grid_x(width) * (uint32_t)(row1 - row0);
  return sort_finish_impl(uv, radius, tiles_touched, n, vt, T, k, false, scratch_n, bytes_n,
                          scratch_k, bytes_k, info, ids_out, tile_range_out, stream);
}

int pgb_band_counts(const float* uv, const int32_t* radius, int64_t n, int width, int height,
                    const int32_t* bands, int nbands, unsigned long long* counts, void* stream) {
  if (n < 0 || width <= 0 || height <= 0 || nbands < 1 || nbands > kMaxBands || !bands ||
      !counts)
    return PGB_ERR_INVALID;
  if (n > 0 && (!uv || !radius)) return PGB_ERR_INVALID;
  if (misaligned(uv, 8) || misaligned(counts, 8)) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(counts, 0, (size_t)nbands * sizeof(unsigned long long), s) != cudaSuccess)
    return PGB_ERR_CUDA;
  if (n == 0) return PGB_OK;
  band_counts_kernel<<<stream_grid(n), kStreamThreads, 0, s>>>(
      uv, radius, n, grid_x(width), grid_y(height), bands, nbands, counts);
  return launch_status();
}

size_t pgb_band_lists_scratch_bytes(int64_t n, int nbands) {
  if (n < 0 || nbands < 1 || nbands > kMaxListBands) return 0;
  return align256((size_t)nbands * (size_t)std::max(1, list_blocks(n)) * sizeof(uint32_t));
}

static int band_lists_check(const float* uv, const int32_t* radius, int64_t n, int width,
                            int height, const int32_t* rows, int nbands, const void* scratch_n,
                            size_t bytes_n, const void* scratch, size_t scratch_bytes,
                            const int64_t* offsets) {
  if (n < 0 || width <= 0 || height <= 0 || nbands < 1 || nbands > kMaxListBands || !rows ||
      !offsets || misaligned(offsets, 8))
    return PGB_ERR_INVALID;
  if (n > 0 && (!uv || !radius || !scratch_n || !scratch || misaligned(uv, 8) ||
                misaligned(scratch_n, 16)))
    return PGB_ERR_INVALID;
  if (n > 0 && (bytes_n < layout_n(n).total ||
                scratch_bytes < pgb_band_lists_scratch_bytes(n, nbands)))
    return PGB_ERR_INVALID;
  return PGB_OK;
}

int pgb_band_lists_count(const float* uv, const int32_t* radius, int64_t n, int width, int height,
                         const int32_t* rows, int nbands, const void* scratch_n, size_t bytes_n,
                         void* scratch, size_t scratch_bytes, int64_t* offsets, void* stream) {
  const int rc = band_lists_check(uv, radius, n, width, height, rows, nbands, scratch_n, bytes_n,
                                  scratch, scratch_bytes, offsets);
  if (rc != PGB_OK) return rc;
  cudaStream_t s = as_stream(stream);
  if (n == 0)
    return cudaMemsetAsync(offsets, 0, (size_t)(nbands + 1) * sizeof(int64_t), s) == cudaSuccess
               ? PGB_OK
               : PGB_ERR_CUDA;
  const int nblocks = list_blocks(n);
  uint32_t* counts = static_cast<uint32_t*>(scratch);
  const uint32_t* order = at<uint32_t>(const_cast<void*>(scratch_n), layout_n(n).dv0);
  band_list_count_kernel<<<nblocks, kListThreads, 0, s>>>(order, uv, radius, n, grid_x(width),
                                                          grid_y(height), rows, nbands, counts);
  band_list_scan_kernel<<<nbands, kListThreads, 0, s>>>(counts, nblocks, offsets);
  band_list_offsets_kernel<<<1, 32, 0, s>>>(offsets, nbands);
  return launch_status();
}

int pgb_band_lists_write(const float* uv, const int32_t* radius, int64_t n, int width, int height,
                         const int32_t* rows, int nbands, const void* scratch_n, size_t bytes_n,
                         const void* scratch, size_t scratch_bytes, const int64_t* offsets,
                         int32_t* lists, void* stream) {
  const int rc = band_lists_check(uv, radius, n, width, height, rows, nbands, scratch_n, bytes_n,
                                  scratch, scratch_bytes, offsets);
  if (rc != PGB_OK) return rc;
  if (n == 0) return PGB_OK;
  if (!lists) return PGB_ERR_INVALID;
  const uint32_t* order = at<uint32_t>(const_cast<void*>(scratch_n), layout_n(n).dv0);
  band_list_write_kernel<<<list_blocks(n), kListThreads, 0, as_stream(stream)>>>(
      order, uv, radius, n, grid_x(width), grid_y(height), rows, nbands,
      static_cast<const uint32_t*>(scratch), offsets, reinterpret_cast<uint32_t*>(lists));
  return launch_status();
}

int pgb_sort_gaussian_finish_band_list(const float* uv, const int32_t* radius, int64_t n,
                                       int width, int height, int row0, int row1, int64_t k,
                                       const int32_t* list, int64_t n_list, void* scratch_n,
                                       size_t bytes_n, void* scratch_k, size_t bytes_k,
                                       int64_t* info, int32_t* ids_out, int32_t* tile_range_out,
                                       void* stream) {
  ViewTable vt;
  if (!band_view(width, height, row0, row1, vt)) return PGB_ERR_INVALID;
  if (n < 0 || n_list < 0 || n_list > n || !info || misaligned(info, 8)) return PGB_ERR_INVALID;
  if (n_list > 0 && !list) return PGB_ERR_INVALID;
  const ScratchN L = layout_n(n);
  if (!scratch_n || bytes_n < L.total || misaligned(scratch_n, 16)) return PGB_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  // the depth order stays; phase two's counters, tile histograms and scan
  // status start again from zero (as pgb_sort_gaussian_rebegin)
  if (cudaMemsetAsync(info, 0, 2 * sizeof(int64_t), s) != cudaSuccess ||
      cudaMemsetAsync(at<char>(scratch_n, L.counters), 0, L.depth_hist - L.counters, s) !=
          cudaSuccess ||
      cudaMemsetAsync(at<char>(scratch_n, L.tile_hist), 0, L.depth_status - L.tile_hist, s) !=
          cudaSuccess ||
      cudaMemsetAsync(at<char>(scratch_n, L.scan_status), 0, L.zero_bytes - L.scan_status, s) !=
          cudaSuccess)
    return PGB_ERR_CUDA;
  const uint32_t T = (uint32_t)grid_x(width) * (uint32_t)(row1 - row0);
  return sort_finish_impl(uv, radius, nullptr, n, vt, T, k, false, scratch_n, bytes_n, scratch_k,
                          bytes_k, info, ids_out, tile_range_out, stream,
                          reinterpret_cast<const uint32_t*>(list), n_list);
}

int pgb_tile_counts_views(const float* uv, const int32_t* radius, int64_t n_per_view,
                          const int32_t* sizes, int nviews, int tile_height, int32_t* tiles_out,
                          void* stream) {
  ViewTable vt;
  uint32_t T = 0;
  int64_t pixels = 0;
  if (!make_views(sizes, nviews, n_per_view, vt, T, pixels, tile_height)) return PGB_ERR_INVALID;
  const int64_t n = n_per_view * nviews;
  if (n > 0 && (!uv || !radius || !tiles_out || misaligned(uv, 8))) return PGB_ERR_INVALID;
  if (n == 0) return PGB_OK;
  view_tiles_kernel<<<stream_grid(n), kStreamThreads, 0, as_stream(stream)>>>(uv, radius, n, vt,
                                                                              tiles_out);
  return launch_status();
}

int pgb_sort_gaussian_finish_views_h(const float* uv, const int32_t* radius,
                                     const int32_t* tiles_touched, int64_t n_per_view,
                                     const int32_t* sizes, int nviews, int tile_height, int64_t k,
                                     int k_on_device, void* scratch_n, size_t bytes_n,
                                     void* scratch_k, size_t bytes_k, int64_t* info,
                                     int32_t* ids_out, int32_t* tile_range_out, void* stream) {
  ViewTable vt;
  uint32_t T = 0;
  int64_t pixels = 0;
  if (!make_views(sizes, nviews, n_per_view, vt, T, pixels, tile_height)) return PGB_ERR_INVALID;
  return sort_finish_impl(uv, radius, tiles_touched, n_per_view * nviews, vt, T, k,
                          k_on_device != 0, scratch_n, bytes_n, scratch_k, bytes_k, info, ids_out,
                          tile_range_out, stream);
}

}  // extern "C"
