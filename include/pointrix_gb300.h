/*
 * pointrix_gb300 -- C ABI of the GB300 (sm_103a) msplat operator kernels.
 *
 * Each entry point replaces one operator of the msplat CUDA extension that
 * Pointrix's MsplatRender calls (pointrix/model/renderer/msplat.py:94-151;
 * the same six calls in examples/supervise/renderer.py:42-85), split into a
 * forward and a backward half so that any host language can bind it.  The
 * Python binding (pointrix_gb300/ops.py) wraps each pair in a
 * torch.autograd.Function with msplat's signature.
 *
 * Conventions for every call:
 *  - all pointers are device pointers (unless stated), float32 unless typed
 *    otherwise, densely packed row-major ([N,3] means 3 floats per row);
 *  - `stream` is a cudaStream_t passed as void*; work is enqueued on it and
 *    the call returns without synchronising (unless stated);
 *  - nothing is allocated and no caller memory is freed: scratch is passed
 *    in, sized by the matching *_scratch_bytes query;
 *  - a buffer may be NULL only where its entry point says so, or when its
 *    array is empty; otherwise the call returns PGB_ERR_INVALID before any
 *    CUDA call.  Arrays the kernels access with vector loads or stores must
 *    start on that vector's boundary, else PGB_ERR_INVALID: 8 bytes for
 *    [N,2] arrays (uv, d_uv), cov3d [N,6], tile ranges [T,2] and the int64
 *    `info` words; 16 bytes for quaternions [N,4], blend records, gradient
 *    records and sort scratch (allocations from cudaMalloc or the torch
 *    allocator always are);
 *  - the return value is a PGB_* status; a non-zero value means nothing
 *    useful was written.  Device-side faults that can only be seen after the
 *    kernels ran are reported through the `info` words named below.
 */
#ifndef POINTRIX_GB300_H
#define POINTRIX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PGB_OK = 0,
  PGB_ERR_INVALID = 1,   /* bad size, shape, pointer or scratch too small */
  PGB_ERR_CUDA = 2,      /* a CUDA API call or kernel launch failed */
  PGB_ERR_OVERFLOW = 3,  /* a device-side bound was exceeded */
  PGB_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up */
  PGB_ERR_MISMATCH = 5   /* tiles_touched disagrees with the uv/radius rectangles */
};

/* Human-readable name of a status code (static string). */
const char* pgb_status_string(int status);
/* ABI version of this library; bumped on any signature change. */
int pgb_abi_version(void);

/* ---------------------------------------------------------------------
 * compute_sh -- replaces msplat.compute_sh
 * (pointrix/model/renderer/msplat.py:104, examples/supervise/renderer.py:42)
 * sh is [N,3,K] addressed through element strides (sn, sc, sk), so the
 * permuted view that render_iter passes (strides 3K,1,3) is read in place;
 * K in {1,4,9,16}.  dirs [N,3] unit view directions.  rgb [N,3] is the raw
 * SH sum (no +0.5, no clamp).  The backward writes d_sh with the same
 * strides as sh, and d_dirs [N,3].
 * ------------------------------------------------------------------- */
int pgb_compute_sh_forward(const float* sh, int64_t n, int k, int64_t sn, int64_t sc, int64_t sk,
                           const float* dirs, float* rgb, void* stream);
int pgb_compute_sh_backward(const float* sh, int64_t n, int k, int64_t sn, int64_t sc, int64_t sk,
                            const float* dirs, const float* d_rgb, float* d_sh, float* d_dirs,
                            void* stream);

/* ---------------------------------------------------------------------
 * project_point -- replaces msplat.project_point
 * (pointrix/model/renderer/msplat.py:109-113)
 * xyz [N,3]; intr [4] = fx,fy,cx,cy; extr [3,4] world->camera.
 * uv [N,2], depth [N,1]; culled points (depth <= nearest, or centre outside
 * `extent` times the half image) get uv = 0, depth = 0.
 * The backward writes d_xyz [N,3], d_intr [4], d_extr [12]; it needs
 * pgb_camera_grad_scratch_bytes() bytes of scratch.
 * ------------------------------------------------------------------- */
size_t pgb_camera_grad_scratch_bytes(void);
int pgb_project_point_forward(const float* xyz, int64_t n, const float* intr, const float* extr,
                              int width, int height, float nearest, float extent,
                              float* uv, float* depth, void* stream);
int pgb_project_point_backward(const float* xyz, int64_t n, const float* intr, const float* extr,
                               int width, int height, float nearest, float extent,
                               const float* d_uv, const float* d_depth,
                               float* d_xyz, float* d_intr, float* d_extr,
                               void* scratch, size_t scratch_bytes, void* stream);

/* ---------------------------------------------------------------------
 * compute_cov3d -- replaces msplat.compute_cov3d
 * (pointrix/model/renderer/msplat.py:118)
 * scales [N,3] (activated), uquats [N,4] unit wxyz, visible [N] bytes
 * (0/1).  cov3d [N,6] = upper triangle xx,xy,xz,yy,yz,zz of R S S^T R^T.
 * ------------------------------------------------------------------- */
int pgb_compute_cov3d_forward(const float* scales, const float* uquats, const uint8_t* visible,
                              int64_t n, float* cov3d, void* stream);
int pgb_compute_cov3d_backward(const float* scales, const float* uquats, const uint8_t* visible,
                               int64_t n, const float* d_cov3d, float* d_scales, float* d_uquats,
                               void* stream);

/* ---------------------------------------------------------------------
 * ewa_project -- replaces msplat.ewa_project
 * (pointrix/model/renderer/msplat.py:121-130)
 * conic [N,3] (inverse 2D covariance a,b,c), radius [N] int32 (pixels),
 * tiles_touched [N] int32 (16x16 tiles).  The backward takes the forward's
 * radius (0 = culled) and writes d_xyz [N,3], d_cov3d [N,6], d_intr [4],
 * d_extr [12]; scratch as for project_point.
 * ------------------------------------------------------------------- */
int pgb_ewa_project_forward(const float* xyz, const float* cov3d, const float* intr,
                            const float* extr, const float* uv, const uint8_t* visible, int64_t n,
                            int width, int height, float* conic, int32_t* radius,
                            int32_t* tiles_touched, void* stream);
int pgb_ewa_project_backward(const float* xyz, const float* cov3d, const float* intr,
                             const float* extr, const int32_t* radius, int64_t n, int width,
                             int height, const float* d_conic, float* d_xyz, float* d_cov3d,
                             float* d_intr, float* d_extr, void* scratch, size_t scratch_bytes,
                             void* stream);

/* ---------------------------------------------------------------------
 * sort_gaussian -- replaces msplat.sort_gaussian
 * (pointrix/model/renderer/msplat.py:133-135)
 * Two calls, because the output length K = sum(tiles_touched) is only known
 * on the device:
 *   1. pgb_sort_gaussian_begin writes info[0] = K and info[1] = 0 (int64
 *      device words) and sorts the Gaussians by depth in scratch_n;
 *   2. the caller reads K back, then pgb_sort_gaussian_finish writes
 *      ids_out [K] int32 (Gaussian ids ordered by tile, then depth, then id)
 *      and tile_range_out [T,2] int32 ([start,end) per 16x16 tile, [0,0] if
 *      empty, T = ceil(W/16) * ceil(H/16)).
 * After finish, info[1] holds a PGB_* status raised on the device
 * (PGB_ERR_TIMEOUT, PGB_ERR_MISMATCH, PGB_ERR_OVERFLOW) or 0.
 * Scratch: bytes_n for (n), bytes_k for (k); pass k = 0 to size bytes_n.
 * bytes_k depends on the tile count of (width, height); for a batch of
 * views pass any (width, height) with the batch's total tile count
 * (e.g. 16 T x 16).
 * ------------------------------------------------------------------- */
int pgb_sort_scratch_bytes(int64_t n, int64_t k, int width, int height, size_t* bytes_n,
                           size_t* bytes_k);
int pgb_sort_gaussian_begin(const float* depth, const int32_t* radius,
                            const int32_t* tiles_touched, int64_t n, int width, int height,
                            void* scratch_n, size_t bytes_n, int64_t* info, void* stream);
int pgb_sort_gaussian_finish(const float* uv, const int32_t* radius, const int32_t* tiles_touched,
                             int64_t n, int width, int height, int64_t k, void* scratch_n,
                             size_t bytes_n, void* scratch_k, size_t bytes_k, int64_t* info,
                             int32_t* ids_out, int32_t* tile_range_out, void* stream);

/* ---------------------------------------------------------------------
 * pgb_sort_gaussian_finish_capacity -- no counterpart in the reference
 * (whose sort_gaussian, pointrix/model/renderer/msplat.py:133-135, always
 * returns K-sized outputs).  Phase two without the host read-back of K:
 * K is read on the device from info[0] (left there by
 * pgb_sort_gaussian_begin), and every K-sized buffer (scratch_k from
 * pgb_sort_scratch_bytes(n, k_capacity, ...), ids_out [k_capacity]) is
 * sized for the capacity.  Only ids_out[0 .. K) is written; tile_range_out
 * is the same as with pgb_sort_gaussian_finish.  A K above k_capacity sets
 * info[1] = PGB_ERR_OVERFLOW and leaves every tile range [0,0].  Nothing on
 * the host depends on device data, so begin + finish_capacity can be
 * captured in a CUDA graph.
 * ------------------------------------------------------------------- */
int pgb_sort_gaussian_finish_capacity(const float* uv, const int32_t* radius,
                                      const int32_t* tiles_touched, int64_t n, int width,
                                      int height, int64_t k_capacity, void* scratch_n,
                                      size_t bytes_n, void* scratch_k, size_t bytes_k,
                                      int64_t* info, int32_t* ids_out, int32_t* tile_range_out,
                                      void* stream);

/* ---------------------------------------------------------------------
 * pgb_sort_gaussian_noalloc -- no counterpart in the reference.
 * The same result as pgb_sort_gaussian_begin + finish, for callers that
 * cannot allocate device memory: code running inside a host application that
 * owns the GPU memory budget, or that must not enter the CUDA allocator on
 * its hot path (cudaMalloc synchronises the device and may fail under memory
 * pressure).  Its scratch is a static device array of
 * PGB_NOALLOC_SCRATCH_BYTES (24 MiB) that every GPU loading this library
 * holds until the process exits; the call allocates nothing.
 * Limits: n <= PGB_NOALLOC_MAX_GAUSSIANS (262,144), else PGB_ERR_INVALID
 * before any GPU work; K (sum of tiles_touched) must fit the rest of the
 * array (about 1.0 million entries at the largest n) and ids_capacity, else
 * PGB_ERR_OVERFLOW with *k_out (host, may be NULL) set to the K needed.
 * Synchronous: returns when the results are complete on `stream`; a
 * device-side fault comes back as the return value.  The first call on a
 * device looks up the array's device address (with that device current).
 * Under CUDA's lazy module
 * loading (the default since CUDA 12.2) that first call is also when the
 * library's device code, and with it the array, is set up on the device, so
 * it can fail with PGB_ERR_CUDA when device memory is short: make one warm-up
 * call per device at start-up, before the memory budget is tight (or load
 * modules eagerly with CUDA_MODULE_LOADING=EAGER).  All calls share the one
 * array (each clears what must start at zero): calls that overlap on the GPU,
 * e.g. from two streams or threads, race and must be serialised by the
 * caller.
 * ------------------------------------------------------------------- */
#define PGB_NOALLOC_MAX_GAUSSIANS 262144
#define PGB_NOALLOC_SCRATCH_BYTES (24u << 20)
int pgb_sort_gaussian_noalloc(const float* uv, const float* depth, const int32_t* radius,
                              const int32_t* tiles_touched, int64_t n, int width, int height,
                              int32_t* ids_out, int64_t ids_capacity, int32_t* tile_range_out,
                              int64_t* k_out, void* stream);

/* ---------------------------------------------------------------------
 * alpha_blending -- replaces msplat.alpha_blending
 * (pointrix/model/renderer/msplat.py:148-151)
 * uv [N,2], conic [N,3], opacity [N,1], feature [N,C] (1 <= C <= 26),
 * ids [K], tile_range [T,2] from sort_gaussian, bg added to every channel
 * with the final transmittance.  The forward packs one record of
 * pgb_blend_record_floats(C) floats per Gaussian into `records` (kept for
 * the backward) and writes out [C,H,W], final_T [H,W] and n_contrib [H,W]
 * (list entries up to the last contributor).  The backward writes d_uv
 * [N,2] (also the gradient msplat routes to its `ndc` argument), d_conic
 * [N,3], d_opacity [N,1], d_feature [N,C]; grad_records is scratch of
 * N * pgb_blend_grad_record_floats(C) floats.  `info` is one device int64 word that the caller
 * zeroes beforehand; a bounded device-side wait that expires writes
 * PGB_ERR_TIMEOUT into it (info may be NULL: that status is then dropped).
 * ------------------------------------------------------------------- */
int pgb_blend_record_floats(int channels);
/* Floats per Gaussian of the backward's gradient scratch (16 or 32). */
int pgb_blend_grad_record_floats(int channels);
int pgb_alpha_blending_forward(const float* uv, const float* conic, const float* opacity,
                               const float* feature, int64_t n, int channels, const int32_t* ids,
                               int64_t k, const int32_t* tile_range, float bg, int width,
                               int height, float* records, float* out, float* final_T,
                               int32_t* n_contrib, int64_t* info, void* stream);
int pgb_alpha_blending_backward(const float* records, int64_t n, int channels,
                                const int32_t* ids, int64_t k, const int32_t* tile_range, float bg,
                                int width, int height, const float* final_T,
                                const int32_t* n_contrib, const float* d_out, float* grad_records,
                                float* d_uv, float* d_conic, float* d_opacity, float* d_feature,
                                int64_t* info, void* stream);

/* ---------------------------------------------------------------------
 * Multi-view batches -- replace the per-view loop of MsplatRender.render_batch
 * (pointrix/model/renderer/msplat.py:185-193): the sort and the blend of V
 * views run as one launch sequence each.  Per-Gaussian arrays hold
 * V * n_per_view elements, element g belonging to view g / n_per_view;
 * `sizes` is a HOST array of V (width, height) pairs, 1 <= V <= 64.  The
 * views own consecutive ranges of one 16x16 tile index space (T = sum of
 * the views' tile counts <= 2^24, tile_range has T rows) and per-pixel
 * arrays hold the views one after another (out: per-view [C,H,W] blocks;
 * final_T, n_contrib: per-view [H,W] blocks).  Phase one of the sort is
 * pgb_sort_gaussian_begin_views (which orders the elements by view, then
 * depth, then id; the finish_views entries require it: a finish after the
 * other kind of phase one sets info[1] = PGB_ERR_INVALID, and its outputs
 * are then undefined).  The batch's pairs
 * are then sorted by their view-local tile id, so ids_out holds, for every
 * local tile t, the lists of view 0, 1, ... one after another, and
 * tile_range_out[tile_base(v) + t] is view v's list of tile t; within a list
 * the order is depth, then element id, so each view's image equals
 * rendering it alone.  Scratch: pgb_sort_scratch_bytes with the largest
 * view's tile count (e.g. width 16 T_v, height 16).
 * ------------------------------------------------------------------- */
int pgb_sort_gaussian_begin_views(const float* depth, const int32_t* radius,
                                  const int32_t* tiles_touched, int64_t n_per_view, int nviews,
                                  void* scratch_n, size_t bytes_n, int64_t* info, void* stream);
int pgb_sort_gaussian_finish_views(const float* uv, const int32_t* radius,
                                   const int32_t* tiles_touched, int64_t n_per_view,
                                   const int32_t* sizes, int nviews, int64_t k, void* scratch_n,
                                   size_t bytes_n, void* scratch_k, size_t bytes_k, int64_t* info,
                                   int32_t* ids_out, int32_t* tile_range_out, void* stream);
/* The batch form of pgb_sort_gaussian_finish_capacity (K on the device). */
int pgb_sort_gaussian_finish_views_capacity(const float* uv, const int32_t* radius,
                                            const int32_t* tiles_touched, int64_t n_per_view,
                                            const int32_t* sizes, int nviews, int64_t k_capacity,
                                            void* scratch_n, size_t bytes_n, void* scratch_k,
                                            size_t bytes_k, int64_t* info, int32_t* ids_out,
                                            int32_t* tile_range_out, void* stream);
int pgb_alpha_blending_forward_views(const float* uv, const float* conic, const float* opacity,
                                     const float* feature, int64_t n_per_view, int channels,
                                     const int32_t* ids, int64_t k, const int32_t* tile_range,
                                     float bg, const int32_t* sizes, int nviews, float* records,
                                     float* out, float* final_T, int32_t* n_contrib,
                                     int64_t* info, void* stream);
int pgb_alpha_blending_backward_views(const float* records, int64_t n_per_view, int channels,
                                      const int32_t* ids, int64_t k, const int32_t* tile_range,
                                      float bg, const int32_t* sizes, int nviews,
                                      const float* final_T, const int32_t* n_contrib,
                                      const float* d_out, float* grad_records, float* d_uv,
                                      float* d_conic, float* d_opacity, float* d_feature,
                                      int64_t* info, void* stream);

/* The four blend entry points with the kernel variant chosen by the caller
 * (the run-time autotuner of pointrix_gb300.autotune).  Forward: 64 or 128
 * records per batch, plus 2048 for the compositing step without per-pixel
 * branches.  Backward: 64, 128 or 256 records per batch with two pixels per
 * thread, or 4096 + 32 / 64 / 128 for four pixels per thread (64 threads per
 * tile, 8x16 pixel boxes per warp); 8192 + 64, 8192 + 512 + 32 and 8192 +
 * 1024 + 32 select the second four-pixel form (d_out in shared memory,
 * packed f32x2 accumulation; butterfly or transposed per-splat reduction; at
 * most 85 registers for the last), 8192 + 2048 + 32 / 64 (and + 1024, at
 * most 102 registers) its replay without per-pixel branches; 16384 + 32 /
 * 64 (and 16384 + 1024 + 32, 16384 + 2048 + 32 at 102 / 85 registers) one
 * warp per 8x16 half as its own CTA; 32768 + 32 one warp per 16x16 tile,
 * eight pixels per lane.  The later forms take up to eight channels; wider
 * features (and, except the one-warp-per-tile form, 16 x 32 tiles) use the
 * first form with the same batch.  0 = the default (128, two pixels per
 * thread).  Every variant gives the same images, final transmittance and
 * contributor counts; the backward's gradient sums are formed in a
 * variant-dependent order (float atomics).
 * pgb_blend_batches(backward, out) lists the compiled variants (returns
 * their count, writes them to out if not NULL). */
int pgb_alpha_blending_forward_with_batch(const float* uv, const float* conic,
                                          const float* opacity, const float* feature, int64_t n,
                                          int channels, const int32_t* ids, int64_t k,
                                          const int32_t* tile_range, float bg, int width,
                                          int height, float* records, float* out, float* final_T,
                                          int32_t* n_contrib, int64_t* info, void* stream,
                                          int batch);
int pgb_alpha_blending_backward_with_batch(const float* records, int64_t n, int channels,
                                           const int32_t* ids, int64_t k,
                                           const int32_t* tile_range, float bg, int width,
                                           int height, const float* final_T,
                                           const int32_t* n_contrib, const float* d_out,
                                           float* grad_records, float* d_uv, float* d_conic,
                                           float* d_opacity, float* d_feature, int64_t* info,
                                           void* stream, int batch);
int pgb_alpha_blending_forward_views_with_batch(
    const float* uv, const float* conic, const float* opacity, const float* feature,
    int64_t n_per_view, int channels, const int32_t* ids, int64_t k, const int32_t* tile_range,
    float bg, const int32_t* sizes, int nviews, float* records, float* out, float* final_T,
    int32_t* n_contrib, int64_t* info, void* stream, int batch);
int pgb_alpha_blending_backward_views_with_batch(
    const float* records, int64_t n_per_view, int channels, const int32_t* ids, int64_t k,
    const int32_t* tile_range, float bg, const int32_t* sizes, int nviews, const float* final_T,
    const int32_t* n_contrib, const float* d_out, float* grad_records, float* d_uv,
    float* d_conic, float* d_opacity, float* d_feature, int64_t* info, void* stream, int batch);
int pgb_blend_batches(int backward, int32_t* out);

/* ---------------------------------------------------------------------
 * Tiles 16 pixels wide and 32 high for a batch of views -- no counterpart
 * in the reference (the batched multi-view path chooses its tile shape; the
 * drop-in operators keep msplat's 16 x 16 tiles).  A 16 x 32 tile's list
 * holds every splat whose 16 x 32 tile rectangle covers it; the blend keeps,
 * per 8-pixel box, exactly the splats whose 16 x 16 rectangle covers the
 * box's 16 x 16 tile, so the images and gradients are those of 16 x 16
 * tiles, with fewer (tile, splat) entries to sort.
 *
 * pgb_tile_counts_views: tiles_out [V*N] = entries of each element for
 * 16 x tile_height tiles (the tiles_touched of the sort below).
 * pgb_sort_gaussian_finish_views_h: pgb_sort_gaussian_finish_views (k_on_device
 * = 0) or _capacity (k_on_device != 0, k the capacity) for 16 x tile_height
 * tiles; tile_range covers the views' 16 x tile_height tiles.
 * pgb_alpha_blending_forward/backward_views_h: the views' blend for those
 * lists; radius [V*N] is required for tile_height 32 (RGB, RGB + depth and
 * RGB + depth + normal channel counts).  pgb_blend_batches_h lists the
 * forward batches of 16 x tile_height tiles (32: 64, 128, 256, and 2048 +
 * 128 / 256 without per-pixel branches).
 * tile_height is 16 or 32.
 * ------------------------------------------------------------------- */
int pgb_tile_counts_views(const float* uv, const int32_t* radius, int64_t n_per_view,
                          const int32_t* sizes, int nviews, int tile_height, int32_t* tiles_out,
                          void* stream);
int pgb_sort_gaussian_finish_views_h(const float* uv, const int32_t* radius,
                                     const int32_t* tiles_touched, int64_t n_per_view,
                                     const int32_t* sizes, int nviews, int tile_height, int64_t k,
                                     int k_on_device, void* scratch_n, size_t bytes_n,
                                     void* scratch_k, size_t bytes_k, int64_t* info,
                                     int32_t* ids_out, int32_t* tile_range_out, void* stream);
int pgb_alpha_blending_forward_views_h(const float* uv, const float* conic, const float* opacity,
                                       const float* feature, int64_t n_per_view, int channels,
                                       const int32_t* ids, int64_t k, const int32_t* tile_range,
                                       float bg, const int32_t* sizes, int nviews,
                                       int tile_height, const int32_t* radius, float* records,
                                       float* out, float* final_T, int32_t* n_contrib,
                                       int64_t* info, void* stream, int batch);
int pgb_alpha_blending_backward_views_h(const float* records, int64_t n_per_view, int channels,
                                        const int32_t* ids, int64_t k, const int32_t* tile_range,
                                        float bg, const int32_t* sizes, int nviews,
                                        int tile_height, const int32_t* radius,
                                        const float* final_T, const int32_t* n_contrib,
                                        const float* d_out, float* grad_records, float* d_uv,
                                        float* d_conic, float* d_opacity, float* d_feature,
                                        int64_t* info, void* stream, int batch);
int pgb_blend_batches_h(int backward, int tile_height, int32_t* out);

/* ---------------------------------------------------------------------
 * Bands of tile rows -- no counterpart in the reference.  They serve the
 * recompute-in-backward mode of large views (ops.rasterize(recompute=True)):
 * one image is sorted and blended one band of tile rows [row0, row1) at a
 * time, so the K-sized sort buffers and id list hold one band's entries
 * instead of the whole image's.  The per-tile lists, images, contributor
 * counts and gradients equal those of the whole-image calls.
 *
 * pgb_band_tiles: tiles_out[g] = entries of Gaussian g inside the band (its
 * tile rectangle clipped to the rows; 0 for radius <= 0).
 * pgb_sort_gaussian_rebegin: after a pgb_sort_gaussian_begin on the same
 * Gaussians (whose depth order scratch_n keeps), prepares phase two for
 * another band: sums the band's tiles_touched into info[0] (K of the band)
 * and clears what phase two counts in.
 * pgb_sort_gaussian_finish_band: phase two for the band, K = k: ids [k] and
 * tile_range [gx * (row1 - row0), 2] with band-local tile ids (row r of the
 * band is tile row row0 + r); scratch as pgb_sort_scratch_bytes(n, k, width,
 * height) gives for the whole image.
 * pgb_alpha_blending_forward_band / _backward_band: the blend of the band's
 * tiles, reading that tile_range, writing (reading) only the band's pixels
 * of the whole-image out, final_T, n_contrib (d_out).  Forward: pack = 0
 * reuses records packed by an earlier band's call.  Backward: first != 0
 * zeroes grad_records, last != 0 unpacks the gradients summed over all bands
 * (d_uv, d_conic, d_opacity, d_feature may be NULL while last == 0).
 * ------------------------------------------------------------------- */
int pgb_band_tiles(const float* uv, const int32_t* radius, int64_t n, int width, int height,
                   int row0, int row1, int32_t* tiles_out, void* stream);
/* K of every band at once: bands (device int32 [nbands + 1], increasing
 * tile rows; band b is rows [bands[b], bands[b + 1])), counts (device
 * uint64 [nbands], overwritten).  nbands <= 1024. */
int pgb_band_counts(const float* uv, const int32_t* radius, int64_t n, int width, int height,
                    const int32_t* bands, int nbands, unsigned long long* counts, void* stream);
int pgb_sort_gaussian_rebegin(const int32_t* radius, const int32_t* tiles_touched, int64_t n,
                              void* scratch_n, size_t bytes_n, int64_t* info, void* stream);
int pgb_sort_gaussian_finish_band(const float* uv, const int32_t* radius,
                                  const int32_t* tiles_touched, int64_t n, int width, int height,
                                  int row0, int row1, int64_t k, void* scratch_n, size_t bytes_n,
                                  void* scratch_k, size_t bytes_k, int64_t* info, int32_t* ids_out,
                                  int32_t* tile_range_out, void* stream);
/* Band lists: the band path above visits all n Gaussians in every band's
 * phase two.  These calls build, once per image, each band's list of the
 * Gaussians with at least one entry in it, in the depth order that
 * pgb_sort_gaussian_begin left in scratch_n (bytes_n for n), so that each
 * band's phase two visits only its own Gaussians:
 * pgb_band_lists_count: rows (device int32 [nbands + 1], increasing tile
 * rows; nbands <= 256), scratch of pgb_band_lists_scratch_bytes(n, nbands)
 * bytes; writes offsets (device int64 [nbands + 1]): band b's list is
 * lists[offsets[b] .. offsets[b + 1]).  The caller reads offsets[nbands]
 * (the total) back to size lists.
 * pgb_band_lists_write: the same arguments after the count, writes lists
 * (device int32 [offsets[nbands]], Gaussian ids).
 * pgb_sort_gaussian_finish_band_list: phase two for band rows [row0, row1)
 * with K = k over that band's list (list [n_list]); clears what phase two
 * counts in (no pgb_sort_gaussian_rebegin or pgb_band_tiles needed).  ids
 * and tile_range equal pgb_sort_gaussian_finish_band's bit for bit. */
size_t pgb_band_lists_scratch_bytes(int64_t n, int nbands);
int pgb_band_lists_count(const float* uv, const int32_t* radius, int64_t n, int width, int height,
                         const int32_t* rows, int nbands, const void* scratch_n, size_t bytes_n,
                         void* scratch, size_t scratch_bytes, int64_t* offsets, void* stream);
int pgb_band_lists_write(const float* uv, const int32_t* radius, int64_t n, int width, int height,
                         const int32_t* rows, int nbands, const void* scratch_n, size_t bytes_n,
                         const void* scratch, size_t scratch_bytes, const int64_t* offsets,
                         int32_t* lists, void* stream);
int pgb_sort_gaussian_finish_band_list(const float* uv, const int32_t* radius, int64_t n,
                                       int width, int height, int row0, int row1, int64_t k,
                                       const int32_t* list, int64_t n_list, void* scratch_n,
                                       size_t bytes_n, void* scratch_k, size_t bytes_k,
                                       int64_t* info, int32_t* ids_out, int32_t* tile_range_out,
                                       void* stream);
int pgb_alpha_blending_forward_band(const float* uv, const float* conic, const float* opacity,
                                    const float* feature, int64_t n, int channels,
                                    const int32_t* ids, int64_t k, const int32_t* tile_range,
                                    float bg, int width, int height, int row0, int row1, int pack,
                                    float* records, float* out, float* final_T,
                                    int32_t* n_contrib, int64_t* info, void* stream, int batch);
int pgb_alpha_blending_backward_band(const float* records, int64_t n, int channels,
                                     const int32_t* ids, int64_t k, const int32_t* tile_range,
                                     float bg, int width, int height, int row0, int row1,
                                     const float* final_T, const int32_t* n_contrib,
                                     const float* d_out, float* grad_records, int first, int last,
                                     float* d_uv, float* d_conic, float* d_opacity,
                                     float* d_feature, int64_t* info, void* stream, int batch);

/* pgb_blend_pair_census -- no counterpart in the reference: a measurement
 * aid, not part of the training path.  For the blend a forward call made
 * (its records, sorted ids, tile ranges and n_contrib [H,W]), adds to
 * counts[0] (device, uint64) the list entries up to each pixel's last
 * contributor -- the (pixel, splat) pairs the backward replays -- and to
 * counts[1] the composited ones among them (alpha >= 1/255 by the forward's
 * own test on the record).  The caller zeroes counts.  One launch. */
int pgb_blend_pair_census(const float* records, int channels, int64_t n, const int32_t* ids,
                          int64_t k, const int32_t* tile_range, int width, int height,
                          const int32_t* n_contrib, unsigned long long* counts, void* stream);

/* Camera pose (the camera model around the path,
 * pointrix/utils/pose.py:40-84): world_to_camera [4,4] row-major and the
 * camera centre [3] from a wxyz quaternion [4] (normalised) and a
 * translation [3]; the backward takes d_world_to_camera and d_centre (either
 * may be NULL) and writes d_quat [4], d_translation [3].  One single-block
 * launch each way. */
int pgb_camera_pose_forward(const float* quat, const float* translation, float* world_to_camera,
                            float* centre, void* stream);
int pgb_camera_pose_backward(const float* quat, const float* translation,
                             const float* d_world_to_camera, const float* d_centre, float* d_quat,
                             float* d_translation, void* stream);

/* Feature pieces (no counterpart in the reference): the single-view blend
 * with the [N,C] feature given as npieces [N,w_p] row-major device tensors
 * (pieces / widths are HOST arrays; sum of widths = C <= 26), e.g. rgb,
 * depth and a normal without concatenating them; the backward writes each
 * piece's gradient to d_pieces[p] ([N,w_p]).  Same results as the [N,C]
 * entry points on the concatenation; `batch` as above. */
int pgb_alpha_blending_forward_pieces(const float* uv, const float* conic, const float* opacity,
                                      const float* const* pieces, const int32_t* widths,
                                      int npieces, int64_t n, const int32_t* ids, int64_t k,
                                      const int32_t* tile_range, float bg, int width, int height,
                                      float* records, float* out, float* final_T,
                                      int32_t* n_contrib, int64_t* info, void* stream, int batch);
int pgb_alpha_blending_backward_pieces(const float* records, int64_t n, const int32_t* widths,
                                       int npieces, const int32_t* ids, int64_t k,
                                       const int32_t* tile_range, float bg, int width, int height,
                                       const float* final_T, const int32_t* n_contrib,
                                       const float* d_out, float* grad_records, float* d_uv,
                                       float* d_conic, float* d_opacity, float* const* d_pieces,
                                       int64_t* info, void* stream, int batch);

/* ---------------------------------------------------------------------
 * Adam step over several parameter tensors in one launch -- replaces the
 * torch Adam update of the training step (pointrix/optimizer/optimizer.py:
 * 128-140; apex FusedAdam hook pointrix/optimizer/__init__.py:56-59).
 * Each segment is a dense float32 tensor with its gradient, both moment
 * buffers, its learning rate and its bias corrections 1 - beta1^t and
 * 1 - beta2^t for its own step count t; at most 32 segments.  Same update as
 * torch.optim.Adam without weight decay or amsgrad.
 * ------------------------------------------------------------------- */
typedef struct {
  float* param;
  const float* grad;
  float* exp_avg;
  float* exp_avg_sq;
  int64_t n;
  float lr;
  float bias_correction1;
  float bias_correction2;
} pgb_adam_segment;
int pgb_adam_step(const pgb_adam_segment* segments, int nsegments, float beta1, float beta2,
                  float eps, void* stream);

/* The same update with the step counts on the device, for a step captured
 * in a CUDA graph: step_counts[i] (int32, device) is segment i's count t,
 * incremented by the call before use; the bias corrections 1 - beta^t are
 * formed on the device in double precision into bias_corrections (float,
 * device, 2 per segment) -- the bias_correction fields of the segments are
 * ignored.  Two launches. */
int pgb_adam_step_device(const pgb_adam_segment* segments, int nsegments, double beta1,
                         double beta2, float eps, int32_t* step_counts, float* bias_corrections,
                         void* stream);

/* ---------------------------------------------------------------------
 * Fused caller-side passes of the training step -- no msplat counterpart.
 * They replace torch glue that surrounds the operators above, with the same
 * arithmetic.
 *
 * pgb_gaussian_activate_*: the parameter activations of GaussianPointCloud
 * (pointrix/model/point_cloud/gaussian_points.py:70-80: exp, sigmoid,
 * F.normalize) and the normal feature of examples/supervise/model.py:50-62
 * (column argmin(log_scale) of the rotation matrix of
 * pointrix/utils/pose.py:40-84, normalised).  log_scale [N,3], quat [N,4]
 * wxyz, opacity_logit [N] -> scaling [N,3], rotation [N,4], opacity [N],
 * normal [N,3] (NULL: not computed).  quat, rotation, d_rotation and d_quat
 * must be 16-byte aligned.  The backward takes the incoming gradients (any of
 * them NULL: zero) and writes the parameter gradients.
 * ------------------------------------------------------------------- */
int pgb_gaussian_activate_forward(const float* log_scale, const float* quat,
                                  const float* opacity_logit, int64_t n, float* scaling,
                                  float* rotation, float* opacity, float* normal, void* stream);
int pgb_gaussian_activate_backward(const float* log_scale, const float* quat,
                                   const float* opacity_logit, int64_t n, const float* d_scaling,
                                   const float* d_rotation, const float* d_opacity,
                                   const float* d_normal, float* d_log_scale, float* d_quat,
                                   float* d_opacity_logit, void* stream);

/* pgb_sh_rgb_*: the view colour of MsplatRender.render_iter
 * (pointrix/model/renderer/msplat.py:94-105): direction = normalise(xyz -
 * center), the SH mask (coefficients k >= active are zero), compute_sh, +0.5
 * and clamp(min=0), in one pass.  sh is the dense [N,K,3] storage (the
 * tensor msplat.py:99 permutes), 16-byte aligned; center [3].  The backward
 * writes d_sh [N,K,3] (zero for k >= active), d_xyz [N,3] and d_center [3]
 * (deterministic, through scratch of pgb_sh_rgb_scratch_floats(n) floats). */
int pgb_sh_rgb_scratch_floats(int64_t n);
int pgb_sh_rgb_forward(const float* sh, int64_t n, int k, int active, const float* xyz,
                       const float* center, float* rgb, void* stream);
int pgb_sh_rgb_backward(const float* sh, int64_t n, int k, int active, const float* xyz,
                        const float* center, const float* d_rgb, float* d_sh, float* d_xyz,
                        float* d_center, float* scratch, int64_t scratch_floats, void* stream);

/* pgb_sh_rgb_views_*: pgb_sh_rgb_* for V cameras in one pass over the
 * coefficients (batches of views).  centres [V,3] on the device (V <= 64),
 * rgb and d_rgb [V][N][3]; the backward writes d_sh and d_xyz summed over
 * the views and d_centres [V,3] (deterministic, scratch of
 * pgb_sh_rgb_views_scratch_floats(n) floats). */
int pgb_sh_rgb_views_scratch_floats(int64_t n);
int pgb_sh_rgb_views_forward(const float* sh, int64_t n, int k, int active, const float* xyz,
                             const float* centres, int nviews, float* rgb, void* stream);
int pgb_sh_rgb_views_backward(const float* sh, int64_t n, int k, int active, const float* xyz,
                              const float* centres, int nviews, const float* d_rgb,
                              float* d_sh, float* d_xyz, float* d_centres, float* scratch,
                              int64_t scratch_floats, void* stream);

/* pgb_l1_l2_loss_*: L = mean|x - t| + w * mean((x - t)^2) over n floats
 * (the L1 term of pointrix/model/loss.py:27-33 plus a weighted L2 term), x
 * and t 16-byte aligned.  The forward writes L to loss[0] (device) through
 * scratch of pgb_l1_l2_loss_scratch_doubles(n) doubles, summed in a fixed
 * order; the backward reads dL from d_loss[0] (device) and writes
 * d_x = sign(x - t) dL / n + (2 / n)(x - t) w dL. */
int pgb_l1_l2_loss_scratch_doubles(int64_t n);
int pgb_l1_l2_loss_forward(const float* x, const float* target, int64_t n, float w,
                           double* scratch, int64_t scratch_doubles, float* loss, void* stream);
int pgb_l1_l2_loss_backward(const float* x, const float* target, int64_t n, float w,
                            const float* d_loss, float* d_x, void* stream);
/* The training step's form: the forward also writes d_x_unit (16-byte
 * aligned, n floats) = the backward for dL = 1, in the pass that reads x and
 * t for the loss; pgb_l1_l2_loss_backward_unit then takes that buffer as d_x
 * and returns at once when d_loss[0] == 1 (no pass over x and t), otherwise
 * rewrites it exactly as pgb_l1_l2_loss_backward does.  The values are bit
 * for bit those of pgb_l1_l2_loss_backward either way. */
int pgb_l1_l2_loss_forward_grad(const float* x, const float* target, int64_t n, float w,
                                double* scratch, int64_t scratch_doubles, float* loss,
                                float* d_x_unit, void* stream);
int pgb_l1_l2_loss_backward_unit(const float* x, const float* target, int64_t n, float w,
                                 const float* d_loss, float* d_x, void* stream);

/* pgb_preprocess_*: project_point + compute_cov3d + ewa_project as the
 * renderer chains them (pointrix/model/renderer/msplat.py:109-130, visible =
 * depth != 0), in one pass forward and one backward.  Outputs are
 * bit-identical to the three operators' (uv [N,2], depth [N,1], conic [N,3],
 * radius [N], tiles_touched [N]); the backward takes d uv, d depth and
 * d conic and writes d xyz (both paths summed), d scales, d quats and the
 * camera gradients d_intr [4], d_extr [12] (scratch of
 * pgb_camera_grad_scratch_bytes()).  uquats / d_uquats 16-byte aligned. */
int pgb_preprocess_forward(const float* xyz, const float* scales, const float* uquats, int64_t n,
                           const float* intr, const float* extr, int width, int height,
                           float nearest, float extent, float* uv, float* depth, float* conic,
                           int32_t* radius, int32_t* tiles_touched, void* stream);
int pgb_preprocess_backward(const float* xyz, const float* scales, const float* uquats, int64_t n,
                            const float* intr, const float* extr, int width, int height,
                            float nearest, float extent, const int32_t* radius, const float* d_uv,
                            const float* d_depth, const float* d_conic, float* d_xyz,
                            float* d_scales, float* d_uquats, float* d_intr, float* d_extr,
                            void* scratch, size_t scratch_bytes, void* stream);

/* pgb_preprocess_views_*: the same for V views of one set of Gaussians (the
 * batched multi-view path; no msplat counterpart): view v's camera is
 * intrs[4v..4v+3] and extrs[12v..12v+11] (device, [V,4] and [V,3,4]), its
 * image size sizes[2v], sizes[2v+1] (host); outputs are view-major [V*N, .]
 * (element v*N + i), each equal bit for bit to the single-view call for that
 * view.  The backward takes the view-major d uv / d depth / d conic and
 * writes d xyz, d scales, d quats summed over the views (in view order, one
 * thread per Gaussian: deterministic) and d_intrs [V,4], d_extrs [V,3,4]
 * (scratch of pgb_camera_grad_views_scratch_bytes(V)).  V <= 64. */
size_t pgb_camera_grad_views_scratch_bytes(int nviews);
int pgb_preprocess_views_forward(const float* xyz, const float* scales, const float* uquats,
                                 int64_t n, const float* intrs, const float* extrs,
                                 const int32_t* sizes, int nviews, float nearest, float extent,
                                 float* uv, float* depth, float* conic, int32_t* radius,
                                 int32_t* tiles_touched, void* stream);
int pgb_preprocess_views_backward(const float* xyz, const float* scales, const float* uquats,
                                  int64_t n, const float* intrs, const float* extrs,
                                  const int32_t* sizes, int nviews, float nearest, float extent,
                                  const int32_t* radius, const float* d_uv, const float* d_depth,
                                  const float* d_conic, float* d_xyz, float* d_scales,
                                  float* d_uquats, float* d_intrs, float* d_extrs, void* scratch,
                                  size_t scratch_bytes, void* stream);

/* pgb_ssim_*: the SSIM of pointrix/model/loss.py:71-125 (11x11 Gaussian
 * window, sigma 1.5, zero padding, C1 = 0.01^2, C2 = 0.03^2, mean over all
 * pixels) of x against the target y, both `planes` contiguous float planes of
 * height x width.  The forward writes the mean to ssim_out[0] (device)
 * through scratch of pgb_ssim_scratch_doubles(...) doubles (fixed-order
 * sum); the backward reads dL from d_out[0] (device) and writes d_x (y is
 * not differentiated). */
int64_t pgb_ssim_scratch_doubles(int planes, int height, int width);
int pgb_ssim_forward(const float* x, const float* y, int planes, int height, int width,
                     double* scratch, int64_t scratch_doubles, float* ssim_out, void* stream);
int pgb_ssim_backward(const float* x, const float* y, int planes, int height, int width,
                      const float* d_out, float* d_x, void* stream);

/* pgb_densify_accumulate: the densification statistics update of
 * DensificationController.preprocess (pointrix/controller/gs.py:318-333,
 * gradient from accumulate_viewspace_grad, gs.py:260-284) for the points
 * with radius > 0: max_radii[i] = max(max_radii[i], radius[i]);
 * grad_accum[i] += |(d_uv[i].x * sx, d_uv[i].y * sy)|; acc_steps[i] += 1.
 * d_uv [N,2] (8-byte aligned) is the screen-space gradient (summed over the
 * views of a batch), sx = W/2, sy = H/2 with normalize_grad (else 1). */
int pgb_densify_accumulate(const float* d_uv, int64_t n, const int32_t* radius, float sx,
                           float sy, float* grad_accum, float* acc_steps, float* max_radii,
                           void* stream);

#ifdef __cplusplus
}
#endif

#endif /* POINTRIX_GB300_H */
