"""Batched multi-view rendering: V views, one sort and one blend launch.

``MsplatRender.render_batch`` renders views one after another
(``pointrix/model/renderer/msplat.py:185-213``): every view pays its own
sort read-back (a host synchronisation), its own launches and, for small
views, an under-filled GPU.  Here the per-Gaussian operators run per view
(their inputs differ per camera) on one stream, and then all V x N
(view, Gaussian) elements go through one sort -- one read-back for the
batch -- and one blend launch forward and one backward over the tiles of
every view.  Within any tile the order is depth, then element id, exactly
as when the view is rendered alone, so each image equals the per-view
result.  Differentiable in every Gaussian parameter and camera, like the
per-view path.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib, autotune, fused, ops
from ._lib import call
from .ops import _c, _ptr, _status_word, _stream, _timed

TILE = 16
MAX_VIEWS = 64


def _sizes_array(sizes):
    arr = (C.c_int32 * (2 * len(sizes)))()
    for i, (W, H) in enumerate(sizes):
        arr[2 * i], arr[2 * i + 1] = int(W), int(H)
    return arr


def _tiles(W, H, th=TILE):
    return ((W + TILE - 1) // TILE) * ((H + th - 1) // th)


TILE_HEIGHTS = (16, 32)


def _blend_batches_h(backward: int, th: int) -> tuple:
    if th == TILE:
        return ops._blend_batches(backward)
    cnt = _lib.lib().pgb_blend_batches_h(backward, th, None)
    buf = (C.c_int32 * max(cnt, 1))()
    cnt = _lib.lib().pgb_blend_batches_h(backward, th, buf)
    return tuple(buf[i] for i in range(cnt))


def tile_counts_views(uv, radius, sizes, n_per_view, tile_height):
    """Entries of each element for 16 x ``tile_height`` tiles [V*N] int32."""
    tiles = torch.empty_like(radius)
    call("pgb_tile_counts_views", _ptr(uv), _ptr(radius), int(n_per_view), _sizes_array(sizes),
         len(sizes), int(tile_height), _ptr(tiles), _stream(uv.device))
    return tiles


class ViewsSortHandle:
    """A views sort between its phases (:func:`sort_views_begin`): the depth
    sort is enqueued and K is being copied to the host; ``ready()`` polls,
    ``finish()`` enqueues the tile passes (on the stream of the begin)."""

    __slots__ = ("h", "sizes", "n_per_view", "th")

    def ready(self) -> bool:
        return self.h.ready()

    def count(self) -> int:
        return self.h.count()

    def finish(self):
        return _sort_views_finish(self.h, self.sizes, self.n_per_view, self.th, None)


def sort_views_begin(uv, depth, radius, tiles_touched, sizes, n_per_view, tile_height=16):
    """Phase one of :func:`sort_views` without blocking the host (for a
    server that overlaps requests): returns a :class:`ViewsSortHandle`."""
    th = int(tile_height)
    if th not in TILE_HEIGHTS:
        raise ValueError(f"tile_height must be one of {TILE_HEIGHTS}, got {th}")
    if th != TILE:
        tiles_touched = tile_counts_views(_c(uv), _c(radius.reshape(-1)), sizes, n_per_view, th)
    W0, H0 = sizes[0]
    hv = ViewsSortHandle()
    hv.h = ops.sort_gaussian_begin(uv, depth, W0, H0, radius, tiles_touched, read_count=True,
                                   views=(len(sizes), n_per_view))
    hv.sizes, hv.n_per_view, hv.th = list(sizes), int(n_per_view), th
    return hv


def _sort_views_finish(h, sizes, n_per_view, th, capacity):
    K = h.count() if capacity is None else int(capacity)
    dev = h.dev
    T = sum(_tiles(W, H, th) for W, H in sizes)
    # the batch sorts local tile ids: its K-sized scratch is that of the
    # largest view's tile count (a 16T x 16 "image" has T tiles)
    T_local = max(_tiles(W, H, th) for W, H in sizes)
    _, bk = ops._sort_scratch(h.n, K, 16 * T_local, 16)
    with torch.cuda.stream(h.stream):
        scratch_k = torch.empty(max(bk, 1), dtype=torch.uint8, device=dev)
        ids = torch.empty(max(K, 1), dtype=torch.int32, device=dev)[:K]
        rng = torch.empty(T, 2, dtype=torch.int32, device=dev)
        with _timed("sort_finish", dev, (3 + ops._tile_passes(T_local)) if (K and h.n) else
                    (0 if capacity is None else 1)):
            call("pgb_sort_gaussian_finish_views_h", _ptr(h.uv), _ptr(h.radius), _ptr(h.tiles),
                 n_per_view, _sizes_array(sizes), len(sizes), th, K, 0 if capacity is None else 1,
                 _ptr(h.scratch_n), h.bn, _ptr(scratch_k), bk, _ptr(h.info),
                 _ptr(ids) if K else None, _ptr(rng), h.stream.cuda_stream)
        if capacity is None:
            ops._defer_check(h.info[1:], "sort_views (tile passes)")
        else:
            ops._fold_status(h.info[1:2], dev)
    return ids, rng


def sort_views(uv, depth, radius, tiles_touched, sizes, n_per_view, capacity=None, tile_height=16):
    """Tile lists of V views at once: ids [K] (element ids v*N + g) and
    tile_range [sum of tiles, 2] over the views' concatenated tile space.
    The pairs are sorted by view-local tile over a view-major emission, so
    ids holds, for each local tile, the views' lists one after another;
    tile_range[base_v + t] selects view v's list of tile t (depth, then id).
    With ``capacity`` K stays on the device (ids has ``capacity`` entries)
    and nothing synchronises, as in :func:`ops.sort_gaussian`.
    ``tile_height`` 32 sorts 16 x 32 tiles (``tiles_touched`` is then
    recounted for them); the blend of :func:`blend_views` with the same
    tile height renders exactly the 16 x 16 images."""
    th = int(tile_height)
    if th not in TILE_HEIGHTS:
        raise ValueError(f"tile_height must be one of {TILE_HEIGHTS}, got {th}")
    if th != TILE:
        tiles_touched = tile_counts_views(_c(uv), _c(radius.reshape(-1)), sizes, n_per_view, th)
    W0, H0 = sizes[0]
    h = ops.sort_gaussian_begin(uv, depth, W0, H0, radius, tiles_touched,
                                read_count=capacity is None, views=(len(sizes), n_per_view))
    return _sort_views_finish(h, sizes, n_per_view, th, capacity)


class _BlendViews(torch.autograd.Function):
    @staticmethod
    def forward(ctx, uv, conic, opacity, feature, ids, tile_range, bg, sizes, n_per_view, th,
                radius):
        n, Cc = feature.shape
        dev = feature.device
        P = sum(W * H for W, H in sizes)
        records = torch.empty(n, _lib.lib().pgb_blend_record_floats(Cc), dtype=torch.float32, device=dev)
        out = torch.empty(Cc * P, dtype=torch.float32, device=dev)
        final_T = torch.empty(P, dtype=torch.float32, device=dev)
        ncon = torch.empty(P, dtype=torch.int32, device=dev)
        sz = _sizes_array(sizes)

        def run(batch):
            call("pgb_alpha_blending_forward_views_h", _ptr(uv), _ptr(conic), _ptr(opacity),
                 _ptr(feature), n_per_view, Cc, _ptr(ids), ids.numel(), _ptr(tile_range), float(bg),
                 sz, len(sizes), th, _ptr(radius), _ptr(records), _ptr(out), _ptr(final_T),
                 _ptr(ncon), _ptr(_status_word(dev)), _stream(dev), batch)

        key = autotune.workload_class(f"blend_fwd_h{th}", Cc, P, ids.numel(), tile_range.shape[0])
        batch = autotune.choose(key, _blend_batches_h(0, th), run, dev) if n else 0
        with _timed("alpha_blending_fwd", dev, 2 if n else 1):
            run(batch)
        ctx.save_for_backward(records, ids, tile_range, final_T, ncon, radius)
        ctx.cfg = (n, Cc, float(bg), tuple(sizes), n_per_view, th)
        return out

    @staticmethod
    def backward(ctx, d_out):
        records, ids, tile_range, final_T, ncon, radius = ctx.saved_tensors
        n, Cc, bg, sizes, n_per_view, th = ctx.cfg
        dev = records.device
        grec = torch.empty(n, _lib.lib().pgb_blend_grad_record_floats(Cc), dtype=torch.float32,
                           device=dev)
        d_uv = torch.empty(n, 2, dtype=torch.float32, device=dev)
        d_conic = torch.empty(n, 3, dtype=torch.float32, device=dev)
        d_op = torch.empty(n, dtype=torch.float32, device=dev)
        d_feat = torch.empty(n, Cc, dtype=torch.float32, device=dev)
        d_out = _c(d_out)
        sz = _sizes_array(sizes)
        P = sum(W * H for W, H in sizes)

        def run(batch):
            call("pgb_alpha_blending_backward_views_h", _ptr(records), n_per_view, Cc,
                 _ptr(ids), ids.numel(), _ptr(tile_range), bg, sz, len(sizes), th, _ptr(radius),
                 _ptr(final_T), _ptr(ncon), _ptr(d_out), _ptr(grec), _ptr(d_uv), _ptr(d_conic),
                 _ptr(d_op), _ptr(d_feat), _ptr(_status_word(dev)), _stream(dev), batch)

        key = autotune.workload_class(f"blend_bwd_h{th}", Cc, P, ids.numel(), tile_range.shape[0])
        batch = autotune.choose(key, _blend_batches_h(1, th), run, dev) if n else 0
        with _timed("alpha_blending_bwd", dev, 2 if n else 0):
            run(batch)
        return d_uv, d_conic, d_op, d_feat, None, None, None, None, None, None, None


def blend_views(uv, conic, opacity, feature, ids, tile_range, bg, sizes, n_per_view,
                tile_height=16, radius=None):
    """Blends V views in one launch; returns the list of [C,H,W] images.
    ``tile_height`` and the lists as :func:`sort_views` made them;
    ``radius`` [V*N] (the elements' radii) is needed for 16 x 32 tiles."""
    n, Cc = feature.shape
    th = int(tile_height)
    if th != TILE and radius is None:
        raise ValueError("blend_views: 16 x 32 tiles need the elements' radii")
    if radius is None:
        radius = torch.zeros(1, dtype=torch.int32, device=feature.device)
    if len(sizes) < 1 or len(sizes) > MAX_VIEWS:
        raise ValueError(f"blend_views takes 1..{MAX_VIEWS} views, got {len(sizes)}")
    if n != n_per_view * len(sizes):
        raise ValueError("feature rows must be n_per_view * number of views")
    flat = _BlendViews.apply(_c(uv), _c(conic), _c(opacity.reshape(n)), _c(feature), _c(ids),
                             _c(tile_range), bg, [tuple(map(int, s)) for s in sizes], int(n_per_view),
                             th, _c(radius.reshape(-1)))
    out, o = [], 0
    for W, H in sizes:
        out.append(flat[o:o + Cc * W * H].view(Cc, H, W))
        o += Cc * W * H
    return out


def render_views(position, scaling, rotation, opacity, shs, cams, bg=0.0, render_depth=True,
                 extra_features=None, nearest=ops.NEAREST_DEFAULT, capacity=None, sh_active=None,
                 tile_height=16):
    """Renders every camera of ``cams`` (objects with W, H, intr [1,4] or [4],
    extr [4,4] world->camera, center [3]) in one batch.  Features are
    rgb (+ depth) (+ ``extra_features`` [N,c]) as in ``MsplatRender``; the
    colour uses the first ``sh_active`` SH coefficients (all when None).
    ``capacity`` keeps the batch's K on the device (see :func:`sort_views`),
    so the whole call can be captured in a CUDA graph.  ``tile_height`` 32
    sorts and blends 16 x 32 tiles (fewer entries, the same images).
    Returns (list of [C,H,W] images, list of per-view uv, list of radius)."""
    n = position.shape[0]
    K = shs.shape[1]
    V = len(cams)
    active = K if sh_active is None else sh_active
    sizes = [(cam.W, cam.H) for cam in cams]
    if V > MAX_VIEWS:
        raise ValueError(f"render_views takes at most {MAX_VIEWS} views, got {V}")
    # every view's colour in one pass over the coefficients, every view's
    # projection in one kernel (gradients summed over views inside it)
    if fused.sh_rgb_supported(shs):
        centres = torch.stack([cam.center.reshape(3) for cam in cams])
        rgb_all = fused.sh_rgb_views(shs, position, centres, active).reshape(V * n, 3)
    else:
        shc = shs.permute(0, 2, 1)
        rgbs = []
        for cam in cams:
            d = position - cam.center.reshape(1, 3)
            d = d / d.norm(dim=1, keepdim=True)
            sh_in = shc
            if active < K:
                mask = torch.zeros_like(shc)
                mask[..., :active] = 1.0
                sh_in = shc * mask
            rgbs.append((ops.compute_sh(sh_in, d) + 0.5).clamp(min=0.0))
        rgb_all = torch.cat(rgbs)
    intrs = torch.stack([cam.intr.reshape(4) for cam in cams])
    extrs = torch.stack([cam.extr[:3, :] for cam in cams])
    uv_all, depth_all, conic_all, radius_all, tiles_all = fused.preprocess_views(
        position, scaling, rotation, intrs, extrs, sizes, nearest=nearest)
    f = [rgb_all] + ([depth_all] if render_depth else [])
    if extra_features is not None:
        f.append(extra_features.repeat(V, 1))
    feat_all = torch.cat(f, 1) if len(f) > 1 else f[0]
    ids, rng = sort_views(uv_all, depth_all, radius_all, tiles_all, sizes, n, capacity=capacity,
                          tile_height=tile_height)
    op_all = opacity.reshape(1, n).expand(V, n).reshape(-1)
    imgs = blend_views(uv_all, conic_all, op_all, feat_all, ids, rng, bg, sizes, n,
                       tile_height=tile_height, radius=radius_all)
    uvs = list(uv_all.split(n))
    radii = list(radius_all.split(n))
    return imgs, uvs, radii
