"""The msplat operators on GB300: torch.autograd.Functions over the C ABI.

Each public function keeps the signature and argument meaning that Pointrix's
``MsplatRender.render_iter`` relies on (``pointrix/model/renderer/msplat.py``
lines 104-151; the same six calls in ``examples/supervise/renderer.py:42-85``),
so ``import msplat`` can resolve to this module unchanged.  Inputs are CUDA
float32 tensors (possibly strided views); outputs are new tensors on the same
device; all work is enqueued on the current CUDA stream.  Errors raise
``ValueError`` (bad arguments) or :class:`pointrix_gb300._lib.PgbError`
(a status from the kernel library).  There is no CPU path.
"""
from __future__ import annotations

import ctypes
import threading

import torch

from . import _lib, autotune
from ._lib import PgbError, call

__all__ = [
    "compute_sh", "project_point", "compute_cov3d", "ewa_project", "sort_gaussian",
    "sort_gaussian_begin", "SortHandle", "rasterize",
    "alpha_blending", "alpha_blending_with_state", "alpha_blending_pieces", "check_device_status",
    "kernel_timing",
    "NEAREST_DEFAULT", "EXTENT_DEFAULT",
]

NEAREST_DEFAULT = 0.2
EXTENT_DEFAULT = 1.3
TILE = 16


def _ptr(t):
    return None if t is None else t.data_ptr()


def _c(t):
    """Contiguous and 16-byte aligned (kernels use 8- and 16-byte vector
    accesses on rows); copies only when the input is neither."""
    t = t.contiguous()
    if t.data_ptr() % 16:
        t = t.clone()
    return t


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _need(t, name, dtype=torch.float32, ndim=None, last=None):
    if not isinstance(t, torch.Tensor):
        raise ValueError(f"{name} must be a tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (pointrix_gb300 has no CPU path)")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if ndim is not None and t.dim() != ndim:
        raise ValueError(f"{name} must have {ndim} dims, got shape {tuple(t.shape)}")
    if last is not None and t.shape[-1] != last:
        raise ValueError(f"{name} must have last dim {last}, got shape {tuple(t.shape)}")


def _intr4(intr):
    _need(intr, "intr")
    if intr.numel() != 4:
        raise ValueError(f"intr must hold 4 values (fx, fy, cx, cy), got shape {tuple(intr.shape)}")
    return _c(intr.reshape(4))


def _extr34(extr):
    _need(extr, "extr")
    if tuple(extr.shape) != (3, 4):
        raise ValueError(f"extr must be [3,4], got {tuple(extr.shape)}")
    return _c(extr)


def _visible_bytes(visible, n):
    if visible.numel() != n:
        raise ValueError(f"visible must have {n} entries, got shape {tuple(visible.shape)}")
    v = visible.reshape(-1)
    if v.dtype != torch.bool:
        v = v != 0
    return _c(v).view(torch.uint8)


# ---------------------------------------------------------------------------
# optional per-operator CUDA-event timing and kernel-launch counting
# ---------------------------------------------------------------------------
class KernelTiming:
    """Records a CUDA event pair around every library call on the calling
    stream, and counts the kernels each call launches.  Enable with
    ``with kernel_timing() as kt: ...``; read after a synchronize."""

    def __init__(self):
        self.events: dict[str, list] = {}
        self.launches: dict[str, int] = {}

    def total_launches(self) -> int:
        return sum(self.launches.values())

    def ms(self, name: str) -> list[float]:
        return [a.elapsed_time(b) for a, b in self.events.get(name, [])]

    def names(self):
        return list(self.events)


_timing: KernelTiming | None = None


class kernel_timing:
    def __enter__(self) -> KernelTiming:
        global _timing
        self.prev, _timing = _timing, KernelTiming()
        return _timing

    def __exit__(self, *exc):
        global _timing
        _timing = self.prev
        return False


class _timed:
    __slots__ = ("name", "dev", "kernels", "ev")

    def __init__(self, name, dev, kernels):
        self.name, self.dev, self.kernels = name, dev, kernels

    def __enter__(self):
        if _timing is not None and not _capturing():
            self.ev = torch.cuda.Event(enable_timing=True)
            self.ev.record(torch.cuda.current_stream(self.dev))
        return self

    def __exit__(self, *exc):
        t = _timing
        if t is not None and exc[0] is None and not _capturing():
            end = torch.cuda.Event(enable_timing=True)
            end.record(torch.cuda.current_stream(self.dev))
            t.events.setdefault(self.name, []).append((self.ev, end))
            t.launches[self.name] = t.launches.get(self.name, 0) + self.kernels
        return False


# ---------------------------------------------------------------------------
# device status words (blend kernels write a PGB status on a device-side
# fault; sort_gaussian's finish step reports through its per-call info words)
# ---------------------------------------------------------------------------
_status_lock = threading.Lock()
_dev_status: dict[int, torch.Tensor] = {}
# Deferred status checks: (event, pinned read-back, what) per call; a caller
# that never drains (a loop of plain sorts) keeps the list short through the
# drain that every _PENDING_DRAIN-th deferral runs.
_pending: list[tuple[torch.cuda.Event, torch.Tensor, str]] = []
_PENDING_DRAIN = 32


def _status_word(device) -> torch.Tensor:
    idx = device.index if device.index is not None else torch.cuda.current_device()
    with _status_lock:
        t = _dev_status.get(idx)
        if t is None:
            t = torch.zeros(4, dtype=torch.int64, device=device)
            _dev_status[idx] = t
    return t


def _capturing() -> bool:
    """True while the current stream is being captured into a CUDA graph:
    nothing may then wait on, or read back, device data."""
    return torch.cuda.is_current_stream_capturing()


def _defer_check(word: torch.Tensor, what: str):
    if _capturing():  # a graph's replays are checked with check_device_status
        return
    host = torch.empty(word.numel(), dtype=torch.int64, pin_memory=True)
    host.copy_(word, non_blocking=True)
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream(word.device))
    with _status_lock:
        _pending.append((ev, host, what))
        drain = len(_pending) >= _PENDING_DRAIN
    if drain:
        _drain_pending(block=False)


def _drain_pending(block: bool):
    with _status_lock:
        items = list(_pending)
        _pending.clear()
    keep, err = [], None
    for i, (ev, host, what) in enumerate(items):
        if block:
            ev.synchronize()
        elif not ev.query():
            # deferred in order: the ones after it are (nearly always) still
            # pending too -- keep them unqueried
            keep = items[i:]
            break
        code = int(host.numpy().max())   # the pinned words, read in place
        if code and err is None:
            err = (code, what)
    if keep:
        with _status_lock:
            _pending[:0] = keep          # older than anything deferred meanwhile
    if err:
        _lib.check(err[0], err[1])


def check_device_status(device=None) -> None:
    """Synchronise ``device`` and raise if any kernel of this library
    recorded a device-side fault (expired bounded wait, overflow, mismatch)."""
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    torch.cuda.synchronize(device)
    _drain_pending(block=True)
    w = _status_word(device)
    code = int(w.max().item())
    if code:
        w.zero_()
        _lib.check(code, "device status")


# ---------------------------------------------------------------------------
# compute_sh
# ---------------------------------------------------------------------------
def _dense_sh(sh):
    if sh.is_contiguous() or sh.permute(0, 2, 1).is_contiguous():
        return sh
    return sh.contiguous()


class _ComputeSH(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sh, dirs):
        n, K = sh.shape[0], sh.shape[2]
        rgb = torch.empty(n, 3, dtype=torch.float32, device=sh.device)
        sn, sc, sk = sh.stride()
        with _timed("compute_sh_fwd", sh.device, 1 if n else 0):
            call("pgb_compute_sh_forward", _ptr(sh), n, K, sn, sc, sk, _ptr(dirs), _ptr(rgb), _stream(sh.device))
        ctx.save_for_backward(sh, dirs)
        return rgb

    @staticmethod
    def backward(ctx, d_rgb):
        sh, dirs = ctx.saved_tensors
        n, K = sh.shape[0], sh.shape[2]
        d_sh = torch.empty_like(sh)
        d_dirs = torch.empty_like(dirs)
        sn, sc, sk = sh.stride()
        with _timed("compute_sh_bwd", sh.device, 1 if n else 0):
            call("pgb_compute_sh_backward", _ptr(sh), n, K, sn, sc, sk, _ptr(dirs),
                 _ptr(_c(d_rgb)), _ptr(d_sh), _ptr(d_dirs), _stream(sh.device))
        return d_sh, d_dirs


def compute_sh(shs, view_dirs):
    """Raw real-SH colour ``sum_k shs[:, c, k] Y_k(view_dirs)`` -> [N,3].

    ``shs`` is [N,3,K] with K in {1,4,9,16} (any strides; the permuted
    ``get_shs`` view is read in place); ``view_dirs`` [N,3] unit vectors.
    No +0.5 offset and no clamp (``msplat.py:103-105`` adds them).
    """
    _need(shs, "shs", ndim=3)
    _need(view_dirs, "view_dirs", ndim=2, last=3)
    if shs.shape[1] != 3 or shs.shape[2] not in (1, 4, 9, 16):
        raise ValueError(f"shs must be [N,3,K] with K in (1,4,9,16), got {tuple(shs.shape)}")
    if view_dirs.shape[0] != shs.shape[0]:
        raise ValueError("shs and view_dirs disagree on N")
    return _ComputeSH.apply(_dense_sh(shs), _c(view_dirs))


# ---------------------------------------------------------------------------
# project_point
# ---------------------------------------------------------------------------
class _ProjectPoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, intr, extr, W, H, nearest, extent, intr_shape):
        n = xyz.shape[0]
        uv = torch.empty(n, 2, dtype=torch.float32, device=xyz.device)
        depth = torch.empty(n, 1, dtype=torch.float32, device=xyz.device)
        with _timed("project_point_fwd", xyz.device, 1 if n else 0):
            call("pgb_project_point_forward", _ptr(xyz), n, _ptr(intr), _ptr(extr), W, H,
                 float(nearest), float(extent), _ptr(uv), _ptr(depth), _stream(xyz.device))
        ctx.save_for_backward(xyz, intr, extr)
        ctx.cfg = (W, H, float(nearest), float(extent), intr_shape)
        return uv, depth

    @staticmethod
    def backward(ctx, d_uv, d_depth):
        xyz, intr, extr = ctx.saved_tensors
        W, H, nearest, extent, intr_shape = ctx.cfg
        n = xyz.shape[0]
        dev = xyz.device
        d_uv = torch.zeros(n, 2, device=dev) if d_uv is None else _c(d_uv)
        d_depth = torch.zeros(n, 1, device=dev) if d_depth is None else _c(d_depth)
        d_xyz = torch.empty_like(xyz)
        d_intr = torch.empty(4, dtype=torch.float32, device=dev)
        d_extr = torch.empty(3, 4, dtype=torch.float32, device=dev)
        nbytes = _lib.lib().pgb_camera_grad_scratch_bytes()
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        with _timed("project_point_bwd", dev, 2):
            call("pgb_project_point_backward", _ptr(xyz), n, _ptr(intr), _ptr(extr), W, H, nearest,
                 extent, _ptr(d_uv), _ptr(d_depth), _ptr(d_xyz), _ptr(d_intr), _ptr(d_extr),
                 _ptr(scratch), nbytes, _stream(dev))
        return d_xyz, d_intr, d_extr, None, None, None, None, None


def project_point(xyz, intr, extr, W, H, nearest=NEAREST_DEFAULT, extent=EXTENT_DEFAULT):
    """Pinhole projection: uv [N,2] = (fx x/z + cx, fy y/z + cy) of the
    camera-space point, depth [N,1] = z.  Points with z <= ``nearest`` or a
    centre outside ``extent`` x the half image get uv = 0 and depth = 0
    (``visible = depth != 0`` at ``msplat.py:115``).  ``intr`` is [4] or
    [1,4] (fx, fy, cx, cy); ``extr`` is the world->camera [3,4]."""
    _need(xyz, "xyz", ndim=2, last=3)
    shape = tuple(intr.shape) if isinstance(intr, torch.Tensor) else None
    intr4, extr34 = _intr4(intr), _extr34(extr)
    return _ProjectPoint.apply(_c(xyz), intr4, extr34, int(W), int(H), nearest, extent, shape)


# ---------------------------------------------------------------------------
# compute_cov3d
# ---------------------------------------------------------------------------
class _ComputeCov3d(torch.autograd.Function):
    @staticmethod
    def forward(ctx, scales, uquats, vis_u8):
        n = scales.shape[0]
        cov = torch.empty(n, 6, dtype=torch.float32, device=scales.device)
        with _timed("compute_cov3d_fwd", scales.device, 1 if n else 0):
            call("pgb_compute_cov3d_forward", _ptr(scales), _ptr(uquats), _ptr(vis_u8), n, _ptr(cov),
                 _stream(scales.device))
        ctx.save_for_backward(scales, uquats, vis_u8)
        return cov

    @staticmethod
    def backward(ctx, d_cov):
        scales, uquats, vis_u8 = ctx.saved_tensors
        n = scales.shape[0]
        d_s = torch.empty_like(scales)
        d_q = torch.empty_like(uquats)
        with _timed("compute_cov3d_bwd", scales.device, 1 if n else 0):
            call("pgb_compute_cov3d_backward", _ptr(scales), _ptr(uquats), _ptr(vis_u8), n,
                 _ptr(_c(d_cov)), _ptr(d_s), _ptr(d_q), _stream(scales.device))
        return d_s, d_q, None


def compute_cov3d(scales, uquats, visible):
    """3D covariance ``(R S)(R S)^T`` as its upper triangle
    (xx, xy, xz, yy, yz, zz) [N,6]; zero rows where ``visible`` is false.
    ``uquats`` are unit wxyz quaternions, ``scales`` activated [N,3]."""
    _need(scales, "scales", ndim=2, last=3)
    _need(uquats, "uquats", ndim=2, last=4)
    n = scales.shape[0]
    if uquats.shape[0] != n:
        raise ValueError("scales and uquats disagree on N")
    return _ComputeCov3d.apply(_c(scales), _c(uquats), _visible_bytes(visible, n))


# ---------------------------------------------------------------------------
# ewa_project
# ---------------------------------------------------------------------------
class _EwaProject(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, cov3d, intr, extr, uv, W, H, vis_u8, intr_shape):
        n = xyz.shape[0]
        dev = xyz.device
        conic = torch.empty(n, 3, dtype=torch.float32, device=dev)
        radius = torch.empty(n, dtype=torch.int32, device=dev)
        tiles = torch.empty(n, dtype=torch.int32, device=dev)
        with _timed("ewa_project_fwd", dev, 1 if n else 0):
            call("pgb_ewa_project_forward", _ptr(xyz), _ptr(cov3d), _ptr(intr), _ptr(extr), _ptr(uv),
                 _ptr(vis_u8), n, W, H, _ptr(conic), _ptr(radius), _ptr(tiles), _stream(dev))
        ctx.save_for_backward(xyz, cov3d, intr, extr, radius)
        ctx.cfg = (W, H, intr_shape)
        ctx.mark_non_differentiable(radius, tiles)
        ctx.set_materialize_grads(False)  # no zero tensors for radius / tiles
        return conic, radius, tiles

    @staticmethod
    def backward(ctx, d_conic, _r, _t):
        xyz, cov3d, intr, extr, radius = ctx.saved_tensors
        W, H, intr_shape = ctx.cfg
        n = xyz.shape[0]
        dev = xyz.device
        if d_conic is None:
            d_conic = torch.zeros(n, 3, device=dev)
        d_xyz = torch.empty_like(xyz)
        d_cov = torch.empty_like(cov3d)
        d_intr = torch.empty(4, dtype=torch.float32, device=dev)
        d_extr = torch.empty(3, 4, dtype=torch.float32, device=dev)
        nbytes = _lib.lib().pgb_camera_grad_scratch_bytes()
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        with _timed("ewa_project_bwd", dev, 2):
            call("pgb_ewa_project_backward", _ptr(xyz), _ptr(cov3d), _ptr(intr), _ptr(extr),
                 _ptr(radius), n, W, H, _ptr(_c(d_conic)), _ptr(d_xyz), _ptr(d_cov),
                 _ptr(d_intr), _ptr(d_extr), _ptr(scratch), nbytes, _stream(dev))
        return d_xyz, d_cov, d_intr, d_extr, None, None, None, None, None


def ewa_project(xyz, cov3d, intr, extr, uv, W, H, visible):
    """EWA projection of the 3D covariance into an image-space conic.

    Returns conic [N,3] (inverse 2D covariance a, b, c), radius [N] int32
    (pixels, 3 sigma of the dilated footprint) and tiles_touched [N] int32
    (16x16 tiles of its rectangle); culled Gaussians get zeros.
    Differentiable in xyz, cov3d, intr and extr.
    """
    _need(xyz, "xyz", ndim=2, last=3)
    _need(cov3d, "cov3d", ndim=2, last=6)
    _need(uv, "uv", ndim=2, last=2)
    n = xyz.shape[0]
    shape = tuple(intr.shape)
    return _EwaProject.apply(_c(xyz), _c(cov3d), _intr4(intr), _extr34(extr),
                             _c(uv.detach()), int(W), int(H), _visible_bytes(visible, n), shape)


# ---------------------------------------------------------------------------
# sort_gaussian
# ---------------------------------------------------------------------------
def _sort_scratch(n, k, W, H):
    import ctypes as C
    bn, bk = C.c_size_t(0), C.c_size_t(0)
    call("pgb_sort_scratch_bytes", n, k, W, H, C.byref(bn), C.byref(bk))
    return bn.value, bk.value


class SortHandle:
    """A sort between its two phases: the depth sort and the count K are
    enqueued, K is being copied to pinned host memory.  ``ready()`` polls
    without blocking; ``finish()`` allocates the K-sized outputs and enqueues
    the tile passes (on the stream that was current at ``begin``)."""

    __slots__ = ("uv", "depth", "radius", "tiles", "W", "H", "n", "dev", "stream", "scratch_n",
                 "bn", "info", "host", "event")

    def ready(self) -> bool:
        return self.event.query()

    def count(self) -> int:
        """K, the number of (Gaussian, tile) entries (waits for phase one)."""
        self.event.synchronize()
        _lib.check(int(self.host[1]), "sort_gaussian (depth passes)")
        return int(self.host[0])

    def finish(self):
        K = self.count()
        W, H, n, dev = self.W, self.H, self.n, self.dev
        T = ((W + TILE - 1) // TILE) * ((H + TILE - 1) // TILE)
        with torch.cuda.stream(self.stream):
            _, bk = _sort_scratch(n, K, W, H)
            scratch_k = torch.empty(max(bk, 1), dtype=torch.uint8, device=dev)
            ids = torch.empty(K, dtype=torch.int32, device=dev)
            rng = torch.empty(T, 2, dtype=torch.int32, device=dev)
            with _timed("sort_finish", dev, (3 + _tile_passes(T)) if (K and n) else 0):
                call("pgb_sort_gaussian_finish", _ptr(self.uv), _ptr(self.radius), _ptr(self.tiles),
                     n, W, H, K, _ptr(self.scratch_n), self.bn, _ptr(scratch_k), bk, _ptr(self.info),
                     _ptr(ids) if K else None, _ptr(rng), self.stream.cuda_stream)
            _defer_check(self.info[1:], "sort_gaussian (tile passes)")
        return ids, rng

    def finish_capacity(self, capacity: int):
        """Phase two with K left on the device: ids [capacity] (entries past K
        unspecified) and tile_range [T,2].  No host read-back, so the whole
        sort can be captured in a CUDA graph.  A K above ``capacity`` leaves
        every tile empty and raises at the next :func:`check_device_status`;
        ``self.info[0]`` holds K on the device."""
        W, H, n, dev = self.W, self.H, self.n, self.dev
        cap = int(capacity)
        if cap < 0:
            raise ValueError(f"sort capacity must be >= 0, got {cap}")
        T = ((W + TILE - 1) // TILE) * ((H + TILE - 1) // TILE)
        with torch.cuda.stream(self.stream):
            _, bk = _sort_scratch(n, cap, W, H)
            scratch_k = torch.empty(max(bk, 1), dtype=torch.uint8, device=dev)
            ids = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)[:cap]
            rng = torch.empty(T, 2, dtype=torch.int32, device=dev)
            with _timed("sort_finish", dev, (3 + _tile_passes(T)) if (cap and n) else 1):
                call("pgb_sort_gaussian_finish_capacity", _ptr(self.uv), _ptr(self.radius),
                     _ptr(self.tiles), n, W, H, cap, _ptr(self.scratch_n), self.bn, _ptr(scratch_k),
                     bk, _ptr(self.info), _ptr(ids) if cap else None, _ptr(rng),
                     self.stream.cuda_stream)
            _fold_status(self.info[1:2], dev)
        return ids, rng


def _tile_passes(T: int) -> int:
    """Tile-sort passes of the library for T tiles (launch accounting)."""
    return 1 if T <= 256 else (2 if T <= (1 << 18) else 3)


def _fold_status(word: torch.Tensor, dev):
    """Merges a per-call device status (int64 [1]) into the device's status
    word on the stream, for :func:`check_device_status` (no host read)."""
    w = _status_word(dev)[1:2]
    torch.maximum(w, word, out=w)


def sort_gaussian_begin(uv, depth, W, H, radius, tiles_touched, read_count=True,
                        views=None) -> SortHandle:
    """Phase one of :func:`sort_gaussian` without blocking the host: sorts the
    Gaussians by depth and (``read_count``) starts the read-back of K.
    ``views`` = (nviews, n_per_view): the elements are a batch of views
    (element v * n_per_view + g), sorted by view, then depth, then id, for
    the batch's tile passes (``multiview.sort_views``)."""
    _need(uv, "uv", ndim=2, last=2)
    _need(depth, "depth")
    _need(radius, "radius", dtype=torch.int32)
    _need(tiles_touched, "tiles_touched", dtype=torch.int32)
    W, H = int(W), int(H)
    n = uv.shape[0]
    if depth.numel() != n or radius.numel() != n or tiles_touched.numel() != n:
        raise ValueError("sort_gaussian: uv, depth, radius and tiles_touched disagree on N")
    h = SortHandle()
    h.dev = uv.device
    h.stream = torch.cuda.current_stream(h.dev)
    h.W, h.H, h.n = W, H, n
    h.uv, h.depth = _c(uv.detach()), _c(depth.detach().reshape(-1))
    h.radius, h.tiles = _c(radius.reshape(-1)), _c(tiles_touched.reshape(-1))
    h.bn, _ = _sort_scratch(n, 0, W, H)
    h.scratch_n = torch.empty(max(h.bn, 1), dtype=torch.uint8, device=h.dev)
    h.info = torch.empty(2, dtype=torch.int64, device=h.dev)
    if views is None:
        with _timed("sort_begin", h.dev, 5 if n else 0):
            call("pgb_sort_gaussian_begin", _ptr(h.depth), _ptr(h.radius), _ptr(h.tiles), n, W, H,
                 _ptr(h.scratch_n), h.bn, _ptr(h.info), h.stream.cuda_stream)
    else:
        nviews, n_per_view = int(views[0]), int(views[1])
        if nviews * n_per_view != n:
            raise ValueError(f"sort_gaussian_begin: {nviews} views of {n_per_view} is not N = {n}")
        with _timed("sort_begin", h.dev, 6 if n else 0):
            call("pgb_sort_gaussian_begin_views", _ptr(h.depth), _ptr(h.radius), _ptr(h.tiles),
                 n_per_view, nviews, _ptr(h.scratch_n), h.bn, _ptr(h.info), h.stream.cuda_stream)
    h.host = h.event = None
    if read_count:
        h.host = torch.empty(2, dtype=torch.int64, pin_memory=True)
        h.host.copy_(h.info, non_blocking=True)
        h.event = torch.cuda.Event()
        h.event.record(h.stream)
    return h


def sort_gaussian(uv, depth, W, H, radius, tiles_touched, capacity=None):
    """Tile binning: ``gaussian_ids_sorted`` [K] int32 (ids ordered by tile,
    then depth, then id) and ``tile_range`` [T,2] int32 ([start, end) per
    16x16 tile, [0,0] when empty), K = sum of ``tiles_touched`` over
    Gaussians with ``radius > 0``.  Reads K back to the host (one sync).

    ``capacity`` (not in the reference signature): K stays on the device and
    ``gaussian_ids_sorted`` has ``capacity`` entries, of which the first K are
    the result (the tile ranges never reach past K); nothing synchronises, so
    the call can be captured in a CUDA graph.  A K above the capacity leaves
    every tile empty and raises at the next :func:`check_device_status`."""
    if capacity is not None:
        h = sort_gaussian_begin(uv, depth, W, H, radius, tiles_touched, read_count=False)
        return h.finish_capacity(capacity)
    h = sort_gaussian_begin(uv, depth, W, H, radius, tiles_touched)
    h.count()
    _drain_pending(block=False)
    return h.finish()


# ---------------------------------------------------------------------------
# alpha_blending
# ---------------------------------------------------------------------------
_BATCHES: dict = {}


def _blend_batches(backward: int) -> tuple:
    """Per-block splat batches the library compiled for the forward (0) or
    the backward (1) blend."""
    hit = _BATCHES.get(backward)
    if hit is None:
        import ctypes as C
        cnt = _lib.lib().pgb_blend_batches(backward, None)   # the count first
        buf = (C.c_int32 * max(cnt, 1))()
        cnt = _lib.lib().pgb_blend_batches(backward, buf)
        hit = _BATCHES[backward] = tuple(buf[i] for i in range(cnt))
    return hit


def _piece_table(tensors):
    """Host arrays (device pointers, widths) of [N,w] pieces."""
    ptrs = (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])
    widths = (ctypes.c_int32 * len(tensors))(*[t.shape[1] for t in tensors])
    return ptrs, widths


def _blend_forward_raw(uv, conic, opacity, feature, ids, tile_range, bg, W, H):
    """``feature``: one [N,C] tensor, or a list of contiguous [N,w] pieces
    (blended as their concatenation, which is never built)."""
    pieces = list(feature) if isinstance(feature, (list, tuple)) else None
    if pieces is None:
        n, C = feature.shape
        dev = feature.device
    else:
        n, C = pieces[0].shape[0], sum(t.shape[1] for t in pieces)
        dev = pieces[0].device
    rf = _lib.lib().pgb_blend_record_floats(C)
    records = torch.empty(n, rf, dtype=torch.float32, device=dev)
    out = torch.empty(C, H, W, dtype=torch.float32, device=dev)
    final_T = torch.empty(H, W, dtype=torch.float32, device=dev)
    ncon = torch.empty(H, W, dtype=torch.int32, device=dev)
    status = _status_word(dev)

    if pieces is None:
        def run(batch):
            call("pgb_alpha_blending_forward_with_batch", _ptr(uv), _ptr(conic), _ptr(opacity),
                 _ptr(feature), n, C, _ptr(ids), ids.numel(), _ptr(tile_range), float(bg), W, H,
                 _ptr(records), _ptr(out), _ptr(final_T), _ptr(ncon), _ptr(status), _stream(dev),
                 batch)
    else:
        ptrs, widths = _piece_table(pieces)

        def run(batch):
            call("pgb_alpha_blending_forward_pieces", _ptr(uv), _ptr(conic), _ptr(opacity), ptrs,
                 widths, len(pieces), n, _ptr(ids), ids.numel(), _ptr(tile_range), float(bg), W, H,
                 _ptr(records), _ptr(out), _ptr(final_T), _ptr(ncon), _ptr(status), _stream(dev),
                 batch)

    key = autotune.workload_class("blend_fwd", C, W * H, ids.numel(), tile_range.shape[0])
    batch = autotune.choose(key, _blend_batches(0), run, dev) if n else 0
    with _timed("alpha_blending_fwd", dev, 2 if n else 1):
        run(batch)
    return records, out, final_T, ncon


def _blend_backward_raw(records, ids, tile_range, final_T, ncon, d_out, n, C, bg, W, H,
                        widths=None):
    """Gradients (uv, conic, opacity, feature); with ``widths`` the feature
    gradient is a list of [N,w] pieces."""
    dev = records.device
    grec = torch.empty(n, _lib.lib().pgb_blend_grad_record_floats(C), dtype=torch.float32, device=dev)
    d_uv = torch.empty(n, 2, dtype=torch.float32, device=dev)
    d_conic = torch.empty(n, 3, dtype=torch.float32, device=dev)
    d_op = torch.empty(n, dtype=torch.float32, device=dev)
    status = _status_word(dev)
    d_out = _c(d_out)

    if widths is None:
        d_feat = torch.empty(n, C, dtype=torch.float32, device=dev)

        def run(batch):
            call("pgb_alpha_blending_backward_with_batch", _ptr(records), n, C, _ptr(ids),
                 ids.numel(), _ptr(tile_range), bg, W, H, _ptr(final_T), _ptr(ncon), _ptr(d_out),
                 _ptr(grec), _ptr(d_uv), _ptr(d_conic), _ptr(d_op), _ptr(d_feat), _ptr(status),
                 _stream(dev), batch)
    else:
        d_feat = [torch.empty(n, w, dtype=torch.float32, device=dev) for w in widths]
        ptrs, wtab = _piece_table(d_feat)

        def run(batch):
            call("pgb_alpha_blending_backward_pieces", _ptr(records), n, wtab, len(d_feat),
                 _ptr(ids), ids.numel(), _ptr(tile_range), bg, W, H, _ptr(final_T), _ptr(ncon),
                 _ptr(d_out), _ptr(grec), _ptr(d_uv), _ptr(d_conic), _ptr(d_op), ptrs,
                 _ptr(status), _stream(dev), batch)

    key = autotune.workload_class("blend_bwd", C, W * H, ids.numel(), tile_range.shape[0])
    batch = autotune.choose(key, _blend_batches(1), run, dev) if n else 0
    with _timed("alpha_blending_bwd", dev, 2 if n else 0):
        run(batch)
    return d_uv, d_conic, d_op, d_feat


class _AlphaBlending(torch.autograd.Function):
    @staticmethod
    def forward(ctx, uv, conic, opacity, feature, ids, tile_range, bg, W, H, ndc):
        n, C = feature.shape
        records, out, final_T, ncon = _blend_forward_raw(uv, conic, opacity, feature, ids,
                                                         tile_range, bg, W, H)
        ctx.save_for_backward(records, ids, tile_range, final_T, ncon)
        ctx.cfg = (n, C, float(bg), W, H, ndc is not None)
        ctx.mark_non_differentiable(final_T, ncon)
        ctx.set_materialize_grads(False)  # no zero images for final_T / ncon
        return out, final_T, ncon

    @staticmethod
    def backward(ctx, d_out, _dT, _dn):
        if d_out is None:
            return (None,) * 10
        records, ids, tile_range, final_T, ncon = ctx.saved_tensors
        n, C, bg, W, H, has_ndc = ctx.cfg
        d_uv, d_conic, d_op, d_feat = _blend_backward_raw(records, ids, tile_range, final_T, ncon,
                                                          d_out, n, C, bg, W, H)
        d_ndc = d_uv.clone() if has_ndc else None
        return d_uv, d_conic, d_op, d_feat, None, None, None, None, None, d_ndc


class _AlphaBlendingPieces(torch.autograd.Function):
    """alpha_blending over the concatenation of [N,w] feature pieces, which
    is never built; each piece gets its own gradient tensor."""

    @staticmethod
    def forward(ctx, uv, conic, opacity, ids, tile_range, bg, W, H, ndc, *pieces):
        n = uv.shape[0]
        widths = [t.shape[1] for t in pieces]
        records, out, final_T, ncon = _blend_forward_raw(uv, conic, opacity, pieces, ids,
                                                         tile_range, bg, W, H)
        ctx.save_for_backward(records, ids, tile_range, final_T, ncon)
        ctx.cfg = (n, sum(widths), widths, float(bg), W, H, ndc is not None)
        ctx.mark_non_differentiable(final_T, ncon)
        ctx.set_materialize_grads(False)  # no zero images for final_T / ncon
        return out, final_T, ncon

    @staticmethod
    def backward(ctx, d_out, _dT, _dn):
        if d_out is None:
            return (None,) * (9 + len(ctx.cfg[2]))
        records, ids, tile_range, final_T, ncon = ctx.saved_tensors
        n, C, widths, bg, W, H, has_ndc = ctx.cfg
        d_uv, d_conic, d_op, d_feat = _blend_backward_raw(records, ids, tile_range, final_T, ncon,
                                                          d_out, n, C, bg, W, H, widths)
        d_ndc = d_uv.clone() if has_ndc else None
        return (d_uv, d_conic, d_op, None, None, None, None, None, d_ndc, *d_feat)


# target entries per band of the recompute mode: ids and sort scratch of
# about 0.7 GB
BAND_ENTRIES = 1 << 25


def band_rows(K: int, H: int, bands=None, max_entries: int = BAND_ENTRIES):
    """Equal-height tile-row bands [(row0, row1), ...] covering an image of
    height H: the given number of bands, or enough that a band holds about
    ``max_entries`` of the image's K entries if they were spread evenly."""
    gy = (int(H) + TILE - 1) // TILE
    nb = int(bands) if bands else -(-int(K) // int(max_entries))
    nb = max(1, min(gy, nb))
    rows = -(-gy // nb)
    return [(r0, min(gy, r0 + rows)) for r0 in range(0, gy, rows)]


def group_rows(row_k, bands=None, max_entries: int = BAND_ENTRIES):
    """Bands from the entries of each tile row (``row_k``): consecutive rows
    grouped front to back, a new band starting when the next row would take
    the band past the target -- ``max_entries``, or K / ``bands`` when a
    band count is given.  Returns [(row0, row1, K of the band), ...]."""
    K = int(sum(row_k))
    gy = len(row_k)
    target = max(1, -(-K // max(1, int(bands)))) if bands else int(max_entries)
    out, r0, acc = [], 0, 0
    for r, k in enumerate(row_k):
        k = int(k)
        if r > r0 and acc + k > target and (not bands or len(out) < int(bands) - 1):
            out.append((r0, r, acc))
            r0, acc = r, 0
        acc += k
    out.append((r0, gy, acc))
    return out


# bands up to which a banded sort builds per-band Gaussian lists (the
# library's limit for pgb_band_lists_*); more bands take the whole-order path
BAND_LIST_MAX = 256
# the band plan [(row0, row1, entries), ...] of the latest banded call (for
# measurements)
last_band_plan: list = []


class _BandSort:
    """The depth sort of one image done once, then phase two of the sort for
    one band of tile rows at a time (``pgb_sort_gaussian_rebegin`` /
    ``pgb_sort_gaussian_finish_band``).  The entries of every tile row are
    counted in one pass and read back once; the bands group rows up to the
    target, and one set of K-sized buffers, sized for the largest band, is
    reused by every band."""

    def __init__(self, uv, depth, W, H, radius, tiles, bands=None,
                 max_entries: int = BAND_ENTRIES):
        self.h = h = sort_gaussian_begin(uv, depth, W, H, radius, tiles, read_count=False)
        dev, n = h.dev, h.n
        gy = (int(H) + TILE - 1) // TILE
        rows = torch.arange(gy + 1, dtype=torch.int32, device=dev)
        row_k = torch.empty(gy, dtype=torch.int64, device=dev)
        call("pgb_band_counts", _ptr(h.uv), _ptr(h.radius), n, h.W, h.H, _ptr(rows), gy,
             _ptr(row_k), h.stream.cuda_stream)
        row_k = row_k.tolist()                      # the first synchronisation
        self.K = int(sum(row_k))
        self.plan = group_rows(row_k, bands, max_entries)
        kmax = max(k for _, _, k in self.plan)
        _, self.bk = _sort_scratch(n, kmax, h.W, h.H)
        self.scratch_k = torch.empty(max(self.bk, 1), dtype=torch.uint8, device=dev)
        self.ids = torch.empty(max(kmax, 1), dtype=torch.int32, device=dev)
        self.lists = self.list_off = self.tiles_b = None
        nb = len(self.plan)
        if n and nb <= BAND_LIST_MAX:
            # every band's Gaussians in depth order, so that a band's phase
            # two visits only its own (one pass over the depth order, and the
            # lists' total read back: the second synchronisation)
            rows_b = torch.tensor([r0 for r0, _, _ in self.plan] + [self.plan[-1][1]],
                                  dtype=torch.int32).to(dev)
            sb = int(_lib.lib().pgb_band_lists_scratch_bytes(n, nb))
            scratch = torch.empty(max(sb, 1), dtype=torch.uint8, device=dev)
            offsets = torch.empty(nb + 1, dtype=torch.int64, device=dev)
            s = h.stream.cuda_stream
            args = (_ptr(h.uv), _ptr(h.radius), n, h.W, h.H, _ptr(rows_b), nb, _ptr(h.scratch_n),
                    h.bn, _ptr(scratch), sb, _ptr(offsets))
            call("pgb_band_lists_count", *args, s)
            self.list_off = offsets.tolist()
            self.lists = torch.empty(max(self.list_off[-1], 1), dtype=torch.int32, device=dev)
            call("pgb_band_lists_write", *args, _ptr(self.lists), s)
        else:
            self.tiles_b = torch.empty_like(h.tiles)

    def band(self, i):
        """(ids [K_b] -- a view of the shared buffer --, tile_range
        [gx * rows, 2]) of band i."""
        h = self.h
        r0, r1, k = self.plan[i]
        dev, n, W, H = h.dev, h.n, h.W, h.H
        gx = (W + TILE - 1) // TILE
        s = h.stream.cuda_stream
        ids = self.ids[:k]
        rng = torch.empty(gx * (r1 - r0), 2, dtype=torch.int32, device=dev)
        launches = (3 + _tile_passes(rng.shape[0])) if (k and n) else 0
        if self.lists is not None:
            a, b = self.list_off[i], self.list_off[i + 1]
            with _timed("sort_finish", dev, launches):
                call("pgb_sort_gaussian_finish_band_list", _ptr(h.uv), _ptr(h.radius), n, W, H,
                     r0, r1, k, self.lists.data_ptr() + 4 * a if b > a else None, b - a,
                     _ptr(h.scratch_n), h.bn, _ptr(self.scratch_k), self.bk, _ptr(h.info),
                     _ptr(ids) if k else None, _ptr(rng), s)
        else:
            call("pgb_band_tiles", _ptr(h.uv), _ptr(h.radius), n, W, H, r0, r1,
                 _ptr(self.tiles_b), s)
            call("pgb_sort_gaussian_rebegin", _ptr(h.radius), _ptr(self.tiles_b), n,
                 _ptr(h.scratch_n), h.bn, _ptr(h.info), s)
            with _timed("sort_finish", dev, launches):
                call("pgb_sort_gaussian_finish_band", _ptr(h.uv), _ptr(h.radius),
                     _ptr(self.tiles_b), n, W, H, r0, r1, k, _ptr(h.scratch_n), h.bn,
                     _ptr(self.scratch_k), self.bk, _ptr(h.info), _ptr(ids) if k else None,
                     _ptr(rng), s)
        _defer_check(h.info[1:], "sort_gaussian (band tile passes)")
        return ids, rng


def _blend_band_forward(uv, conic, opacity, feature, ids, rng, bg, W, H, r0, r1, pack, records,
                        out, final_T, ncon):
    n, C = feature.shape
    dev = feature.device
    status = _status_word(dev)

    def run(batch):
        call("pgb_alpha_blending_forward_band", _ptr(uv), _ptr(conic), _ptr(opacity),
             _ptr(feature), n, C, _ptr(ids), ids.numel(), _ptr(rng), float(bg), W, H, r0, r1,
             1 if pack else 0, _ptr(records), _ptr(out), _ptr(final_T), _ptr(ncon),
             _ptr(status), _stream(dev), batch)

    key = autotune.workload_class("blend_fwd", C, W * (r1 - r0) * TILE, ids.numel(),
                                  rng.shape[0])
    batch = autotune.choose(key, _blend_batches(0), run, dev) if n else 0
    with _timed("alpha_blending_fwd", dev, 2 if (pack and n) else 1):
        run(batch)


def _rasterize_banded_forward(uv, conic, opacity, feature, depth, radius, tiles, bg, W, H, bands,
                              backward=None):
    """Sort and blend one band of tile rows at a time.  ``backward`` =
    (d_out, grad outputs...) runs each band's blend backward right after the
    band's forward, while its lists are alive."""
    n, C = feature.shape
    dev = feature.device
    bs = _BandSort(uv, depth, W, H, radius, tiles, bands)
    plan = bs.plan
    last_band_plan[:] = plan
    rf = _lib.lib().pgb_blend_record_floats(C)
    records = torch.empty(n, rf, dtype=torch.float32, device=dev)
    out = torch.empty(C, H, W, dtype=torch.float32, device=dev)
    final_T = torch.empty(H, W, dtype=torch.float32, device=dev)
    ncon = torch.empty(H, W, dtype=torch.int32, device=dev)
    for i, (r0, r1, _) in enumerate(plan):
        ids, rng = bs.band(i)
        _blend_band_forward(uv, conic, opacity, feature, ids, rng, bg, W, H, r0, r1, i == 0,
                            records, out, final_T, ncon)
        if backward is not None:
            backward(records, ids, rng, final_T, ncon, r0, r1, i == 0, i == len(plan) - 1)
        del ids, rng
    return out, len(plan)


class _RasterizeRecompute(torch.autograd.Function):
    """Sort + blend whose backward recomputes the tile lists, the records and
    the per-pixel final transmittance / last-contributor counts instead of
    keeping them alive between forward and backward.  Both directions work
    one band of tile rows at a time (``band_rows``), so the K-sized sort
    buffers and id list hold one band's entries."""

    @staticmethod
    def forward(ctx, uv, conic, opacity, feature, depth, radius, tiles, bg, W, H, ndc, bands):
        out, _ = _rasterize_banded_forward(uv, conic, opacity, feature, depth, radius, tiles, bg,
                                           W, H, bands)
        ctx.save_for_backward(uv, conic, opacity, feature, depth, radius, tiles)
        ctx.cfg = (float(bg), W, H, ndc is not None, bands)
        return out

    @staticmethod
    def backward(ctx, d_out):
        uv, conic, opacity, feature, depth, radius, tiles = ctx.saved_tensors
        bg, W, H, has_ndc, bands = ctx.cfg
        n, C = feature.shape
        dev = feature.device
        d_out = _c(d_out)
        grec = torch.empty(n, _lib.lib().pgb_blend_grad_record_floats(C), dtype=torch.float32,
                           device=dev)
        d_uv = torch.empty(n, 2, dtype=torch.float32, device=dev)
        d_conic = torch.empty(n, 3, dtype=torch.float32, device=dev)
        d_op = torch.empty(n, dtype=torch.float32, device=dev)
        d_feat = torch.empty(n, C, dtype=torch.float32, device=dev)
        status = _status_word(dev)

        def band_backward(records, ids, rng, final_T, ncon, r0, r1, first, last):
            def run(batch, first=first, last=last):
                call("pgb_alpha_blending_backward_band", _ptr(records), n, C, _ptr(ids),
                     ids.numel(), _ptr(rng), bg, W, H, r0, r1, _ptr(final_T), _ptr(ncon),
                     _ptr(d_out), _ptr(grec), 1 if first else 0, 1 if last else 0, _ptr(d_uv),
                     _ptr(d_conic), _ptr(d_op), _ptr(d_feat), _ptr(status), _stream(dev), batch)
            key = autotune.workload_class("blend_bwd", C, W * (r1 - r0) * TILE, ids.numel(),
                                          rng.shape[0])
            if key not in autotune.table() and autotune._enabled and not _capturing():
                # timing runs add into the records: time them on a scratch copy
                saved = grec.clone() if not first else None
                batch = autotune.choose(key, _blend_batches(1),
                                        lambda b: run(b, first=True, last=False), dev)
                if saved is not None:
                    grec.copy_(saved)
            else:
                batch = autotune.choose(key, _blend_batches(1), run, dev)
            with _timed("alpha_blending_bwd", dev, 2 if last else 1):
                run(batch)

        _rasterize_banded_forward(uv, conic, opacity, feature, depth, radius, tiles, bg, W, H,
                                  bands, backward=band_backward)
        d_ndc = d_uv.clone() if has_ndc else None
        return d_uv, d_conic, d_op, d_feat, None, None, None, None, None, None, d_ndc, None


def rasterize(uv, conic, opacity, feature, depth, radius, tiles_touched, bg, W, H, ndc=None,
              recompute=False, capacity=None, bands=None):
    """``sort_gaussian`` followed by ``alpha_blending`` -> [C,H,W].
    ``feature`` is [N,C] or a list of [N,w] pieces (blended as their
    concatenation, without building it).

    With ``recompute=False`` this is exactly the two operators.  With
    ``recompute=True`` the backward re-runs the sort and the blend forward
    instead of keeping the tile lists, records and per-pixel state alive from
    the forward: less memory held between forward and backward (what limits
    4K views of millions of Gaussians), one more sort and blend forward per
    step.  Gradients are the same in both modes.  The recompute mode also
    sorts and blends one band of tile rows at a time, in both directions
    (``bands`` of them, or as many as keep a band near ``BAND_ENTRIES``
    entries), so the K-sized sort buffers and id list -- the peak of a large
    view -- hold one band's entries.  ``capacity`` is passed to
    :func:`sort_gaussian` in the stored mode (K kept on the device, no
    synchronisation); the recompute mode reads each band's K back."""
    if not recompute:
        ids, rng = sort_gaussian(uv, depth, W, H, radius, tiles_touched, capacity=capacity)
        if isinstance(feature, (list, tuple)):
            return alpha_blending_pieces(uv, conic, opacity, feature, ids, rng, bg, W, H, ndc)
        return alpha_blending(uv, conic, opacity, feature, ids, rng, bg, W, H, ndc)
    if isinstance(feature, (list, tuple)):
        feature = torch.cat(list(feature), dim=-1)
    _need(feature, "feature", ndim=2)
    n, C = feature.shape
    if C < 1 or C > 26:
        raise ValueError(f"rasterize supports 1..26 feature channels, got {C}")
    if isinstance(bg, torch.Tensor):
        bg = float(bg)
    return _RasterizeRecompute.apply(_c(uv), _c(conic), _c(opacity.reshape(n)), _c(feature),
                                     depth, radius, tiles_touched, bg, int(W), int(H), ndc,
                                     bands)


def alpha_blending_with_state(uv, conic, opacity, feature, gaussian_ids_sorted, tile_range, bg, W, H,
                              ndc=None):
    """As :func:`alpha_blending`, also returning the final transmittance
    [H,W] and the per-pixel count of list entries up to the last
    contributor [H,W] (what the backward replays from)."""
    _need(uv, "uv", ndim=2, last=2)
    _need(conic, "conic", ndim=2, last=3)
    _need(opacity, "opacity")
    _need(feature, "feature", ndim=2)
    _need(gaussian_ids_sorted, "gaussian_ids_sorted", dtype=torch.int32)
    _need(tile_range, "tile_range", dtype=torch.int32, ndim=2, last=2)
    n, C = feature.shape
    if C < 1 or C > 26:
        raise ValueError(f"alpha_blending supports 1..26 feature channels, got {C}")
    if uv.shape[0] != n or conic.shape[0] != n or opacity.numel() != n:
        raise ValueError("alpha_blending: uv, conic, opacity and feature disagree on N")
    W, H = int(W), int(H)
    T = ((W + TILE - 1) // TILE) * ((H + TILE - 1) // TILE)
    if tile_range.shape[0] != T:
        raise ValueError(f"tile_range has {tile_range.shape[0]} rows, the {W}x{H} image has {T} tiles")
    if isinstance(bg, torch.Tensor):
        bg = float(bg)
    if ndc is not None and tuple(ndc.shape) != (n, 2):
        raise ValueError(f"ndc must be [N,2], got {tuple(ndc.shape)}")
    return _AlphaBlending.apply(_c(uv), _c(conic), _c(opacity.reshape(n)), _c(feature),
                                _c(gaussian_ids_sorted), _c(tile_range), bg, W, H, ndc)


def alpha_blending_pieces(uv, conic, opacity, pieces, gaussian_ids_sorted, tile_range, bg, W, H,
                          ndc=None):
    """:func:`alpha_blending` of ``torch.cat(pieces, 1)`` without building
    the concatenation: ``pieces`` are [N,w] feature tensors (at most 26
    channels in all), each receiving its own gradient."""
    pieces = [t if t.dim() == 2 else t.reshape(t.shape[0], -1) for t in pieces]
    if not pieces:
        raise ValueError("alpha_blending_pieces needs at least one feature piece")
    n = uv.shape[0]
    for t in pieces:
        if not (t.is_cuda and t.dtype == torch.float32) or t.shape[0] != n or t.shape[1] < 1:
            raise ValueError(f"feature pieces must be CUDA float32 [N,w], got {tuple(t.shape)}")
    C = sum(t.shape[1] for t in pieces)
    if C > 26:
        raise ValueError(f"alpha_blending supports 1..26 feature channels, got {C}")
    _need(uv, "uv", ndim=2, last=2)
    _need(conic, "conic", ndim=2, last=3)
    _need(opacity, "opacity")
    _need(gaussian_ids_sorted, "gaussian_ids_sorted", dtype=torch.int32)
    _need(tile_range, "tile_range", dtype=torch.int32, ndim=2, last=2)
    if conic.shape[0] != n or opacity.numel() != n:
        raise ValueError("alpha_blending: uv, conic, opacity and feature disagree on N")
    W, H = int(W), int(H)
    T = ((W + TILE - 1) // TILE) * ((H + TILE - 1) // TILE)
    if tile_range.shape[0] != T:
        raise ValueError(f"tile_range has {tile_range.shape[0]} rows, the {W}x{H} image has {T} tiles")
    if isinstance(bg, torch.Tensor):
        bg = float(bg)
    if ndc is not None and tuple(ndc.shape) != (n, 2):
        raise ValueError(f"ndc must be [N,2], got {tuple(ndc.shape)}")
    return _AlphaBlendingPieces.apply(_c(uv), _c(conic), _c(opacity.reshape(n)),
                                      _c(gaussian_ids_sorted), _c(tile_range), bg, W, H, ndc,
                                      *[t.contiguous() for t in pieces])[0]


def alpha_blending(uv, conic, opacity, feature, gaussian_ids_sorted, tile_range, bg, W, H, ndc=None):
    """Front-to-back alpha compositing of ``feature`` [N,C] per 16x16 tile ->
    [C,H,W], plus ``bg`` times the final transmittance in every channel.

    Differentiable in uv, conic, opacity and feature; ``ndc`` ([N,2], the
    zero leaf that ``msplat.py:141-145`` creates) receives d(loss)/d(uv) in
    pixel units, which the densification controller reads as ``ndc.grad``.
    """
    return alpha_blending_with_state(uv, conic, opacity, feature, gaussian_ids_sorted, tile_range,
                                     bg, W, H, ndc)[0]


def blend_pair_census(uv, conic, opacity, feature, gaussian_ids_sorted, tile_range, W, H):
    """(evaluated, composited): the (pixel, splat) pairs of this blend up to
    each pixel's last contributor, and the composited ones among them
    (``pgb_blend_pair_census``).  A measurement aid for the benchmark's
    roofline: runs one forward to get the records and contributor counts."""
    ids = _c(gaussian_ids_sorted.to(torch.int32))
    rng = _c(tile_range.to(torch.int32))
    with torch.no_grad():
        records, _, _, ncon = _blend_forward_raw(uv.detach(), conic.detach(), opacity.detach(),
                                                 feature.detach(), ids, rng, 0.0, W, H)
    counts = torch.zeros(2, dtype=torch.int64, device=records.device)
    call("pgb_blend_pair_census", _ptr(records), int(feature.shape[1]), int(records.shape[0]),
         _ptr(ids), int(ids.numel()), _ptr(rng), int(W), int(H), _ptr(ncon), _ptr(counts),
         _stream(records.device))
    c = counts.tolist()
    return int(c[0]), int(c[1])
